"""The restatement of trimesh's default processing of the stage-2 output (``safe_project.mesh_process``) on CPU:
faces on non-finite vertices dropped, vertices equal after rounding to 8 decimals merged, unreferenced vertices
dropped, survivors in order of first occurrence."""

import numpy as np

from tests import meshes


def test_clean_mesh_is_unchanged():
    from pamo_gb300.safe_project import mesh_process

    V, F = meshes.octahedron()
    V2, F2 = mesh_process(V, F)
    assert V2.dtype == np.float64 and F2.dtype == np.int64
    assert np.array_equal(V2, V.astype(np.float64)) and np.array_equal(F2, F)


def test_duplicates_merge_in_first_occurrence_order():
    from pamo_gb300.safe_project import mesh_process

    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1.000000000001, 0, 0], [5, 5, 5], [0, 0, 1]], np.float64)
    F = np.array([[0, 1, 2], [0, 3, 5], [3, 2, 5]], np.int32)  # vertex 3 duplicates 1, vertex 4 is unreferenced
    V2, F2 = mesh_process(V, F)
    assert np.array_equal(V2, V[[0, 1, 2, 5]])
    assert np.array_equal(F2, [[0, 1, 2], [0, 1, 3], [1, 2, 3]])


def test_faces_on_non_finite_vertices_are_dropped():
    from pamo_gb300.safe_project import mesh_process

    V = np.array([[0, 0, 0], [1, 0, 0], [np.nan, 0, 0], [0, 1, 0], [0, 0, 1]], np.float64)
    F = np.array([[0, 1, 3], [0, 2, 3], [1, 3, 4]], np.int64)
    V2, F2 = mesh_process(V, F)
    assert np.isfinite(V2).all()
    assert np.array_equal(V2, V[[0, 1, 3, 4]])
    assert np.array_equal(F2, [[0, 1, 2], [1, 2, 3]])


def test_empty_inputs_pass_through():
    from pamo_gb300.safe_project import mesh_process

    V2, F2 = mesh_process(np.zeros((0, 3)), np.zeros((0, 3), np.int64))
    assert V2.shape == (0, 3) and F2.shape == (0, 3)


def _native_process(lib, V, F):
    import ctypes

    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    Vo = np.zeros_like(V)
    Fo = np.zeros_like(F)
    nv, nf = ctypes.c_int32(0), ctypes.c_int32(0)
    st = lib.pamo_mesh_process(V.ctypes.data, len(V), F.ctypes.data, len(F), Vo.ctypes.data, ctypes.byref(nv),
                               Fo.ctypes.data, ctypes.byref(nf))
    return st, Vo[: nv.value], Fo[: nf.value]


def test_server_processing_equals_the_python_restatement(native_lib):
    """pamo_mesh_process (the C++ processing the server applies to each stage-2 result before stage 3) gives
    safe_project.mesh_process's vertices and faces, bit for bit, on meshes with near-duplicate vertices (inside and
    just outside the 1e-8 rounding), unreferenced and non-finite vertices."""
    from pamo_gb300.safe_project import mesh_process

    rng = np.random.default_rng(5)
    for trial in range(40):
        n = int(rng.integers(4, 300))
        V = rng.normal(size=(n, 3))
        dup = rng.integers(0, n, n // 3)
        V = np.concatenate([V, V[dup] + rng.choice([0.0, 2e-9, -4e-9, 3e-8], size=(len(dup), 1))])
        if trial % 3 == 0:
            V[rng.integers(0, len(V), 2)] = np.nan
        if trial % 5 == 0:
            V[rng.integers(0, len(V))] = np.inf
        F = rng.integers(0, len(V), size=(int(rng.integers(1, 2 * n)), 3)).astype(np.int32)
        st, Vn, Fn = _native_process(native_lib, V, F)
        assert st == 0
        Vp, Fp = mesh_process(V, F)
        assert np.array_equal(Vn, Vp), trial
        assert np.array_equal(Fn, Fp), trial


def test_server_processing_rejects_bad_indices(native_lib):
    V, F = meshes.octahedron()
    F = F.copy()
    F[0, 0] = len(V)
    st, _, _ = _native_process(native_lib, V, F)
    assert st != 0
