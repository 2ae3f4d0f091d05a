"""The topology a stage-3 call builds on the host (pamo_stage3_topology, no GPU) against brute-force restatements:
trimesh's edges_unique (rows with sorted endpoints, grouped by the hash u ^ (v << 32) that trimesh uses for two
integer columns, in ascending hash order) and hinge_preprocess_slow_kernel (safe_project/.../hinge_energy.py:21-57:
every directed edge (a, b), a < b, of a face t0 paired with every face t1 holding (b, a), in face and corner order)."""

import ctypes

import numpy as np

from tests import meshes


def _native(lib, F, n_points, hinge_capacity=None):
    F = np.ascontiguousarray(F, np.int32)
    cap = 9 * len(F) * len(F) if hinge_capacity is None else hinge_capacity
    E = np.zeros((3 * len(F), 2), np.int32)
    H = np.zeros((max(cap, 1), 4), np.int32)
    ne, nh = ctypes.c_int32(0), ctypes.c_int32(0)
    st = lib.pamo_stage3_topology(F.ctypes.data, n_points, len(F), E.ctypes.data, ctypes.byref(ne), H.ctypes.data, cap,
                                  ctypes.byref(nh))
    return st, E[: ne.value], H[: min(nh.value, cap)], nh.value


def _edges_unique(F):
    rows = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1).astype(np.int64)
    h = rows[:, 0] ^ (rows[:, 1] << 32)
    _, first = np.unique(h, return_index=True)
    return rows[first]


def _hinges(F):
    out = []
    for t0 in F:
        for k in range(3):
            a, b, c = int(t0[k]), int(t0[(k + 1) % 3]), int(t0[(k + 2) % 3])
            if not a < b:
                continue
            for t1 in F:
                for k1 in range(3):
                    if int(t1[k1]) == b and int(t1[(k1 + 1) % 3]) == a:
                        out.append((c, a, b, int(t1[(k1 + 2) % 3])))
    return np.array(out, np.int64).reshape(-1, 4)


def _cases():
    V, F = meshes.octahedron()
    yield len(V), F
    V, F = meshes.sphere(3)
    yield len(V), F
    V, F = meshes.open_patch()
    yield len(V), F
    V, F = meshes.sheet_pair(n=4)
    yield len(V), F
    rng = np.random.default_rng(8)
    for _ in range(6):  # triangle soups on few vertices: non-manifold edges with several hinges each
        n = int(rng.integers(4, 9))
        F = np.array([rng.choice(n, 3, replace=False) for _ in range(int(rng.integers(2, 30)))], np.int32)
        yield n, F


def test_edges_and_hinges_match_the_restatements(native_lib):
    for n, F in _cases():
        st, E, H, nh = _native(native_lib, F, n)
        assert st == 0
        assert np.array_equal(E, _edges_unique(np.asarray(F))), F
        ref = _hinges(np.asarray(F))
        assert nh == len(ref)
        assert np.array_equal(H, ref), F


def test_closed_mesh_counts(native_lib):
    """Closed orientable mesh: E = 3F/2 and one hinge per edge."""
    V, F = meshes.sphere(4)
    st, E, H, nh = _native(native_lib, F, len(V))
    assert st == 0 and len(E) == 3 * len(F) // 2 and nh == len(E)


def test_capacity_and_bad_index(native_lib):
    V, F = meshes.octahedron()
    st, _, _, nh = _native(native_lib, F, len(V), hinge_capacity=3)
    assert st != 0 and nh == 12  # full count reported
    F = np.asarray(F).copy()
    F[2, 1] = -1
    st, _, _, _ = _native(native_lib, F, len(V))
    assert st != 0
