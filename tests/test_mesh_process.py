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
