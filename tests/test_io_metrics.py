"""OBJ reading/writing and the host parts of the evaluation metrics (pamo_gb300.mesh_io, pamo_gb300.metrics)."""

import numpy as np
import pytest

from pamo_gb300 import mesh_io, metrics
from tests import meshes


def test_obj_round_trip(tmp_path):
    V, F = meshes.sphere(6)
    p = tmp_path / "m.obj"
    mesh_io.save_obj(str(p), V, F)
    V2, F2 = mesh_io.load_obj(str(p))
    assert np.array_equal(V2, V.astype(np.float64)) and np.array_equal(F2, F)


def test_obj_polygons_and_index_forms(tmp_path):
    p = tmp_path / "q.obj"
    p.write_text("# quad and a triangle\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\n"
                 "f 1/1 2/1 3/1 4/1\nf -4//1 -2//1 -1//1\n")
    V, F = mesh_io.load_obj(str(p))
    assert V.shape == (4, 3)
    assert F.tolist() == [[0, 1, 2], [0, 2, 3], [0, 2, 3]]


def test_obj_bad_index(tmp_path):
    p = tmp_path / "b.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nf 1 2 3\n")
    with pytest.raises(ValueError):
        mesh_io.load_obj(str(p))


def test_sample_surface_points_lie_on_their_faces():
    V, F = meshes.sphere(5)
    V = V.astype(np.float64)
    s1 = metrics.sample_surface(V, F, 2000, seed=42)
    s2 = metrics.sample_surface(V, F, 2000, seed=42)
    assert np.array_equal(s1, s2)
    # every sample is within rounding of some triangle's plane and inside it (barycentric test, brute force)
    A, B, C = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    n = np.cross(B - A, C - A)
    for p in s1[:200]:
        d = np.abs(np.einsum("ij,ij->i", p - A, n)) / np.linalg.norm(n, axis=1)
        k = np.argmin(d)
        assert d[k] < 1e-12
        w = np.linalg.lstsq(np.stack([B[k] - A[k], C[k] - A[k]], 1), p - A[k], rcond=None)[0]
        assert w.min() > -1e-9 and w.sum() < 1 + 1e-9


def test_sample_surface_is_area_weighted():
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [10, 0, 0], [13, 0, 0], [10, 3, 0]], np.float64)
    F = np.array([[0, 1, 2], [3, 4, 5]])  # areas 0.5 and 4.5
    s = metrics.sample_surface(V, F, 20000, seed=1)
    frac_big = np.mean(s[:, 0] >= 10)
    assert abs(frac_big - 0.9) < 0.01
