"""GPU evaluation kernels against NumPy brute force, and the command line end to end."""

import os
import subprocess
import sys

import numpy as np
import pytest

from pamo_gb300 import mesh_io, metrics
from tests import meshes

pytestmark = pytest.mark.gpu


def _point_tri_sqdist(P, A, B, C):
    n = np.cross(B - A, C - A)
    nn = n / np.linalg.norm(n)
    h = (P - A) @ nn
    foot = P - h[:, None] * nn
    inside = np.ones(len(P), bool)
    for u, v in ((A, B), (B, C), (C, A)):
        inside &= (np.cross(v - u, foot - u) @ n) >= 0
    best = np.where(inside, h * h, np.inf)
    for u, v in ((A, B), (B, C), (C, A)):
        t = np.clip(((P - u) @ (v - u)) / ((v - u) @ (v - u)), 0, 1)
        best = np.minimum(best, np.sum((P - (u + t[:, None] * (v - u))) ** 2, axis=1))
    return best


def test_point_mesh_sqdist_matches_brute_force():
    V, F = meshes.tangled(n=7, seed=4)
    V = V.astype(np.float64)
    rng = np.random.default_rng(0)
    P = np.vstack([rng.normal(0, 1.5, (400, 3)), V[:50] + 1e-9, metrics.sample_surface(V, F, 100, seed=3)])
    d2, fi = metrics.point_mesh_sqdist(P, V, F)
    want = np.full(len(P), np.inf)
    for f in F:
        want = np.minimum(want, _point_tri_sqdist(P, V[f[0]], V[f[1]], V[f[2]]))
    assert np.allclose(d2, want, rtol=1e-9, atol=1e-20)
    # the reported face attains the distance
    for i in range(0, len(P), 37):
        f = F[fi[i]]
        assert _point_tri_sqdist(P[i:i + 1], V[f[0]], V[f[1]], V[f[2]])[0] == pytest.approx(d2[i], rel=1e-9, abs=1e-20)


def test_face_min_angles_match_the_reference_formulas():
    V, F = meshes.with_degenerate_face()
    V = V.astype(np.float64)
    edge_form, igl_form = metrics.face_min_angles(V, F)
    mask = (F[:, 0] != F[:, 1]) & (F[:, 1] != F[:, 2]) & (F[:, 2] != F[:, 0])
    assert np.isnan(edge_form[~mask]).all() and np.isnan(igl_form[~mask]).all()
    Fm = F[mask]
    e = np.stack([V[Fm[:, 0]] - V[Fm[:, 1]], V[Fm[:, 1]] - V[Fm[:, 2]], V[Fm[:, 2]] - V[Fm[:, 0]]], 1)
    L = np.linalg.norm(e, axis=-1)
    cos = -np.sum(e * np.roll(e, 1, axis=1), axis=-1) / (L * np.roll(L, 1, axis=1))
    want = np.arccos(np.clip(cos, -1, 1)).min(axis=1)
    assert np.allclose(edge_form[mask], want, rtol=0, atol=1e-12)
    assert np.allclose(igl_form[mask], want, rtol=0, atol=1e-9)
    assert metrics.compute_min_angle_VF(V, F) == pytest.approx(want.min(), abs=1e-12)


def test_command_line_end_to_end(tmp_path):
    V, F = meshes.sphere(16)
    src, dst = tmp_path / "in.obj", tmp_path / "out.obj"
    mesh_io.save_obj(str(src), V, F)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-m", "pamo_gb300", "-i", str(src), "-o", str(dst), "-r", "0.1",
                        "--disable_stage1", "--metrics"], capture_output=True, text=True, cwd=root, timeout=600)
    assert r.returncode == 0, r.stderr
    V2, F2 = mesh_io.load_obj(str(dst))
    assert 0 < len(F2) <= 0.1 * len(F) + 2
    assert "Chamfer distance" in r.stdout and "Faces in self-intersecting pairs: 0" in r.stdout
