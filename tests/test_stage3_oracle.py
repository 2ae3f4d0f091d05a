"""The float64 stage-3 oracle (oracle/stage3_oracle.cpp) against the mathematics it restates.

The reference's stage 3 needs a fork of Warp that is not available, so its outputs cannot be used as golden
data (parity unpinned). These tests pin the restatement instead: every energy's gradient equals a central
finite difference of that energy, the topology counts follow from the mesh, and the do-nothing rule and
the projection itself behave as the reference's processing.py describes.
"""

import numpy as np
import pytest

from oracle import oracle as orc
from tests import meshes

ONLY = {
    "distance": dict(elas_young_modulus=0, hinge_stiffness=0, coll_stiffness=0),
    "elastic": dict(mesh2gt_dist_stiffness=0, hinge_stiffness=0, coll_stiffness=0),
    "hinge": dict(mesh2gt_dist_stiffness=0, elas_young_modulus=0, coll_stiffness=0),
    "contact": dict(mesh2gt_dist_stiffness=0, elas_young_modulus=0, hinge_stiffness=0),
}


@pytest.mark.parametrize("energy", sorted(ONLY))
def test_gradient_matches_finite_differences(energy):
    V, F = meshes.sheet_pair()
    rng = np.random.default_rng(2)
    q0 = orc.stage3_probe(V, F, V, F, np.zeros_like(V))["q"]
    x0 = q0 + rng.normal(0, 2e-3, V.shape)  # off the rest shape; the sheets stay apart
    dx = rng.normal(0, 1, V.shape)
    prm = ONLY[energy]
    pr = orc.stage3_probe(V, F, V, F, dx, prm, x0=x0)
    assert pr["n_contacts"] > 100
    h = 1e-9 if energy == "contact" else 1e-7  # the barrier is steep near d -> 0
    ep = orc.stage3_energy_at(V, F, V, F, x0 + h * dx, prm, x0=x0)
    em = orc.stage3_energy_at(V, F, V, F, x0 - h * dx, prm, x0=x0)
    fd = (ep - em) / (2 * h)
    an = float((pr["grad"] * dx).sum())
    assert abs(fd - an) <= 1e-5 * abs(an) + 1e-12


def test_elastic_hessian_product_at_rest_matches_finite_differences():
    # At the rest shape the StVK stress vanishes and the reference's Hessian product (fixed local basis) is
    # the exact second derivative.
    V, F = meshes.sheet_pair()
    rng = np.random.default_rng(4)
    dx = rng.normal(0, 1, V.shape)
    prm = ONLY["elastic"]
    q0 = orc.stage3_probe(V, F, V, F, dx, prm)
    h = 1e-6
    gp = orc.stage3_probe(V, F, V, F, dx, prm, x0=q0["q"] + h * dx)["grad"]
    gm = orc.stage3_probe(V, F, V, F, dx, prm, x0=q0["q"] - h * dx)["grad"]
    hfd = (gp - gm) / (2 * h)
    assert np.linalg.norm(hfd - q0["hvp"]) <= 1e-6 * np.linalg.norm(hfd)


def test_topology_counts():
    GV, GF, V, F = meshes.stage3_pair()
    out, st = orc.stage3_run(GV, GF, V, F, 0)
    # closed genus-0 triangle mesh: E = 3F/2, one hinge per edge, V - E + F = 2
    assert st["edges"] == 3 * len(F) // 2
    assert st["hinges"] == st["edges"]
    assert len(V) - st["edges"] + len(F) == 2
    # zero steps: only the normalisation round trip
    assert np.allclose(out, V, rtol=0, atol=1e-12)
    V2, F2 = meshes.sheet_pair()
    _, st2 = orc.stage3_run(V2, F2, V2, F2, 0)
    n = 8
    assert st2["edges"] == 2 * (2 * n * (n - 1) + (n - 1) ** 2)
    assert st2["hinges"] == 2 * (2 * (n - 1) * (n - 2) + (n - 1) ** 2)


def test_projection_moves_vertices_onto_gt():
    GV, GF, V, F = meshes.stage3_pair()
    out, st = orc.stage3_run(GV, GF, V, F, 2)
    assert st["steps"] == 2 and not st["do_nothing"]
    r_gt = np.linalg.norm(GV, axis=1).mean()
    # the coarse mesh was inflated by 2 %: after projection its radius is back at the GT's
    before = abs(np.linalg.norm(V, axis=1).mean() / r_gt - 1)
    after = abs(np.linalg.norm(out, axis=1).mean() / r_gt - 1)
    assert before > 0.015 and after < 0.25 * before


def _octahedron_with(extra_faces):
    GV, GF = meshes.octahedron()
    GV = GV.astype(np.float64)
    # three extra collinear points; every coordinate stays exact through the normalisation (scale 1/2, t 0)
    V = np.vstack([GV, [[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [0.25, 0.0, 0.0]]])
    F = np.vstack([GF, extra_faces]).astype(np.int32)
    return GV, GF, V, F


def test_do_nothing_on_zero_angle():
    # system.py:214-221: a minimum internal angle <= 0 degrees skips every step
    GV, GF, V, F = _octahedron_with([[6, 7, 8]])
    out, st = orc.stage3_run(GV, GF, V, F, 2)
    assert st["do_nothing"] == 1 and st["steps"] == 0
    assert np.array_equal(out, V)


def test_nan_angle_disables_do_nothing():
    # numpy's min propagates NaN (a zero-length edge gives acos(0/0)), and NaN <= 0 is false
    GV, GF, V, F = _octahedron_with([[6, 7, 8], [6, 6, 7]])
    _, st = orc.stage3_run(GV, GF, V, F, 0)
    assert st["do_nothing"] == 0


def test_contacts_keep_sheets_apart():
    V, F = meshes.sheet_pair()
    GV = V.copy()
    # GT: the lower sheet only, lifted to the upper one: distance energy pulls the lower sheet into the upper
    n = len(V) // 2
    GV[:n, 2] += 0.0012
    out, st = orc.stage3_run(GV, F, V, F, 1)
    assert st["total_contacts"] > 0
    gap = out[n:, 2].mean() - out[:n, 2].mean()
    assert gap > 0  # the barrier keeps the order of the sheets
