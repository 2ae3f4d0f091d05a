"""The legacy simplifier without rollback (``CUDSP.forward`` / ``PaSP.run``, reference simp_cuda/src/cusimp.cu and
simp_cuda/pamo/__init__.py:181-227) on the GPU against the CPU oracle's restatement: every output of every round
bit-exact, and the whole loop."""

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests import meshes

pytestmark = pytest.mark.gpu


def _cases():
    return {
        "octahedron": meshes.octahedron(),
        "sphere6": meshes.sphere(6),
        "sphere10": meshes.sphere(10, L=5, sigma=0.05, seed=3),
        "open_patch": meshes.open_patch(),
        "degenerate_face": meshes.with_degenerate_face(),
        "tangled": meshes.tangled(10, seed=9, amp=0.25),
    }


@pytest.mark.parametrize("name", sorted(_cases()))
def test_rounds_match_oracle(name):
    import pamo_gb300

    v, f = _cases()[name]
    scale = float(np.max(v.max(0) - v.min(0)))
    gpu, cpu = pamo_gb300.CUDSP(), orc.Oracle()
    vg, fg = v.astype(np.float32), f.astype(np.int32)
    for r in range(10):
        outs_g = [t.cpu().numpy() for t in gpu.forward(torch.from_numpy(vg).cuda(), torch.from_numpy(fg).cuda(), scale,
                                                       1e-3, r == 0)]
        outs_c = cpu.forward_legacy(vg, fg, scale, 1e-3, r == 0)
        for k, (a, b) in enumerate(zip(outs_g, outs_c)):
            assert a.shape == b.shape, (r, k)
            assert np.array_equal(a, b), (name, r, k)
        verts, tris, occ, vmap = outs_c
        vg = verts[occ[:, 0].astype(bool)]
        fg = vmap[:, 0][tris[tris[:, 0] >= 0]].astype(np.int32)
        if len(fg) < 4:
            break


@pytest.mark.parametrize("name", ["sphere10", "tangled"])
def test_pasp_run_matches_oracle(name):
    import pamo_gb300

    v, f = _cases()[name]
    model = pamo_gb300.PaSP()
    V, F = model.run(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda())
    Vo, Fo, rounds = orc.Oracle().run_legacy(v, f)
    assert model.iterations == rounds
    assert np.array_equal(F.cpu().numpy(), Fo)
    assert np.array_equal(V.cpu().numpy(), Vo)
