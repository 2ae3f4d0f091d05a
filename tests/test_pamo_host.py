"""Host logic of PaMO.run on CPU, with the GPU calls replaced by recorders: the stage-2 target, the stage-3
hand-over (trimesh-style processing, then the projection onto the input mesh) and the projection target uploaded
once and kept across runs."""

import numpy as np
import torch

from tests import meshes


def test_run_hands_stage2_to_stage3_and_keeps_the_target(monkeypatch):
    import pamo_gb300.api as api
    from pamo_gb300 import safe_project

    V, F = meshes.octahedron()
    calls = {"simplify": [], "process": []}

    class FakeContext:
        def __init__(self, device):
            self.device = device

    def fake_simplify(points, triangles, ratio, tolerance, threshold, iter, min_verts, ctx=None):
        calls["simplify"].append((len(triangles), ratio, tolerance, threshold, min_verts))
        return points[:4].clone(), torch.tensor([[0, 1, 2], [0, 2, 3]], dtype=torch.int32), 3

    class FakeSystem:
        def __init__(self, config, device):
            self.device = device

    def fake_process(gt_V, gt_F, V2, F2, n_iters, system=None):
        calls["process"].append((gt_V, gt_F, n_iters))
        return np.asarray(V2, np.float64) + 1.0, F2

    monkeypatch.setattr(api, "Context", FakeContext)
    monkeypatch.setattr(api, "simplify", fake_simplify)
    monkeypatch.setattr(safe_project, "Stage3System", FakeSystem)
    monkeypatch.setattr(safe_project, "process", fake_process)

    model = api.PaMO((V, F), use_stage1=False, use_stage3=True)
    pts, tri = torch.from_numpy(V).float(), torch.from_numpy(F).int()
    for _ in range(2):
        out_V, out_F = model.run(pts, tri, ratio=0.5, min_verts=0)
        assert out_V.shape == (4, 3) and np.array_equal(out_F, [[0, 1, 2], [0, 2, 3]])
        assert np.allclose(out_V, V[:4] + 1.0)
    assert calls["simplify"] == [(len(F), 0.5, 4, 1e-3, 0)] * 2
    assert model.target_faces == len(F) // 2 and model.last_rounds == 3
    (g0, f0, n0), (g1, f1, n1) = calls["process"]
    assert n0 == n1 == 5
    assert g0.dtype == torch.float64 and f0.dtype == torch.int32
    assert torch.equal(g0, torch.from_numpy(V).double()) and torch.equal(f0, torch.from_numpy(F).int())
    assert g1 is g0 and f1 is f0  # uploaded once, reused by the next run
