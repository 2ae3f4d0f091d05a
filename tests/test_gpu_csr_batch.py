"""Batched rounds (pamo_csr_*, CsrBatch): many meshes in one CSR batch run the PaMO.run loop together, every round one
pass over all live meshes. Each result must equal the mesh's plain-path result alone, bit for bit, and the
reference's own results where the fixtures hold them; meshes that take undo passes, stuck rounds, open boundaries,
degenerate faces and zero-length edges are mixed into the batches."""

import numpy as np
import pytest
import torch

from tests import meshes
from tests.golden import make_ref_round_golden as gen

pytestmark = pytest.mark.gpu


def _alone(v, f, ratio, tol=4, thr=1e-3, iters=1000000):
    import pamo_gb300

    ctx = pamo_gb300.Context("cuda:0")
    V, F, rounds = pamo_gb300.simplify(torch.tensor(v, device="cuda"),
                                       torch.tensor(f, device="cuda", dtype=torch.int32), ratio, tol, thr, iters, 0,
                                       ctx=ctx)
    return V.cpu().numpy(), F.cpu().numpy(), rounds


def _mixed():
    from pamo_gb300 import synth

    ms = [synth.star_mesh(n, 5, lambda l: 0.04, seed) for n, seed in [(12, 1), (20, 2), (6, 3), (16, 4), (9, 5)]]
    ms += [meshes.open_patch(), meshes.octahedron(), meshes.tangled(10, seed=9, amp=0.25),
           meshes.tangled(10, seed=10, amp=0.4), meshes.with_degenerate_face(), meshes.with_coincident_edge(),
           meshes.sphere(4)]
    ratios = [0.05, 0.02, 0.1, 0.01, 0.2, 0.1, 0.5, 0.02, 0.02, 0.05, 0.05, 0.05]
    return ms, ratios


def test_csr_batch_equals_alone():
    from pamo_gb300.batch import CsrBatch, simplify_batch

    ms, ratios = _mixed()
    b = CsrBatch("cuda:0")
    for _ in range(2):  # the same engine twice: every job starts from a new context's state
        res = simplify_batch(ms, ratios, batch=b)
        rounds = b.rounds(len(ms))
        assert len(res) == len(ms)
        for i, ((v, f), r, (V, F)) in enumerate(zip(ms, ratios, res)):
            Va, Fa, ra = _alone(v, f, r)
            assert rounds[i] == ra, i
            assert np.array_equal(F, Fa), i
            assert np.array_equal(V, Va), i


def test_csr_batch_equals_reference_rounds():
    """The final meshes of the reference's own loop (tests/golden/ref_rounds.npz) from one batch of those meshes."""
    from pamo_gb300.batch import CsrBatch, simplify_batch

    g = np.load(gen.__file__.replace("make_ref_round_golden.py", "ref_rounds.npz"))
    names = ["plain_small", "tangled", "tangled_strong", "tangled_dense", "sphere12_rough", "open_patch",
             "degenerate_face", "coincident_edge", "sphere8", "sphere4"]
    cases = gen.cases()
    # the reference loop's own threshold and tolerance are the same for these cases (1e-3, 4)
    assert all(cases[n][3] == 4 and cases[n][4] == 1e-3 for n in names)
    ms = [(cases[n][0], cases[n][1]) for n in names]
    ratios = [cases[n][2] for n in names]
    iters = min(cases[n][5] for n in names)
    res = simplify_batch(ms, ratios, iter=iters, batch=CsrBatch("cuda:0"))
    for n, (V, F) in zip(names, res):
        if cases[n][5] != iters:  # a case whose loop the fixture caps at a different round count
            continue
        assert np.array_equal(F, g[f"{n}.final_faces"]), n
        assert np.array_equal(V, g[f"{n}.final_verts"]), n


def test_csr_batch_many_meshes():
    from pamo_gb300 import synth
    from pamo_gb300.batch import CsrBatch, simplify_batch

    rng = np.random.default_rng(3)
    ms = [synth.star_mesh(int(n), 6, lambda l: 0.03, 100 + i) for i, n in enumerate(rng.integers(3, 28, 70))]
    ratios = rng.uniform(0.001, 0.05, len(ms))
    res = simplify_batch(ms, ratios, batch=CsrBatch("cuda:0"))
    for (v, f), r, (V, F) in zip(ms, ratios, res):
        Va, Fa, _ = _alone(v, f, float(r))
        assert np.array_equal(F, Fa)
        assert np.array_equal(V, Va)
