"""Many meshes on one GPU: the batch and the request server return, for every mesh, the result of the plain
path on a new context (bit-exact), whatever else runs beside it."""

import numpy as np
import pytest
import torch

from tests import meshes

pytestmark = pytest.mark.gpu


def _meshes():
    from pamo_gb300 import synth

    out = [synth.star_mesh(n, 5, lambda l: 0.04, seed) for n, seed in [(12, 1), (20, 2), (6, 3), (16, 4), (9, 5)]]
    out.append(meshes.open_patch())
    out.append(meshes.octahedron())
    return out


def _alone(v, f, ratio):
    import pamo_gb300

    ctx = pamo_gb300.Context("cuda:0")
    V, F, _ = pamo_gb300.simplify(torch.tensor(v, device="cuda"), torch.tensor(f, device="cuda", dtype=torch.int32),
                                  ratio, 4, 1e-3, 1000000, 0, ctx=ctx)
    return V.cpu().numpy(), F.cpu().numpy()


def test_batch_equals_alone():
    from pamo_gb300.batch import Batch, simplify_batch

    ms = _meshes()
    ratios = [0.05, 0.02, 0.1, 0.01, 0.2, 0.1, 0.5]
    b = Batch("cuda:0", workers=4)
    for _ in range(2):  # a second batch on the same workers: every job starts from a new context's state
        res = simplify_batch(ms, ratios, batch=b)
        assert len(res) == len(ms)
        for (v, f), r, (V, F) in zip(ms, ratios, res):
            Va, Fa = _alone(v, f, r)
            assert np.array_equal(F, Fa)
            assert np.array_equal(V, Va)


def test_batch_matches_oracle():
    from oracle import oracle as orc
    from pamo_gb300.batch import simplify_batch

    ms = _meshes()[:3]
    res = simplify_batch(ms, [0.05, 0.02, 0.1], workers=3)
    for (v, f), r, (V, F) in zip(ms, [0.05, 0.02, 0.1], res):
        Vo, Fo, _ = orc.Oracle().run(v, f, r, 4, 1e-3, 1000000, 0)
        assert np.array_equal(F, Fo)
        assert np.array_equal(V, Vo)


def test_server_results_and_admission():
    from pamo_gb300.batch import Server

    ms = _meshes()
    jb = [Server.job_bytes(len(v), len(f)) for v, f in ms]
    budget = 2 * max(jb)  # at most a few jobs in flight at once
    srv = Server("cuda:0", workers=4, hbm_budget_bytes=budget)
    ids = {srv.submit(v, f, 0.05): i for i, (v, f) in enumerate(ms)}
    got = {}
    while len(got) < len(ms):
        w = srv.wait(10000)
        assert w is not None, "server stalled"
        rid, st, npt, ntr, times = w
        assert st == 0
        assert times[2] >= times[1] >= 0
        got[ids[rid]] = srv.fetch(rid, npt, ntr)
    st = srv.stats()
    assert st["finished"] == len(ms) and st["queued"] == 0 and st["in_use"] == 0
    assert st["max_in_use"] <= budget
    srv.close()
    for i, (v, f) in enumerate(ms):  # each result equals the mesh alone
        Va, Fa = _alone(v, f, 0.05)
        assert np.array_equal(got[i][1], Fa)
        assert np.array_equal(got[i][0], Va)


def test_job_bytes_covers_a_context():
    import pamo_gb300
    from pamo_gb300.batch import Server
    from pamo_gb300 import synth

    for n in (8, 32):
        v, f = synth.star_mesh(n, 4, lambda l: 0.04, 7)
        ctx = pamo_gb300.Context("cuda:0")
        pamo_gb300.simplify(torch.tensor(v, device="cuda"), torch.tensor(f, device="cuda", dtype=torch.int32), 0.05,
                            4, 1e-3, 1000000, 0, ctx=ctx)
        need = ctx.device_bytes() + 2 * (12 * len(v) + 12 * len(f))
        assert need <= Server.job_bytes(len(v), len(f))


def test_autotune_picks_a_candidate_and_caches_it(tmp_path, monkeypatch):
    from pamo_gb300 import autotune
    from pamo_gb300.synth import star_mesh

    monkeypatch.setenv("PAMO_GB300_TUNE", str(tmp_path / "tune.json"))
    meshes = [star_mesh(8 + i, 4, lambda l: 0.03, i) for i in range(6)]
    res = autotune.tune_batch(meshes, 0.05, candidates=(2, 4), repeats=1)
    assert res["best"] in (2, 4) and res[2] > 0 and res[4] > 0
    assert autotune.best_workers() == res["best"]
    assert (tmp_path / "tune.json").exists()


def test_server_stage3_equals_pamo_run():
    """Requests with stage 3 (PaMO(use_stage3=True) per request, the projection onto the request's own input): each
    result has PaMO.run's faces and positions, bit for bit (stage 3 sums in a fixed order, and the server's second
    attempt after a grid barrier time-out uses launch shapes with the same bits), among other requests."""
    import pamo_gb300
    from pamo_gb300.batch import Server
    from pamo_gb300 import synth

    ms = [synth.star_mesh(n, 4, lambda l: 0.04, seed) for n, seed in [(10, 1), (14, 2), (8, 3)]]
    srv = Server("cuda:0", workers=3, hbm_budget_bytes=8 << 30)
    ids = {srv.submit(v, f, 0.05, stage3=True): i for i, (v, f) in enumerate(ms)}
    got = {}
    while len(got) < len(ms):
        w = srv.wait(20000)
        assert w is not None, "server stalled"
        rid, st, npt, ntr, _ = w
        assert st == 0
        got[ids[rid]] = srv.fetch(rid, npt, ntr, float64=True)
    assert srv.stats()["stage3_reruns"] >= 0
    srv.close()
    for i, (v, f) in enumerate(ms):
        pm = pamo_gb300.PaMO((v.astype(np.float64), f), use_stage1=False, use_stage3=True)
        V, F = pm.run(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda(), ratio=0.05, min_verts=0)
        V, F = np.asarray(V), np.asarray(F)
        assert got[i][0].dtype == np.float64
        assert np.array_equal(got[i][1], F)
        assert np.array_equal(got[i][0], V)
