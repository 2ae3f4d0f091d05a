"""Parity of the CUDA path (through the C ABI) with the CPU oracle, round by round and over the whole loop.

Integer outputs (faces, occupancy, maps, undo lists, collapse sets) must be bit-exact; positions are
compared exactly too because both sides evaluate the same float32 operations in the same order.
"""

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests import meshes

pytestmark = pytest.mark.gpu


def _cases():
    return {
        "octahedron": meshes.octahedron(),
        "sphere4": meshes.sphere(4),
        "sphere8": meshes.sphere(8, L=5, sigma=0.05, seed=3),
        "open_patch": meshes.open_patch(),
        "degenerate_face": meshes.with_degenerate_face(),
        "coincident_edge": meshes.with_coincident_edge(),
        "tangled": meshes.tangled(10, seed=9, amp=0.25),
        "tangled_strong": meshes.tangled(10, seed=10, amp=0.4),
    }


def _compact(verts, tris, occ, vmap):
    v = verts[occ[:, 0].astype(bool)]
    f = tris[tris[:, 0] >= 0]
    return v, vmap[:, 0][f].astype(np.int32)


def _chain(v, f, rounds, gpu: bool):
    import pamo_gb300

    op = pamo_gb300.CUDSP_Free() if gpu else orc.Oracle()
    scale = float(np.max(v.max(0) - v.min(0)))
    undo = np.zeros(0, np.int32)
    outs = []
    count, stuck, nprev = 0, False, len(f)
    for r in range(rounds):
        if gpu:
            res = op.forward(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda(), torch.from_numpy(undo).cuda(),
                             len(undo), scale, 1e-3, stuck, r == 0)
            res = [t.cpu().numpy() for t in res]
        else:
            res = op.forward(v, f, undo, len(undo), scale, 1e-3, stuck, r == 0)
        outs.append(res)
        verts, tris, occ, vmap, undo = res
        v, f = _compact(verts, tris, occ, vmap)
        if len(f) == nprev:
            count += 1
        else:
            count, stuck = 0, False
        if count >= 2:
            stuck = True
        nprev = len(f)
        if len(f) <= 10:
            break
    return outs


@pytest.mark.parametrize("name", ["octahedron", "sphere4", "sphere8", "open_patch", "degenerate_face", "coincident_edge",
                                  "tangled", "tangled_strong"])
def test_rounds_match_oracle(name):
    v, f = _cases()[name]
    g = _chain(v, f, 12, gpu=True)
    c = _chain(v, f, 12, gpu=False)
    assert len(g) == len(c)
    for r, (a, b) in enumerate(zip(g, c)):
        for k, (x, y) in enumerate(zip(a, b)):
            assert x.shape == y.shape, (name, r, k)
            assert np.array_equal(x, y), (name, r, k)


def test_plain_small_first_rounds_match_oracle():
    from pamo_gb300 import synth

    v, f = synth.config_mesh("plain_small", seed=0)
    g = _chain(v, f, 6, gpu=True)
    c = _chain(v, f, 6, gpu=False)
    for r, (a, b) in enumerate(zip(g, c)):
        for k, (x, y) in enumerate(zip(a, b)):
            assert np.array_equal(x, y), (r, k)


@pytest.mark.parametrize("name,ratio", [("sphere8", 0.05), ("plain_small", 0.01)])
def test_run_matches_oracle(name, ratio):
    import pamo_gb300
    from pamo_gb300 import synth

    v, f = synth.config_mesh("plain_small", seed=0) if name == "plain_small" else _cases()[name]
    pamo = pamo_gb300.PaMO((v, f), use_stage1=False, use_stage3=False)
    V, F = pamo.run(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda(), ratio=ratio, min_verts=0)
    V0, F0, fpr = orc.Oracle().run(v, f, ratio, min_verts=0)
    assert pamo.last_rounds == len(fpr)
    assert np.array_equal(F, F0)
    assert np.array_equal(V, V0)


def test_bad_index_is_an_error():
    import pamo_gb300

    v, f = meshes.octahedron()
    f = f.copy()
    f[3, 1] = 99
    op = pamo_gb300.CUDSP_Free()
    with pytest.raises(pamo_gb300.PamoError):
        op.forward(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda(), torch.zeros(0, dtype=torch.int32).cuda(), 0,
                   2.0, 1e-3, False, True)


def test_operator_input_checks():
    import pamo_gb300

    v, f = meshes.octahedron()
    op = pamo_gb300.CUDSP_Free()
    with pytest.raises(RuntimeError):
        op.forward(torch.from_numpy(v), torch.from_numpy(f).cuda(), torch.zeros(0, dtype=torch.int32).cuda(), 0, 2.0,
                   1e-3, False, True)
    with pytest.raises(RuntimeError):
        op.forward(torch.from_numpy(v).double().cuda(), torch.from_numpy(f).cuda(),
                   torch.zeros(0, dtype=torch.int32).cuda(), 0, 2.0, 1e-3, False, True)


@pytest.mark.parametrize("name", ["sphere8", "plain_small"])
def test_blender_entry_matches_oracle(name):
    """pamo_simplify (the Blender add-on's host-pointer whole loop) against the oracle's restatement of
    pamo_blender/cusimpinterface.cu:57-161, twice in a row on the kept context (its state carries over)."""
    import pamo_gb300
    from pamo_gb300 import synth

    v, f = meshes.sphere(8, L=5, sigma=0.05, seed=3) if name == "sphere8" else synth.config_mesh("plain_small")
    o = orc.Oracle()
    for _ in range(2):
        V, F = pamo_gb300.pamo_simplify(v, f, 1e-3)
        Vo, Fo, fpr = o.run_blender(v, f, 1e-3)
        assert len(fpr) >= 5 and np.all(fpr[-4:] == fpr[-1])  # stopped after 4 rounds without progress
        assert np.array_equal(F, Fo)
        assert np.array_equal(V, Vo)


@pytest.mark.parametrize("mode", [(1, 1, 1), (1, 1, 0), (1, 0, 1), (0, 0, 0)])
@pytest.mark.parametrize("name,ratio", [("plain_small", 0.01), ("tangled", 0.05), ("tangled_strong", 0.05)])
def test_loop_execution_modes_agree(mode, name, ratio):
    """The whole loop gives the oracle's result with device-driven rounds as graphs (with the carried LBVH and
    with one built every round), as direct launches, and with the host-sized rounds; the tangled meshes take
    undo passes in many rounds."""
    import pamo_gb300
    from pamo_gb300 import synth

    v, f = synth.config_mesh("plain_small") if name == "plain_small" else _cases()[name]
    ctx = pamo_gb300.Context("cuda:0")
    ctx.set_option("device_rounds", mode[0])
    ctx.set_option("graphs", mode[1])
    ctx.set_option("bvh_reuse", mode[2])
    pts = torch.tensor(v, device="cuda")
    tri = torch.tensor(f, device="cuda", dtype=torch.int32)
    Vo, Fo, fpr = orc.Oracle().run(v, f, ratio, 4, 1e-3, 1000000, 0)
    for _ in range(2):  # the second run replays the cached graphs
        ctx.reset()
        V, F, rounds = pamo_gb300.simplify(pts, tri, ratio, 4, 1e-3, 1000000, 0, ctx=ctx)
        assert rounds == len(fpr)
        assert np.array_equal(F.cpu().numpy(), Fo)
        assert np.array_equal(V.cpu().numpy(), Vo)


@pytest.mark.parametrize("name,cap", [("tangled_strong", 16), ("plain_small", 256)])
def test_pair_list_overflow_matches_oracle(name, cap):
    """With the candidate-pair list cut to a few entries, the queries that overflow it walk the tree again and
    decide their pairs in place; the whole loop still gives the oracle's result."""
    import pamo_gb300
    from pamo_gb300 import synth

    v, f = synth.config_mesh("plain_small") if name == "plain_small" else _cases()[name]
    ctx = pamo_gb300.Context("cuda:0")
    ctx.set_option("pair_cap", cap)
    pts = torch.tensor(v, device="cuda")
    tri = torch.tensor(f, device="cuda", dtype=torch.int32)
    Vo, Fo, fpr = orc.Oracle().run(v, f, 0.05, 4, 1e-3, 1000000, 0)
    V, F, rounds = pamo_gb300.simplify(pts, tri, 0.05, 4, 1e-3, 1000000, 0, ctx=ctx)
    assert rounds == len(fpr)
    assert np.array_equal(F.cpu().numpy(), Fo)
    assert np.array_equal(V.cpu().numpy(), Vo)


def _tris_mean_cases():
    from pamo_gb300 import synth

    rng = np.random.default_rng(5)
    cases = {"plain_small": synth.config_mesh("plain_small", seed=0)}
    v, f = meshes.sphere(40)
    cases["sphere40"] = (v, f)
    # sums that wander through zero and across many binades, with offsets, signs and magnitudes mixed
    n = 300000
    fr = rng.integers(0, n, (n, 3)).astype(np.int32)
    for name, pts in {
        "centred_noise": rng.normal(0, 1, (n, 3)),
        "offset": rng.normal(0, 1, (n, 3)) + [1e3, -2e2, 0.5],
        "mixed_scales": rng.normal(0, 1, (n, 3)) * 10.0 ** rng.integers(-6, 6, (n, 1)),
        "dyadic": rng.integers(-64, 64, (n, 3)) / 8.0,  # many exact ties in the sum
    }.items():
        cases[name] = (pts.astype(np.float32), fr)
    return cases


@pytest.mark.parametrize("name", sorted(_tris_mean_cases()))
def test_tris_mean_matches_numpy(name):
    """The centring sum (exact sequential float32 order, computed with window parallelism) equals numpy's
    float32 tris.mean(axis=1).mean(axis=0) bit for bit."""
    import pamo_gb300

    v, f = _tris_mean_cases()[name]
    got = pamo_gb300.tris_mean(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda())
    want = np.asarray(v, np.float32)[f].mean(axis=1).mean(axis=0)
    assert want.dtype == np.float32
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (got, want)
    assert np.array_equal(got, orc.tris_mean(v, f))


def test_midsize_loop_matches_oracle():
    """The whole device loop on a 327,680-face mesh (icosphere frequency 128, SH l <= 16, sigma 0.05/l) to 0.1 %:
    faces per round, final faces and positions bit-identical to the oracle's loop (run with every host core)."""
    import os

    import pamo_gb300
    from pamo_gb300 import synth

    v, f = synth.star_mesh(128, 16, lambda l: 0.05 / l, 0)
    assert len(f) == 327680
    Vo, Fo, fpr = orc.Oracle(threads=os.cpu_count() or 1).run(v, f, 0.001, 4, 1e-3, 1000000, 0)
    ctx = pamo_gb300.Context("cuda:0")
    V, F, rounds = pamo_gb300.simplify(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda(), 0.001, 4, 1e-3,
                                       1000000, 0, ctx=ctx)
    assert rounds == len(fpr)
    assert np.array_equal(pamo_gb300.api.round_faces(ctx, rounds), fpr)
    assert np.array_equal(F.cpu().numpy(), Fo)
    assert np.array_equal(V.cpu().numpy(), Vo)
