"""CPU oracle checks: pinned against thrust's own shuffle, plus invariants of the restated round."""

import hashlib
import os

import numpy as np
import pytest

from oracle import oracle as orc
from tests import meshes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_shuffle_matches_thrust_golden():
    g = np.load(os.path.join(GOLDEN, "thrust_shuffle.npz"))
    assert int(g["thrust_version"]) == 300001
    full = [k for k in g.files if k.startswith("perm_")]
    assert full
    for k in full:
        m = int(k.split("_")[1])
        assert np.array_equal(orc.shuffle_perm(m), g[k]), m
    for k in [k for k in g.files if k.startswith("sha256_")]:
        m = int(k.split("_")[1])
        d = hashlib.sha256(orc.shuffle_perm(m).tobytes()).digest()
        assert np.frombuffer(d, np.uint8).tolist() == g[k].tolist(), m


def test_tris_mean_matches_numpy_float32():
    v, f = meshes.sphere(6)
    ref = v[f].mean(axis=1).mean(axis=0)  # the reference's preprocess_mesh, pamo/__init__.py:61-64
    assert np.array_equal(orc.tris_mean(v, f), ref)


def _round_chain(o, v, f, rounds):
    scale = float(np.max(v.max(0) - v.min(0)))
    undo = np.zeros(0, np.int32)
    outs = []
    for r in range(rounds):
        out = o.forward(v, f, undo, len(undo), scale, 1e-3, False, r == 0)
        verts, tris, occ, vmap, undo = out
        outs.append([a.copy() for a in out])
        v = verts[occ[:, 0].astype(bool)]
        f = tris[tris[:, 0] >= 0]
        f = vmap[:, 0][f]
    return outs, v, f


def test_round_is_deterministic_across_threads():
    v, f = meshes.sphere(8)
    a, va, fa = _round_chain(orc.Oracle(threads=1), v, f, 6)
    b, vb, fb = _round_chain(orc.Oracle(threads=4), v, f, 6)
    for x, y in zip(a, b):
        for p, q in zip(x, y):
            assert np.array_equal(p, q)


def test_round_preserves_topology_and_compaction():
    v, f = meshes.sphere(10)
    o = orc.Oracle()
    outs, v2, f2 = _round_chain(o, v, f, 8)
    assert len(f2) < len(f)
    assert meshes.euler(f2) == 2  # closed genus-0 stays genus-0
    assert f2.min() >= 0 and f2.max() < len(v2)
    for verts, tris, occ, vmap, undo in outs:
        # verts_map is the exclusive scan of verts_occ
        assert np.array_equal(vmap[:, 0], np.concatenate([[0], np.cumsum(occ[:, 0])[:-1]]))
        # removed vertices are zeroed, removed faces are -1 rows
        assert np.all(verts[occ[:, 0] == 0] == 0)
        dead = tris[:, 0] < 0
        assert np.all(tris[dead] == -1)


def test_run_loop_reaches_target_or_stalls():
    v, f = meshes.sphere(8)
    V, F, fpr = orc.Oracle().run(v, f, 0.1, min_verts=0)
    target = int(0.1 * len(f))
    assert F.shape[0] == fpr[-1]
    assert F.shape[0] <= target or (len(fpr) >= 4 and len(set(fpr[-4:].tolist())) == 1)
    assert np.all(np.diff(fpr) <= 0)


def test_open_mesh_boundary_uses_stale_costs():
    # boundary edges (link count != 2) keep the fresh-buffer (zero) cost in the first round
    v, f = meshes.open_patch()
    o = orc.Oracle()
    scale = float(np.max(v.max(0) - v.min(0)))
    o.forward(v, f, np.zeros(0, np.int32), 0, scale, 1e-3, False, True)
    e = o.edges()
    c = o.edge_costs()
    ee = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    uniq, cnt = np.unique(ee, axis=0, return_counts=True)
    boundary = {tuple(x) for x in uniq[cnt == 1]}
    isb = np.array([tuple(x) in boundary for x in e])
    assert isb.any()
    assert np.all(c[isb] == 0)


def _slots(c, q, ci, qi):
    ids, pts = {}, []
    for tri, idx in ((c, ci), (q, qi)):
        for p, i in zip(tri, idx):
            if int(i) not in ids:
                ids[int(i)] = len(pts)
                pts.append(p)
    return (np.array(pts, np.float32), np.array([ids[int(i)] for i in ci], np.int32),
            np.array([ids[int(i)] for i in qi], np.int32))


def test_pair_decision_matches_reference_golden():
    g = np.load(os.path.join(GOLDEN, "tritri_cases.npz"))
    exp = g["expected"]
    assert exp.sum() > 1000 and (exp == 0).sum() > 1000
    for k in range(len(exp)):
        P, c, q = _slots(g["cur"][k], g["qry"][k], g["cur_ids"][k], g["qry_ids"][k])
        assert orc.pair_intersects(P, c, q, 1e-3) == bool(exp[k]), k


def test_legacy_round_outputs_are_consistent():
    """One legacy CUSimp round (no rollback): the map is the exclusive scan of the occupancy, removed vertices are
    zeroed, the surviving faces reference occupied vertices, and the loop converges."""
    v, f = meshes.sphere(10)
    o = orc.Oracle()
    scale = float(np.max(v.max(0) - v.min(0)))
    verts, tris, occ, vmap = o.forward_legacy(v, f, scale, 1e-3, True)
    occ = occ[:, 0]
    assert np.array_equal(vmap[:, 0], np.concatenate([[0], np.cumsum(occ)[:-1]]))
    assert occ.sum() < len(v)
    assert np.all(verts[occ == 0] == 0)
    live = tris[tris[:, 0] >= 0]
    assert len(live) < len(f) and np.all(occ[live] == 1)
    V, F, rounds = orc.Oracle().run_legacy(v, f)
    assert 1 < rounds < 1000 and len(F) < len(f)
    assert F.min() >= 0 and F.max() < len(V)
