"""Generates tests/golden/tritri_cases.npz: triangle pairs with the reference's own per-pair
self-intersection decision.

The decisions come from oracle/_ref/ref_tritri, the reference's tri-tri code (simp_cuda/src/bvh of the reference
checkout named by $PAMO_REFERENCE_ROOT) compiled for the host by oracle/build_ref.py. The script also checks that the oracle's
restatement agrees on every generated case before writing the fixture (all positive cases and a sample of
negatives are stored).

Cases: random nearby pairs, every AABB-overlapping face pair of spheres with randomly displaced vertices
(shared vertices and edges by index), coplanar pairs, pairs sharing coordinates but not indices, vertices
exactly on the other triangle's plane, slivers and points straddling the integer translation boundaries.

    python tests/golden/make_tritri_golden.py
"""

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from pamo_gb300 import synth  # noqa: E402


def run_ref(exe, cur, qry, ci, qi):
    n = len(cur)
    rec = np.zeros(n, dtype=[("c", "<f4", 9), ("q", "<f4", 9), ("ci", "<i4", 3), ("qi", "<i4", 3)])
    rec["c"], rec["q"], rec["ci"], rec["qi"] = cur.reshape(n, 9), qry.reshape(n, 9), ci, qi
    data = np.int32(n).tobytes() + rec.tobytes()
    out = subprocess.run([exe], input=data, capture_output=True, check=True).stdout
    return np.frombuffer(out, np.int32).copy()


def oracle_decisions(cur, qry, ci, qi):
    out = np.zeros(len(cur), np.int32)
    for k in range(len(cur)):
        # give the six vertices slots so that shared indices share a slot
        ids = {}
        pts = []
        for tri, idx in ((cur[k], ci[k]), (qry[k], qi[k])):
            for p, i in zip(tri, idx):
                if int(i) not in ids:
                    ids[int(i)] = len(pts)
                    pts.append(p)
        P = np.array(pts, np.float32)
        c = np.array([ids[int(i)] for i in ci[k]], np.int32)
        q = np.array([ids[int(i)] for i in qi[k]], np.int32)
        out[k] = orc.pair_intersects(P, c, q, 1e-3)
    return out


def cases(rng):
    C, Q, CI, QI = [], [], [], []

    def add(c, q, ci, qi):
        C.append(np.asarray(c, np.float32)); Q.append(np.asarray(q, np.float32))
        CI.append(np.asarray(ci, np.int32)); QI.append(np.asarray(qi, np.int32))

    # random nearby pairs (distinct indices)
    for _ in range(4000):
        c = rng.uniform(-1.5, 1.5, 3) + rng.normal(0, 0.05, (3, 3))
        q = c.mean(0) + rng.normal(0, 0.05, (3, 3))
        add(c, q, [0, 1, 2], [3, 4, 5])
    # meshes with displaced vertices: every AABB-overlapping face pair, both orders
    for seed in range(3):
        v, f = synth.star_mesh(10, 4, lambda l: 0.05, 100 + seed)
        v = v.copy()
        pick = rng.choice(len(v), 25, replace=False)
        v[pick] *= rng.uniform(0.85, 1.15, (25, 1)).astype(np.float32)
        tri = v[f]
        lo, hi = tri.min(1), tri.max(1)
        for a in range(len(f)):
            ov = np.all((hi[a] >= lo) & (hi >= lo[a]), axis=1)
            ov[a] = False
            for b in np.nonzero(ov)[0]:
                add(tri[b], tri[a], f[b], f[a])
    # coplanar and on-plane configurations
    for _ in range(600):
        c = np.c_[rng.uniform(-1, 1, (3, 2)), np.zeros(3)]
        q = np.c_[rng.uniform(-1, 1, (3, 2)), np.zeros(3)]
        if rng.random() < 0.5:
            q[0, 2] = rng.choice([0.0, 1e-9, -1e-9, 1e-4])
        add(c, q, [0, 1, 2], [3, 4, 5])
    # shared vertex (by index or by coordinates), shared edge by coordinates only
    for _ in range(1500):
        s = rng.uniform(-1.2, 1.2, 3)
        c = np.stack([s, s + rng.normal(0, 0.1, 3), s + rng.normal(0, 0.1, 3)])
        q = np.stack([s, s + rng.normal(0, 0.1, 3), s + rng.normal(0, 0.1, 3)])
        mode = rng.integers(3)
        if mode == 0:
            add(c, q, [0, 1, 2], [0, 4, 5])
        elif mode == 1:
            add(c, q, [0, 1, 2], [3, 4, 5])
        else:
            q[1] = c[1]
            add(c, q, [0, 1, 2], [3, 4, 5])
    # slivers, repeated points, translation boundaries
    for _ in range(600):
        base = rng.choice([0.0, 1.0, -1.0, 0.999999, 1e-7])
        c = base + rng.normal(0, 0.01, (3, 3))
        c[2] = c[0] + (c[1] - c[0]) * rng.uniform(0, 1)  # collinear sliver
        q = base + rng.normal(0, 0.01, (3, 3))
        add(c, q, [0, 1, 2], [3, 4, 5])
    return np.array(C), np.array(Q), np.array(CI), np.array(QI)


def main():
    exe = build_ref.build()
    rng = np.random.default_rng(20241203)
    C, Q, CI, QI = cases(rng)
    ref = run_ref(exe, C, Q, CI, QI)
    ora = oracle_decisions(C, Q, CI, QI)
    bad = np.nonzero(ref != ora)[0]
    print(f"{len(C)} cases, {int(ref.sum())} intersecting, {len(bad)} oracle disagreements")
    if len(bad):
        raise SystemExit(f"oracle disagrees with the reference on cases {bad[:20]}")
    pos = np.nonzero(ref == 1)[0]
    neg = np.nonzero(ref == 0)[0]
    keep = np.concatenate([pos, rng.choice(neg, min(len(neg), max(3000, len(pos))), replace=False)])
    keep.sort()
    np.savez_compressed(os.path.join(HERE, "tritri_cases.npz"), cur=C[keep], qry=Q[keep], cur_ids=CI[keep],
                        qry_ids=QI[keep], expected=ref[keep], n_generated=np.array(len(C)))


if __name__ == "__main__":
    main()
