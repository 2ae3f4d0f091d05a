"""Generates tests/golden/ref_rounds.npz: the reference's own stage-2 rounds on the test meshes, from the
reference's CUSimp_Free::forward (simp_cuda/src/cusimp_free.cu:891-1048 with simp_cuda/src/bvh/) compiled for the
host by oracle/build_ref.py (build_round_emu) and driven through the stage-2 loop of PaMO.run
(simp_cuda/pamo/__init__.py:95-163, restated below with numpy in the reference's order of operations).

For every case and round it stores the round's counts (points, faces, undo vertices, collapsed edges, faces after
compaction, the is_stuck flag it ran with) and a
SHA-256 digest of each of the five outputs of the operator (pybind.cpp:74-100: positions, faces with removed rows
at -1, occupancy, compaction map, undo vertices), the faces left after compaction, and the final mesh of the loop.
tests/test_ref_rounds.py checks the oracle's restatement against them, round by round and bit for bit.

Needs the reference checkout ($PAMO_REFERENCE_ROOT, default /root/reference):

    python tests/golden/make_ref_round_golden.py [--check]

--check also runs the oracle on every case and prints the first difference (the test does the same).
"""

from __future__ import annotations

import argparse
import ctypes
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "ref_rounds.npz")
OUTPUT_NAMES = ["verts", "tris", "occ", "map", "undo"]


def cases():
    """name -> (points float32 [V,3], triangles int32 [F,3], ratio, tolerance, threshold, max rounds)."""
    from pamo_gb300 import synth
    from tests import meshes

    c1v, c1f = synth.star_mesh(32, 6, lambda l: 0.03, 0)  # level-5 icosphere, SH l<=6, sigma 0.03, seed 0
    out = {
        "plain_small": (c1v, c1f, 0.01, 4, 1e-3, 1000),
        "octahedron": (*meshes.octahedron(), 0.1, 4, 1e-3, 50),
        "sphere4": (*meshes.sphere(4), 0.05, 4, 1e-3, 50),
        "sphere8": (*meshes.sphere(8, L=5, sigma=0.05, seed=3), 0.02, 4, 1e-3, 50),
        "sphere12_rough": (*meshes.sphere(12, L=8, sigma=0.08, seed=21), 0.01, 4, 1e-3, 60),
        "open_patch": (*meshes.open_patch(), 0.05, 4, 1e-3, 50),
        "degenerate_face": (*meshes.with_degenerate_face(), 0.05, 4, 1e-3, 50),
        "coincident_edge": (*meshes.with_coincident_edge(), 0.05, 4, 1e-3, 50),
        "tangled": (*meshes.tangled(10, seed=9, amp=0.25), 0.02, 4, 1e-3, 50),
        "tangled_strong": (*meshes.tangled(10, seed=10, amp=0.4), 0.02, 4, 1e-3, 50),
        "tangled_dense": (*meshes.tangled(14, seed=12, frac=0.05, amp=0.15), 0.01, 4, 1e-3, 60),
        "high_threshold": (*meshes.sphere(10, L=6, sigma=0.06, seed=7), 0.01, 4, 5e-2, 60),
    }
    return out


def legacy_cases():
    """name -> (points, triangles, threshold, max rounds) for the legacy round and PaSP.run."""
    from pamo_gb300 import synth
    from tests import meshes

    c1v, c1f = synth.star_mesh(32, 6, lambda l: 0.03, 0)
    return {
        "legacy_plain_small": (c1v, c1f, 1e-3, 1000),
        "legacy_sphere8": (*meshes.sphere(8, L=5, sigma=0.05, seed=3), 1e-3, 1000),
        "legacy_sphere12_rough": (*meshes.sphere(12, L=8, sigma=0.08, seed=21), 1e-3, 1000),
        "legacy_open_patch": (*meshes.open_patch(), 1e-3, 1000),
        "legacy_tangled": (*meshes.tangled(10, seed=9, amp=0.25), 1e-3, 1000),
        "legacy_high_threshold": (*meshes.sphere(10, L=6, sigma=0.06, seed=7), 5e-2, 1000),
    }


def digest(a: np.ndarray) -> np.ndarray:
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), dtype=np.uint8)


class RefRound:
    """ctypes view of oracle/_ref/libref_round_emu.so (one reference CUSimp_Free)."""

    def __init__(self, path: str):
        L = ctypes.CDLL(path)
        P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.ref_create.restype = P
        L.ref_destroy.argtypes = [P]
        L.ref_forward.argtypes = [P, P, P, P, I, I, I, F, F, I, I]
        L.ref_counts.argtypes = [P, P]
        L.ref_outputs.argtypes = [P, P, P, P, P, P]
        L.ref_collapsed.argtypes = [P, P]
        self.L = L
        self.h = ctypes.c_void_p(L.ref_create())

    def __del__(self):
        try:
            self.L.ref_destroy(self.h)
        except Exception:
            pass

    @staticmethod
    def _p(a):
        return a.ctypes.data_as(ctypes.c_void_p)

    def counts(self):
        c = np.zeros(5, np.int64)
        self.L.ref_counts(self.h, self._p(c))
        return c

    def forward(self, points, triangles, verts_undo, n_verts_undo, scale, threshold, is_stuck, init):
        pts = np.ascontiguousarray(points, np.float32)
        tri = np.ascontiguousarray(triangles, np.int32)
        und = np.ascontiguousarray(verts_undo, np.int32)
        if und.size == 0:
            und = np.zeros(1, np.int32)
        self.L.ref_forward(self.h, self._p(pts), self._p(tri), self._p(und), int(n_verts_undo), len(pts), len(tri),
                           float(scale), float(threshold), int(bool(is_stuck)), int(bool(init)))
        nP, nT, nU = (int(x) for x in self.counts()[:3])
        verts = np.zeros((nP, 3), np.float32)
        tris = np.zeros((nT, 3), np.int32)
        occ = np.zeros((nP, 1), np.int32)
        vmap = np.zeros((nP, 1), np.int32)
        undo = np.zeros(max(nU, 1), np.int32)
        self.L.ref_outputs(self.h, self._p(verts), self._p(tris), self._p(occ), self._p(vmap), self._p(undo))
        return verts, tris, occ, vmap, undo[:nU]

    def n_collapsed(self):
        return int(self.counts()[3])


class RefLegacy:
    """ctypes view of the legacy round in oracle/_ref/libref_round_emu.so (one reference CUSimp)."""

    def __init__(self, path: str):
        L = ctypes.CDLL(path)
        P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.ref_legacy_create.restype = P
        L.ref_legacy_destroy.argtypes = [P]
        L.ref_legacy_forward.argtypes = [P, P, P, I, I, F, F, I]
        L.ref_legacy_counts.argtypes = [P, P]
        L.ref_legacy_outputs.argtypes = [P, P, P, P, P]
        self.L = L
        self.h = ctypes.c_void_p(L.ref_legacy_create())

    def __del__(self):
        try:
            self.L.ref_legacy_destroy(self.h)
        except Exception:
            pass

    def forward_legacy(self, points, triangles, scale, threshold, init):
        p = RefRound._p
        pts = np.ascontiguousarray(points, np.float32)
        tri = np.ascontiguousarray(triangles, np.int32)
        self.L.ref_legacy_forward(self.h, p(pts), p(tri), len(pts), len(tri), float(scale), float(threshold),
                                  int(bool(init)))
        c = np.zeros(2, np.int64)
        self.L.ref_legacy_counts(self.h, p(c))
        nP, nT = int(c[0]), int(c[1])
        verts = np.zeros((nP, 3), np.float32)
        tris = np.zeros((nT, 3), np.int32)
        occ = np.zeros((nP, 1), np.int32)
        vmap = np.zeros((nP, 1), np.int32)
        self.L.ref_legacy_outputs(self.h, p(verts), p(tris), p(occ), p(vmap))
        return verts, tris, occ, vmap


def legacy_loop(op, points, triangles, threshold=1e-3, iters=1000, on_round=None):
    """PaSP.run (pamo/__init__.py:197-227) over an operator with CUDSP.forward's contract: no centring, stop at the
    first round without progress. on_round(r, outputs, faces_after_compaction). Returns (verts, faces)."""
    verts, faces = points, triangles
    ext = verts.max(0) - verts.min(0)
    scale = max(max(ext[0], ext[1]), ext[2])
    init = True
    for it in range(iters):
        n_prev = faces.shape[0]
        res = op.forward_legacy(verts, faces, scale, threshold, init)
        v_out, t_out, occ, vmap = res
        verts = v_out[occ.reshape(-1).astype(bool)]
        faces = t_out[t_out[:, 0] >= 0].copy()
        faces[:, 0] = vmap.reshape(-1)[faces[:, 0]]
        faces[:, 1] = vmap.reshape(-1)[faces[:, 1]]
        faces[:, 2] = vmap.reshape(-1)[faces[:, 2]]
        init = False
        if on_round is not None:
            on_round(it, res, faces)
        if faces.shape[0] == n_prev:
            break
    return verts, faces


def record_legacy(op, v, f, thr, iters):
    rows = []

    def on_round(r, res, faces):
        verts, tris, occ, vmap = res
        rows.append(([len(verts), len(tris), len(faces)], [digest(a) for a in res]))

    V, F = legacy_loop(op, v, f, thr, iters, on_round)
    return (np.array([c for c, _ in rows], np.int64), np.stack([np.stack(d) for _, d in rows]), V, F)


def centre(points: np.ndarray, triangles: np.ndarray):
    """PaMO.preprocess_mesh's mean (pamo/__init__.py:60-65, numpy float32) and the centred points (:117)."""
    tris = points[triangles]
    tris_mean = tris.mean(axis=1).mean(axis=0)
    return points - tris_mean, tris_mean


def stage2_loop(op, points, triangles, ratio, tolerance=4, threshold=1e-3, iters=1000000, min_verts=0,
                on_round=None):
    """The stage-2 loop of PaMO.run (pamo/__init__.py:96-158) over an operator with CUDSP_Free.forward's contract.

    on_round(r, outputs, faces_after_compaction, op, is_stuck) is called after every round, with the is_stuck flag
    the round ran with. Returns (verts, faces) as PaMO.run does (:161-162): the mean added back to the positions."""
    target = max(int(ratio * len(triangles)), min_verts)
    verts, tris_mean = centre(points, triangles)
    faces = triangles
    verts_undo = np.zeros(0, np.int32)
    n_verts_undo, count, is_stuck, init = 0, 0, 0, True
    ext = verts.max(0) - verts.min(0)
    scale = max(max(ext[0], ext[1]), ext[2])
    for it in range(iters):
        n_prev = faces.shape[0]
        res = op.forward(verts, faces, verts_undo, n_verts_undo, scale, threshold, is_stuck, init)
        stuck_used = is_stuck
        init = False
        v_out, t_out, occ, vmap, verts_undo = res
        n_verts_undo = verts_undo.shape[0]
        verts = v_out[occ.reshape(-1).astype(bool)]
        faces = t_out[t_out[:, 0] >= 0].copy()
        faces[:, 0] = vmap.reshape(-1)[faces[:, 0]]
        faces[:, 1] = vmap.reshape(-1)[faces[:, 1]]
        faces[:, 2] = vmap.reshape(-1)[faces[:, 2]]
        if on_round is not None:
            on_round(it, res, faces, op, stuck_used)
        n_cur = faces.shape[0]
        if n_cur <= target or n_cur <= 10:
            break
        if n_cur == n_prev:
            count += 1
        else:
            count = 0
            is_stuck = 0
        if count >= 2:
            is_stuck = 1
        if count == tolerance:
            break
    return verts + tris_mean, faces


def record(op, v, f, ratio, tol, thr, iters):
    rows = []

    def on_round(r, res, faces, o, stuck):
        verts, tris, occ, vmap, undo = res
        counts = [len(verts), len(tris), len(undo), o.n_collapsed(), len(faces), int(stuck)]
        rows.append((counts, [digest(a) for a in res]))

    V, F = stage2_loop(op, v, f, ratio, tol, thr, iters, 0, on_round)
    counts = np.array([c for c, _ in rows], np.int64)
    digests = np.stack([np.stack(d) for _, d in rows])  # [R, 5, 32]
    return counts, digests, V, F


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--check", action="store_true", help="also compare the oracle with the reference per round")
    ap.add_argument("--only", default="", help="comma-separated case names")
    args = ap.parse_args()
    from oracle import build_ref

    lib = build_ref.build_round_emu()
    out = {}
    sel = set(args.only.split(",")) if args.only else None
    for name, (v, f, ratio, tol, thr, iters) in cases().items():
        if sel and name not in sel:
            continue
        counts, digests, V, F = record(RefRound(lib), v, f, ratio, tol, thr, iters)
        out[f"{name}.input"] = np.concatenate([digest(np.ascontiguousarray(v, np.float32)),
                                               digest(np.ascontiguousarray(f, np.int32))])
        out[f"{name}.params"] = np.array([ratio, tol, thr, iters], np.float64)
        out[f"{name}.counts"] = counts
        out[f"{name}.digests"] = digests
        out[f"{name}.final_verts"] = V
        out[f"{name}.final_faces"] = F
        print(f"{name}: {len(f)} -> {len(F)} faces in {len(counts)} rounds, {int(counts[:, 5].sum())} stuck; "
              f"undo vertices per round {counts[:, 2].tolist()[:12]}")
        if args.check:
            from oracle import oracle as orc

            oc, od, OV, OF = record(_OracleOp(orc.Oracle()), v, f, ratio, tol, thr, iters)
            same = oc.shape == counts.shape and np.array_equal(oc, counts) and np.array_equal(od, digests)
            if not same:
                r = next((i for i in range(min(len(oc), len(counts)))
                          if not (np.array_equal(oc[i], counts[i]) and np.array_equal(od[i], digests[i]))), None)
                print(f"  oracle differs: first at round {r}: ref {counts[r] if r is not None else counts.shape} "
                      f"oracle {oc[r] if r is not None else oc.shape}; outputs differing: "
                      f"{[OUTPUT_NAMES[k] for k in range(5) if r is not None and not np.array_equal(od[r, k], digests[r, k])]}")
            else:
                print("  oracle identical")
    for name, (v, f, thr, iters) in legacy_cases().items():
        if sel and name not in sel:
            continue
        counts, digests, V, F = record_legacy(RefLegacy(lib), v, f, thr, iters)
        out[f"{name}.input"] = np.concatenate([digest(np.ascontiguousarray(v, np.float32)),
                                               digest(np.ascontiguousarray(f, np.int32))])
        out[f"{name}.params"] = np.array([thr, iters], np.float64)
        out[f"{name}.counts"] = counts
        out[f"{name}.digests"] = digests
        out[f"{name}.final_verts"] = V
        out[f"{name}.final_faces"] = F
        print(f"{name}: {len(f)} -> {len(F)} faces in {len(counts)} rounds")
        if args.check:
            from oracle import oracle as orc

            oc, od, OV, OF = record_legacy(orc.Oracle(), v, f, thr, iters)
            same = oc.shape == counts.shape and np.array_equal(oc, counts) and np.array_equal(od, digests)
            if not same:
                r = next((i for i in range(min(len(oc), len(counts)))
                          if not (np.array_equal(oc[i], counts[i]) and np.array_equal(od[i], digests[i]))), None)
                print(f"  oracle differs: first at round {r} of {len(counts)}: ref {counts[r] if r is not None else counts.shape} "
                      f"oracle {oc[r] if r is not None else oc.shape}")
            else:
                print("  oracle identical")
    if not args.only:
        np.savez_compressed(OUT, **out)
        print("wrote", OUT)


class _OracleOp:
    def __init__(self, o):
        self.o = o

    def forward(self, *a):
        return self.o.forward(*a)

    def n_collapsed(self):
        return self.o.counts()["n_collapsed"]


if __name__ == "__main__":
    main()
