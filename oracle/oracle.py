"""ctypes wrapper of the CPU oracle (oracle/pamo_oracle.cpp).

Test infrastructure only: used as the checker by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline; the product path never imports it.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import build as _build

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(_build.build())
        P, I, F, D, LL = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_longlong
        L.oracle_create.restype = P
        L.oracle_destroy.argtypes = [P]
        L.oracle_set_threads.argtypes = [P, I]
        L.oracle_forward.argtypes = [P, P, P, P, I, I, I, F, F, I, I]
        L.oracle_counts.argtypes = [P, P]
        L.oracle_forward_legacy.argtypes = [P, P, P, I, I, F, F, I]
        L.oracle_outputs.argtypes = [P, P, P, P, P, P]
        L.oracle_collapsed.argtypes = [P, P]
        L.oracle_edge_costs.argtypes = [P, P]
        L.oracle_edges.argtypes = [P, P]
        L.oracle_shuffle_perm.argtypes = [LL, P]
        L.oracle_pair_intersects.argtypes = [P, P, P, F]
        L.oracle_tris_mean.argtypes = [P, P, I, P]
        L.oracle_run.argtypes = [P, P, P, I, I, D, I, F, I, LL, P, P]
        L.oracle_run_result.argtypes = [P, P, P, P]
        L.oracle_run_round_seconds.argtypes = [P, P, I]
        L.oracle_run_round_seconds.restype = I
        L.oracle_run_blender.argtypes = [P, P, P, I, I, F, P, P]
        L.oracle_self_intersect.argtypes = [P, P, P, I, I, P]
        L.oracle_self_intersect.restype = LL
        L.check_self_intersections.argtypes = [P, I, P, I, P, I]
        L.check_self_intersections.restype = LL
        L.check_self_intersections_all_pairs.argtypes = [P, I, P, I]
        L.check_self_intersections_all_pairs.restype = LL
        L.hausdorff.argtypes = [P, I, P, I, P, I, P, I, P]
        L.hausdorff.restype = D
        L.cpu_qem_simplify.argtypes = [P, I, P, I, LL, D, P]
        L.oracle_cost_fp64.argtypes = [P, P, I, I, P, I, D, D, I, I, P, P]
        L.oracle_cost_fp64.restype = I
        L.cpu_qem_simplify.restype = LL
        L.exact_orient3d.argtypes = [P]
        L.exact_orient3d.restype = I
        L.s3_oracle_run.argtypes = [P, P, I, I, P, P, I, I, I, P, P, P]
        L.s3_oracle_probe.argtypes = [P, P, I, I, P, P, I, I, P, P, P, P, P, P, P, P, P]
        L.s3_oracle_energy_at.argtypes = [P, P, I, I, P, P, I, I, P, P, P, P]
        _LIB = L
    return _LIB


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def shuffle_perm(m: int) -> np.ndarray:
    out = np.zeros(m, np.int32)
    lib().oracle_shuffle_perm(m, _p(out))
    return out


def pair_intersects(points: np.ndarray, cur, qry, eps: float = 1e-3) -> bool:
    pts = np.ascontiguousarray(points, np.float32)
    c = np.ascontiguousarray(cur, np.int32)
    q = np.ascontiguousarray(qry, np.int32)
    return bool(lib().oracle_pair_intersects(_p(pts), _p(c), _p(q), eps))


def tris_mean(points: np.ndarray, tris: np.ndarray) -> np.ndarray:
    out = np.zeros(3, np.float32)
    p = np.ascontiguousarray(points, np.float32)
    t = np.ascontiguousarray(tris, np.int32)
    lib().oracle_tris_mean(_p(p), _p(t), len(t), _p(out))
    return out


class Oracle:
    """Stateful CPU restatement of one reference CUSimp_Free (simp_cuda/src/cusimp_free.cu:891-1048)."""

    COUNT_KEYS = ["n_pts", "n_tris", "n_vertices_undo", "n_edges", "n_win", "n_collapsed", "n_considered", "passes",
                  "n_intersect_pairs", "status"]

    def __init__(self, threads: int = 1):
        self._h = ctypes.c_void_p(lib().oracle_create())
        lib().oracle_set_threads(self._h, threads)

    def __del__(self):
        try:
            if self._h:
                lib().oracle_destroy(self._h)
        except Exception:
            pass

    def forward_legacy(self, points, triangles, scale, threshold, init):
        """One round of the legacy CUSimp (simp_cuda/src/cusimp.cu:587-720): (verts, tris, occ, map)."""
        pts = np.ascontiguousarray(points, np.float32)
        tri = np.ascontiguousarray(triangles, np.int32)
        lib().oracle_forward_legacy(self._h, _p(pts), _p(tri), len(pts), len(tri), float(scale), float(threshold),
                                    int(bool(init)))
        nP, nT = len(pts), len(tri)
        verts = np.zeros((nP, 3), np.float32)
        tris = np.zeros((nT, 3), np.int32)
        occ = np.zeros((nP, 1), np.int32)
        vmap = np.zeros((nP, 1), np.int32)
        undo = np.zeros(1, np.int32)
        lib().oracle_outputs(self._h, _p(verts), _p(tris), _p(occ), _p(vmap), _p(undo))
        return verts, tris, occ, vmap

    def run_legacy(self, points, triangles, threshold=0.001, iters=1000):
        """PaSP.run (simp_cuda/pamo/__init__.py:197-227): (verts, faces, rounds)."""
        v = np.ascontiguousarray(points, np.float32)
        f = np.ascontiguousarray(triangles, np.int32)
        ext = v.max(0) - v.min(0)
        scale = max(max(ext[0], ext[1]), ext[2])
        rounds = 0
        for it in range(iters):
            n0 = len(f)
            verts, tris, occ, vmap = self.forward_legacy(v, f, scale, threshold, it == 0)
            rounds = it + 1
            v = verts[occ[:, 0].astype(bool)]
            f = vmap[:, 0][tris[tris[:, 0] >= 0]].astype(np.int32)
            if len(f) == n0:
                break
        return v, f, rounds

    def forward(self, points, triangles, verts_undo, n_verts_undo, scale, threshold, is_stuck, init):
        pts = np.ascontiguousarray(points, np.float32)
        tri = np.ascontiguousarray(triangles, np.int32)
        und = np.ascontiguousarray(verts_undo, np.int32)
        if und.size == 0:
            und = np.zeros(1, np.int32)
        lib().oracle_forward(self._h, _p(pts), _p(tri), _p(und), int(n_verts_undo), len(pts), len(tri), float(scale),
                             float(threshold), int(bool(is_stuck)), int(bool(init)))
        c = self.counts()
        nP, nT, nU = c["n_pts"], c["n_tris"], c["n_vertices_undo"]
        verts = np.zeros((nP, 3), np.float32)
        tris = np.zeros((nT, 3), np.int32)
        occ = np.zeros((nP, 1), np.int32)
        vmap = np.zeros((nP, 1), np.int32)
        undo = np.zeros(max(nU, 1), np.int32)
        lib().oracle_outputs(self._h, _p(verts), _p(tris), _p(occ), _p(vmap), _p(undo))
        return verts, tris, occ, vmap, undo[:nU]

    def counts(self) -> dict:
        c = np.zeros(10, np.int64)
        lib().oracle_counts(self._h, _p(c))
        return {k: int(v) for k, v in zip(self.COUNT_KEYS, c)}

    def collapsed(self) -> np.ndarray:
        n = self.counts()["n_collapsed"]
        out = np.zeros(max(n, 1), np.int32)
        lib().oracle_collapsed(self._h, _p(out))
        return out[:n]

    def edges(self) -> np.ndarray:
        n = self.counts()["n_edges"]
        out = np.zeros((max(n, 1), 2), np.int32)
        lib().oracle_edges(self._h, _p(out))
        return out[:n]

    def edge_costs(self) -> np.ndarray:
        n = self.counts()["n_edges"]
        out = np.zeros(max(n, 1), np.uint32)
        lib().oracle_edge_costs(self._h, _p(out))
        return out[:n]

    def self_intersect(self, points, triangles):
        """Per-face flags of the reference's global self-intersection check; returns (flags, hit tests)."""
        pts = np.ascontiguousarray(points, np.float32)
        tri = np.ascontiguousarray(triangles, np.int32)
        out = np.zeros(len(tri), np.uint8)
        n = lib().oracle_self_intersect(self._h, _p(pts), _p(tri), len(pts), len(tri), _p(out))
        return out, int(n)

    def run(self, points, triangles, ratio, tolerance=4, threshold=1e-3, iters=1000000, min_verts=10000000000):
        """The stage-2 loop of PaMO.run: returns (verts, faces, faces_per_round)."""
        pts = np.ascontiguousarray(points, np.float32)
        tri = np.ascontiguousarray(triangles, np.int32)
        onp, ont = ctypes.c_int(), ctypes.c_int()
        rounds = lib().oracle_run(self._h, _p(pts), _p(tri), len(pts), len(tri), float(ratio), int(tolerance),
                                  float(threshold), int(iters), int(min_verts), ctypes.byref(onp), ctypes.byref(ont))
        V = np.zeros((onp.value, 3), np.float32)
        F = np.zeros((ont.value, 3), np.int32)
        fpr = np.zeros(max(rounds, 1), np.int32)
        lib().oracle_run_result(self._h, _p(V), _p(F), _p(fpr))
        return V, F, fpr[:rounds]

    def round_seconds(self) -> np.ndarray:
        """Wall time of each round of the last run()/run_blender() (seconds)."""
        n = lib().oracle_run_round_seconds(self._h, None, 0)
        out = np.zeros(max(n, 1), np.float64)
        lib().oracle_run_round_seconds(self._h, _p(out), n)
        return out[:n]

    def run_blender(self, points, triangles, threshold=1e-3):
        """The Blender add-on's pamo_simplify loop: returns (verts, faces, faces_per_round)."""
        pts = np.ascontiguousarray(points, np.float32)
        tri = np.ascontiguousarray(triangles, np.int32)
        onp, ont = ctypes.c_int(), ctypes.c_int()
        rounds = lib().oracle_run_blender(self._h, _p(pts), _p(tri), len(pts), len(tri), float(threshold),
                                          ctypes.byref(onp), ctypes.byref(ont))
        V = np.zeros((onp.value, 3), np.float32)
        F = np.zeros((ont.value, 3), np.int32)
        fpr = np.zeros(max(rounds, 1), np.int32)
        lib().oracle_run_result(self._h, _p(V), _p(F), _p(fpr))
        return V, F, fpr[:rounds]


# ------------------------------------------------------------------------------------------ stage 3
STAGE3_PARAMS = ["n_newton_iters", "n_cg_iters", "n_line_search_iters", "d_hat", "coll_stiffness",
                 "contact_detection_radius", "ee_classify_thres", "ccd_slackness", "ccd_thickness", "ccd_max_iters",
                 "spd_max_iters", "elas_young_modulus", "elas_poisson_ratio", "hinge_stiffness",
                 "mesh2gt_dist_stiffness", "min_angle_thres", "max_blocks"]
STAGE3_DEFAULTS = dict(n_newton_iters=10, n_cg_iters=40, n_line_search_iters=10, d_hat=1e-3, coll_stiffness=1e2,
                       contact_detection_radius=1e-2, ee_classify_thres=1e-3, ccd_slackness=0.7, ccd_thickness=1e-6,
                       ccd_max_iters=100, spd_max_iters=3, elas_young_modulus=0.1, elas_poisson_ratio=0.0,
                       hinge_stiffness=1e-2, mesh2gt_dist_stiffness=1e3, min_angle_thres=0.0, max_blocks=1 << 25)
STAGE3_STATS = ["particles", "triangles", "edges", "hinges", "steps", "newton_iters", "max_contacts",
                "radius_halvings", "do_nothing", "energy", "total_contacts"]  # the oracle's 11 entries


def _s3_args(gt_V, gt_F, V, F, params):
    P = dict(STAGE3_DEFAULTS)
    P.update(params or {})
    prm = np.array([float(P[k]) for k in STAGE3_PARAMS], np.float64)
    gv = np.ascontiguousarray(gt_V, np.float64)
    gf = np.ascontiguousarray(gt_F, np.int32)
    v = np.ascontiguousarray(V, np.float64)
    f = np.ascontiguousarray(F, np.int32)
    return gv, gf, v, f, prm


def stage3_run(gt_V, gt_F, V, F, n_iters: int, params: dict | None = None):
    """Float64 restatement of process(gt_V, gt_F, V, F, n_iters): returns (V_out float64, stats dict)."""
    gv, gf, v, f, prm = _s3_args(gt_V, gt_F, V, F, params)
    out = np.zeros_like(v)
    st = np.zeros(len(STAGE3_STATS), np.float64)
    rc = lib().s3_oracle_run(_p(gv), _p(gf), len(gv), len(gf), _p(v), _p(f), len(v), len(f), int(n_iters), _p(prm),
                             _p(out), _p(st))
    if rc:
        raise RuntimeError(f"stage-3 oracle failed with status {rc}")
    return out, dict(zip(STAGE3_STATS, st.tolist()))


def _opt(x):
    return (None, None) if x is None else (np.ascontiguousarray(x, np.float64),) * 2


def stage3_probe(gt_V, gt_F, V, F, dx, params: dict | None = None, x0=None):
    """Energy, dE/dq, Hessian diagonal and H dx at x0 (normalised frame; None: the registered mesh)."""
    gv, gf, v, f, prm = _s3_args(gt_V, gt_F, V, F, params)
    x0a, _ = _opt(x0)
    dxa = np.ascontiguousarray(dx, np.float64)
    qn, g, h, hv = (np.zeros_like(v) for _ in range(4))
    e = np.zeros(1, np.float64)
    nc = ctypes.c_int(0)
    rc = lib().s3_oracle_probe(_p(gv), _p(gf), len(gv), len(gf), _p(v), _p(f), len(v), len(f), _p(prm),
                               None if x0a is None else _p(x0a), _p(dxa),
                               _p(qn), _p(e), _p(g), _p(h), _p(hv), ctypes.byref(nc))
    if rc:
        raise RuntimeError(f"stage-3 oracle probe failed with status {rc}")
    return dict(q=qn, energy=float(e[0]), grad=g, hdiag=h, hvp=hv, n_contacts=nc.value)


def stage3_energy_at(gt_V, gt_F, V, F, x, params: dict | None = None, x0=None) -> float:
    """Energy at x (normalised frame) with the targets and contacts of stage3_probe at x0."""
    gv, gf, v, f, prm = _s3_args(gt_V, gt_F, V, F, params)
    x0a, _ = _opt(x0)
    xa = np.ascontiguousarray(x, np.float64)
    e = np.zeros(1, np.float64)
    rc = lib().s3_oracle_energy_at(_p(gv), _p(gf), len(gv), len(gf), _p(v), _p(f), len(v), len(f), _p(prm),
                                   None if x0a is None else _p(x0a), _p(xa), _p(e))
    if rc:
        raise RuntimeError(f"stage-3 oracle energy failed with status {rc}")
    return float(e[0])


def exact_orient3d(a, b, c, d) -> int:
    """Sign of det[a-d; b-d; c-d], exact for double inputs (expansion arithmetic)."""
    p = np.ascontiguousarray(np.concatenate([a, b, c, d]), np.float64)
    return int(lib().exact_orient3d(_p(p)))


def self_intersections(points, tris, max_pairs: int = 64):
    """(count, pairs [k,2]) of face pairs of the mesh that meet beyond their shared vertices and edge, decided
    with exact orientation predicates."""
    P = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
    T = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
    pairs = np.zeros((max(max_pairs, 1), 2), np.int32)
    n = int(lib().check_self_intersections(_p(P), len(P), _p(T), len(T), _p(pairs), max_pairs))
    if n < 0:
        raise ValueError("triangle index out of range")
    return n, pairs[: min(n, max_pairs)]


def self_intersections_all_pairs(points, tris) -> int:
    """The same count as self_intersections, testing every pair of faces (small meshes only)."""
    P = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
    T = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
    return int(lib().check_self_intersections_all_pairs(_p(P), len(P), _p(T), len(T)))


def hausdorff(va, fa, vb, fb):
    """(two-sided, A->B, B->A) vertex Hausdorff distances between two triangle meshes."""
    A = np.ascontiguousarray(va, np.float64).reshape(-1, 3)
    B = np.ascontiguousarray(vb, np.float64).reshape(-1, 3)
    FA = np.ascontiguousarray(fa, np.int32).reshape(-1, 3)
    FB = np.ascontiguousarray(fb, np.int32).reshape(-1, 3)
    out = np.zeros(2, np.float64)
    h = lib().hausdorff(_p(A), len(A), _p(FA), len(FA), _p(B), len(B), _p(FB), len(FB), _p(out))
    return float(h), float(out[0]), float(out[1])


def cost_fp64(points, tris, edges, scale: float, threshold: float, optimal: bool = False, threads: int = 0):
    """The reference's edge cost of each edge (u, v) in float64, before clamp and quantisation, with its placement
    (the midpoint, or the quadric's minimiser with optimal): (cost [E], place [E,3])."""
    import os

    P = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    T = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
    E = np.ascontiguousarray(edges, np.int32).reshape(-1, 2)
    cost = np.zeros(len(E), np.float64)
    place = np.zeros((len(E), 3), np.float64)
    rc = lib().oracle_cost_fp64(_p(P), _p(T), len(P), len(T), _p(E), len(E), float(scale), float(threshold),
                                int(bool(optimal)), int(threads or os.cpu_count() or 1), _p(cost), _p(place))
    if rc:
        raise ValueError("triangle index out of range")
    return cost, place


def cpu_qem(points, tris, target_faces: int, time_budget_s: float = 0.0):
    """The sequential priority-queue QEM baseline (oracle/cpu_qem.cpp): (collapses, faces left)."""
    P = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    T = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
    left = ctypes.c_longlong()
    n = lib().cpu_qem_simplify(_p(P), len(P), _p(T), len(T), int(target_faces), float(time_budget_s),
                               ctypes.byref(left))
    return int(n), int(left.value)
