"""Small test meshes shared by the tests."""

import numpy as np

from pamo_gb300 import synth


def octahedron():
    v = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    f = np.array([[0, 2, 4], [2, 1, 4], [1, 3, 4], [3, 0, 4], [2, 0, 5], [1, 2, 5], [3, 1, 5], [0, 3, 5]], np.int32)
    return v, f


def sphere(n, L=4, sigma=0.03, seed=1):
    return synth.star_mesh(n, L, lambda l: sigma, seed)


def open_patch(n=12, seed=3):
    """A bumpy open grid (has boundary edges)."""
    rng = np.random.default_rng(seed)
    xs, ys = np.meshgrid(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1), indexing="ij")
    z = 0.05 * np.sin(3 * xs) * np.cos(2 * ys) + 0.002 * rng.standard_normal(xs.shape)
    v = np.stack([xs, ys, z], -1).reshape(-1, 3).astype(np.float32)
    idx = np.arange((n + 1) * (n + 1)).reshape(n + 1, n + 1)
    a, b, c, d = idx[:-1, :-1].ravel(), idx[1:, :-1].ravel(), idx[1:, 1:].ravel(), idx[:-1, 1:].ravel()
    f = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)]).astype(np.int32)
    return v, f


def euler(f):
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    ne = len(np.unique(e, axis=0))
    nv = len(np.unique(f))
    return nv - ne + len(f)


def with_degenerate_face(seed=5):
    """A sphere with one face whose vertex repeats (index-degenerate)."""
    v, f = sphere(5, seed=seed)
    f = f.copy()
    f[7] = [f[7, 0], f[7, 0], f[7, 2]]
    return v, f


def with_coincident_edge(seed=6):
    """A sphere where one edge has both endpoints at the same position (zero length)."""
    v, f = sphere(5, seed=seed)
    v = v.copy()
    a, b = f[11, 0], f[11, 1]
    v[b] = v[a]
    return v, f


def tangled(n=8, seed=9, frac=0.08, amp=0.25):
    """A sphere with a fraction of vertices moved in random directions by up to `amp` (about two edge
    lengths at n = 10), which folds the surface so that faces intersect."""
    rng = np.random.default_rng(seed)
    v, f = sphere(n, seed=seed)
    v = v.copy()
    pick = rng.choice(len(v), max(1, int(frac * len(v))), replace=False)
    v[pick] += rng.uniform(-amp, amp, (len(pick), 3)).astype(np.float32)
    return v, f


def sheet_pair(n=8, gap=0.0006, shift=0.031, seed=1):
    """Two parallel square grids (n x n vertices each) a small gap apart, slightly shifted in the plane, so
    that point-triangle and edge-edge pairs across the gap are inside the contact barrier's range."""
    def grid(z, off):
        xs = np.linspace(0, 1, n)
        X, Y = np.meshgrid(xs, xs, indexing="ij")
        V = np.stack([X.ravel() + off, Y.ravel() + off * 0.7, np.full(n * n, z)], 1)
        F = []
        for i in range(n - 1):
            for j in range(n - 1):
                a, b, c, d = i * n + j, (i + 1) * n + j, (i + 1) * n + j + 1, i * n + j + 1
                F += [(a, b, c), (a, c, d)]
        return V, np.array(F, dtype=np.int32)

    V1, F1 = grid(0.0, 0.0)
    V2, F2 = grid(gap, shift)
    V = np.vstack([V1, V2])
    F = np.vstack([F1, F2 + len(V1)]).astype(np.int32)
    rng = np.random.default_rng(seed)
    V = V + rng.normal(0, 5e-5, V.shape) * np.array([1.0, 1.0, 0.0])
    return V, F


def stage3_pair(n_gt=16, n_mesh=6, noise=0.003, seed=11):
    """A fine star-shaped GT mesh and a coarse, inflated and jittered star mesh of the same shape, as the
    stage-2 output a projection starts from (float64)."""
    GV, GF = synth.star_mesh(n_gt, 4, lambda l: 0.04, seed)
    V, F = synth.star_mesh(n_mesh, 4, lambda l: 0.04, seed)
    rng = np.random.default_rng(seed + 1)
    V = V.astype(np.float64) * 1.02 + rng.normal(0, noise, V.shape)
    return GV.astype(np.float64), GF, V, F
