"""Seeded synthetic star-shaped genus-0 meshes.

A geodesic icosphere of frequency ``n`` (each icosahedron face split into n^2 triangles and projected to
the unit sphere: V = 10 n^2 + 2, F = 20 n^2) whose radius is perturbed by real orthonormal spherical
harmonics, r(theta, phi) = 1 + sum_{l=1..L} sum_{m=-l..l} c_lm Y_lm(theta, phi), with the coefficients drawn
from ``numpy.random.default_rng(seed)`` (in the order l = 1..L, m = -l..l) and redrawn while min r < 0.2.
Vertices are float32 xyz, faces int32 with outward counter-clockwise winding. Because every vertex lies on
its own ray from the origin and every face keeps a positive orientation with respect to the origin, the
surface is star-shaped and free of self-intersections.

Frequency 32 is the level-5 subdivided icosahedron (10 242 V / 20 480 F); frequency 512 is level 9
(2 621 442 V / 5 242 880 F).
"""

from __future__ import annotations

import math

import numpy as np

__all__ = ["icosphere", "sh_radius", "star_mesh", "config_mesh", "frequency_for_faces"]

_PHI = (1.0 + math.sqrt(5.0)) / 2.0


def _icosahedron():
    v = []
    for a in (-1.0, 1.0):
        for b in (-_PHI, _PHI):
            v += [(0.0, a, b), (a, b, 0.0), (b, 0.0, a)]
    v = np.array(v, dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    d = np.linalg.norm(v[:, None, :] - v[None, :, :], axis=2)
    edge = d[d > 1e-9].min()
    faces = []
    for i in range(12):
        for j in range(i + 1, 12):
            for k in range(j + 1, 12):
                if abs(d[i, j] - edge) < 1e-9 and abs(d[j, k] - edge) < 1e-9 and abs(d[i, k] - edge) < 1e-9:
                    n = np.cross(v[j] - v[i], v[k] - v[i])
                    faces.append((i, j, k) if n @ (v[i] + v[j] + v[k]) > 0 else (i, k, j))
    faces = np.array(faces, dtype=np.int64)
    assert faces.shape == (20, 3)
    return v, faces


def icosphere(n: int):
    """Unit geodesic icosphere of frequency ``n``: returns (float64 [V,3], int32 [F,3]), outward CCW."""
    if n < 1:
        raise ValueError("frequency must be >= 1")
    base, bfaces = _icosahedron()
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    mask = ii + jj <= n
    ii, jj = ii[mask], jj[mask]
    npts = ii.size
    lid = -np.ones((n + 1, n + 1), dtype=np.int64)
    lid[ii, jj] = np.arange(npts)
    # local lattice triangles (shared by all 20 faces)
    tri = []
    for i in range(n):
        j = np.arange(n - i)
        tri.append(np.stack([lid[i, j], lid[i + 1, j], lid[i, j + 1]], axis=1))
        j = np.arange(n - i - 1)
        if j.size:
            tri.append(np.stack([lid[i + 1, j], lid[i + 1, j + 1], lid[i, j + 1]], axis=1))
    tri = np.concatenate(tri, axis=0)
    keys = np.empty((20, npts), dtype=np.int64)
    vid_w = []
    for f, (a, b, c) in enumerate(bfaces):
        vid = np.stack([np.full(npts, a), np.full(npts, b), np.full(npts, c)], axis=1)
        w = np.stack([n - ii - jj, ii, jj], axis=1)
        vid = np.where(w > 0, vid, 12)
        order = np.argsort(vid, axis=1, kind="stable")
        vid = np.take_along_axis(vid, order, axis=1)
        w = np.take_along_axis(w, order, axis=1)
        keys[f] = ((vid[:, 0] * 13 + vid[:, 1]) * 13 + vid[:, 2]) * (n + 1) ** 2 + w[:, 0] * (n + 1) + w[:, 1]
        vid_w.append((vid, w))
    uk, first, inv = np.unique(keys.ravel(), return_index=True, return_inverse=True)
    inv = inv.reshape(20, npts)
    allvid = np.concatenate([vw[0] for vw in vid_w], axis=0)[first]
    allw = np.concatenate([vw[1] for vw in vid_w], axis=0)[first].astype(np.float64)
    padded = np.concatenate([base, np.zeros((1, 3))], axis=0)
    pos = (allw[:, :, None] * padded[allvid]).sum(axis=1)
    pos /= np.linalg.norm(pos, axis=1, keepdims=True)
    faces = np.concatenate([inv[f][tri] for f in range(20)], axis=0).astype(np.int32)
    assert pos.shape[0] == 10 * n * n + 2 and faces.shape[0] == 20 * n * n
    return pos, faces


def sh_radius(dirs: np.ndarray, coeffs: dict) -> np.ndarray:
    """1 + sum c_lm Y_lm at unit directions ``dirs`` [N,3]; ``coeffs`` maps (l, m) -> c_lm.

    Real orthonormal harmonics: Y_l0 = P_l^0, Y_lm = sqrt(2) P_l^m cos(m phi) (m > 0),
    Y_l,-m = sqrt(2) P_l^m sin(m phi), with P_l^m the associated Legendre functions normalised so that
    each Y_lm has unit L2 norm on the sphere.
    """
    x, y, z = dirs[:, 0], dirs[:, 1], np.clip(dirs[:, 2], -1.0, 1.0)
    st = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = np.arctan2(y, x)
    L = max((l for l, _ in coeffs), default=0)
    r = np.ones_like(z)
    pmm = np.full_like(z, math.sqrt(1.0 / (4.0 * math.pi)))
    for m in range(0, L + 1):
        if m > 0:
            pmm = -math.sqrt((2.0 * m + 1.0) / (2.0 * m)) * st * pmm
        cm, sm = (np.cos(m * phi), np.sin(m * phi)) if m > 0 else (None, None)
        p_lm2, p_lm1 = None, pmm
        for l in range(m, L + 1):
            if l == m:
                p = pmm
            elif l == m + 1:
                p = math.sqrt(2.0 * m + 3.0) * z * pmm
            else:
                a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
                b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
                p = a * (z * p_lm1 - b * p_lm2)
            if l >= 1:
                if m == 0:
                    r += coeffs.get((l, 0), 0.0) * p
                else:
                    r += coeffs.get((l, m), 0.0) * math.sqrt(2.0) * p * cm
                    r += coeffs.get((l, -m), 0.0) * math.sqrt(2.0) * p * sm
            if l > m:
                p_lm2, p_lm1 = p_lm1, p
            else:
                p_lm1 = p
    return r


def _draw(rng, L, sigma):
    c = {}
    for l in range(1, L + 1):
        s = sigma(l)
        for m in range(-l, l + 1):
            c[(l, m)] = float(rng.normal(0.0, s))
    return c


def star_mesh(n: int, L: int, sigma, seed: int, min_radius: float = 0.2):
    """Star-shaped mesh: icosphere(n) with radius 1 + SH(l <= L), c_lm ~ N(0, sigma(l)^2), seeded.

    Returns (float32 [V,3], int32 [F,3]).
    """
    dirs, faces = icosphere(n)
    rng = np.random.default_rng(seed)
    while True:
        coeffs = _draw(rng, L, sigma)
        r = sh_radius(dirs, coeffs)
        if r.min() >= min_radius:
            break
    pts = (dirs * r[:, None]).astype(np.float32)
    return pts, faces


def frequency_for_faces(nfaces: float) -> int:
    """Icosphere frequency whose face count 20 n^2 is nearest to ``nfaces``."""
    return max(1, int(round(math.sqrt(nfaces / 20.0))))


def config_mesh(name: str, seed: int = 0):
    """Input meshes of the benchmark configurations.

    ``plain_small``: frequency 32 (level 5), L = 6, c ~ N(0, 0.03^2).
    ``plain_large``: frequency 512 (level 9), L = 16, c_lm ~ N(0, (0.05 / l)^2).
    """
    if name == "plain_small":
        return star_mesh(32, 6, lambda l: 0.03, seed)
    if name == "plain_large":
        return star_mesh(512, 16, lambda l: 0.05 / l, seed)
    raise KeyError(name)


def is_star_shaped(pts: np.ndarray, faces: np.ndarray) -> bool:
    """True when every face has positive orientation seen from the origin (det[v0, v1, v2] > 0)."""
    p = pts.astype(np.float64)
    a, b, c = p[faces[:, 0]], p[faces[:, 1]], p[faces[:, 2]]
    return bool((np.einsum("ij,ij->i", a, np.cross(b, c)) > 0).all())
