"""The output checks of oracle/mesh_check.cpp: exact orientation predicates, the self-intersection count of
a mesh and the two-sided Hausdorff distance, against exact rational arithmetic, hand-made configurations and
brute force."""

from fractions import Fraction

import numpy as np
import pytest

from oracle import oracle as orc
from tests import meshes


def _orient3d_exact(a, b, c, d):
    a, b, c, d = ([Fraction(float(x)) for x in p] for p in (a, b, c, d))
    m = [[a[i] - d[i] for i in range(3)], [b[i] - d[i] for i in range(3)], [c[i] - d[i] for i in range(3)]]
    det = (m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0])
           + m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]))
    return (det > 0) - (det < 0)


def test_orient3d_is_exact_near_degenerate():
    rng = np.random.default_rng(0)
    disagree_naive = 0
    for _ in range(400):
        a, b, c = rng.uniform(-1, 1, (3, 3)) * 10.0 ** rng.integers(-3, 4)
        w = rng.uniform(0, 1, 3)
        w /= w.sum()
        d = w[0] * a + w[1] * b + w[2] * c  # on the plane up to rounding
        d = d + np.spacing(d) * rng.integers(-2, 3, 3)
        want = _orient3d_exact(a, b, c, d)
        assert orc.exact_orient3d(a, b, c, d) == want
        naive = np.linalg.det(np.stack([a - d, b - d, c - d]))
        disagree_naive += int(np.sign(naive) != want)
    assert disagree_naive > 0  # the cases are hard enough that a plain double determinant gets some wrong


def _count(V, F):
    n, _ = orc.self_intersections(V, F)
    assert n == orc.self_intersections_all_pairs(V, F)
    return n


T0 = [[0, 0, 0], [1, 0, 0], [0, 1, 0]]


@pytest.mark.parametrize("d,want", [
    ([0.3, 0.3, 0.0], 1),    # common edge, coplanar, same side: folded over
    ([0.3, -0.3, 0.0], 0),   # coplanar, opposite sides: a flat pair
    ([0.3, 0.3, 0.5], 0),    # a dihedral angle
])
def test_common_edge(d, want):
    V = np.array(T0 + [d], np.float64)
    assert _count(V, np.array([[0, 1, 2], [0, 1, 3]])) == want


@pytest.mark.parametrize("pts,want", [
    ([[0.2, 0.5, 0.0], [0.5, 0.2, 0.0]], 1),    # common vertex, coplanar, overlapping
    ([[-0.2, -0.5, 0.0], [-0.5, -0.2, 0.0]], 0),  # coplanar, touching only at the vertex
    ([[0.6, 0.2, 0.5], [0.2, 0.6, -0.5]], 1),   # piercing: the second face crosses the first's interior
    ([[0.6, 0.2, 0.5], [0.2, 0.6, 0.5]], 0),    # leaning away, touching at the vertex
    ([[0.5, 0.0, 0.0], [0.2, 0.0, 0.7]], 1),    # an edge of the second along an edge of the first
])
def test_common_vertex(pts, want):
    V = np.array(T0 + pts, np.float64)
    assert _count(V, np.array([[0, 1, 2], [0, 3, 4]])) == want


def test_disjoint_faces_touching_and_one_ulp_apart():
    T = np.array(T0, np.float64) + [0.0, 0.0, 0.5]
    V = np.vstack([T, [[0.25, 0.25, 0.5], [0.25, 0.3, 1.5], [0.3, 0.25, 1.5]]])
    F = np.array([[0, 1, 2], [3, 4, 5]])
    assert _count(V, F) == 1  # a vertex on the other face's interior
    V[3, 2] = np.nextafter(0.5, 1.0)
    assert _count(V, F) == 0
    V[3, 2] = np.nextafter(0.5, 0.0)
    assert _count(V, F) == 1


def test_duplicated_face():
    V = np.array(T0, np.float64)
    assert _count(V, np.array([[0, 1, 2], [1, 2, 0]])) == 1


@pytest.mark.parametrize("mesh", ["octahedron", "sphere", "open_patch"])
def test_clean_meshes_have_none(mesh):
    V, F = getattr(meshes, mesh)(*([] if mesh != "sphere" else [12]))
    assert _count(V, F) == 0


def test_tangled_mesh_grid_equals_all_pairs():
    V, F = meshes.tangled(n=6)
    n, pairs = orc.self_intersections(V, F, max_pairs=10000)
    assert n > 0 and len(pairs) == n
    assert n == orc.self_intersections_all_pairs(V, F)
    assert (pairs[:, 0] < pairs[:, 1]).all()


def test_index_out_of_range():
    with pytest.raises(ValueError):
        orc.self_intersections(np.zeros((3, 3)), np.array([[0, 1, 3]]))


def _point_tri_dist(P, A, B, C):
    """Distances from points P [n,3] to the triangle (A, B, C): the plane when the foot is inside, else the
    nearest edge."""
    n = np.cross(B - A, C - A)
    nn = n / np.linalg.norm(n)
    h = (P - A) @ nn
    foot = P - h[:, None] * nn
    inside = np.ones(len(P), bool)
    for u, v in ((A, B), (B, C), (C, A)):
        inside &= (np.cross(v - u, foot - u) @ n) >= 0
    best = np.where(inside, np.abs(h), np.inf)
    for u, v in ((A, B), (B, C), (C, A)):
        t = np.clip(((P - u) @ (v - u)) / ((v - u) @ (v - u)), 0, 1)
        best = np.minimum(best, np.linalg.norm(P - (u + t[:, None] * (v - u)), axis=1))
    return best


def _hausdorff_brute(VA, FA, VB, FB):
    def one(P, V, F):
        d = np.full(len(P), np.inf)
        for f in F:
            d = np.minimum(d, _point_tri_dist(P, V[f[0]], V[f[1]], V[f[2]]))
        return d.max()
    return one(VA, VB, FB), one(VB, VA, FA)


def test_hausdorff_octahedron_scaled():
    V, F = meshes.octahedron()
    V = V.astype(np.float64)
    h, ab, ba = orc.hausdorff(V * 1.1, F, V, F)
    assert ab == pytest.approx(0.1, abs=1e-12)
    assert ba == pytest.approx(0.1 / np.sqrt(3), abs=1e-12)
    assert h == ab
    assert orc.hausdorff(V, F, V, F)[0] == 0.0


def test_hausdorff_matches_brute_force():
    VA, FA = meshes.sphere(10, seed=1)
    VB, FB = meshes.tangled(n=7, seed=4)
    VB = VB * 1.3 + 0.2  # partly outside A's grid
    h, ab, ba = orc.hausdorff(VA, FA, VB, FB)
    bab, bba = _hausdorff_brute(VA.astype(np.float64), FA, VB.astype(np.float64), FB)
    assert ab == pytest.approx(bab, rel=1e-9)
    assert ba == pytest.approx(bba, rel=1e-9)
    assert h == max(ab, ba)


@pytest.mark.parametrize("ratio", [0.2, 0.05])
def test_oracle_simplification_is_intersection_free(ratio):
    """The restated algorithm keeps a clean input clean under the exact check (its own rollback test is a
    float test with a tolerance); the GPU path is bit-identical to it."""
    V, F = meshes.sphere(14, seed=3)
    v2, f2 = orc.Oracle(threads=4).run(V, F, ratio, min_verts=0)[:2]
    assert len(f2) < len(F)
    assert orc.self_intersections(v2, f2)[0] == 0
    h, ab, ba = orc.hausdorff(v2, f2, V, F)
    assert 0 < h < 0.05 * float(np.linalg.norm(V.max(0) - V.min(0)))
