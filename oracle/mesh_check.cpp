// Independent checks of output meshes: self-intersections with exact orientation predicates, and the
// two-sided vertex Hausdorff distance between two meshes.
//
// TEST INFRASTRUCTURE ONLY: used by tests/ and by bench.py to check results; the product never loads it.
//
// Exact predicates: orient3d and orient2d evaluated with floating-point expansion arithmetic (Shewchuk,
// "Adaptive precision floating-point arithmetic and fast robust geometric predicates", 1997): every input
// coordinate is a double (float32 inputs convert exactly), differences and products are kept as nonoverlapping
// expansions (two_sum, two_product by fma), so the sign of the determinant is exact. A double evaluation with a
// static error bound answers first and the expansion runs only when that bound cannot decide. Exact as long as
// no product underflows, which holds for every float32 input (products of float32 differences stay far above
// the double range's lower end).
//
// Self-intersection semantics (those of common mesh-repair tools, e.g. CGAL's self_intersections): two faces
// intersect when they share a point other than the vertices and edge they have in common. Faces with no
// common vertex: any common point. One common vertex v: a common point other than v. One common edge: the two
// faces are coplanar and lie on the same side of the edge. Three common vertices: a duplicated face.
//
// Hausdorff distance: max over the vertices of each mesh of the distance to the other mesh's surface, both
// ways (the definition of igl::hausdorff, used by the reference's metrics.py:49).

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace mc {

// ------------------------------------------------------------------ expansion arithmetic
typedef std::vector<double> Exp;

static inline void two_sum(double a, double b, double& x, double& y) {
    x = a + b;
    const double bv = x - a, av = x - bv;
    y = (a - av) + (b - bv);
}
static inline void two_prod(double a, double b, double& x, double& y) {
    x = a * b;
    y = std::fma(a, b, -x);
}
// e + b (e nonoverlapping, increasing magnitude) -> nonoverlapping expansion (grow_expansion)
static Exp grow(const Exp& e, double b) {
    Exp h;
    h.reserve(e.size() + 1);
    double q = b;
    for (double ei : e) {
        double x, y;
        two_sum(q, ei, x, y);
        if (y != 0.0) h.push_back(y);
        q = x;
    }
    if (q != 0.0 || h.empty()) h.push_back(q);
    return h;
}
static Exp add(const Exp& e, const Exp& f) {
    Exp h = e;
    for (double fi : f) h = grow(h, fi);
    return h;
}
static Exp neg(Exp e) {
    for (double& x : e) x = -x;
    return e;
}
static Exp scale(const Exp& e, double b) {  // scale_expansion
    Exp h;
    for (double ei : e) {
        double p, q;
        two_prod(ei, b, p, q);
        h = grow(h, q);
        h = grow(h, p);
    }
    if (h.empty()) h.push_back(0.0);
    return h;
}
static Exp mul(const Exp& e, const Exp& f) {
    Exp h{0.0};
    for (double fi : f) h = add(h, scale(e, fi));
    return h;
}
static Exp diff(double a, double b) {
    double x, y;
    two_sum(a, -b, x, y);
    Exp e;
    if (y != 0.0) e.push_back(y);
    e.push_back(x);
    return e;
}
static int sign(const Exp& e) {
    for (size_t i = e.size(); i-- > 0;)
        if (e[i] != 0.0) return e[i] > 0 ? 1 : -1;
    return 0;
}

struct P3 {
    double x, y, z;
};

// orient3d(a, b, c, d): sign of det[a-d; b-d; c-d] (positive when d is below the plane of a, b, c seen with
// a, b, c counter-clockwise)
static int orient3d(const P3& a, const P3& b, const P3& c, const P3& d) {
    const double adx = a.x - d.x, ady = a.y - d.y, adz = a.z - d.z;
    const double bdx = b.x - d.x, bdy = b.y - d.y, bdz = b.z - d.z;
    const double cdx = c.x - d.x, cdy = c.y - d.y, cdz = c.z - d.z;
    const double t1 = bdx * cdy - bdy * cdx, t2 = cdx * ady - cdy * adx, t3 = adx * bdy - ady * bdx;
    const double det = adz * t1 + bdz * t2 + cdz * t3;
    const double perm = (std::fabs(bdx * cdy) + std::fabs(bdy * cdx)) * std::fabs(adz) +
                        (std::fabs(cdx * ady) + std::fabs(cdy * adx)) * std::fabs(bdz) +
                        (std::fabs(adx * bdy) + std::fabs(ady * bdx)) * std::fabs(cdz);
    const double bound = 1e-14 * perm;  // far above the static error of this evaluation (Shewchuk: ~7.8e-16)
    if (det > bound) return 1;
    if (det < -bound) return -1;
    const Exp ax = diff(a.x, d.x), ay = diff(a.y, d.y), az = diff(a.z, d.z);
    const Exp bx = diff(b.x, d.x), by = diff(b.y, d.y), bz = diff(b.z, d.z);
    const Exp cx = diff(c.x, d.x), cy = diff(c.y, d.y), cz = diff(c.z, d.z);
    const Exp e1 = add(mul(bx, cy), neg(mul(by, cx)));
    const Exp e2 = add(mul(cx, ay), neg(mul(cy, ax)));
    const Exp e3 = add(mul(ax, by), neg(mul(ay, bx)));
    return sign(add(add(mul(az, e1), mul(bz, e2)), mul(cz, e3)));
}

// orient2d in the coordinate plane that drops axis `drop` (0: x, 1: y, 2: z)
static void proj(const P3& p, int drop, double& u, double& v) {
    if (drop == 0) { u = p.y; v = p.z; }
    else if (drop == 1) { u = p.z; v = p.x; }
    else { u = p.x; v = p.y; }
}
static int orient2d(const P3& a, const P3& b, const P3& c, int drop) {
    double ax, ay, bx, by, cx, cy;
    proj(a, drop, ax, ay);
    proj(b, drop, bx, by);
    proj(c, drop, cx, cy);
    const double det = (ax - cx) * (by - cy) - (ay - cy) * (bx - cx);
    const double bound = 1e-14 * (std::fabs((ax - cx) * (by - cy)) + std::fabs((ay - cy) * (bx - cx)));
    if (det > bound) return 1;
    if (det < -bound) return -1;
    const Exp e = add(mul(diff(ax, cx), diff(by, cy)), neg(mul(diff(ay, cy), diff(bx, cx))));
    return sign(e);
}

// a projection plane in which the triangle a, b, c is not degenerate (-1 when it is degenerate in all three)
static int drop_axis(const P3& a, const P3& b, const P3& c) {
    for (int d = 0; d < 3; ++d)
        if (orient2d(a, b, c, d) != 0) return d;
    return -1;
}

// ------------------------------------------------------------------ 2D primitives (in a projection plane)
static bool on_segment2(const P3& p, const P3& a, const P3& b, int drop) {  // p collinear with a, b assumed
    double pu, pv, au, av, bu, bv;
    proj(p, drop, pu, pv);
    proj(a, drop, au, av);
    proj(b, drop, bu, bv);
    return std::min(au, bu) <= pu && pu <= std::max(au, bu) && std::min(av, bv) <= pv && pv <= std::max(av, bv);
}
static bool seg_seg2(const P3& p, const P3& q, const P3& a, const P3& b, int drop) {
    const int o1 = orient2d(p, q, a, drop), o2 = orient2d(p, q, b, drop);
    const int o3 = orient2d(a, b, p, drop), o4 = orient2d(a, b, q, drop);
    if (o1 * o2 < 0 && o3 * o4 < 0) return true;
    if (o1 == 0 && on_segment2(a, p, q, drop)) return true;
    if (o2 == 0 && on_segment2(b, p, q, drop)) return true;
    if (o3 == 0 && on_segment2(p, a, b, drop)) return true;
    if (o4 == 0 && on_segment2(q, a, b, drop)) return true;
    return false;
}
static bool point_in_tri2(const P3& p, const P3& a, const P3& b, const P3& c, int drop) {
    const int o1 = orient2d(a, b, p, drop), o2 = orient2d(b, c, p, drop), o3 = orient2d(c, a, p, drop);
    return (o1 >= 0 && o2 >= 0 && o3 >= 0) || (o1 <= 0 && o2 <= 0 && o3 <= 0);
}

// closed segment [p, q] against closed triangle (a, b, c), exact
static bool seg_tri(const P3& p, const P3& q, const P3& a, const P3& b, const P3& c) {
    const int dr = drop_axis(a, b, c);
    if (dr < 0) {  // degenerate triangle: its edges
        auto seg_seg3 = [&](const P3& s0, const P3& s1) {
            // coplanar segments meet iff they meet in some projection where neither is a point... test all
            if (orient3d(p, q, s0, s1) != 0) return false;
            for (int d = 0; d < 3; ++d) {
                if (!seg_seg2(p, q, s0, s1, d)) return false;
            }
            return true;
        };
        return seg_seg3(a, b) || seg_seg3(b, c) || seg_seg3(c, a);
    }
    const int o1 = orient3d(a, b, c, p), o2 = orient3d(a, b, c, q);
    if (o1 * o2 > 0) return false;
    if (o1 == 0 && o2 == 0) {  // segment in the triangle's plane
        if (point_in_tri2(p, a, b, c, dr) || point_in_tri2(q, a, b, c, dr)) return true;
        return seg_seg2(p, q, a, b, dr) || seg_seg2(p, q, b, c, dr) || seg_seg2(p, q, c, a, dr);
    }
    // the line pq meets the plane at a point of the segment; it lies in the triangle iff the three edge
    // orientations agree (zeros allowed)
    const int s1 = orient3d(p, q, a, b), s2 = orient3d(p, q, b, c), s3 = orient3d(p, q, c, a);
    return (s1 >= 0 && s2 >= 0 && s3 >= 0) || (s1 <= 0 && s2 <= 0 && s3 <= 0);
}

static bool tri_tri(const P3 t[3], const P3 u[3]) {
    for (int k = 0; k < 3; ++k) {
        if (seg_tri(t[k], t[(k + 1) % 3], u[0], u[1], u[2])) return true;
        if (seg_tri(u[k], u[(k + 1) % 3], t[0], t[1], t[2])) return true;
    }
    return false;
}

// direction w - v inside the closed angle (a - v, b - v) of a triangle (v, a, b), all coplanar
static bool ray_in_angle(const P3& v, const P3& w, const P3& a, const P3& b, int drop) {
    const int oab = orient2d(v, a, b, drop);
    const int oaw = orient2d(v, a, w, drop), owb = orient2d(v, w, b, drop);
    if (oab == 0) return false;
    if (oab > 0) return oaw >= 0 && owb >= 0 && !(oaw == 0 && owb == 0);
    return oaw <= 0 && owb <= 0 && !(oaw == 0 && owb == 0);
}

// the pair (f, g) of a mesh intersects beyond what the two faces share
static bool faces_intersect(const int* F, const P3* V, int f, int g) {
    const int* a = F + 3 * f;
    const int* b = F + 3 * g;
    int shared = 0, sa[3] = {-1, -1, -1}, sb[3] = {-1, -1, -1};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (a[i] == b[j]) {
                sa[shared] = i;
                sb[shared] = j;
                ++shared;
            }
    const P3 t[3] = {V[a[0]], V[a[1]], V[a[2]]}, u[3] = {V[b[0]], V[b[1]], V[b[2]]};
    if (shared == 0) return tri_tri(t, u);
    if (shared >= 3) return true;  // a duplicated face
    if (shared == 2) {
        // common edge (e0, e1); the opposite vertices
        const int ia = 3 - sa[0] - sa[1], ib = 3 - sb[0] - sb[1];
        const P3& e0 = t[sa[0]];
        const P3& e1 = t[sa[1]];
        if (orient3d(e0, e1, t[ia], u[ib]) != 0) return false;
        const int dr = drop_axis(e0, e1, t[ia]) >= 0 ? drop_axis(e0, e1, t[ia]) : drop_axis(e0, e1, u[ib]);
        if (dr < 0) return true;  // both faces degenerate onto the edge's line
        return orient2d(e0, e1, t[ia], dr) * orient2d(e0, e1, u[ib], dr) > 0;
    }
    // one common vertex
    const int va = sa[0], vb = sb[0];
    const P3& v = t[va];
    const P3& a1 = t[(va + 1) % 3];
    const P3& b1 = t[(va + 2) % 3];
    const P3& a2 = u[(vb + 1) % 3];
    const P3& b2 = u[(vb + 2) % 3];
    if (seg_tri(a1, b1, u[0], u[1], u[2]) || seg_tri(a2, b2, t[0], t[1], t[2])) return true;
    // an edge from v lying in the other face's plane and pointing into its angle at v
    const int d2 = drop_axis(v, a2, b2), d1 = drop_axis(v, a1, b1);
    for (const P3* w : {&a1, &b1})
        if (d2 >= 0 && orient3d(v, a2, b2, *w) == 0 && ray_in_angle(v, *w, a2, b2, d2)) return true;
    for (const P3* w : {&a2, &b2})
        if (d1 >= 0 && orient3d(v, a1, b1, *w) == 0 && ray_in_angle(v, *w, a1, b1, d1)) return true;
    return false;
}

// ------------------------------------------------------------------ closest point (Ericson 5.1.5), in double
static P3 sub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static P3 addp(P3 a, P3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static P3 mulp(double s, P3 a) { return {s * a.x, s * a.y, s * a.z}; }
static double dotp(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static P3 closest_tri(P3 p, P3 a, P3 b, P3 c) {
    const P3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    const double d1 = dotp(ab, ap), d2 = dotp(ac, ap);
    if (d1 <= 0 && d2 <= 0) return a;
    const P3 bp = sub(p, b);
    const double d3 = dotp(ab, bp), d4 = dotp(ac, bp);
    if (d3 >= 0 && d4 <= d3) return b;
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) return addp(a, mulp(d1 / (d1 - d3), ab));
    const P3 cp = sub(p, c);
    const double d5 = dotp(ab, cp), d6 = dotp(ac, cp);
    if (d6 >= 0 && d5 <= d6) return c;
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) return addp(a, mulp(d2 / (d2 - d6), ac));
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0)
        return addp(b, mulp((d4 - d3) / ((d4 - d3) + (d5 - d6)), sub(c, b)));
    const double den = 1.0 / (va + vb + vc);
    return addp(a, addp(mulp(vb * den, ab), mulp(vc * den, ac)));
}

// uniform grid over triangle boxes: sorted (cell, face) pairs
struct Grid {
    double h = 1, lo[3] = {0, 0, 0};
    long long dims[3] = {1, 1, 1};
    std::vector<std::pair<long long, int>> cells;
    long long key(long long i, long long j, long long k) const { return (i * dims[1] + j) * dims[2] + k; }
    void cell_of(double x, double y, double z, long long* c) const {
        const double v[3] = {x, y, z};
        for (int d = 0; d < 3; ++d)
            c[d] = std::min(dims[d] - 1, std::max(0ll, (long long)std::floor((v[d] - lo[d]) / h)));
    }
    void build(const P3* V, int nv, const int* F, int nf) {
        double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300}, el = 0;
        for (int i = 0; i < nv; ++i) {
            const double c[3] = {V[i].x, V[i].y, V[i].z};
            for (int d = 0; d < 3; ++d) {
                mn[d] = std::min(mn[d], c[d]);
                mx[d] = std::max(mx[d], c[d]);
            }
        }
        for (int f = 0; f < nf; ++f) el += std::sqrt(dotp(sub(V[F[3 * f + 1]], V[F[3 * f]]), sub(V[F[3 * f + 1]], V[F[3 * f]])));
        el /= std::max(1, nf);
        double ext = 0;
        for (int d = 0; d < 3; ++d) ext = std::max(ext, mx[d] - mn[d]);
        h = std::max(2.0 * el, ext / 1024.0);
        if (!(h > 0)) h = 1;
        for (int d = 0; d < 3; ++d) {
            lo[d] = mn[d];
            dims[d] = (long long)std::floor((mx[d] - mn[d]) / h) + 1;
        }
        cells.clear();
        for (int f = 0; f < nf; ++f) {
            const P3 p0 = V[F[3 * f]], p1 = V[F[3 * f + 1]], p2 = V[F[3 * f + 2]];
            long long a[3], b[3];
            cell_of(std::min({p0.x, p1.x, p2.x}), std::min({p0.y, p1.y, p2.y}), std::min({p0.z, p1.z, p2.z}), a);
            cell_of(std::max({p0.x, p1.x, p2.x}), std::max({p0.y, p1.y, p2.y}), std::max({p0.z, p1.z, p2.z}), b);
            for (long long i = a[0]; i <= b[0]; ++i)
                for (long long j = a[1]; j <= b[1]; ++j)
                    for (long long k = a[2]; k <= b[2]; ++k) cells.push_back({key(i, j, k), f});
        }
        std::sort(cells.begin(), cells.end());
    }
    double nearest_sq(P3 p, const P3* V, const int* F) const {
        long long c[3];
        cell_of(p.x, p.y, p.z, c);
        double best = 1e300;
        const long long rmax = std::max({dims[0], dims[1], dims[2]}) + 1;
        for (long long r = 0; r <= rmax; ++r) {
            for (long long i = c[0] - r; i <= c[0] + r; ++i) {
                if (i < 0 || i >= dims[0]) continue;
                for (long long j = c[1] - r; j <= c[1] + r; ++j) {
                    if (j < 0 || j >= dims[1]) continue;
                    for (long long k = c[2] - r; k <= c[2] + r; ++k) {
                        if (k < 0 || k >= dims[2]) continue;
                        if (std::max({std::llabs(i - c[0]), std::llabs(j - c[1]), std::llabs(k - c[2])}) != r) continue;
                        const long long kk = key(i, j, k);
                        for (auto it = std::lower_bound(cells.begin(), cells.end(), std::make_pair(kk, -1));
                             it != cells.end() && it->first == kk; ++it) {
                            const int f = it->second;
                            const P3 q = closest_tri(p, V[F[3 * f]], V[F[3 * f + 1]], V[F[3 * f + 2]]);
                            best = std::min(best, dotp(sub(q, p), sub(q, p)));
                        }
                    }
                }
            }
            // every point of a cell outside ring r is more than r * h from p (p lies in cell c, or outside the
            // grid beyond it), and a face's nearest point lies in one of the cells its box covers
            const double reach = r * h;
            if (best < 1e300 && reach > 0 && best <= reach * reach) break;
        }
        return best;
    }
};

}  // namespace mc

using namespace mc;

extern "C" {

// Number of intersecting face pairs of the mesh (and up to cap of them in pairs_out as (f, g), f < g, in no
// particular order); -1 for an index out of range. Candidate pairs are the faces whose boxes share a grid cell,
// each pair tested in the lowest cell common to both boxes only.
long long check_self_intersections(const double* pts, int nv, const int* tris, int nf, int* pairs_out, int cap) {
    for (long long i = 0; i < 3ll * nf; ++i)
        if (tris[i] < 0 || tris[i] >= nv) return -1;
    std::vector<P3> V(nv);
    for (int i = 0; i < nv; ++i) V[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    Grid g;
    g.build(V.data(), nv, tris, nf);
    // per face: box and cell range
    std::vector<std::array<double, 6>> box(nf);
    std::vector<std::array<long long, 6>> rng(nf);
    for (int f = 0; f < nf; ++f) {
        const P3 p0 = V[tris[3 * f]], p1 = V[tris[3 * f + 1]], p2 = V[tris[3 * f + 2]];
        box[f] = {std::min({p0.x, p1.x, p2.x}), std::min({p0.y, p1.y, p2.y}), std::min({p0.z, p1.z, p2.z}),
                  std::max({p0.x, p1.x, p2.x}), std::max({p0.y, p1.y, p2.y}), std::max({p0.z, p1.z, p2.z})};
        long long a[3], b[3];
        g.cell_of(box[f][0], box[f][1], box[f][2], a);
        g.cell_of(box[f][3], box[f][4], box[f][5], b);
        rng[f] = {a[0], a[1], a[2], b[0], b[1], b[2]};
    }
    // cell starts
    std::vector<size_t> starts;
    for (size_t i = 0; i < g.cells.size(); ++i)
        if (i == 0 || g.cells[i].first != g.cells[i - 1].first) starts.push_back(i);
    starts.push_back(g.cells.size());
    const long long ncell = (long long)starts.size() - 1;
    long long found = 0;
    std::vector<std::pair<int, int>> hits;
#pragma omp parallel
    {
        std::vector<std::pair<int, int>> mine;
        long long cnt = 0;
#pragma omp for schedule(dynamic, 64)
        for (long long c = 0; c < ncell; ++c) {
            const long long key = g.cells[starts[c]].first;
            const long long ck[3] = {key / (g.dims[1] * g.dims[2]), (key / g.dims[2]) % g.dims[1], key % g.dims[2]};
            for (size_t a = starts[c]; a < starts[c + 1]; ++a)
                for (size_t b = a + 1; b < starts[c + 1]; ++b) {
                    const int f = std::min(g.cells[a].second, g.cells[b].second);
                    const int h = std::max(g.cells[a].second, g.cells[b].second);
                    bool first = true;
                    for (int d = 0; d < 3; ++d) first = first && std::max(rng[f][d], rng[h][d]) == ck[d];
                    if (!first) continue;
                    bool sep = false;
                    for (int d = 0; d < 3; ++d) sep = sep || box[f][d + 3] < box[h][d] || box[h][d + 3] < box[f][d];
                    if (sep || !faces_intersect(tris, V.data(), f, h)) continue;
                    ++cnt;
                    if (pairs_out && (long long)mine.size() < cap) mine.push_back({f, h});
                }
        }
#pragma omp critical
        {
            found += cnt;
            hits.insert(hits.end(), mine.begin(), mine.end());
        }
    }
    if (pairs_out) {
        std::sort(hits.begin(), hits.end());
        for (long long i = 0; i < (long long)hits.size() && i < cap; ++i) {
            pairs_out[2 * i] = hits[i].first;
            pairs_out[2 * i + 1] = hits[i].second;
        }
    }
    return found;
}

// Two-sided vertex Hausdorff distance (igl::hausdorff): out[0] = max over A's vertices of the distance to
// B's surface, out[1] = the same from B to A; returns max(out[0], out[1]).
double hausdorff(const double* pa, int nva, const int* fa, int nfa, const double* pb, int nvb, const int* fb, int nfb,
                 double* out) {
    std::vector<P3> A(nva), B(nvb);
    for (int i = 0; i < nva; ++i) A[i] = {pa[3 * i], pa[3 * i + 1], pa[3 * i + 2]};
    for (int i = 0; i < nvb; ++i) B[i] = {pb[3 * i], pb[3 * i + 1], pb[3 * i + 2]};
    Grid ga, gb;
    ga.build(A.data(), nva, fa, nfa);
    gb.build(B.data(), nvb, fb, nfb);
    double hab = 0, hba = 0;
#pragma omp parallel for reduction(max : hab) schedule(dynamic, 256)
    for (int i = 0; i < nva; ++i) hab = std::max(hab, gb.nearest_sq(A[i], B.data(), fb));
#pragma omp parallel for reduction(max : hba) schedule(dynamic, 256)
    for (int i = 0; i < nvb; ++i) hba = std::max(hba, ga.nearest_sq(B[i], A.data(), fa));
    if (out) {
        out[0] = std::sqrt(hab);
        out[1] = std::sqrt(hba);
    }
    return std::sqrt(std::max(hab, hba));
}

// All pairs, no grid: the check of the grid's candidate pairs on small meshes.
long long check_self_intersections_all_pairs(const double* pts, int nv, const int* tris, int nf) {
    for (long long i = 0; i < 3ll * nf; ++i)
        if (tris[i] < 0 || tris[i] >= nv) return -1;
    std::vector<P3> V(nv);
    for (int i = 0; i < nv; ++i) V[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    long long found = 0;
    for (int f = 0; f < nf; ++f)
        for (int h = f + 1; h < nf; ++h) found += faces_intersect(tris, V.data(), f, h) ? 1 : 0;
    return found;
}

// exact predicate for tests: orient3d on 12 doubles
int exact_orient3d(const double* p) {
    return orient3d({p[0], p[1], p[2]}, {p[3], p[4], p[5]}, {p[6], p[7], p[8]}, {p[9], p[10], p[11]});
}

}  // extern "C"
