// PaMO stage-3 oracle: a float64 CPU restatement of the reference's safe projection
// (pamo_safe_project.process with the default Stage3Config).
//
// TEST INFRASTRUCTURE ONLY. This file is the checker of the CUDA path: it is linked by tests/ and by
// __graft_entry__.smoke(); the product library (pamo_gb300/) never loads it.
//
// PARITY UNPINNED: the reference runs on a fork of NVIDIA Warp (it calls wp.spd_project_blocks, which
// released Warp does not have) and that fork is not available, so the reference cannot be run to produce
// golden outputs. This restatement follows the reference's source step by step in float64; where the
// reference calls a fork-only or library routine, the routine's mathematical operation is restated:
//   * wp.spd_project_blocks(3, block, it_max): projection of the 9x9 matrix of hinge blocks [0..2][0..2]
//     onto the positive semi-definite cone, here by it_max cyclic Jacobi sweeps and clamping of negative
//     eigenvalues (the CUDA path does the same in float32);
//   * wp.mesh_query_point_no_sign + mesh_eval_position: the closest point of the GT surface (uniform grid);
//   * wp.bvh_query_aabb: candidate pairs whose boxes overlap, then the reference's distance filter; the
//     filter alone decides, so a uniform grid gives the same contact set;
//   * igl::massmatrix(VORONOI), igl::internal_angles: restated from libigl's published formulas;
//   * trimesh.edges_unique: unique sorted edges ordered by (larger, smaller) endpoint.
//
// Reference files (inside simp_cuda/safe_project/src/pamo_safe_project/):
//   processing.py:15-106   normalisation and the step loop
//   system.py:167-272      register_mesh; :325-470 energy/diff/hess_dx/clamp/CCD/line search/step
//   cg_solver.py:46-158    Jacobi-preconditioned CG
//   kernels/energy_kernels/distance_energy.py:6-45, elastic_energy.py:7-220, hinge_energy.py:4-274,
//   collision_energy.py:8-99,186-254,379-409, contact_detection.py:120-216
//   kernels/distance_kernels/distance_kernels.py (classification and distances), kernels/ccd_kernels.py:9-111,
//   kernels/solver_kernels.py, kernels/utils_kernels.py:21-39, config.py:6-73

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <unordered_map>
#include <vector>

namespace s3o {

struct V3 {
    double x = 0, y = 0, z = 0;
};
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
static inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
static inline V3 operator*(V3 a, double s) { return {s * a.x, s * a.y, s * a.z}; }
static inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
static inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static inline double len2(V3 a) { return dot(a, a); }
static inline double len(V3 a) { return std::sqrt(dot(a, a)); }
static inline V3 nrm(V3 a) {
    const double l = len(a);
    return l > 0 ? a / l : V3{};
}
static inline double stp(double x) { return x < 0 ? 1.0 : 0.0; }

struct Params {
    int n_newton_iters = 10, n_cg_iters = 40, n_line_search_iters = 10, ccd_max_iters = 100, spd_max_iters = 3;
    double d_hat = 1e-3, coll_stiffness = 1e2, radius = 1e-2, ee_thres = 1e-3, ccd_slackness = 0.7,
           ccd_thickness = 1e-6, young = 0.1, poisson = 0.0, hinge_k = 1e-2, m2gt_k = 1e3, min_angle = 0.0;
    long long max_blocks = 1ll << 25;
};

// ---------------------------------------------------------------- distances (distance_kernels.py)
enum { PT_PT = 0, PT_PP01, PT_PP02, PT_PE012, PT_PP03, PT_PE031, PT_PE023 };
enum { EE_PP02 = 0, EE_PP03, EE_PP12, EE_PP13, EE_PE023, EE_PE123, EE_PE201, EE_PE301, EE_EE };
enum { BLOCK_PT = 3, BLOCK_EE = 4 };

static double d_pt(V3 x0, V3 x1, V3 x2, V3 x3) { return std::fabs(dot(x0 - x1, nrm(cross(x2 - x1, x3 - x1)))); }
static double d_ee(V3 x0, V3 x1, V3 x2, V3 x3) { return std::fabs(dot(x0 - x2, nrm(cross(x1 - x0, x3 - x2)))); }
static double d_pe(V3 x0, V3 x1, V3 x2) { return len(cross(x1 - x0, x2 - x0)) / len(x1 - x2); }
static double d_pp(V3 x0, V3 x1) { return len(x1 - x0); }

static int pt_classify(V3 x0, V3 x1, V3 x2, V3 x3) {
    V3 x10 = x0 - x1;
    const V3 x12 = x2 - x1, x13 = x3 - x1;
    const double a2 = len2(cross(x12, x13));
    if (a2 <= 1e-6 * (len2(x12) * len2(x13)) || a2 <= 1e-16) {
        const double d1 = len(x10), d2 = len(x0 - x2), d3 = len(x0 - x3);
        if (d1 < d2) return d1 < d3 ? PT_PP01 : PT_PP03;
        return d2 < d3 ? PT_PP02 : PT_PP03;
    }
    const V3 n = nrm(cross(x12, x13));
    const V3 xp = x0 - dot(n, x10) * n;
    x10 = xp - x1;
    const V3 x20 = xp - x2, x30 = xp - x3;
    const double a00 = dot(x12, x12), a01 = dot(x12, x13), a11 = dot(x13, x13);
    const double b0 = dot(x10, x12), b1 = dot(x10, x13);
    const double det = a00 * a11 - a01 * a01;
    const double beta = b0 * a11 - b1 * a01, gamma = a00 * b1 - b0 * a01, alpha = det - beta - gamma;
    const double nneg = stp(alpha) + stp(beta) + stp(gamma);
    if (nneg == 0) return PT_PT;
    if (nneg == 1) {
        if (alpha < 0) {
            const V3 x23 = x3 - x2;
            const double dr = dot(x23, x0 - x2);
            return dr < 0 ? PT_PP02 : (dr > dot(x23, x23) ? PT_PP03 : PT_PE023);
        } else if (beta < 0) {
            const V3 x31 = x1 - x3;
            const double dr = dot(x31, x0 - x3);
            return dr < 0 ? PT_PP03 : (dr > dot(x31, x31) ? PT_PP01 : PT_PE031);
        } else if (gamma < 0) {
            const double dr = dot(x12, x10);
            return dr < 0 ? PT_PP01 : (dr > dot(x12, x12) ? PT_PP02 : PT_PE012);
        }
        return -1;
    }
    if (alpha >= 0) {
        const double d12 = dot(x12, x10), d13 = dot(x13, x10);
        if (d12 > 0 && d13 <= 0) return dot(x12, x20) > 0 ? PT_PP02 : PT_PE012;
        if (d13 > 0 && d12 <= 0) return dot(x13, x30) > 0 ? PT_PP03 : PT_PE031;
        return PT_PP01;
    } else if (beta >= 0) {
        const V3 x23 = x3 - x2, x21 = x1 - x2;
        const double d23 = dot(x23, x20), d21 = dot(x21, x20);
        if (d23 > 0 && d21 <= 0) return dot(x23, x30) > 0 ? PT_PP03 : PT_PE023;
        if (d21 > 0 && d23 <= 0) return dot(x21, x10) > 0 ? PT_PP01 : PT_PE012;
        return PT_PP02;
    }
    const V3 x31 = x1 - x3, x32 = x2 - x3;
    const double d31 = dot(x31, x30), d32 = dot(x32, x30);
    if (d31 > 0 && d32 <= 0) return dot(x31, x10) > 0 ? PT_PP01 : PT_PE031;
    if (d32 > 0 && d31 <= 0) return dot(x32, x20) > 0 ? PT_PP02 : PT_PE023;
    return PT_PP03;
}

static double pt_dist(V3 x0, V3 x1, V3 x2, V3 x3, int t) {
    switch (t) {
        case PT_PT: return d_pt(x0, x1, x2, x3);
        case PT_PP01: return d_pp(x0, x1);
        case PT_PP02: return d_pp(x0, x2);
        case PT_PE012: return d_pe(x0, x1, x2);
        case PT_PP03: return d_pp(x0, x3);
        case PT_PE031: return d_pe(x0, x3, x1);
        case PT_PE023: return d_pe(x0, x2, x3);
    }
    return 1e9;
}

static int ee_classify(V3 x0, V3 x1, V3 x2, V3 x3, double thres) {
    const V3 e0 = x0 - x1, e1 = x2 - x3;
    const double e0s = dot(e0, e0), e1s = dot(e1, e1);
    const double a00 = e0s, a01 = -dot(e0, e1), a10 = dot(e0, e1), a11 = -e1s;
    const double b0 = dot(x3 - x1, e0), b1 = dot(x3 - x1, e1);
    const double mu0 = -(b0 * a11 - b1 * a01), mu1 = -(a00 * b1 - a10 * b0), detA = -(a00 * a11 - a01 * a10);
    const double sn = len(cross(nrm(e0), nrm(e1)));
    if (mu0 >= 0 && mu0 <= detA && mu1 >= 0 && mu1 <= detA && sn >= thres && len2(e0) > 1e-15 && len2(e1) > 1e-15)
        return EE_EE;
    double best = 1e9;
    int type = -1;
    auto c = [&](double d, int t) {
        if (d < best) {
            best = d;
            type = t;
        }
    };
    const double t0 = dot(x0 - x3, e1);
    if (t0 >= e1s) c(d_pp(x0, x2), EE_PP02);
    else if (t0 <= 0) c(d_pp(x0, x3), EE_PP03);
    else c(d_pe(x0, x2, x3), EE_PE023);
    const double t1 = dot(x1 - x3, e1);
    if (t1 >= e1s) c(d_pp(x1, x2), EE_PP12);
    else if (t1 <= 0) c(d_pp(x1, x3), EE_PP13);
    else c(d_pe(x1, x2, x3), EE_PE123);
    const double t2 = dot(x2 - x1, e0);
    if (t2 >= e0s) c(d_pp(x2, x0), EE_PP02);
    else if (t2 <= 0) c(d_pp(x2, x1), EE_PP12);
    else c(d_pe(x2, x0, x1), EE_PE201);
    const double t3 = dot(x3 - x1, e0);
    if (t3 >= e0s) c(d_pp(x3, x0), EE_PP03);
    else if (t3 <= 0) c(d_pp(x3, x1), EE_PP13);
    else c(d_pe(x3, x0, x1), EE_PE301);
    return type;
}

static double ee_dist(V3 x0, V3 x1, V3 x2, V3 x3, int t) {
    switch (t) {
        case EE_PP02: return d_pp(x0, x2);
        case EE_PP03: return d_pp(x0, x3);
        case EE_PP12: return d_pp(x1, x2);
        case EE_PP13: return d_pp(x1, x3);
        case EE_PE023: return d_pe(x0, x2, x3);
        case EE_PE123: return d_pe(x1, x2, x3);
        case EE_PE201: return d_pe(x2, x0, x1);
        case EE_PE301: return d_pe(x3, x0, x1);
        case EE_EE: return d_ee(x0, x1, x2, x3);
    }
    return 1e9;
}

// gradients of the unsigned distances (the reference's grad_funcs.py evaluates the same derivatives from
// generated expressions)
static void g_pp(V3 a, V3 b, int ia, int ib, V3* g) {
    const V3 u = nrm(a - b);
    g[ia] = u;
    g[ib] = -u;
}
static void g_pe(V3 a, V3 b, V3 c, int ia, int ib, int ic, V3* g) {
    const V3 e = c - b;
    const double ee = dot(e, e);
    const double t = ee > 0 ? dot(a - b, e) / ee : 0;
    const V3 n = nrm(a - (b + t * e));
    g[ia] = n;
    g[ib] = -(1 - t) * n;
    g[ic] = -t * n;
}
static void g_ptp(V3 x0, V3 x1, V3 x2, V3 x3, V3* g) {
    const V3 e1 = x2 - x1, e2 = x3 - x1;
    const V3 n = nrm(cross(e1, e2));
    const double sd = dot(n, x0 - x1);
    const V3 sn = (sd < 0 ? -1.0 : 1.0) * n;
    const V3 pr = x0 - sd * n - x1;
    const double a00 = dot(e1, e1), a01 = dot(e1, e2), a11 = dot(e2, e2), b0 = dot(pr, e1), b1 = dot(pr, e2);
    const double det = a00 * a11 - a01 * a01;
    const double l2 = det != 0 ? (b0 * a11 - b1 * a01) / det : 0, l3 = det != 0 ? (a00 * b1 - b0 * a01) / det : 0;
    g[0] = sn;
    g[1] = -(1 - l2 - l3) * sn;
    g[2] = -l2 * sn;
    g[3] = -l3 * sn;
}
static void g_eel(V3 x0, V3 x1, V3 x2, V3 x3, V3* g) {
    const V3 d1 = x1 - x0, d2 = x3 - x2, r0 = x0 - x2;
    const V3 n = nrm(cross(d1, d2));
    const V3 sn = (dot(n, r0) < 0 ? -1.0 : 1.0) * n;
    const double A = dot(d1, d1), B = dot(d1, d2), C = dot(d2, d2), D = dot(d1, r0), E = dot(d2, r0);
    const double den = A * C - B * B;
    const double a = den != 0 ? (B * E - C * D) / den : 0, b = den != 0 ? (A * E - B * D) / den : 0;
    g[0] = (1 - a) * sn;
    g[1] = a * sn;
    g[2] = -(1 - b) * sn;
    g[3] = -b * sn;
}
static void pt_grad(V3 x0, V3 x1, V3 x2, V3 x3, int t, V3* g) {
    g[0] = g[1] = g[2] = g[3] = V3{};
    switch (t) {
        case PT_PT: g_ptp(x0, x1, x2, x3, g); break;
        case PT_PP01: g_pp(x0, x1, 0, 1, g); break;
        case PT_PP02: g_pp(x0, x2, 0, 2, g); break;
        case PT_PE012: g_pe(x0, x1, x2, 0, 1, 2, g); break;
        case PT_PP03: g_pp(x0, x3, 0, 3, g); break;
        case PT_PE031: g_pe(x0, x3, x1, 0, 3, 1, g); break;
        case PT_PE023: g_pe(x0, x2, x3, 0, 2, 3, g); break;
    }
}
static void ee_grad(V3 x0, V3 x1, V3 x2, V3 x3, int t, V3* g) {
    g[0] = g[1] = g[2] = g[3] = V3{};
    switch (t) {
        case EE_PP02: g_pp(x0, x2, 0, 2, g); break;
        case EE_PP03: g_pp(x0, x3, 0, 3, g); break;
        case EE_PP12: g_pp(x1, x2, 1, 2, g); break;
        case EE_PP13: g_pp(x1, x3, 1, 3, g); break;
        case EE_PE023: g_pe(x0, x2, x3, 0, 2, 3, g); break;
        case EE_PE123: g_pe(x1, x2, x3, 1, 2, 3, g); break;
        case EE_PE201: g_pe(x2, x0, x1, 2, 0, 1, g); break;
        case EE_PE301: g_pe(x3, x0, x1, 3, 0, 1, g); break;
        case EE_EE: g_eel(x0, x1, x2, x3, g); break;
    }
}

// barrier (collision_energy.py:8-28); Warp's select(c, a, b) is a when c is false
static double bar(double d, double h) { return d >= h ? 0 : -(d - h) * (d - h) * std::log(d / h); }
static double bar1(double d, double h) {
    const double t = d - h;
    return d >= h ? 0 : -2.0 * t * std::log(d / h) - t * t / d;
}
static double bar2(double d, double h) {
    return d >= h ? 0 : -2.0 * std::log(d / h) - 2.0 * (d - h) / d - 1.0 + (h * h) / (d * d);
}

// closest point on a triangle (Ericson, Real-Time Collision Detection 5.1.5)
static V3 closest_tri(V3 p, V3 a, V3 b, V3 c) {
    const V3 ab = b - a, ac = c - a, ap = p - a;
    const double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0 && d2 <= 0) return a;
    const V3 bp = p - b;
    const double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) return b;
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) return a + (d1 / (d1 - d3)) * ab;
    const V3 cp = p - c;
    const double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) return c;
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) return a + (d2 / (d2 - d6)) * ac;
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) return b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b);
    const double den = 1.0 / (va + vb + vc);
    return a + (vb * den) * ab + (vc * den) * ac;
}

struct M2 {
    double a, b, c, d;
};
static M2 mm(M2 x, M2 y) { return {x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d}; }
static M2 mt(M2 x) { return {x.a, x.c, x.b, x.d}; }
static M2 ma(M2 x, M2 y) { return {x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d}; }
static M2 ms(double s, M2 x) { return {s * x.a, s * x.b, s * x.c, s * x.d}; }
static double mtr(M2 x) { return x.a + x.d; }

typedef std::array<std::array<double, 3>, 3> M3;
static M3 outer(V3 a, V3 b) {
    const double A[3] = {a.x, a.y, a.z}, B[3] = {b.x, b.y, b.z};
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[i][j] = A[i] * B[j];
    return r;
}
static M3 T(M3 a) {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[i][j] = a[j][i];
    return r;
}
static M3 lin(double s, M3 a, double t, M3 b) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = s * a[i][j] + t * b[i][j];
    return a;
}
static M3 sc(double s, M3 a) { return lin(s, a, 0, a); }
static M3 add(M3 a, M3 b) { return lin(1, a, 1, b); }
static M3 sub(M3 a, M3 b) { return lin(1, a, -1, b); }
static M3 sym(M3 a) { return add(a, T(a)); }

static double hinge_angle(V3 x0, V3 x1, V3 x2, V3 x3) {
    const V3 e12 = nrm(x2 - x1);
    const V3 n1 = nrm(cross(e12, x0 - x1)), n2 = nrm(cross(x3 - x1, e12));
    return std::atan2(dot(cross(n1, n2), e12), dot(n1, n2));
}

struct Elastic {
    V3 b1, b2;
    M2 F, inv;
    double W;
};

// Closest point on the GT surface by a uniform grid: triangles binned by their boxes into cells of side h
// (sorted (cell, triangle) pairs); a query scans Chebyshev rings of cells around its own until the best
// distance found is below the distance to the next ring. Gives the exact nearest point (as the reference's
// BVH query does), in any order of equally near triangles.
struct GtGrid {
    double h = 1, lo[3] = {0, 0, 0};
    long long dims[3] = {1, 1, 1};
    std::vector<std::pair<long long, int>> cells;
    long long key(long long i, long long j, long long k) const { return (i * dims[1] + j) * dims[2] + k; }
    void build(const std::vector<V3>& P, const std::vector<std::array<int, 3>>& T) {
        double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300}, el = 0;
        for (auto& p : P) {
            const double c[3] = {p.x, p.y, p.z};
            for (int d = 0; d < 3; ++d) {
                mn[d] = std::min(mn[d], c[d]);
                mx[d] = std::max(mx[d], c[d]);
            }
        }
        for (auto& t : T) el += len(P[t[1]] - P[t[0]]);
        el /= std::max<size_t>(1, T.size());
        double ext = 0;
        for (int d = 0; d < 3; ++d) ext = std::max(ext, mx[d] - mn[d]);
        h = std::max(2.0 * el, ext / 1024.0);
        if (!(h > 0)) h = 1;
        for (int d = 0; d < 3; ++d) {
            lo[d] = mn[d];
            dims[d] = (long long)std::floor((mx[d] - mn[d]) / h) + 1;
        }
        cells.clear();
        for (int f = 0; f < (int)T.size(); ++f) {
            long long a[3], b[3];
            const V3 p0 = P[T[f][0]], p1 = P[T[f][1]], p2 = P[T[f][2]];
            const double l[3] = {std::min({p0.x, p1.x, p2.x}), std::min({p0.y, p1.y, p2.y}), std::min({p0.z, p1.z, p2.z})};
            const double u[3] = {std::max({p0.x, p1.x, p2.x}), std::max({p0.y, p1.y, p2.y}), std::max({p0.z, p1.z, p2.z})};
            for (int d = 0; d < 3; ++d) {
                a[d] = std::min(dims[d] - 1, std::max(0ll, (long long)std::floor((l[d] - lo[d]) / h)));
                b[d] = std::min(dims[d] - 1, std::max(0ll, (long long)std::floor((u[d] - lo[d]) / h)));
            }
            for (long long i = a[0]; i <= b[0]; ++i)
                for (long long j = a[1]; j <= b[1]; ++j)
                    for (long long k = a[2]; k <= b[2]; ++k) cells.push_back({key(i, j, k), f});
        }
        std::sort(cells.begin(), cells.end());
    }
    V3 nearest(V3 p, const std::vector<V3>& P, const std::vector<std::array<int, 3>>& T) const {
        long long c[3];
        const double pc[3] = {p.x, p.y, p.z};
        for (int d = 0; d < 3; ++d) c[d] = (long long)std::floor((pc[d] - lo[d]) / h);
        double best = 1e300;
        V3 bp = p;
        const long long rmax = std::max({dims[0], dims[1], dims[2]}) + std::max({std::llabs(c[0]), std::llabs(c[1]), std::llabs(c[2])}) + 1;
        for (long long r = 0; r <= rmax; ++r) {
            for (long long i = c[0] - r; i <= c[0] + r; ++i) {
                if (i < 0 || i >= dims[0]) continue;
                for (long long j = c[1] - r; j <= c[1] + r; ++j) {
                    if (j < 0 || j >= dims[1]) continue;
                    for (long long k = c[2] - r; k <= c[2] + r; ++k) {
                        if (k < 0 || k >= dims[2]) continue;
                        if (std::max({std::llabs(i - c[0]), std::llabs(j - c[1]), std::llabs(k - c[2])}) != r) continue;
                        const long long kk = key(i, j, k);
                        auto it = std::lower_bound(cells.begin(), cells.end(), std::make_pair(kk, -1));
                        for (; it != cells.end() && it->first == kk; ++it) {
                            const auto& t = T[it->second];
                            const V3 q = closest_tri(p, P[t[0]], P[t[1]], P[t[2]]);
                            const double d = len2(q - p);
                            if (d < best) {
                                best = d;
                                bp = q;
                            }
                        }
                    }
                }
            }
            // every cell of ring r + 1 or beyond is at least r * h away from p
            if (best < 1e300 && best <= ((double)r * h) * ((double)r * h)) break;
        }
        return bp;
    }
};

struct System {
    Params P;
    GtGrid grid;
    int NP = 0, NT = 0, NE = 0, NH = 0, NGT = 0;
    std::vector<V3> gt, q, q_rest, qpn, qpd, p, target, grad, hd, r, z, v, Av;
    std::vector<double> w;
    std::vector<std::array<int, 3>> tri, gtri;
    std::vector<std::array<int, 2>> edge;
    std::vector<std::array<int, 4>> hinge;
    std::vector<double> elW, hang, hlen;
    std::vector<M2> elInv;
    std::vector<std::array<double, 144>> blocks;
    std::vector<std::array<int, 4>> cidx;
    std::vector<int> ct1, ct2;
    std::vector<double> cd;
    std::vector<std::array<V3, 4>> cdd;
    double radius = 1e-2, energy = 0, energy_prev = 0, ccd_step = 1;
    double mu = 0, la = 0;
    long long total_contacts = 0;
    int max_contacts = 0, halvings = 0;
    bool do_nothing = false;

    Elastic local(int f, const std::vector<V3>& x) const {
        Elastic L;
        const V3 x0 = x[tri[f][0]], x1 = x[tri[f][1]], x2 = x[tri[f][2]];
        const V3 x01 = x1 - x0, x02 = x2 - x0;
        L.b1 = nrm(x01);
        L.b2 = nrm(x02 - dot(x02, L.b1) * L.b1);
        const M2 Ds = {dot(L.b1, x01), dot(L.b1, x02), dot(L.b2, x01), dot(L.b2, x02)};
        L.inv = elInv[f];
        L.F = mm(Ds, L.inv);
        L.W = elW[f];
        return L;
    }

    // ------------------------------------------------------------ contacts (contact_detection.py:120-216)
    struct Grid {
        double cell = 1, lo[3] = {0, 0, 0};
        std::unordered_map<long long, std::vector<int>> cells;
        long long key(long long i, long long j, long long k) const { return (i * 73856093ll) ^ (j * 19349663ll) ^ (k * 83492791ll); }
        void idx(V3 p, long long* o) const {
            o[0] = (long long)std::floor((p.x - lo[0]) / cell);
            o[1] = (long long)std::floor((p.y - lo[1]) / cell);
            o[2] = (long long)std::floor((p.z - lo[2]) / cell);
        }
    };

    int detect() {
        const double thr = 2.0 * radius + P.d_hat;
        cidx.clear();
        ct1.clear();
        // boxes of triangles and edges, binned in a grid with cells >= thr
        Grid g;
        V3 mn{1e300, 1e300, 1e300};
        double ext = 0;
        for (auto& x : q) {
            mn.x = std::min(mn.x, x.x);
            mn.y = std::min(mn.y, x.y);
            mn.z = std::min(mn.z, x.z);
        }
        for (auto& x : q) ext = std::max({ext, x.x - mn.x, x.y - mn.y, x.z - mn.z});
        g.cell = std::max(thr, ext / 64.0);
        g.lo[0] = mn.x - 1;
        g.lo[1] = mn.y - 1;
        g.lo[2] = mn.z - 1;
        auto bin = [&](Grid& G, int id, V3 lo, V3 hi) {
            long long a[3], b[3];
            G.idx(lo, a);
            G.idx(hi, b);
            for (long long i = a[0]; i <= b[0]; ++i)
                for (long long j = a[1]; j <= b[1]; ++j)
                    for (long long k = a[2]; k <= b[2]; ++k) G.cells[G.key(i, j, k)].push_back(id);
        };
        auto lo3 = [](V3 a, V3 b) { return V3{std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; };
        auto hi3 = [](V3 a, V3 b) { return V3{std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; };
        Grid gt_ = g, ge = g;
        for (int f = 0; f < NT; ++f) {
            const V3 a = q[tri[f][0]], b = q[tri[f][1]], c = q[tri[f][2]];
            bin(gt_, f, lo3(lo3(a, b), c), hi3(hi3(a, b), c));
        }
        for (int e = 0; e < NE; ++e) {
            const V3 a = q[edge[e][0]], b = q[edge[e][1]];
            bin(ge, e, lo3(a, b), hi3(a, b));
        }
        const V3 T3{thr, thr, thr};
        std::vector<int> stamp(std::max(NT, NE), -1);
        long long raw = 0;
        for (int i0 = 0; i0 < NP; ++i0) {
            const V3 x0 = q[i0];
            long long a[3], b[3];
            g.idx(x0 - T3, a);
            g.idx(x0 + T3, b);
            std::vector<int> cand;
            for (long long i = a[0]; i <= b[0]; ++i)
                for (long long j = a[1]; j <= b[1]; ++j)
                    for (long long k = a[2]; k <= b[2]; ++k) {
                        auto it = gt_.cells.find(gt_.key(i, j, k));
                        if (it == gt_.cells.end()) continue;
                        for (int f : it->second)
                            if (stamp[f] != i0) {
                                stamp[f] = i0;
                                cand.push_back(f);
                            }
                    }
            std::sort(cand.begin(), cand.end());
            for (int f : cand) {
                const int i1 = tri[f][0], i2 = tri[f][1], i3 = tri[f][2];
                if (i0 == i1 || i0 == i2 || i0 == i3) continue;
                const int t = pt_classify(x0, q[i1], q[i2], q[i3]);
                if (pt_dist(x0, q[i1], q[i2], q[i3], t) <= thr) {
                    ++raw;
                    cidx.push_back({i0, i1, i2, i3});
                    ct1.push_back(BLOCK_PT);
                }
            }
        }
        std::fill(stamp.begin(), stamp.end(), -1);
        for (int e0 = 0; e0 < NE; ++e0) {
            const int i0 = edge[e0][0], i1 = edge[e0][1];
            const V3 x0 = q[i0], x1 = q[i1];
            long long a[3], b[3];
            g.idx(lo3(x0, x1) - T3, a);
            g.idx(hi3(x0, x1) + T3, b);
            std::vector<int> cand;
            for (long long i = a[0]; i <= b[0]; ++i)
                for (long long j = a[1]; j <= b[1]; ++j)
                    for (long long k = a[2]; k <= b[2]; ++k) {
                        auto it = ge.cells.find(ge.key(i, j, k));
                        if (it == ge.cells.end()) continue;
                        for (int e1 : it->second)
                            if (e1 > e0 && stamp[e1] != e0) {
                                stamp[e1] = e0;
                                cand.push_back(e1);
                            }
                    }
            std::sort(cand.begin(), cand.end());
            for (int e1 : cand) {
                const int i2 = edge[e1][0], i3 = edge[e1][1];
                if (i0 == i2 || i0 == i3 || i1 == i2 || i1 == i3) continue;
                const int t = ee_classify(x0, x1, q[i2], q[i3], P.ee_thres);
                if (ee_dist(x0, x1, q[i2], q[i3], t) <= thr) {
                    ++raw;
                    cidx.push_back({i0, i1, i2, i3});
                    ct1.push_back(BLOCK_EE);
                }
            }
        }
        if (raw > P.max_blocks) return -1;
        const int n = (int)cidx.size();
        ct2.assign(n, 0);
        cd.assign(n, 0);
        cdd.assign(n, {});
        max_contacts = std::max(max_contacts, n);
        total_contacts += n;
        return 0;
    }

    // ------------------------------------------------------------ energy (system.py:325-339)
    double compute_energy(const std::vector<V3>& x) {
        double e = 0;
        for (int i = 0; i < NP; ++i) e += 0.5 * len2(x[i] - target[i]) * (w[i] * P.m2gt_k);
        for (int f = 0; f < NT; ++f) {
            const Elastic L = local(f, x);
            const M2 E = ms(0.5, ma(mm(mt(L.F), L.F), M2{-1, 0, 0, -1}));
            const double trE = mtr(E);
            e += L.W * (mu * mtr(mm(E, mt(E))) + 0.5 * la * trE * trE);
        }
        for (int h = 0; h < NH; ++h) {
            const auto& i = hinge[h];
            const double dth = hinge_angle(x[i[0]], x[i[1]], x[i[2]], x[i[3]]) - hang[h];
            e += 0.5 * P.hinge_k * dth * dth * hlen[h];
        }
        for (size_t b = 0; b < cidx.size(); ++b) {
            const auto& i = cidx[b];
            const V3 x0 = x[i[0]], x1 = x[i[1]], x2 = x[i[2]], x3 = x[i[3]];
            double d;
            if (ct1[b] == BLOCK_PT) {
                ct2[b] = pt_classify(x0, x1, x2, x3);
                d = pt_dist(x0, x1, x2, x3, ct2[b]);
            } else {
                ct2[b] = ee_classify(x0, x1, x2, x3, P.ee_thres);
                d = ee_dist(x0, x1, x2, x3, ct2[b]);
            }
            cd[b] = d;
            if (d < P.d_hat) e += bar(d, P.d_hat) * P.coll_stiffness;
        }
        return e;
    }

    // ------------------------------------------------------------ gradient (coeff -1) and Hessian diagonal
    void compute_diff() {
        const double coeff = -1.0;
        std::fill(grad.begin(), grad.end(), V3{});
        std::fill(hd.begin(), hd.end(), V3{});
        for (int i = 0; i < NP; ++i) {
            const double wi = w[i] * P.m2gt_k;
            grad[i] = grad[i] + (q[i] - target[i]) * wi * coeff;
            hd[i] = hd[i] + V3{wi, wi, wi};
        }
        for (int f = 0; f < NT; ++f) {
            const Elastic L = local(f, q);
            const M2 E = ms(0.5, ma(mm(mt(L.F), L.F), M2{-1, 0, 0, -1}));
            const double trE = mtr(E);
            const M2 Pm = mm(L.F, ma(ms(2 * mu, E), ms(la * trE, M2{1, 0, 0, 1})));
            const M2 H = mm(ms(coeff * L.W, Pm), mt(L.inv));
            const V3 f1 = H.a * L.b1 + H.c * L.b2, f2 = H.b * L.b1 + H.d * L.b2;
            grad[tri[f][0]] = grad[tri[f][0]] + (-f1 - f2);
            grad[tri[f][1]] = grad[tri[f][1]] + f1;
            grad[tri[f][2]] = grad[tri[f][2]] + f2;
        }
        for (int h = 0; h < NH; ++h) hinge_diff(h, coeff);
        for (size_t b = 0; b < cidx.size(); ++b) {
            const double d = cd[b];
            if (d >= P.d_hat) continue;
            const auto& i = cidx[b];
            V3 g[4];
            if (ct1[b] == BLOCK_PT) pt_grad(q[i[0]], q[i[1]], q[i[2]], q[i[3]], ct2[b], g);
            else ee_grad(q[i[0]], q[i[1]], q[i[2]], q[i[3]], ct2[b], g);
            const double c1 = bar1(d, P.d_hat) * P.coll_stiffness * coeff, c2 = bar2(d, P.d_hat) * P.coll_stiffness;
            for (int k = 0; k < 4; ++k) {
                cdd[b][k] = g[k];
                grad[i[k]] = grad[i[k]] + g[k] * c1;
                hd[i[k]] = hd[i[k]] + c2 * V3{g[k].x * g[k].x, g[k].y * g[k].y, g[k].z * g[k].z};
            }
        }
    }

    void hinge_diff(int h, double coeff) {
        const auto& id = hinge[h];
        const V3 x0 = q[id[0]], x1 = q[id[1]], x2 = q[id[2]], x3 = q[id[3]];
        const V3 e0 = x2 - x1, e1 = x0 - x2, e2 = x0 - x1, e1_ = x3 - x2, e2_ = x3 - x1;
        const double e0l2 = len2(e0), e0l = std::sqrt(e0l2), e1l = len(e1), e2l = len(e2), e1l_ = len(e1_), e2l_ = len(e2_);
        const V3 e0u = nrm(e0), e1u = nrm(e1), e2u = nrm(e2), e1u_ = nrm(e1_), e2u_ = nrm(e2_);
        const double ca1 = dot(e2u, e0u), ca2 = -dot(e1u, e0u), ca1_ = dot(e2u_, e0u), ca2_ = -dot(e1u_, e0u);
        const double h0 = len(cross(e1, e2)) / e0l, h1 = len(cross(e0, e2)) / e1l, h2 = len(cross(e0, e1)) / e2l;
        const double h0_ = len(cross(e1_, e2_)) / e0l, h1_ = len(cross(e0, e2_)) / e1l_, h2_ = len(cross(e0, e1_)) / e2l_;
        const V3 n = nrm(cross(e0, e2)), n_ = nrm(cross(e2_, e0));
        const double theta = std::atan2(dot(cross(n, n_), e0) / e0l, dot(n, n_));
        const double dE = P.hinge_k * (theta - hang[h]) * hlen[h], d2E = P.hinge_k * hlen[h];
        const V3 g1 = n * (ca2 / h1) + n_ * (ca2_ / h1_), g2 = n * (ca1 / h2) + n_ * (ca1_ / h2_);
        const V3 g0 = n * (-1.0 / h0), g3 = n_ * (-1.0 / h0_);
        const V3 gg[4] = {g0, g1, g2, g3};
        for (int a = 0; a < 4; ++a) grad[id[a]] = grad[id[a]] + dE * gg[a] * coeff;
        const V3 m0 = nrm(cross(e0, n)), m1 = nrm(cross(e1, n)), m2 = nrm(cross(n, e2));
        const V3 m0_ = nrm(cross(n_, e0)), m1_ = nrm(cross(n_, e1_)), m2_ = nrm(cross(e2_, n_));
        const M3 M0 = outer(n, m0), M1 = outer(n, m1), M2_ = outer(n, m2);
        const M3 M0b = outer(n_, m0_), M1b = outer(n_, m1_), M2b = outer(n_, m2_);
        const M3 N0 = sc(1 / e0l2, M0), N0b = sc(1 / e0l2, M0b);
        const M3 P10 = sc(ca1 / (h1 * h0), T(M0)), P11 = sc(ca1 / (h1 * h1), T(M1)), P12 = sc(ca1 / (h1 * h2), T(M2_));
        const M3 P20 = sc(ca2 / (h2 * h0), T(M0)), P21 = sc(ca2 / (h2 * h1), T(M1)), P22 = sc(ca2 / (h2 * h2), T(M2_));
        const M3 P10b = sc(ca1_ / (h1_ * h0_), T(M0b)), P11b = sc(ca1_ / (h1_ * h1_), T(M1b)), P12b = sc(ca1_ / (h1_ * h2_), T(M2b));
        const M3 P20b = sc(ca2_ / (h2_ * h0_), T(M0b)), P21b = sc(ca2_ / (h2_ * h1_), T(M1b)), P22b = sc(ca2_ / (h2_ * h2_), T(M2b));
        const M3 Q0 = sc(1 / (h0 * h0), M0), Q1 = sc(1 / (h0 * h1), M1), Q2 = sc(1 / (h0 * h2), M2_);
        const M3 Q0b = sc(1 / (h0_ * h0_), M0b), Q1b = sc(1 / (h0_ * h1_), M1b), Q2b = sc(1 / (h0_ * h2_), M2b);
        M3 B[4][4];
        B[0][0] = add(sc(-dE, sym(Q0)), sc(d2E, outer(g0, g0)));
        B[3][3] = add(sc(-dE, sym(Q0b)), sc(d2E, outer(g3, g3)));
        B[1][1] = add(sc(dE, sub(add(sub(sym(P11), N0), sym(P11b)), N0b)), sc(d2E, outer(g1, g1)));
        B[2][2] = add(sc(dE, sub(add(sub(sym(P22), N0), sym(P22b)), N0b)), sc(d2E, outer(g2, g2)));
        B[1][0] = add(sc(dE, sub(P10, Q1)), sc(d2E, outer(g1, g0)));
        B[2][0] = add(sc(dE, sub(P20, Q2)), sc(d2E, outer(g2, g0)));
        B[1][3] = add(sc(dE, sub(P10b, Q1b)), sc(d2E, outer(g1, g3)));
        B[2][3] = add(sc(dE, sub(P20b, Q2b)), sc(d2E, outer(g2, g3)));
        B[1][2] = add(sc(dE, add(add(add(add(add(P12, T(P21)), N0), P12b), T(P21b)), N0b)), sc(d2E, outer(g1, g2)));
        B[0][3] = sc(d2E, outer(g0, g3));
        B[0][1] = T(B[1][0]);
        B[0][2] = T(B[2][0]);
        B[3][1] = T(B[1][3]);
        B[3][2] = T(B[2][3]);
        B[2][1] = T(B[1][2]);
        B[3][0] = T(B[0][3]);
        for (int a = 0; a < 4; ++a) hd[id[a]] = hd[id[a]] + V3{B[a][a][0][0], B[a][a][1][1], B[a][a][2][2]};
        auto& out = blocks[h];
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) out[((a * 4 + b) * 3 + i) * 3 + j] = B[a][b][i][j];
        spd_project(out.data());
    }

    // block_spd_project_kernel (utils_kernels.py:21-39) with the PSD projection restated as Jacobi sweeps
    void spd_project(double* B) const {
        double A[9][9], V[9][9];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) A[a * 3 + i][b * 3 + j] = B[((a * 4 + b) * 3 + i) * 3 + j];
        for (int i = 0; i < 9; ++i)
            for (int j = 0; j < 9; ++j) V[i][j] = i == j;
        for (int i = 0; i < 9; ++i)
            for (int j = i + 1; j < 9; ++j) A[i][j] = A[j][i] = 0.5 * (A[i][j] + A[j][i]);
        for (int sw = 0; sw < P.spd_max_iters; ++sw)
            for (int p = 0; p < 8; ++p)
                for (int qq = p + 1; qq < 9; ++qq) {
                    const double apq = A[p][qq];
                    if (std::fabs(apq) < 1e-30) continue;
                    const double th = (A[qq][qq] - A[p][p]) / (2 * apq);
                    const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
                    const double c = 1 / std::sqrt(t * t + 1), s = t * c;
                    for (int k = 0; k < 9; ++k) {
                        const double akp = A[k][p], akq = A[k][qq];
                        A[k][p] = c * akp - s * akq;
                        A[k][qq] = s * akp + c * akq;
                    }
                    for (int k = 0; k < 9; ++k) {
                        const double apk = A[p][k], aqk = A[qq][k];
                        A[p][k] = c * apk - s * aqk;
                        A[qq][k] = s * apk + c * aqk;
                    }
                    for (int k = 0; k < 9; ++k) {
                        const double vkp = V[k][p], vkq = V[k][qq];
                        V[k][p] = c * vkp - s * vkq;
                        V[k][qq] = s * vkp + c * vkq;
                    }
                }
        double lam[9];
        for (int i = 0; i < 9; ++i) lam[i] = std::max(A[i][i], 0.0);
        for (int i = 0; i < 9; ++i)
            for (int j = 0; j < 9; ++j) {
                double s = 0;
                for (int k = 0; k < 9; ++k) s += V[i][k] * lam[k] * V[j][k];
                A[i][j] = s;
            }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) B[((a * 4 + b) * 3 + i) * 3 + j] = A[a * 3 + i][b * 3 + j];
        for (int b = 0; b < 3; ++b)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double s = 0;
                    for (int a = 0; a < 3; ++a) s -= B[((a * 4 + b) * 3 + i) * 3 + j];
                    B[((12 + b) * 3 + i) * 3 + j] = s;
                }
        for (int b = 0; b < 3; ++b)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) B[((b * 4 + 3) * 3 + i) * 3 + j] = B[((12 + b) * 3 + j) * 3 + i];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int b = 0; b < 3; ++b) s -= B[((b * 4 + 3) * 3 + i) * 3 + j];
                B[((15) * 3 + i) * 3 + j] = s;
            }
    }

    // ------------------------------------------------------------ Hessian-vector product (system.py:348-352)
    void hess_dx(const std::vector<V3>& dx, std::vector<V3>& out) const {
        std::fill(out.begin(), out.end(), V3{});
        for (int i = 0; i < NP; ++i) out[i] = out[i] + dx[i] * (w[i] * P.m2gt_k);
        for (int f = 0; f < NT; ++f) {
            const Elastic L = local(f, q);
            const int i0 = tri[f][0], i1 = tri[f][1], i2 = tri[f][2];
            const V3 d01 = dx[i1] - dx[i0], d02 = dx[i2] - dx[i0];
            const M2 dDs = {dot(L.b1, d01), dot(L.b1, d02), dot(L.b2, d01), dot(L.b2, d02)};
            const M2 dF = mm(dDs, L.inv);
            const M2 I = {1, 0, 0, 1};
            const M2 E = ms(0.5, ma(mm(mt(L.F), L.F), ms(-1, I)));
            const double trE = mtr(E);
            const M2 dE = ms(0.5, ma(mm(mt(dF), L.F), mm(mt(L.F), dF)));
            const double trdE = mtr(dE);
            const M2 dP = ma(mm(dF, ma(ms(2 * mu, E), ms(la * trE, I))), mm(L.F, ma(ms(2 * mu, dE), ms(la * trdE, I))));
            const M2 dH = mm(ms(L.W, dP), mt(L.inv));
            const V3 df1 = dH.a * L.b1 + dH.c * L.b2, df2 = dH.b * L.b1 + dH.d * L.b2;
            out[i0] = out[i0] + (-df1 - df2);
            out[i1] = out[i1] + df1;
            out[i2] = out[i2] + df2;
        }
        for (int h = 0; h < NH; ++h) {
            const auto& id = hinge[h];
            const double* B = blocks[h].data();
            for (int a = 0; a < 4; ++a) {
                V3 acc{};
                for (int b = 0; b < 4; ++b) {
                    const double* M = B + (a * 4 + b) * 9;
                    const V3 d = dx[id[b]];
                    acc = acc + V3{M[0] * d.x + M[1] * d.y + M[2] * d.z, M[3] * d.x + M[4] * d.y + M[5] * d.z,
                                   M[6] * d.x + M[7] * d.y + M[8] * d.z};
                }
                out[id[a]] = out[id[a]] + acc;
            }
        }
        for (size_t b = 0; b < cidx.size(); ++b) {
            if (cd[b] >= P.d_hat) continue;
            const double c = bar2(cd[b], P.d_hat) * P.coll_stiffness;
            double s = 0;
            for (int k = 0; k < 4; ++k) s += dot(cdd[b][k], dx[cidx[b][k]]);
            for (int k = 0; k < 4; ++k) out[cidx[b][k]] = out[cidx[b][k]] + cdd[b][k] * (s * c);
        }
    }

    static double vdot(const std::vector<V3>& a, const std::vector<V3>& b) {
        double s = 0;
        for (size_t i = 0; i < a.size(); ++i) s += dot(a[i], b[i]);
        return s;
    }

    // cg_solver.py:46-158
    void cg() {
        for (int i = 0; i < NP; ++i) {
            p[i] = V3{};
            r[i] = grad[i];
            z[i] = V3{r[i].x / (hd[i].x + 1e-6), r[i].y / (hd[i].y + 1e-6), r[i].z / (hd[i].z + 1e-6)};
            v[i] = z[i];
        }
        double zr = vdot(z, r);
        for (int it = 0; it < P.n_cg_iters; ++it) {
            hess_dx(v, Av);
            const double vAv = vdot(v, Av);
            const double zr_last = zr;
            for (int i = 0; i < NP; ++i) {
                if (vAv > 1e-16) {
                    const double alpha = zr_last / vAv;
                    p[i] = p[i] + alpha * v[i];
                    r[i] = r[i] - alpha * Av[i];
                }
                z[i] = V3{r[i].x / hd[i].x, r[i].y / hd[i].y, r[i].z / hd[i].z};
            }
            zr = vdot(z, r);
            const double s = zr / zr_last;
            for (int i = 0; i < NP; ++i) v[i] = z[i] + s * v[i];
        }
    }

    // accd_kernel (ccd_kernels.py:9-111)
    void accd() {
        ccd_step = 1.0;
        for (size_t b = 0; b < cidx.size(); ++b) {
            const auto& id = cidx[b];
            V3 x0 = q[id[0]], x1 = q[id[1]], x2 = q[id[2]], x3 = q[id[3]];
            V3 v0 = p[id[0]], v1 = p[id[1]], v2 = p[id[2]], v3 = p[id[3]];
            const V3 va = (v0 + v1 + v2 + v3) / 4.0;
            v0 = v0 - va;
            v1 = v1 - va;
            v2 = v2 - va;
            v3 = v3 - va;
            double lv;
            if (ct1[b] == BLOCK_PT) lv = len(v0) + std::max(len(v1), std::max(len(v2), len(v3)));
            else lv = std::max(len(v0), len(v1)) + std::max(len(v2), len(v3));
            if (lv < 1e-12) continue;
            auto dist = [&]() {
                if (ct1[b] == BLOCK_PT) return pt_dist(x0, x1, x2, x3, pt_classify(x0, x1, x2, x3));
                return ee_dist(x0, x1, x2, x3, ee_classify(x0, x1, x2, x3, P.ee_thres));
            };
            const double th = P.ccd_thickness;
            double d = dist();
            double dmt = std::max((d * d - th * th) / (std::sqrt(d * d) + th), 0.0);
            const double gap = (1.0 - P.ccd_slackness) * dmt;
            double t = 0, tl = P.ccd_slackness * dmt / lv;
            int it = 0;
            while (true) {
                x0 = x0 + tl * v0;
                x1 = x1 + tl * v1;
                x2 = x2 + tl * v2;
                x3 = x3 + tl * v3;
                d = dist();
                dmt = std::max((d * d - th * th) / (std::sqrt(d * d) + th), 0.0);
                if ((it > 0 && dmt <= gap) || it >= P.ccd_max_iters) {
                    ccd_step = std::min(ccd_step, t);
                    break;
                }
                t += tl;
                if (t > 1.0) break;
                tl = 0.8 * dmt / lv;
                ++it;
            }
        }
    }

    void update_targets() {
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < NP; ++i) target[i] = grid.nearest(q[i], gt, gtri);
    }

    int step() {
        // _update_vertex_target (geometry_kernels.py:81-93)
        update_targets();
        for (int it = 0; it < P.n_newton_iters; ++it) {
            qpn = q;
            int guard = 0;
            while (detect() == -1) {
                radius *= 0.5;
                ++halvings;
                if (++guard > 40) return 3;
            }
            qpd = q;
            energy = compute_energy(q);
            compute_diff();
            cg();
            for (int i = 0; i < NP; ++i) {  // clamp_p_kernel
                const V3 dq = qpn[i] + p[i] - qpd[i];
                if (len(dq) > P.radius) p[i] = nrm(dq) * P.radius + qpd[i] - qpn[i];
            }
            accd();
            energy_prev = energy;
            for (int n = 0; n < P.n_line_search_iters; ++n) {
                if (!(n > 0 && energy < energy_prev)) {
                    const double a = ccd_step * std::pow(0.5, (double)n);
                    for (int i = 0; i < NP; ++i) q[i] = qpn[i] + a * p[i];
                }
                energy = compute_energy(q);
            }
        }
        return 0;
    }
};

}  // namespace s3o

using namespace s3o;

extern "C" {

// params (17 doubles, the order of Stage3Params): n_newton_iters, n_cg_iters, n_line_search_iters, d_hat,
// coll_stiffness, contact_detection_radius, ee_classify_thres, ccd_slackness, ccd_thickness, ccd_max_iters,
// spd_max_iters, elas_young_modulus, elas_poisson_ratio, hinge_stiffness, mesh2gt_dist_stiffness,
// min_angle_thres, max_blocks.  stats (11 doubles): particles, triangles, edges, hinges, steps, Newton
// iterations, most contacts, halvings, do_nothing, final energy, total contacts.  Returns 0, or 1 for a bad
// index, 3 when contacts stay above max_blocks.
static int s3_setup(System& S, double& scale, double* t, const double* gt_pts, const int* gt_tris, int ngp, int ngt,
                    const double* pts, const int* tris, int np, int nt, const double* params) {
    Params& P = S.P;
    P.n_newton_iters = (int)params[0];
    P.n_cg_iters = (int)params[1];
    P.n_line_search_iters = (int)params[2];
    P.d_hat = params[3];
    P.coll_stiffness = params[4];
    P.radius = params[5];
    P.ee_thres = params[6];
    P.ccd_slackness = params[7];
    P.ccd_thickness = params[8];
    P.ccd_max_iters = (int)params[9];
    P.spd_max_iters = (int)params[10];
    P.young = params[11];
    P.poisson = params[12];
    P.hinge_k = params[13];
    P.m2gt_k = params[14];
    P.min_angle = params[15];
    P.max_blocks = (long long)params[16];
    S.radius = P.radius;
    S.mu = P.young / (2.0 * (1.0 + P.poisson));
    S.la = P.young * P.poisson / ((1.0 + P.poisson) * (1.0 - 2.0 * P.poisson));
    for (int i = 0; i < 3 * nt; ++i)
        if (tris[i] < 0 || tris[i] >= np) return 1;
    for (int i = 0; i < 3 * ngt; ++i)
        if (gt_tris[i] < 0 || gt_tris[i] >= ngp) return 1;
    // normalisation (processing.py:15-21)
    double c[3] = {0, 0, 0}, mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < ngp; ++i)
        for (int d = 0; d < 3; ++d) {
            c[d] += gt_pts[3 * i + d];
            mn[d] = std::min(mn[d], gt_pts[3 * i + d]);
            mx[d] = std::max(mx[d], gt_pts[3 * i + d]);
        }
    double ext = 0;
    for (int d = 0; d < 3; ++d) {
        c[d] /= ngp;
        ext = std::max(ext, mx[d] - mn[d]);
    }
    scale = 1.0 / ext;
    for (int d = 0; d < 3; ++d) t[d] = -c[d] * scale;
    auto normed = [&](const double* a, int i) { return V3{a[3 * i] * scale + t[0], a[3 * i + 1] * scale + t[1], a[3 * i + 2] * scale + t[2]}; };
    S.NP = np;
    S.NT = nt;
    S.NGT = ngt;
    S.gt.resize(ngp);
    for (int i = 0; i < ngp; ++i) S.gt[i] = normed(gt_pts, i);
    S.gtri.resize(ngt);
    for (int f = 0; f < ngt; ++f) S.gtri[f] = {gt_tris[3 * f], gt_tris[3 * f + 1], gt_tris[3 * f + 2]};
    S.grid.build(S.gt, S.gtri);
    S.q.resize(np);
    for (int i = 0; i < np; ++i) S.q[i] = normed(pts, i);
    S.q_rest = S.q;
    S.tri.resize(nt);
    for (int f = 0; f < nt; ++f) S.tri[f] = {tris[3 * f], tris[3 * f + 1], tris[3 * f + 2]};
    // edges_unique ordered by (larger, smaller); hinges of hinge_preprocess_slow_kernel
    std::vector<long long> uk;
    std::vector<std::pair<long long, int>> dk;
    for (int f = 0; f < nt; ++f)
        for (int k = 0; k < 3; ++k) {
            const long long a = tris[3 * f + k], b = tris[3 * f + (k + 1) % 3];
            uk.push_back(std::max(a, b) * np + std::min(a, b));
            dk.push_back({a * np + b, 3 * f + k});
        }
    std::sort(uk.begin(), uk.end());
    uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
    std::sort(dk.begin(), dk.end());
    for (long long k : uk) S.edge.push_back({(int)(k % np), (int)(k / np)});
    for (int f = 0; f < nt; ++f)
        for (int k = 0; k < 3; ++k) {
            const int a = tris[3 * f + k], b = tris[3 * f + (k + 1) % 3], cc = tris[3 * f + (k + 2) % 3];
            if (!(a < b)) continue;
            const long long key = (long long)b * np + a;
            for (auto it = std::lower_bound(dk.begin(), dk.end(), std::make_pair(key, -1)); it != dk.end() && it->first == key; ++it)
                S.hinge.push_back({cc, a, b, tris[3 * (it->second / 3) + (it->second % 3 + 2) % 3]});
        }
    S.NE = (int)S.edge.size();
    S.NH = (int)S.hinge.size();
    // Voronoi weights (igl::massmatrix VORONOI) in float64
    S.w.assign(np, 0.0);
    for (int f = 0; f < nt; ++f) {
        V3 pp[3];
        for (int k = 0; k < 3; ++k) pp[k] = S.q[S.tri[f][k]];
        double l[3];
        for (int k = 0; k < 3; ++k) l[k] = std::sqrt(len2(pp[(k + 1) % 3] - pp[(k + 2) % 3]));
        double a = l[0], b = l[1], cc = l[2];
        if (a < b) std::swap(a, b);
        if (b < cc) std::swap(b, cc);
        if (a < b) std::swap(a, b);
        double dblA = 0.5 * std::sqrt((a + (b + cc)) * (cc - (a - b)) * (cc + (a - b)) * (a + (b - cc)));
        if (dblA != dblA) dblA = 0;
        double cs[3], bc[3];
        for (int k = 0; k < 3; ++k) {
            const int j = (k + 1) % 3, m = (k + 2) % 3;
            cs[k] = (l[m] * l[m] + l[j] * l[j] - l[k] * l[k]) / (l[j] * l[m] * 2.0);
            bc[k] = cs[k] * l[k];
        }
        const double sum = bc[0] + bc[1] + bc[2];
        double part[3], quad[3];
        for (int k = 0; k < 3; ++k) part[k] = (bc[k] / sum) * (dblA * 0.5);
        for (int k = 0; k < 3; ++k) quad[k] = (part[(k + 1) % 3] + part[(k + 2) % 3]) * 0.5;
        for (int o = 0; o < 3; ++o)
            if (cs[o] < 0)
                for (int k = 0; k < 3; ++k) quad[k] = (k == o) ? 0.25 * dblA : 0.125 * dblA;
        for (int k = 0; k < 3; ++k) S.w[S.tri[f][k]] += quad[k];
    }
    // StVK rest shapes (elastic_energy.py:7-37), Warp's 2x2 inverse: adjugate times 1/det, zero if det == 0
    S.elW.resize(nt);
    S.elInv.resize(nt);
    for (int f = 0; f < nt; ++f) {
        const V3 x0 = S.q_rest[S.tri[f][0]], x1 = S.q_rest[S.tri[f][1]], x2 = S.q_rest[S.tri[f][2]];
        const V3 x01 = x1 - x0, x02 = x2 - x0;
        S.elW[f] = 0.5 * len(cross(x01, x02));
        const V3 b1 = nrm(x01), b2 = nrm(x02 - dot(x02, b1) * b1);
        const double a = dot(b1, x01), b = dot(b1, x02), c2 = dot(b2, x01), d = dot(b2, x02);
        const double det = a * d - c2 * b;
        S.elInv[f] = det != 0 ? M2{d * (1.0 / det), -b * (1.0 / det), -c2 * (1.0 / det), a * (1.0 / det)} : M2{0, 0, 0, 0};
    }
    S.hang.resize(S.NH);
    S.hlen.resize(S.NH);
    for (int h = 0; h < S.NH; ++h) {
        const auto& i = S.hinge[h];
        S.hang[h] = hinge_angle(S.q_rest[i[0]], S.q_rest[i[1]], S.q_rest[i[2]], S.q_rest[i[3]]);
        S.hlen[h] = len(S.q_rest[i[1]] - S.q_rest[i[2]]);
    }
    S.blocks.assign(S.NH, {});
    // minimum internal angle (system.py:214-221) with numpy's NaN propagation
    bool any_nan = false, any_small = false;
    for (int f = 0; f < nt; ++f) {
        double s[3];
        for (int k = 0; k < 3; ++k) s[k] = len2(S.q[S.tri[f][(k + 1) % 3]] - S.q[S.tri[f][(k + 2) % 3]]);
        for (int d = 0; d < 3; ++d) {
            const double deg = std::acos((s[(d + 2) % 3] + s[(d + 1) % 3] - s[d]) / (2. * std::sqrt(s[(d + 2) % 3] * s[(d + 1) % 3]))) * 180.0 / 3.141592653589793;
            if (deg != deg) any_nan = true;
            else if (deg <= P.min_angle) any_small = true;
        }
    }
    S.do_nothing = any_small && !any_nan;
    for (auto* vec : {&S.qpn, &S.qpd, &S.p, &S.target, &S.grad, &S.hd, &S.r, &S.z, &S.v, &S.Av}) vec->assign(np, V3{});
    return 0;
}

int s3_oracle_run(const double* gt_pts, const int* gt_tris, int ngp, int ngt, const double* pts, const int* tris,
                  int np, int nt, int n_iters, const double* params, double* out, double* stats) {
    System S;
    const Params& P = S.P;
    double scale = 1, t[3] = {0, 0, 0};
    const int rs = s3_setup(S, scale, t, gt_pts, gt_tris, ngp, ngt, pts, tris, np, nt, params);
    if (rs) return rs;
    int steps = 0;
    if (!S.do_nothing)
        for (int it = 0; it < n_iters; ++it) {
            ++steps;
            const int rc = S.step();
            if (rc) return rc;
        }
    for (int i = 0; i < np; ++i) {
        out[3 * i] = (S.q[i].x - t[0]) / scale;
        out[3 * i + 1] = (S.q[i].y - t[1]) / scale;
        out[3 * i + 2] = (S.q[i].z - t[2]) / scale;
    }
    if (stats) {
        const double v[11] = {(double)np, (double)nt, (double)S.NE, (double)S.NH, (double)steps,
                              (double)steps * P.n_newton_iters, (double)S.max_contacts, (double)S.halvings,
                              (double)S.do_nothing, S.energy, (double)S.total_contacts};
        std::memcpy(stats, v, sizeof(v));
    }
    return 0;
}

// Energy, gradient (dE/dq, normalised frame), Hessian diagonal and Hessian-vector product for the direction
// dx after one target update and one contact detection at x0 (normalised frame; NULL: the registered mesh),
// with the rest state of the registered mesh: the pieces a Newton iteration consumes (system.py:325-352),
// for finite-difference checks of the restated formulas. out arrays are np x 3; qn receives the evaluation
// point.
int s3_oracle_probe(const double* gt_pts, const int* gt_tris, int ngp, int ngt, const double* pts, const int* tris,
                    int np, int nt, const double* params, const double* x0, const double* dx, double* qn,
                    double* energy, double* grad, double* hdiag, double* hvp, int* n_contacts) {
    System S;
    double scale = 1, t[3] = {0, 0, 0};
    const int rs = s3_setup(S, scale, t, gt_pts, gt_tris, ngp, ngt, pts, tris, np, nt, params);
    if (rs) return rs;
    if (x0)
        for (int i = 0; i < np; ++i) S.q[i] = V3{x0[3 * i], x0[3 * i + 1], x0[3 * i + 2]};
    S.update_targets();
    if (S.detect() == -1) return 3;
    *n_contacts = (int)S.cidx.size();
    energy[0] = S.compute_energy(S.q);
    S.compute_diff();
    std::vector<V3> d(np), o(np);
    for (int i = 0; i < np; ++i) d[i] = V3{dx[3 * i], dx[3 * i + 1], dx[3 * i + 2]};
    S.hess_dx(d, o);
    for (int i = 0; i < np; ++i) {
        const double g[3] = {-S.grad[i].x, -S.grad[i].y, -S.grad[i].z};  // grad holds -dE/dq (coeff -1)
        const double h[3] = {S.hd[i].x, S.hd[i].y, S.hd[i].z}, a[3] = {o[i].x, o[i].y, o[i].z};
        const double qq[3] = {S.q[i].x, S.q[i].y, S.q[i].z};
        for (int k = 0; k < 3; ++k) {
            grad[3 * i + k] = g[k];
            hdiag[3 * i + k] = h[k];
            hvp[3 * i + k] = a[k];
            qn[3 * i + k] = qq[k];
        }
    }
    return 0;
}

// Energy at normalised positions x (np x 3) with the targets and contact set of s3_oracle_probe at x0
// (recomputed the same way), for finite differences.
int s3_oracle_energy_at(const double* gt_pts, const int* gt_tris, int ngp, int ngt, const double* pts, const int* tris,
                        int np, int nt, const double* params, const double* x0, const double* x, double* energy) {
    System S;
    double scale = 1, t[3] = {0, 0, 0};
    const int rs = s3_setup(S, scale, t, gt_pts, gt_tris, ngp, ngt, pts, tris, np, nt, params);
    if (rs) return rs;
    if (x0)
        for (int i = 0; i < np; ++i) S.q[i] = V3{x0[3 * i], x0[3 * i + 1], x0[3 * i + 2]};
    S.update_targets();
    if (S.detect() == -1) return 3;
    std::vector<V3> xv(np);
    for (int i = 0; i < np; ++i) xv[i] = V3{x[3 * i], x[3 * i + 1], x[3 * i + 2]};
    energy[0] = S.compute_energy(xv);
    return 0;
}

}  // extern "C"
