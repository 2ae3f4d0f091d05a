// Device triangle-triangle decision of the reference's self-intersection check
// (simp_cuda/src/bvh/self_intersect.cuh:129-149 and :233-377, tri_tri_3d.cuh:20-297, math.cuh:42-51).
//
// The reference evaluates, for every candidate (query f, hit g): translate both triangles by the floored
// mean of their coordinates, skip coplanar pairs (fp64 plane test), skip pairs that share an edge by index
// or by coordinates, run the Blender-style fp64/fp32 segment test, and drop a hit whose segment is shorter
// than eps (L-inf) when the pair shares one vertex. The decision below returns the same boolean. It is
// reordered only where every branch it skips returns "no intersection" in the reference as well:
//   * two or three shared vertex indices -> no intersection whatever the coplanarity test says;
//   * two coordinate-shared vertices      -> no intersection whatever the coplanarity test says;
//   * a float certificate of the reference's own coplanarity test (whose normal is not normalised, so on
//     fine meshes nearly every pair of neighbours counts as coplanar and is skipped);
//   * a float orientation filter with a rigorous error bound (Shewchuk's orient3d static bound written
//     for binary32) that proves one triangle lies strictly on one side of the other's plane. For pairs
//     with no shared vertex the reference then returns at its first or second side test (or earlier at
//     the coplanar test). For pairs sharing one vertex both triangles' free vertices must pass: the
//     segment the reference computes then degenerates to the shared vertex and the eps rule drops it.
// Only pairs the filter cannot decide take the fp64 path.
#pragma once
#include "pamo_common.cuh"

namespace pamo {

struct Tri9 {
    float v[3][3];
};

__device__ __forceinline__ int floor_mean6(float a, float b, float c, float d, float e, float f) {
    float mean = (a + b + c + d + e + f) / 6.0f;
    return (int)floorf(mean);
}

__device__ __forceinline__ bool same_eps(const float* a, const float* b, float eps) {
    return fabsf(a[0] - b[0]) < eps && fabsf(a[1] - b[1]) < eps && fabsf(a[2] - b[2]) < eps;
}

__device__ __forceinline__ void plane_db(const Tri9& T, double pl[4]) {
    double ba0 = (double)T.v[0][0] - (double)T.v[1][0], ba1 = (double)T.v[0][1] - (double)T.v[1][1],
           ba2 = (double)T.v[0][2] - (double)T.v[1][2];
    double bc0 = (double)T.v[2][0] - (double)T.v[1][0], bc1 = (double)T.v[2][1] - (double)T.v[1][1],
           bc2 = (double)T.v[2][2] - (double)T.v[1][2];
    pl[0] = ba1 * bc2 - ba2 * bc1;
    pl[1] = ba2 * bc0 - ba0 * bc2;
    pl[2] = ba0 * bc1 - ba1 * bc0;
    pl[3] = -(pl[0] * (double)T.v[1][0] + pl[1] * (double)T.v[1][1] + pl[2] * (double)T.v[1][2]);
}

__device__ __forceinline__ double dot_dbfl(const double* a, const float* b) {
    return a[0] * (double)b[0] + a[1] * (double)b[1] + a[2] * (double)b[2];
}

__device__ __noinline__ bool coplanar_db(const Tri9& A, const Tri9& B) {
    float scale = 0.0f;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) scale = fmaxf(scale, fabsf(A.v[i][j]));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) scale = fmaxf(scale, fabsf(B.v[i][j]));
    double pa[4];
    plane_db(A, pa);
    double s0 = dot_dbfl(pa, B.v[0]) + pa[3];
    double s1 = dot_dbfl(pa, B.v[1]) + pa[3];
    double s2 = dot_dbfl(pa, B.v[2]) + pa[3];
    double eps = (double)scale * 1e-6;
    return fabs(s0) <= eps && fabs(s1) <= eps && fabs(s2) <= eps;
}

__device__ __forceinline__ void lerp3(float* r, const float* a, const float* b, float t) {
    const float s = 1.0f - t;
    r[0] = s * a[0] + t * b[0];
    r[1] = s * a[1] + t * b[1];
    r[2] = s * a[2] + t * b[2];
}

__device__ __forceinline__ void cp3(float* r, const float* a) {
    r[0] = a[0];
    r[1] = a[1];
    r[2] = a[2];
}

// isect_tri_tri_v3_ex: returns true with the shared segment in r1, r2
__device__ __noinline__ bool isect_tri_tri_db(const Tri9& A, const Tri9& B, float* r1, float* r2) {
    float rmn[2], rmx[2], loc[2][2][3];
    float side[2][3];
    double pa[4], pb[4];
    plane_db(A, pa);
    side[1][0] = (float)(dot_dbfl(pa, B.v[0]) + pa[3]);
    side[1][1] = (float)(dot_dbfl(pa, B.v[1]) + pa[3]);
    side[1][2] = (float)(dot_dbfl(pa, B.v[2]) + pa[3]);
    if (side[1][0] == 0.0f && side[1][1] == 0.0f && side[1][2] == 0.0f) return false;
    if ((side[1][0] != 0.0f && side[1][1] != 0.0f && side[1][2] != 0.0f) && (side[1][0] < 0.0f) == (side[1][1] < 0.0f) &&
        (side[1][0] < 0.0f) == (side[1][2] < 0.0f))
        return false;
    plane_db(B, pb);
    side[0][0] = (float)(dot_dbfl(pb, A.v[0]) + pb[3]);
    side[0][1] = (float)(dot_dbfl(pb, A.v[1]) + pb[3]);
    side[0][2] = (float)(dot_dbfl(pb, A.v[2]) + pb[3]);
    if ((side[0][0] != 0.0f && side[0][1] != 0.0f && side[0][2] != 0.0f) && (side[0][0] < 0.0f) == (side[0][1] < 0.0f) &&
        (side[0][0] < 0.0f) == (side[0][2] < 0.0f))
        return false;
    double dir[3] = {pa[1] * pb[2] - pa[2] * pb[1], pa[2] * pb[0] - pa[0] * pb[2], pa[0] * pb[1] - pa[1] * pb[0]};
    for (int i = 0; i < 2; ++i) {
        const Tri9& T = (i == 0) ? A : B;
        const float* s = side[i];
        int t0, t1, t2;
        if ((s[0] != 0.0f && s[1] != 0.0f) && (s[0] < 0.0f) == (s[1] < 0.0f)) {
            t0 = 1; t1 = 2; t2 = 0;
        } else if ((s[1] != 0.0f && s[2] != 0.0f) && (s[1] < 0.0f) == (s[2] < 0.0f)) {
            t0 = 2; t1 = 0; t2 = 1;
        } else if (s[1] == 0.0f && (s[2] < 0.0f) != (s[0] < 0.0f)) {
            t0 = 1; t1 = 2; t2 = 0;
        } else {
            t0 = 0; t1 = 1; t2 = 2;
        }
        double dot_b = dot_dbfl(dir, T.v[t1]);
        float sidec = s[t1];
        if (sidec != 0.0f) {
            double dot_a = dot_dbfl(dir, T.v[t0]);
            double dot_c = dot_dbfl(dir, T.v[t2]);
            float fac0 = sidec / (sidec - s[t0]);
            float fac1 = sidec / (sidec - s[t2]);
            double off0 = (double)fac0 * (dot_a - dot_b);
            double off1 = (double)fac1 * (dot_c - dot_b);
            if (off0 > off1) {
                double td = off0; off0 = off1; off1 = td;
                float tf = fac0; fac0 = fac1; fac1 = tf;
                int ti = t0; t0 = t2; t2 = ti;
            }
            rmn[i] = (float)(dot_b + off0);
            rmx[i] = (float)(dot_b + off1);
            lerp3(loc[i][0], T.v[t1], T.v[t0], fac0);
            lerp3(loc[i][1], T.v[t1], T.v[t2], fac1);
        } else {
            rmn[i] = rmx[i] = (float)dot_b;
            cp3(loc[i][0], T.v[t1]);
            cp3(loc[i][1], T.v[t1]);
        }
    }
    if ((rmx[0] > rmn[1]) && (rmn[0] < rmx[1])) {
        if (rmn[0] >= rmn[1]) {
            cp3(r1, loc[0][0]);
            if (rmx[0] <= rmx[1]) cp3(r2, loc[0][1]);
            else cp3(r2, loc[1][1]);
        } else {
            if (rmx[0] <= rmx[1]) {
                cp3(r1, loc[0][1]);
                cp3(r2, loc[1][0]);
            } else {
                cp3(r1, loc[1][0]);
                cp3(r2, loc[1][1]);
            }
        }
        return true;
    }
    return false;
}

// Float orientation of p against A's plane: the sign of det[a0 - p, a1 - p, a2 - p], which equals the
// reference's plane value n_a . (p - a1) with n_a = (a0 - a1) x (a2 - a1). Returns +1 / -1 when the sign is
// certain, 0 otherwise. The error bound is Shewchuk's orient3d static filter, (7 + 56 eps) eps * permanent
// with eps = 2^-24 (taken as 8e-7), plus abs_err, which covers the cancellation of the reference's fp64
// evaluation dot(n_a, p) - dot(n_a, a1) with a 1e5 margin, so that a certain float sign is also the sign of
// the reference's value and, for a vertex shared by both faces, the reference's near-zero value is at most
// 1e-5 of the others.
__device__ __forceinline__ int orient_f(const float* a0, const float* a1, const float* a2, const float* p, float abs_err) {
    const float adx = a0[0] - p[0], ady = a0[1] - p[1], adz = a0[2] - p[2];
    const float bdx = a1[0] - p[0], bdy = a1[1] - p[1], bdz = a1[2] - p[2];
    const float cdx = a2[0] - p[0], cdy = a2[1] - p[1], cdz = a2[2] - p[2];
    const float bc = bdx * cdy - bdy * cdx, ca = cdx * ady - cdy * adx, ab = adx * bdy - ady * bdx;
    const float det = adz * bc + bdz * ca + cdz * ab;
    const float perm = (fabsf(bdx * cdy) + fabsf(bdy * cdx)) * fabsf(adz) + (fabsf(cdx * ady) + fabsf(cdy * adx)) * fabsf(bdz) +
                       (fabsf(adx * bdy) + fabsf(ady * bdx)) * fabsf(cdz);
    const float err = 8.0e-7f * perm + abs_err + 1e-30f;
    if (det > err) return 1;
    if (det < -err) return -1;
    return 0;
}

// every vertex of B except index `skip` lies strictly on one side of A's plane
__device__ __forceinline__ bool strictly_one_side(const Tri9& A, const Tri9& B, int skip, float cmax) {
    const float e0x = A.v[0][0] - A.v[1][0], e0y = A.v[0][1] - A.v[1][1], e0z = A.v[0][2] - A.v[1][2];
    const float e1x = A.v[2][0] - A.v[1][0], e1y = A.v[2][1] - A.v[1][1], e1z = A.v[2][2] - A.v[1][2];
    const float nsum = fabsf(e0y * e1z - e0z * e1y) + fabsf(e0z * e1x - e0x * e1z) + fabsf(e0x * e1y - e0y * e1x);
    const float abs_err = 1e-10f * nsum * (cmax + 1.0f);
    int sgn = 0;
    for (int k = 0; k < 3; ++k) {
        if (k == skip) continue;
        int o = orient_f(A.v[0], A.v[1], A.v[2], B.v[k], abs_err);
        if (o == 0) return false;
        if (sgn == 0) sgn = o;
        else if (o != sgn) return false;
    }
    return true;
}

// Float certificate for the reference's coplanarity test (tri_tri_3d.cuh:99-129): +1 when every vertex of B
// certainly has |n_a . (b - a1)| <= scale * 1e-6 in the reference's fp64 evaluation, -1 when one certainly
// exceeds it, 0 when undecided. `scale` is the largest absolute coordinate of the six (exact in float).
__device__ __forceinline__ int coplanar_f(const Tri9& A, const Tri9& B, float cmax) {
    const float e0x = A.v[0][0] - A.v[1][0], e0y = A.v[0][1] - A.v[1][1], e0z = A.v[0][2] - A.v[1][2];
    const float e1x = A.v[2][0] - A.v[1][0], e1y = A.v[2][1] - A.v[1][1], e1z = A.v[2][2] - A.v[1][2];
    const float nsum = fabsf(e0y * e1z - e0z * e1y) + fabsf(e0z * e1x - e0x * e1z) + fabsf(e0x * e1y - e0y * e1x);
    const float abs_err = 1e-10f * nsum * (cmax + 1.0f);
    const float eps_lo = cmax * 1e-6f * (1.0f - 1e-5f), eps_hi = cmax * 1e-6f * (1.0f + 1e-5f);
    bool all_in = true;
    for (int k = 0; k < 3; ++k) {
        const float* a0 = A.v[0];
        const float* a1 = A.v[1];
        const float* a2 = A.v[2];
        const float* p = B.v[k];
        const float adx = a0[0] - p[0], ady = a0[1] - p[1], adz = a0[2] - p[2];
        const float bdx = a1[0] - p[0], bdy = a1[1] - p[1], bdz = a1[2] - p[2];
        const float cdx = a2[0] - p[0], cdy = a2[1] - p[1], cdz = a2[2] - p[2];
        const float bc = bdx * cdy - bdy * cdx, ca = cdx * ady - cdy * adx, ab = adx * bdy - ady * bdx;
        const float det = adz * bc + bdz * ca + cdz * ab;
        const float perm = (fabsf(bdx * cdy) + fabsf(bdy * cdx)) * fabsf(adz) + (fabsf(cdx * ady) + fabsf(cdy * adx)) * fabsf(bdz) +
                           (fabsf(adx * bdy) + fabsf(ady * bdx)) * fabsf(cdz);
        const float err = 8.0e-7f * perm + abs_err + 1e-30f;
        const float m = fabsf(det);
        if (m - err > eps_hi) return -1;  // this vertex certainly lies off the plane
        if (m + err >= eps_lo) all_in = false;
    }
    return all_in ? 1 : 0;
}

// Translated pair geometry shared by the float filter and the fp64 path.
struct PairGeom {
    Tri9 A, B;  // A = BVH hit ("current"), B = querying face, both translated
    int shared, sa, sb;
    float cmax;
};

__device__ __forceinline__ void pair_geom(const float4 c0, const float4 c1, const float4 c2, const int4 ct, const float4 q0,
                                          const float4 q1, const float4 q2, const int4 qt, PairGeom& g) {
    g.A = {{{c0.x, c0.y, c0.z}, {c1.x, c1.y, c1.z}, {c2.x, c2.y, c2.z}}};
    g.B = {{{q0.x, q0.y, q0.z}, {q1.x, q1.y, q1.z}, {q2.x, q2.y, q2.z}}};
    const int mx = floor_mean6(g.A.v[0][0], g.A.v[1][0], g.A.v[2][0], g.B.v[0][0], g.B.v[1][0], g.B.v[2][0]);
    const int my = floor_mean6(g.A.v[0][1], g.A.v[1][1], g.A.v[2][1], g.B.v[0][1], g.B.v[1][1], g.B.v[2][1]);
    const int mz = floor_mean6(g.A.v[0][2], g.A.v[1][2], g.A.v[2][2], g.B.v[0][2], g.B.v[1][2], g.B.v[2][2]);
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        g.A.v[v][0] -= mx; g.A.v[v][1] -= my; g.A.v[v][2] -= mz;
        g.B.v[v][0] -= mx; g.B.v[v][1] -= my; g.B.v[v][2] -= mz;
    }
    const int ca[3] = {ct.x, ct.y, ct.z}, qb[3] = {qt.x, qt.y, qt.z};
    g.shared = 0;
    g.sa = -1;
    g.sb = -1;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
            if (ca[a] == qb[b]) {
                ++g.shared;
                g.sa = a;
                g.sb = b;
            }
    g.cmax = 0.0f;
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
        for (int d = 0; d < 3; ++d) g.cmax = fmaxf(g.cmax, fmaxf(fabsf(g.A.v[v][d]), fabsf(g.B.v[v][d])));
}

// true when the reference's decision is certainly "no intersection" without the fp64 path
__device__ __forceinline__ bool pair_certainly_disjoint(const PairGeom& g) {
    if (g.shared >= 2) return true;
    {
        const float e6 = 1e-6f;
        int s = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i)
            s += (same_eps(g.A.v[i], g.B.v[0], e6) || same_eps(g.A.v[i], g.B.v[1], e6) || same_eps(g.A.v[i], g.B.v[2], e6)) ? 1 : 0;
        if (s >= 2) return true;
    }
    if (coplanar_f(g.A, g.B, g.cmax) == 1) return true;
    if (g.shared == 0) return strictly_one_side(g.A, g.B, -1, g.cmax) || strictly_one_side(g.B, g.A, -1, g.cmax);
    return strictly_one_side(g.A, g.B, g.sb, g.cmax) && strictly_one_side(g.B, g.A, g.sa, g.cmax);
}

// the reference's fp64 decision on a translated pair
__device__ __forceinline__ bool pair_exact(const PairGeom& g, float eps) {
    if (g.shared >= 2) return false;
    if (coplanar_db(g.A, g.B)) return false;
    {
        const float e6 = 1e-6f;
        int s = 0;
        for (int i = 0; i < 3; ++i)
            s += (same_eps(g.A.v[i], g.B.v[0], e6) || same_eps(g.A.v[i], g.B.v[1], e6) || same_eps(g.A.v[i], g.B.v[2], e6)) ? 1 : 0;
        if (s >= 2) return false;
    }
    float r1[3], r2[3];
    if (!isect_tri_tri_db(g.A, g.B, r1, r2)) return false;
    const float dx = fabsf(r2[0] - r1[0]), dy = fabsf(r2[1] - r1[1]), dz = fabsf(r2[2] - r1[2]);
    float d = -INFINITY;
    if (dx > d) d = dx;
    if (dy > d) d = dy;
    if (dz > d) d = dz;
    if (d < eps && g.shared == 1) return false;
    return true;
}

// The reference's full per-pair decision through the fp64 path: "cur" is the BVH hit, "qry" the querying
// face. Arguments by value so that callers keep their own geometry in registers.
__device__ __noinline__ bool pair_decide_exact(const float4 c0, const float4 c1, const float4 c2, const int4 ct,
                                               const float4 q0, const float4 q1, const float4 q2, const int4 qt,
                                               float eps) {
    PairGeom g;
    pair_geom(c0, c1, c2, ct, q0, q1, q2, qt, g);
    return pair_exact(g, eps);
}

}  // namespace pamo
