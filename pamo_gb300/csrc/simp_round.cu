// Kernels of one PaMO stage-2 collapse round on GB300.
//
// Reference round: CUSimp_Free::forward (simp_cuda/src/cusimp_free.cu:891-1048). Differences in form, not in
// result:
//   * vertex->face lists are filled with atomics and then sorted per vertex, so every float sum over a ring
//     runs in ascending face order and the round is deterministic;
//   * the per-face minimum key of propagate_edge_cost_kernel (:587-610) is computed as the minimum over the
//     face's three vertices of a per-vertex minimum (two 64-bit atomicMin per edge instead of one per ring
//     face); both are the minimum over all edges touching the face;
//   * winners are listed in ascending edge order through a scan instead of an atomic counter;
//   * the undo check marks intersecting faces in a flag array and tests ring membership in O(ring) instead
//     of scanning the whole intersection list per collapsed edge (:776-827).
#include <cstdint>
#include <type_traits>
#include "scan.cuh"
#include "simp_round.cuh"
#include "round_ops.cuh"

namespace pamo {

namespace {

constexpr int kT = 256;
constexpr float kCostRange = 10.0f;            // cusimp_free.cu:15
constexpr float kU32MaxF = 4294967296.0f;      // (float)UINT32_MAX

// ------------------------------------------------------------------ set-up
__global__ void k_undo_stuck(const int* __restrict__ verts_undo, int n, int* tmp_undo, int* undo_list,
                             const int* __restrict__ pts_map, int map_len) {
    for (int a = gtid(); a < n; a += gstride()) {
        const int x = verts_undo[a];
        tmp_undo[a] = x;
        undo_list[a] = (x >= 0 && x < map_len) ? pts_map[x] : 0;  // rearrange_index_of_undo_vertices, :869-878
    }
}

__global__ void k_invalid_mark(const int* __restrict__ verts_undo, int n, unsigned char* invalid, int len) {
    for (int a = gtid(); a < n; a += gstride()) {
        const int x = verts_undo[a];
        if (x >= 0 && x < len) invalid[x] = 1;  // compute_invalid_vertices_table, :880-889
    }
}

__global__ void k_load_points(const float* __restrict__ pts, int n, float4* pos, float4* orig, int* occ) {
    for (int v = gtid(); v < n; v += gstride()) {
        const float4 p = make_float4(pts[3 * v], pts[3 * v + 1], pts[3 * v + 2], 0.f);
        pos[v] = p;
        orig[v] = p;
        occ[v] = 1;
    }
    if (gtid() == 0) occ[n] = 0;
}

__global__ void k_load_points4(const float4* __restrict__ pts, int n, float4* pos, float4* orig, int* occ) {
    for (int v = gtid(); v < n; v += gstride()) {
        const float4 p = pts[v];
        pos[v] = p;
        orig[v] = p;
        occ[v] = 1;
    }
    if (gtid() == 0) occ[n] = 0;
}

__global__ void k_load_tris(const int* __restrict__ tris, int n, int n_pts, int4* tri, RoundCounters* rc) {
    for (int f = gtid(); f < n; f += gstride()) {
        const int a = tris[3 * f], b = tris[3 * f + 1], c = tris[3 * f + 2];
        const bool dead = (a == -1 && b == -1 && c == -1);
        const bool ok = dead || (a >= 0 && a < n_pts && b >= 0 && b < n_pts && c >= 0 && c < n_pts);
        if (!ok) atomicOr(&rc->status, kErrBadIndex);
        tri[f] = ok ? make_int4(a, b, c, 0) : make_int4(-1, -1, -1, 0);
    }
}

__global__ void k_copy4(const int4* __restrict__ src, int4* dst, int n) {
    for (int f = gtid(); f < n; f += gstride()) dst[f] = src[f];
}

__device__ __forceinline__ unsigned long long feistel(const Feistel& fb, unsigned long long idx) {
    uint32_t s0 = (uint32_t)(idx >> fb.rbits), s1 = (uint32_t)(idx & fb.rmask);
#pragma unroll 4
    for (int r = 0; r < 24; ++r) {
        const unsigned long long prod = 0xD2B74407B1CE6E93ull * (unsigned long long)s0;
        const uint32_t hi = (uint32_t)(prod >> 32);
        uint32_t lo = (uint32_t)prod;
        lo = (lo << (fb.rbits - fb.lbits)) | (s1 >> fb.lbits);
        s0 = ((hi ^ fb.key[r]) ^ s1) & fb.lmask;
        s1 = lo & fb.rmask;
    }
    return ((unsigned long long)s0 << fb.rbits) | (unsigned long long)s1;
}

__global__ void k_shuffle_flags(Feistel fb, int* flags) {
    const long long n = (long long)fb.n;
    for (long long i = gtid(); i < n; i += gstride()) flags[i] = feistel(fb, (unsigned long long)i) < fb.m ? 1 : 0;
    if (gtid() == 0) flags[n] = 0;
}

__global__ void k_shuffle_gather(Feistel fb, const int* __restrict__ scan, const int4* __restrict__ src, int4* dst) {
    const long long n = (long long)fb.n;
    for (long long i = gtid(); i < n; i += gstride()) {
        const unsigned long long g = feistel(fb, (unsigned long long)i);
        if (g < fb.m) dst[scan[i]] = src[g];
    }
}

// ------------------------------------------------------------------ adjacency
// Per-face values that the vertex rings read many times (every face lies in three rings and every ring is
// read once per incident edge), each computed by the same operations as where the reference computes it. One
// aligned 64-byte record per face, fgeo[4f .. 4f + 3]:
//   (l01, l12, l20, L1)        the edge lengths |p_x - p_y|, |p_y - p_z|, |p_z - p_x| (the ring edge-length
//                              terms, :449-484) and the L1 norm of the unnormalised normal;
//   (o.x, o.y, o.z, p_x.x), (p_x.y, p_x.z, p_y.x, p_y.y), (p_y.z, p_z.x, p_z.y, p_z.z)
//                              the unnormalised normal cross(p_y - p_x, p_z - p_x) (the flip test) and the three
//                              corner positions, so that a ring face needs no gather of its vertices;
// then, after all n records (n = the round's face count), the face planes of tri2plane (:337-346), fgeo[4n + f]
// (precision mode: a double-float pair, fgeo[4n + 2f] and fgeo[4n + 2f + 1]), which only the quadrics read.
// The buffer holds 6 float4 per face.
__device__ __forceinline__ void face_plane(const float4* __restrict__ pos, int4 t, float p[4]);

// ---- precision mode: error-free transforms (Knuth's TwoSum; TwoProd with an explicit fused multiply-add, which
// --fmad=false leaves alone) and a compensated float accumulator (Ogita, Rump and Oishi's Sum2/Dot2)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = a * b;
    e = __fmaf_rn(a, b, -p);
}
struct CSum {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        float t, e;
        two_sum(s, x, t, e);
        s = t;
        c += e;
    }
    __device__ __forceinline__ void add_prod(float a, float b) {
        float p, pe;
        two_prod(a, b, p, pe);
        add(p);
        c += pe;
    }
    __device__ __forceinline__ float value() const { return s + c; }
};
// Double-float numbers (hi + lo, |lo| <= ulp(hi) / 2) from FP32 operations only (Dekker; Hida, Li and Bailey's
// double-double algorithms), for the precision mode's face planes: about 44 significant bits without FP64.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_fast(float a, float b) {  // |a| >= |b|
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    return df_fast(s, e);
}
__device__ __forceinline__ DF df_neg(DF a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ DF df_mul(DF a, DF b) {
    float p, e;
    two_prod(a.hi, b.hi, p, e);
    e += a.hi * b.lo + a.lo * b.hi;
    return df_fast(p, e);
}
__device__ __forceinline__ DF df_diff(float a, float b) {  // a - b exactly
    float s, e;
    two_sum(a, -b, s, e);
    return {s, e};
}
__device__ __forceinline__ DF df_sqrt(DF a) {
    if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
    const float r = sqrtf(a.hi);
    float p, e;
    two_prod(r, r, p, e);
    return df_fast(r, ((a.hi - p) - e + a.lo) / (2.0f * r));
}
__device__ __forceinline__ DF df_div(DF a, DF b) {
    const float q1 = a.hi / b.hi;
    const DF r = df_add(a, df_neg(df_mul(b, DF{q1, 0.0f})));
    return df_fast(q1, r.hi / b.hi);
}

// The face plane of tri2plane (unit normal of cross(p_y - p_x, p_z - p_x), offset -n.p_x) in double-float
__device__ __forceinline__ void face_plane_df(const float4* __restrict__ pos, int4 t, DF p[4]) {
    const float4 a = pos[t.x], b = pos[t.y], c = pos[t.z];
    const DF e1[3] = {df_diff(b.x, a.x), df_diff(b.y, a.y), df_diff(b.z, a.z)};
    const DF e2[3] = {df_diff(c.x, a.x), df_diff(c.y, a.y), df_diff(c.z, a.z)};
    DF n[3];
    n[0] = df_add(df_mul(e1[1], e2[2]), df_neg(df_mul(e1[2], e2[1])));
    n[1] = df_add(df_mul(e1[2], e2[0]), df_neg(df_mul(e1[0], e2[2])));
    n[2] = df_add(df_mul(e1[0], e2[1]), df_neg(df_mul(e1[1], e2[0])));
    const DF len = df_sqrt(df_add(df_add(df_mul(n[0], n[0]), df_mul(n[1], n[1])), df_mul(n[2], n[2])));
    for (int k = 0; k < 3; ++k) p[k] = df_div(n[k], len);
    const DF d = df_add(df_add(df_mul(p[0], DF{a.x, 0.0f}), df_mul(p[1], DF{a.y, 0.0f})), df_mul(p[2], DF{a.z, 0.0f}));
    p[3] = df_neg(d);
}

__device__ __forceinline__ void acc_add(float& a, float x) { a += x; }
__device__ __forceinline__ void acc_add(CSum& a, float x) { a.add(x); }
__device__ __forceinline__ float acc_value(float a) { return a; }
__device__ __forceinline__ float acc_value(const CSum& a) { return a.value(); }

// plane_df (precision mode): the planes as double-float pairs, fgeo[4n + 2f] (hi) and fgeo[4n + 2f + 1] (lo)
__global__ void __launch_bounds__(kT) k_face_counts(const int4* __restrict__ tri, const RoundCounters* rc, int* valence,
                                                    int* ecount, int* vedges, const float4* __restrict__ pos,
                                                    float4* fgeo, int plane_df) {
    const int n = rc->n_tris;
    for (int f = gtid(); f < n; f += gstride()) {
        const int4 t = tri[f];
        if (face_killed(t)) {
            ecount[f] = 0;
            continue;
        }
        if (fgeo) {
            const V3 o0 = v3(pos[t.x]), o1 = v3(pos[t.y]), o2 = v3(pos[t.z]);
            const V3 ou = vcross(vsub(o1, o0), vsub(o2, o0));
            float4* r = fgeo + 4 * (size_t)f;
            r[0] = make_float4(vnorm(vsub(o0, o1)), vnorm(vsub(o1, o2)), vnorm(vsub(o2, o0)),
                               fabsf(ou.x) + fabsf(ou.y) + fabsf(ou.z));
            r[1] = make_float4(ou.x, ou.y, ou.z, o0.x);
            r[2] = make_float4(o0.y, o0.z, o1.x, o1.y);
            r[3] = make_float4(o1.z, o2.x, o2.y, o2.z);
            if (plane_df) {
                DF pd[4];
                face_plane_df(pos, t, pd);
                fgeo[4 * (size_t)n + 2 * (size_t)f] = make_float4(pd[0].hi, pd[1].hi, pd[2].hi, pd[3].hi);
                fgeo[4 * (size_t)n + 2 * (size_t)f + 1] = make_float4(pd[0].lo, pd[1].lo, pd[2].lo, pd[3].lo);
            } else {
                float pl[4];
                face_plane(pos, t, pl);
                fgeo[4 * (size_t)n + f] = make_float4(pl[0], pl[1], pl[2], pl[3]);
            }
        }
        atomicAdd(&valence[t.x], 1);
        atomicAdd(&valence[t.y], 1);
        atomicAdd(&valence[t.z], 1);
        ecount[f] = (t.x > t.y) + (t.y > t.z) + (t.z > t.x);  // count_edge_kernel, :306-316
        // edges per lower endpoint, for the vertex-grouped processing order
        if (t.x > t.y) atomicAdd(&vedges[t.y], 1);
        if (t.y > t.z) atomicAdd(&vedges[t.z], 1);
        if (t.z > t.x) atomicAdd(&vedges[t.x], 1);
    }
    if (gtid() == 0) ecount[n] = 0;
}

__global__ void __launch_bounds__(kT) k_fill_adjacency(const int4* __restrict__ tri, const RoundCounters* rc,
                                                       const int* __restrict__ nt_off, int* cursor, int* nt,
                                                       const int* __restrict__ edge_off, int2* edges,
                                                       const int* __restrict__ voff, int* vcursor, int* eorder) {
    const int n = rc->n_tris;
    for (int f = gtid(); f < n; f += gstride()) {
        const int4 t = tri[f];
        if (face_killed(t)) continue;
        nt[nt_off[t.x] + atomicAdd(&cursor[t.x], 1)] = f;
        nt[nt_off[t.y] + atomicAdd(&cursor[t.y], 1)] = f;
        nt[nt_off[t.z] + atomicAdd(&cursor[t.z], 1)] = f;
        int e = edge_off[f];  // create_edge_kernel, :318-335
        if (t.x > t.y) {
            eorder[voff[t.y] + atomicAdd(&vcursor[t.y], 1)] = e;
            edges[e++] = make_int2(t.y, t.x);
        }
        if (t.y > t.z) {
            eorder[voff[t.z] + atomicAdd(&vcursor[t.z], 1)] = e;
            edges[e++] = make_int2(t.z, t.y);
        }
        if (t.z > t.x) {
            eorder[voff[t.x] + atomicAdd(&vcursor[t.x], 1)] = e;
            edges[e++] = make_int2(t.x, t.z);
        }
    }
}

__global__ void __launch_bounds__(kT) k_sort_adjacency(const RoundCounters* rc, const int* __restrict__ nt_off, int* nt) {
    const int n = rc->n_pts;
    for (int v = gtid(); v < n; v += gstride()) {
        const int a = nt_off[v], b = nt_off[v + 1];
        for (int i = a + 1; i < b; ++i) {
            const int x = nt[i];
            int j = i - 1;
            while (j >= a && nt[j] > x) {
                nt[j + 1] = nt[j];
                --j;
            }
            nt[j + 1] = x;
        }
    }
}

// ------------------------------------------------------------------ quadrics (compute_vert_Q_kernel, :337-366)
__device__ __forceinline__ void face_plane(const float4* __restrict__ pos, int4 t, float p[4]) {
    const V3 v0 = v3(pos[t.x]), v1 = v3(pos[t.y]), v2 = v3(pos[t.z]);
    V3 n = vcross(vsub(v1, v0), vsub(v2, v0));
    n = vdiv(n, vnorm(n));
    p[0] = n.x;
    p[1] = n.y;
    p[2] = n.z;
    p[3] = -vdot(n, v0);
}

// Quadrics from the face planes of fgeo; also, per ring slot s of v (face t = tri[nt[s]]), nxt[s] = the vertex
// after v in t (the link condition's per-slot value) and spc[s] = (the vertex before v, the corner c of v: the
// first of t.x, t.y, t.z equal to v), from which the ring passes rebuild t without reading it.
// kComp (precision mode): every entry summed with compensation (products by TwoProd, sums by TwoSum), rounded once
template <bool kComp>
__global__ void __launch_bounds__(kT) k_quadrics(const RoundCounters* rc, const int* __restrict__ nt_off,
                                                 const int* __restrict__ nt, const int4* __restrict__ tri,
                                                 const float4* __restrict__ fgeo, Quadric* q, int* nxt,
                                                 int2* spc, Quadric* qlo) {
    const int n = rc->n_pts;
    const size_t planes = 4 * (size_t)rc->n_tris;
    for (int v = gtid(); v < n; v += gstride()) {
        float m00 = 0.f, m01 = 0.f, m02 = 0.f, m03 = 0.f, m11 = 0.f, m12 = 0.f, m13 = 0.f, m22 = 0.f, m23 = 0.f, m33 = 0.f;
        CSum c[10];
        const int b = nt_off[v + 1];
        for (int s = nt_off[v]; s < b; ++s) {
            const int f = nt[s];
            const int4 t = tri[f];
            const int corner = t.x == v ? 0 : (t.y == v ? 1 : 2);
            nxt[s] = corner == 0 ? t.y : (corner == 1 ? t.z : t.x);
            spc[s] = make_int2(corner == 0 ? t.z : (corner == 1 ? t.x : t.y), corner);
            if constexpr (kComp) {  // double-float planes (face_plane_df), double-float products and sums
                const float4 ph = fgeo[planes + 2 * (size_t)f], pl = fgeo[planes + 2 * (size_t)f + 1];
                const DF d[4] = {{ph.x, pl.x}, {ph.y, pl.y}, {ph.z, pl.z}, {ph.w, pl.w}};
                const int ij[10][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 3}, {1, 1}, {1, 2}, {1, 3}, {2, 2}, {2, 3}, {3, 3}};
#pragma unroll
                for (int k = 0; k < 10; ++k) {
                    const DF pr = df_mul(d[ij[k][0]], d[ij[k][1]]);
                    c[k].add(pr.hi);
                    c[k].c += pr.lo;
                }
            } else {
                const float4 pl = fgeo[planes + f];
                const float p[4] = {pl.x, pl.y, pl.z, pl.w};
                m00 += p[0] * p[0]; m01 += p[0] * p[1]; m02 += p[0] * p[2]; m03 += p[0] * p[3];
                m11 += p[1] * p[1]; m12 += p[1] * p[2]; m13 += p[1] * p[3];
                m22 += p[2] * p[2]; m23 += p[2] * p[3];
                m33 += p[3] * p[3];
            }
        }
        if constexpr (kComp) {  // each entry as hi (q) + lo (qlo)
            float l[10];
#pragma unroll
            for (int k = 0; k < 10; ++k) {
                const DF e = df_fast(c[k].s, c[k].c);
                c[k].s = e.hi;
                l[k] = e.lo;
            }
            m00 = c[0].s; m01 = c[1].s; m02 = c[2].s; m03 = c[3].s; m11 = c[4].s;
            m12 = c[5].s; m13 = c[6].s; m22 = c[7].s; m23 = c[8].s; m33 = c[9].s;
            Quadric L;
            L.a = make_float4(l[0], l[1], l[2], l[3]);
            L.b = make_float4(l[4], l[5], l[6], l[7]);
            L.c = make_float4(l[8], l[9], 0.f, 0.f);
            qlo[v] = L;
        }
        Quadric Q;
        Q.a = make_float4(m00, m01, m02, m03);
        Q.b = make_float4(m11, m12, m13, m22);
        Q.c = make_float4(m23, m33, 0.f, 0.f);
        q[v] = Q;
    }
}

// ------------------------------------------------------------------ edge cost (compute_edge_cost_kernel, :382-585)

// The squared lengths of the skinny term: the reference squares with the device's pow(float, int)
// (cusimp_free.cu:533,573, cusimp.cu:423,463), which on the GPU differs from x * x by one ulp for a few floats in
// a million and costs far more; kPow = false squares by multiplication (the oracle's form).
template <bool kPow>
__device__ __forceinline__ float sq_len(float x) {
    if constexpr (kPow) return pow(x, 2);
    else return x * x;
}

// The skinny sum 4*sqrt(3)*A/l01^2 + l12^2 + l20^2 + 1e-7 (only the first square divides: the reference's
// precedence), in float, or in double for the legacy round (cusimp.cu:423,463: `4.0f * sqrt(3)` takes the
// integer overload of sqrt).
template <bool kLegacy>
__device__ __forceinline__ float skinny_sum(float k4s3, float area, float p01, float p12, float p20) {
    if constexpr (kLegacy)
        return (float)((double)4.0f * sqrt(3.0) * (double)area / (double)p01 + (double)p12 + (double)p20 +
                       (double)0.0000001f);
    else
        return k4s3 * area / p01 + p12 + p20 + 0.0000001f;
}

// The term 1 - clamp(sum, 0, 1) with the reference's squares. The sum is first taken with x * x: the device's
// pow(float, int) is within 2 ulp of it (CUDA's documented powf bound) for squares in the normal range, the sum is
// monotone in each square (area >= 0) and rounding is monotone, so a sum of at least 1 + 1e-5 with x * x is at
// least 1 with the device's squares too, and the term is 0 either way. Only other sums (below the margin, tiny
// squares, NaN) are evaluated again with the device's pow.
template <bool kLegacy, bool kPow>
__device__ __forceinline__ float skinny_term(float k4s3, float area, float l01, float l12, float l20) {
    const float q01 = l01 * l01, q12 = l12 * l12, q20 = l20 * l20;
    float e = skinny_sum<kLegacy>(k4s3, area, q01, q12, q20);
    if constexpr (kPow) {
        const bool saturated = e >= 1.00001f && q01 >= 1e-30f && q12 >= 1e-30f && q20 >= 1e-30f;
        if (!saturated) e = skinny_sum<kLegacy>(k4s3, area, sq_len<true>(l01), sq_len<true>(l12), sq_len<true>(l20));
    }
    return 1.0f - rclamp(e, 0.0f, 1.0f);
}

// One pass over the ring of w (slots in face-index order) for both ring sums of the edge (w, other):
// * the edge-length term (:449-484): every ring face adds the lengths of its edges whose first vertex is the larger
//   (t.x > t.y, t.y > t.z, t.z > t.x), to len and their count to cnt;
// * the flip test and the skinny term with w moved to vm, over the ring faces without `other`: false as soon as a
//   face's normal flips (the edge is invalid), else each face adds its skinny term to qa and 1 to ntri.
// Called for the ring of u, then of v, each sum runs in the order of the two separate loops of the reference. The face
// t is rebuilt from w, nxt[s] and spc[s], and its corners come from the face record, so a slot costs two aligned
// 32-byte sectors of the record and contiguous per-slot words.
// The flip test dot(n_old/|n_old|, n_new/|n_new|) < 0 takes its sign from the unnormalised normals when a
// float bound proves it (|dot| > 1e-5 |n_old|_1 |n_new|_1, far above the ~1e-6 relative rounding of the
// normalised form); otherwise the normalised form is evaluated exactly as the reference does.
template <bool kLegacy, bool kPow, class Acc>
__device__ __forceinline__ bool ring_pass(int w, int other, V3 vm, const int* __restrict__ nt_off,
                                          const int* __restrict__ nt, const int* __restrict__ nxt,
                                          const int2* __restrict__ spc, const float4* __restrict__ fgeo, Acc& len,
                                          int& cnt, Acc& qa, int& ntri) {
    const float k4s3 = 4.0f * sqrtf(3.0f);
    const int b = nt_off[w + 1];
    for (int s = nt_off[w]; s < b; ++s) {
        const float4* r = fgeo + 4 * (size_t)nt[s];
        const int nx = nxt[s];
        const int2 pc = spc[s];
        const int4 t = pc.y == 0 ? make_int4(w, nx, pc.x, 0) : (pc.y == 1 ? make_int4(pc.x, w, nx, 0)
                                                                          : make_int4(nx, pc.x, w, 0));
        const float4 g = r[0];
        if (t.x > t.y) { acc_add(len, g.x); cnt++; }
        if (t.y > t.z) { acc_add(len, g.y); cnt++; }
        if (t.z > t.x) { acc_add(len, g.z); cnt++; }
        if (t.x == other || t.y == other || t.z == other) continue;
        const float4 r1 = r[1], r2 = r[2], r3 = r[3];
        const bool wx = t.x == w, wy = t.y == w, wz = t.z == w;
        const V3 n0 = wx ? vm : V3{r1.w, r2.x, r2.y}, n1 = wy ? vm : V3{r2.z, r2.w, r3.x},
                 n2 = wz ? vm : V3{r3.y, r3.z, r3.w};
        const V3 ou = {r1.x, r1.y, r1.z};
        const V3 nu = vcross(vsub(n1, n0), vsub(n2, n0));
        const float du = vdot(ou, nu);
        const float bound = 1e-5f * g.w * (fabsf(nu.x) + fabsf(nu.y) + fabsf(nu.z));
        if (du < -bound) return false;
        if (!(du > bound)) {
            const V3 on = vdiv(ou, vnorm(ou));
            const V3 nn = vdiv(nu, vnorm(nu));
            if (vdot(on, nn) < 0) return false;
        }
        // an edge without w keeps its length (same operations as the per-face value)
        const float l01 = (wx || wy) ? vnorm(vsub(n0, n1)) : g.x;
        const float l12 = (wy || wz) ? vnorm(vsub(n1, n2)) : g.y;
        const float l20 = (wz || wx) ? vnorm(vsub(n2, n0)) : g.z;
        const float sh = (l01 + l12 + l20) / 2;  // triangle_area (Heron), :368-375
        const float heron = sh * (sh - l01) * (sh - l12) * (sh - l20);
        // A face with area >= l01^2 / (4 sqrt 3) makes the first quotient of the skinny sum at least 1, so the clamped
        // sum is 1 and the term exactly 0. Most faces are that fat; it is proven here from Heron's product against
        // (l01^2 / (4 sqrt 3))^2 with a 1e-4 relative margin (far above the few ulps of rounding on either side, the
        // 2-ulp difference of the device's pow and the double-precision constant of the legacy sum), which skips the
        // square root and the division. A bound that is not a normal positive number, or a NaN, takes the full path.
        const float tb = l01 * l01 * 0.144337567f;  // l01^2 / (4 sqrt 3)
        const float tb2 = tb * tb;
        if (tb2 > 1e-30f && tb2 < 1e30f && heron >= tb2 * 1.0001f) {
            acc_add(qa, 0.0f);  // the saturated term
        } else {
            const float area = sqrtf(heron);
            acc_add(qa, skinny_term<kLegacy, kPow>(k4s3, area, l01, l12, l20));
        }
        ntri++;
    }
    return true;
}

__device__ __forceinline__ uint32_t f2u_sat(float f) {
    return __float2uint_rz(f);  // round toward zero, saturating like the reference's uint32_t(float) on the GPU
}

// Minimiser of v^T Q v over v = (x, y, z, 1) for the quadric Q of an edge (precision mode 2, optimal placement; the
// reference places at the midpoint, cusimp_free.cu:491,687): A x = -b with A the upper 3x3 block and b the last
// column, by the adjugate. A is positive semi-definite, so its largest diagonal entry bounds its entries: a
// determinant above 1e-2 of its cube (a well-conditioned A) is solved in float, one down to 1e-10 of it (near
// singular) in double from the compensated entries (hi + lo), and a singular one (flat or cylindrical rings) keeps
// the midpoint. Returns 0 (midpoint), 1 (float) or 2 (double).
__device__ __forceinline__ int qem_optimum(const float* m, const float* lo, V3 mid, V3& x) {
    const float m00 = m[0], m01 = m[1], m02 = m[2], m03 = m[3], m11 = m[4], m12 = m[5], m13 = m[6], m22 = m[7],
                m23 = m[8];
    const float nrm = fmaxf(fabsf(m00), fmaxf(fabsf(m11), fabsf(m22)));
    const float n3 = nrm * nrm * nrm;
    const float c00 = m11 * m22 - m12 * m12, c01 = m02 * m12 - m01 * m22, c02 = m01 * m12 - m11 * m02;
    const float det = m00 * c00 + m01 * c01 + m02 * c02;
    if (nrm > 0.0f && fabsf(det) > 1e-2f * n3) {
        const float c11 = m00 * m22 - m02 * m02, c12 = m01 * m02 - m00 * m12, c22 = m00 * m11 - m01 * m01;
        x.x = -(c00 * m03 + c01 * m13 + c02 * m23) / det;
        x.y = -(c01 * m03 + c11 * m13 + c12 * m23) / det;
        x.z = -(c02 * m03 + c12 * m13 + c22 * m23) / det;
        return 1;
    }
    double d[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) d[i] = (double)m[i] + (double)lo[i];
    const double e00 = d[4] * d[7] - d[5] * d[5], e01 = d[2] * d[5] - d[1] * d[7], e02 = d[1] * d[5] - d[4] * d[2];
    const double det64 = d[0] * e00 + d[1] * e01 + d[2] * e02;
    if (nrm > 0.0f && fabs(det64) > 1e-10 * (double)n3) {
        const double e11 = d[0] * d[7] - d[2] * d[2], e12 = d[1] * d[2] - d[0] * d[5], e22 = d[0] * d[4] - d[1] * d[1];
        x.x = (float)(-(e00 * d[3] + e01 * d[6] + e02 * d[8]) / det64);
        x.y = (float)(-(e01 * d[3] + e11 * d[6] + e12 * d[8]) / det64);
        x.z = (float)(-(e02 * d[3] + e12 * d[6] + e22 * d[8]) / det64);
        return 2;
    }
    x = mid;
    return 0;
}

// The edge's quadric Q_u + Q_v: in float (mode 0), or as hi + lo by two-sum with the quadrics' own lo parts added
// (precision modes)
template <int kMode>
__device__ __forceinline__ void edge_quadric(int u, int v, const Quadric* __restrict__ q,
                                             const Quadric* __restrict__ qlo, float m[10], float mlo[10]) {
    const Quadric Qu = q[u], Qv = q[v];
    const float qu[10] = {Qu.a.x, Qu.a.y, Qu.a.z, Qu.a.w, Qu.b.x, Qu.b.y, Qu.b.z, Qu.b.w, Qu.c.x, Qu.c.y};
    const float qv[10] = {Qv.a.x, Qv.a.y, Qv.a.z, Qv.a.w, Qv.b.x, Qv.b.y, Qv.b.z, Qv.b.w, Qv.c.x, Qv.c.y};
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        if constexpr (kMode == 0) {
            m[i] = qu[i] + qv[i];
            mlo[i] = 0.0f;
        } else {
            two_sum(qu[i], qv[i], m[i], mlo[i]);
        }
    }
    if constexpr (kMode != 0) {
        const Quadric Lu = qlo[u], Lv = qlo[v];
        const float lu[10] = {Lu.a.x, Lu.a.y, Lu.a.z, Lu.a.w, Lu.b.x, Lu.b.y, Lu.b.z, Lu.b.w, Lu.c.x, Lu.c.y};
        const float lv[10] = {Lv.a.x, Lv.a.y, Lv.a.z, Lv.a.w, Lv.b.x, Lv.b.y, Lv.b.z, Lv.b.w, Lv.c.x, Lv.c.y};
#pragma unroll
        for (int i = 0; i < 10; ++i) mlo[i] += lu[i] + lv[i];
    }
}

// returns false when the reference leaves the stale cost in place. kLegacy: the cost of CUSimp
// (cusimp.cu:270-471): the mean ring length is counted twice (`edge_len += edge_len + |e|`) and the skinny term
// has no penalty factor. kMode (precision mode, not the reference's arithmetic): 0 the reference's float order;
// 1 quadric, ring-length, skinny and cost sums compensated (TwoSum/TwoProd, rounded once); 2 as 1 with the
// placement at the quadric's minimiser (qem_optimum) instead of the midpoint. raw: the cost before its clamp and
// quantisation; place: the placement.
template <bool kLegacy, bool kPow, int kMode>
__device__ __forceinline__ bool edge_cost_value(int u, int v, const int* __restrict__ nt_off, const int* __restrict__ nt,
                                                const int4* __restrict__ tri, const float4* __restrict__ pos,
                                                const Quadric* __restrict__ q, const float4* __restrict__ fgeo,
                                                const int* __restrict__ nxt, const int2* __restrict__ spc, float scale,
                                                float tres, uint32_t& out, float& raw, V3& place,
                                                const Quadric* __restrict__ qlo) {
    raw = __int_as_float(0x7fc00000);  // NaN: no finite cost (invalid)
    // link condition
    int dup = 0;
    const int ua = nt_off[u], ub = nt_off[u + 1], va = nt_off[v], vb = nt_off[v + 1];
    for (int a = ua; a < ub; ++a) {
        const int iu = nxt[a];
        for (int b = va; b < vb; ++b) {
            const int iv = nxt[b];
            if (iu == iv) dup++;
            if (dup > 2) {
                out = 0xFFFFFFFFu;
                return true;
            }
        }
    }
    if (dup != 2) return false;
    typedef typename std::conditional<kMode == 0, float, CSum>::type Acc;
    const V3 v0 = v3(pos[u]), v1 = v3(pos[v]);
    float m[10], mlo[10];
    V3 vm = vdiv(vadd(v0, v1), 2.0f);
    if constexpr (kMode == 2) {
        edge_quadric<kMode>(u, v, q, qlo, m, mlo);
        qem_optimum(m, mlo, vm, vm);
    }
    place = vm;
    Acc lacc{}, qacc{};
    int cnt = 0, ntri = 0;
    if (!ring_pass<kLegacy, kPow>(u, v, vm, nt_off, nt, nxt, spc, fgeo, lacc, cnt, qacc, ntri) ||
        !ring_pass<kLegacy, kPow>(v, u, vm, nt_off, nt, nxt, spc, fgeo, lacc, cnt, qacc, ntri)) {
        out = 0xFFFFFFFFu;
        return true;
    }
    float len = acc_value(lacc);
    len = len / (float)cnt / scale * tres;
    if (kLegacy) len = len + (len + vnorm(vsub(v0, v1)) / scale * tres);
    else len = len + vnorm(vsub(v0, v1)) / scale * tres;
    edge_quadric<kMode>(u, v, q, qlo, m, mlo);  // after the ring passes: not live across them
    float qa = acc_value(qacc);
    if (!kLegacy) qa = 5.0f * qa;  // SKINNY_TRIANGLE_PENALTY
    const float x = vm.x, y = vm.y, z = vm.z, w = 1.0f;
    float qem;
    if constexpr (kMode == 0) {
        const float m00 = m[0], m01 = m[1], m02 = m[2], m03 = m[3], m11 = m[4], m12 = m[5], m13 = m[6], m22 = m[7],
                    m23 = m[8], m33 = m[9];
        // Mat4x4::vTMv (cusimp_free.h:145-152) on the symmetric matrix
        const float c0 = m00 * x + m01 * y + m02 * z + m03 * w;
        const float c1 = m01 * x + m11 * y + m12 * z + m13 * w;
        const float c2 = m02 * x + m12 * y + m22 * z + m23 * w;
        const float c3 = m03 * x + m13 * y + m23 * z + m33 * w;
        qem = c0 * x + c1 * y + c2 * z + c3 * w;
    } else {
        // the same products with the matrix as hi + lo, each dot compensated
        const int row[4][4] = {{0, 1, 2, 3}, {1, 4, 5, 6}, {2, 5, 7, 8}, {3, 6, 8, 9}};
        const float vv[4] = {x, y, z, w};
        CSum outer;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            CSum inner;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                inner.add_prod(m[row[r][c]], vv[c]);
                inner.add_prod(mlo[row[r][c]], vv[c]);
            }
            outer.add_prod(inner.s, vv[r]);
            outer.add_prod(inner.c, vv[r]);
        }
        qem = outer.value();
    }
    const float cost = qem / (scale * scale);
    float tot;
    if constexpr (kMode == 0) {
        tot = cost + len + qa / (float)ntri * tres;
    } else {
        CSum t;
        t.add(cost);
        t.add(len);
        t.add(qa / (float)ntri * tres);
        tot = t.value();
    }
    raw = tot;
    out = f2u_sat(rclamp(tot, 0.0f, kCostRange) / kCostRange * kU32MaxF);
    return true;
}

// kBatch: many meshes in one vertex numbering; the scale and is_stuck of an edge's mesh come from per-mesh arrays
// (mesh of the lower vertex from vmesh) instead of d_scale and the single flag. kOut: raw_out / place_out are
// written (probe and precision modes; a compile-time flag so that the default variant keeps its register budget).
template <bool kLegacy, bool kPow, bool kBatch, int kMode = 0, bool kOut = false>
__global__ void __launch_bounds__(kT) k_edge_cost(const RoundCounters* rc, const int* __restrict__ eorder,
                                                  const int2* __restrict__ edges,
                                                  const int* __restrict__ nt_off, const int* __restrict__ nt,
                                                  const int4* __restrict__ tri, const float4* __restrict__ pos,
                                                  const Quadric* __restrict__ q, const float4* __restrict__ fgeo,
                                                  const int* __restrict__ nxt, const int2* __restrict__ spc,
                                                  const unsigned char* __restrict__ invalid,
                                                  uint32_t* cost, unsigned long long* vmin, const float* d_scale,
                                                  float tres, int is_stuck_host, const int* is_stuck_dev,
                                                  const int* __restrict__ vmesh, const int* __restrict__ mesh_stuck,
                                                  float* raw_out = nullptr, float4* place_out = nullptr,
                                                  const Quadric* __restrict__ qlo = nullptr) {
    int is_stuck = 0;
    float scale = 0.0f;
    if constexpr (!kBatch) {
        is_stuck = is_stuck_dev ? *is_stuck_dev : is_stuck_host;
        scale = *d_scale;
    }
    const int n = rc->n_edges;
    for (int i = gtid(); i < n; i += gstride()) {
        const int e = eorder[i];  // edges grouped by their lower vertex: neighbouring threads share rings
        const int2 ed = edges[e];
        const int u = ed.x, v = ed.y;
        if constexpr (kBatch) {
            const int m = vmesh[u];
            scale = d_scale[m];
            is_stuck = mesh_stuck[m];
        }
        uint32_t c = 0;
        bool write;
        if (!kLegacy && invalid[u] && invalid[v]) {
            c = 0xFFFFFFFFu;
            write = true;
        } else if (!kLegacy && is_stuck) {
            write = false;
        } else {
            float raw;
            V3 place;
            write = edge_cost_value<kLegacy, kPow, kMode>(u, v, nt_off, nt, tri, pos, q, fgeo, nxt, spc, scale, tres, c,
                                                          raw, place, qlo);
            if constexpr (kOut) {
                if (raw_out) raw_out[e] = write ? raw : __int_as_float(0x7fc00000);
                if (place_out) place_out[e] = make_float4(place.x, place.y, place.z, 0.f);
            }
        }
        if (write) cost[e] = c;
        else c = cost[e];  // stale value of an earlier round
        const unsigned long long key = ((unsigned long long)c << 32) | (unsigned)e;
        atomicMin(&vmin[u], key);
        atomicMin(&vmin[v], key);
    }
}

__global__ void k_edge_cost_capacity(RoundCounters* rc, int* d_cap) {
    const int n = rc->n_edges;
    int grow = 0;
    if (n > *d_cap) {
        *d_cap = n + n / 5;
        grow = 1;
    }
    rc->pad[0] = grow;
}

__global__ void k_edge_cost_zero(const RoundCounters* rc, uint32_t* cost, int len) {
    if (!rc->pad[0]) return;
    for (int i = gtid(); i < len; i += gstride()) cost[i] = 0u;
}

__global__ void __launch_bounds__(kT) k_face_keys(const RoundCounters* rc, const int4* __restrict__ tri,
                                                  const unsigned long long* __restrict__ vmin, unsigned long long* fkey) {
    const int n = rc->n_tris;
    for (int f = gtid(); f < n; f += gstride()) {
        const int4 t = tri[f];
        if (face_killed(t)) continue;
        unsigned long long k = vmin[t.x];
        k = min(k, vmin[t.y]);
        k = min(k, vmin[t.z]);
        fkey[f] = k;
    }
}

// ------------------------------------------------------------------ collapse (collapse_edge_kernel, :639-774)
__device__ __forceinline__ bool is_skinny(V3 p, V3 q, V3 r) {  // :617-637
    const V3 pq = vsub(q, p), pr = vsub(r, p), qr = vsub(r, q);
    const float lpq = sqrtf(vdot(pq, pq)), lpr = sqrtf(vdot(pr, pr)), lqr = sqrtf(vdot(qr, qr));
    const float maxl = fmaxf(lpq, fmaxf(lpr, lqr));
    const V3 c = {pq.y * pr.z - pq.z * pr.y, pq.z * pr.x - pq.x * pr.z, pq.x * pr.y - pq.y * pr.x};
    const float thr = (float)(1e-6 * (double)maxl * (double)maxl);
    const float area = 0.5f * sqrtf(c.x * c.x + c.y * c.y + c.z * c.z);
    return area < thr;
}


__device__ __forceinline__ bool ring_has_skinny(int w, const int* __restrict__ nt_off, const int* __restrict__ nt,
                                                const int4* tri, const float4* pos) {
    for (int s = nt_off[w]; s < nt_off[w + 1]; ++s) {
        const int4 t = tri[nt[s]];
        if (t.x == -1) continue;
        if (is_skinny(v3(pos[t.x]), v3(pos[t.y]), v3(pos[t.z]))) return true;
    }
    return false;
}


// kRestore = false: CUSimp's collapse (cusimp.cu:512-585), without the skinny-ring restore
// kOpt (precision mode 2): the collapse places at the edge's precomputed placement instead of the midpoint
template <bool kRestore, bool kOpt = false>
__global__ void __launch_bounds__(kT) k_collapse(RoundCounters* rc, const int* __restrict__ eorder,
                                                 const int2* __restrict__ edges,
                                                 const uint32_t* __restrict__ cost, uint32_t collapse_t,
                                                 const unsigned long long* __restrict__ fkey, const int* __restrict__ nt_off,
                                                 const int* __restrict__ nt, int4* tri, const int4* __restrict__ orig_tri,
                                                 float4* pos, const float4* __restrict__ orig_pos, int* occ, int* win,
                                                 const float4* __restrict__ place = nullptr) {
    const int n = rc->n_edges;
    if (gtid() == 0) win[n] = 0;
    for (int i = gtid(); i < n; i += gstride()) {
        const int e = eorder[i];
        int w = 0;
        const uint32_t c = cost[e];
        if (c <= collapse_t) {
            const int2 ed = edges[e];
            const int u = ed.x, v = ed.y;
            const unsigned long long key = ((unsigned long long)c << 32) | (unsigned)e;
            bool ok = true;
            for (int s = nt_off[u]; s < nt_off[u + 1] && ok; ++s) ok = (fkey[nt[s]] == key);
            for (int s = nt_off[v]; s < nt_off[v + 1] && ok; ++s) ok = (fkey[nt[s]] == key);
            if (ok) {
                w = 1;
                const V3 v0 = v3(pos[u]), v1 = v3(pos[v]);
                V3 vm = vdiv(vadd(v0, v1), 2.0f);
                if constexpr (kOpt) vm = v3(place[e]);
                pos[u] = make_float4(vm.x, vm.y, vm.z, 0.f);
                pos[v] = make_float4(0.f, 0.f, 0.f, 0.f);
                occ[v] = 0;
                rewire(u, v, nt_off, nt, tri);
                bool sk = kRestore && ring_has_skinny(u, nt_off, nt, tri, pos);
                if (kRestore && !sk) sk = ring_has_skinny(v, nt_off, nt, tri, pos);
                if (sk) {
                    occ[v] = 1;
                    pos[u] = orig_pos[u];
                    pos[v] = orig_pos[v];
                    restore_ring(u, nt_off, nt, tri, orig_tri);
                    restore_ring(v, nt_off, nt, tri, orig_tri);
                }
            }
        }
        win[e] = w;
    }
}

__global__ void k_compact_winners(const RoundCounters* rc, const int* __restrict__ scan, int* collapsed) {
    const int n = rc->n_edges;
    for (int e = gtid(); e < n; e += gstride())
        if (scan[e + 1] != scan[e]) collapsed[scan[e]] = e;
}

__global__ void __launch_bounds__(kT) k_remove_invalid(const RoundCounters* rc, int4* tri) {  // :218-232
    const int n = rc->n_tris;
    for (int f = gtid(); f < n; f += gstride()) {
        const int4 t = tri[f];
        if (face_killed(t)) continue;
        if (t.x == t.y || t.y == t.z || t.z == t.x) tri[f] = make_int4(-1, -1, -1, 0);
    }
}

__global__ void __launch_bounds__(kT) k_line_detect(RoundCounters* rc, const int2* __restrict__ edges, const float4* pos) {
    const int n = rc->n_edges;
    int found = 0;
    for (int e = gtid(); e < n; e += gstride()) {
        const int2 ed = edges[e];
        const float4 p = pos[ed.x], q = pos[ed.y];
        if (p.x == q.x && p.y == q.y && p.z == q.z) found = 1;
    }
    if (__any_sync(0xffffffffu, found) && (threadIdx.x & 31) == 0) atomicAdd(&rc->n_line, 1);
}

// remove_line_edge_collapse (:234-274), applied in edge order by one thread when any coincident edge exists;
// then the collapsed-list bookkeeping of forward() (:1004-1016).
__global__ void k_line_apply(RoundCounters* rc, const int2* __restrict__ edges, const int* __restrict__ nt_off,
                             const int* __restrict__ nt, int4* tri, float4* pos, int* occ, int* collapsed, int cap) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int h = rc->n_win;
    int k = h;
    if (rc->n_line > 0) {
        const int n = rc->n_edges;
        for (int e = 0; e < n; ++e) {
            const int2 ed = edges[e];
            const float4 p = pos[ed.x], q = pos[ed.y];
            if (!(p.x == q.x && p.y == q.y && p.z == q.z)) continue;
            if (k >= cap) {
                atomicOr(&rc->status, kErrCapacity);
                break;
            }
            collapsed[k++] = e;
            pos[ed.y] = make_float4(0.f, 0.f, 0.f, 0.f);
            occ[ed.y] = 0;
            rewire(ed.x, ed.y, nt_off, nt, tri);
        }
    }
    rc->n_collapsed = k;
    const int roundup = ((h + 511) / 512) * 512;
    rc->n_considered = (h == 0) ? 0 : (k < roundup ? k : roundup);
}

// ------------------------------------------------------------------ rollback
__global__ void k_mark_query(const RoundCounters* rc, const int* __restrict__ collapsed, const int2* __restrict__ edges,
                             const int* __restrict__ nt_off, const int* __restrict__ nt, int* qflag) {
    const int n = rc->n_considered;
    for (int c = gtid(); c < n; c += gstride()) {
        const int2 ed = edges[collapsed[c]];
        for (int s = nt_off[ed.x]; s < nt_off[ed.x + 1]; ++s) qflag[nt[s]] = 1;
        for (int s = nt_off[ed.y]; s < nt_off[ed.y + 1]; ++s) qflag[nt[s]] = 1;
    }
}

__global__ void k_compact_flags(const int* __restrict__ scan, const int* d_n, int* out) {
    const int n = *d_n;
    for (int i = gtid(); i < n; i += gstride())
        if (scan[i + 1] != scan[i]) out[scan[i]] = i;
}

__global__ void k_undo_check(RoundCounters* rc, const int* __restrict__ collapsed, const int2* __restrict__ edges,
                             const int* __restrict__ nt_off, const int* __restrict__ nt, const unsigned char* __restrict__ hit,
                             int* uflag) {
    const int n = rc->n_considered;
    if (gtid() == 0) uflag[n] = 0;
    for (int c = gtid(); c < n; c += gstride()) {
        const int2 ed = edges[collapsed[c]];
        int f = 0;
        for (int s = nt_off[ed.x]; s < nt_off[ed.x + 1] && !f; ++s) f = hit[nt[s]];
        for (int s = nt_off[ed.y]; s < nt_off[ed.y + 1] && !f; ++s) f = hit[nt[s]];
        uflag[c] = f ? 1 : 0;
    }
}

__global__ void k_after_check(RoundCounters* rc) {
    const int nu = rc->n_undo;
    if (rc->passes < 8) rc->undo_per_pass[rc->passes] = nu;
    rc->passes += 1;
    rc->n_vertices_undo += 2 * nu;
}

// undo_collapse_kernel (:829-867) + rearrange_index_of_undo_vertices (:869-878). The map is the compaction
// map of the previous call, as in the reference.
__global__ void k_undo_apply(RoundCounters* rc, const int* __restrict__ collapsed, const int* __restrict__ uscan,
                             const int2* __restrict__ edges, const int* __restrict__ nt_off, const int* __restrict__ nt,
                             int4* tri, const int4* __restrict__ orig_tri, float4* pos, const float4* __restrict__ orig_pos,
                             int* occ, int* tmp_undo, int* undo_list, const int* __restrict__ pts_map, int map_len,
                             int list_cap) {
    const int n = rc->n_considered;
    const int first = rc->first_undo;
    for (int c = gtid(); c < n; c += gstride()) {
        if (uscan[c + 1] == uscan[c]) continue;
        const int a = uscan[c];
        const int2 ed = edges[collapsed[c]];
        const int u = ed.x, v = ed.y;
        occ[v] = 1;
        pos[u] = orig_pos[u];
        pos[v] = orig_pos[v];
        restore_ring(u, nt_off, nt, tri, orig_tri);
        restore_ring(v, nt_off, nt, tri, orig_tri);
        if (first + 2 * a + 1 < list_cap) {
            tmp_undo[2 * a] = u;
            tmp_undo[2 * a + 1] = v;
            undo_list[first + 2 * a] = (u < map_len) ? pts_map[u] : 0;
            undo_list[first + 2 * a + 1] = (v < map_len) ? pts_map[v] : 0;
        } else {
            atomicOr(&rc->status, kErrCapacity);
        }
    }
}

__global__ void k_after_apply(RoundCounters* rc) { rc->first_undo += 2 * rc->n_undo; }

// ------------------------------------------------------------------ outputs
__global__ void k_live_flags(const RoundCounters* rc, const int4* __restrict__ tri, int* flags) {
    const int n = rc->n_tris;
    for (int f = gtid(); f < n; f += gstride()) flags[f] = (tri[f].x >= 0) ? 1 : 0;
    if (gtid() == 0) flags[n] = 0;
}

__global__ void k_compact_mesh(RoundCounters* rc, const float4* __restrict__ pos, const int* __restrict__ occ,
                               const int* __restrict__ pts_map, const int4* __restrict__ tri, const int* __restrict__ fscan,
                               float4* out_pos, int4* out_tri) {
    const int np = rc->n_pts, nf = rc->n_tris;
    for (int v = gtid(); v < np; v += gstride())
        if (occ[v]) out_pos[pts_map[v]] = pos[v];
    for (int f = gtid(); f < nf; f += gstride()) {
        if (fscan[f + 1] == fscan[f]) continue;
        const int4 t = tri[f];
        out_tri[fscan[f]] = make_int4(pts_map[t.x], pts_map[t.y], pts_map[t.z], 0);
    }
    if (gtid() == 0) {
        rc->n_pts_out = pts_map[np];
        rc->n_tris_out = fscan[nf];
    }
}

__global__ void k_export_round(int np, int nf, const float4* __restrict__ pos, const int4* __restrict__ tri,
                               const int* __restrict__ occ, const int* __restrict__ pts_map, const int* __restrict__ undo,
                               float* verts, int* tris, int* vocc, int* vmap, int* vundo, int nu) {
    for (int v = gtid(); v < np; v += gstride()) {
        const float4 p = pos[v];
        verts[3 * v] = p.x;
        verts[3 * v + 1] = p.y;
        verts[3 * v + 2] = p.z;
        if (vocc) vocc[v] = occ[v];
        if (vmap) vmap[v] = pts_map[v];
    }
    for (int f = gtid(); f < nf; f += gstride()) {
        const int4 t = tri[f];
        tris[3 * f] = t.x;
        tris[3 * f + 1] = t.y;
        tris[3 * f + 2] = t.z;
    }
    if (vundo)
        for (int a = gtid(); a < nu; a += gstride()) vundo[a] = undo[a];
}

__global__ void k_export_mesh(int np, int nf, const float4* __restrict__ pos, const int4* __restrict__ tri,
                              const float* __restrict__ add, float* verts, int* tris) {
    const float ax = add ? add[0] : 0.f, ay = add ? add[1] : 0.f, az = add ? add[2] : 0.f;
    for (int v = gtid(); v < np; v += gstride()) {
        const float4 p = pos[v];
        verts[3 * v] = p.x + ax;
        verts[3 * v + 1] = p.y + ay;
        verts[3 * v + 2] = p.z + az;
    }
    for (int f = gtid(); f < nf; f += gstride()) {
        const int4 t = tri[f];
        tris[3 * f] = t.x;
        tris[3 * f + 1] = t.y;
        tris[3 * f + 2] = t.z;
    }
}

// ------------------------------------------------------------------ centring (pamo/__init__.py:60-72, 117, 126)
// numpy float32 semantics: per-face ((a + b) + c) / 3, then a sequential float32 sum over faces / F.
// Face means are written per coordinate (SoA) so that the sequential pass can stage them through shared
// memory with coalesced loads; three lanes of one warp then run the three dependent add chains while the
// other warps fetch the next tile.
__global__ void k_face_means(const float* __restrict__ pts, const int* __restrict__ tris, int nf, float* fm) {
    for (int f = gtid(); f < nf; f += gstride()) {
        const int a = tris[3 * f], b = tris[3 * f + 1], c = tris[3 * f + 2];
#pragma unroll
        for (int d = 0; d < 3; ++d) fm[(size_t)d * nf + f] = ((pts[3 * a + d] + pts[3 * b + d]) + pts[3 * c + d]) / 3.0f;
    }
}


// The sequential float32 sum s_k = fl(s_(k-1) + x_k) of numpy's axis-0 reduction, exact, with window
// parallelism (one block per coordinate). While the running sum stays inside one binade [2^e, 2^(e+1)) (float
// spacing u = 2^(e-23)) and off its end points, fl(s + x) = s + u * round(x / u): the rounded increments are
// integers, so a window's running sums are s + u * (prefix sums of the increments), exact in int64. Each element
// is checked (its running sum inside [2^23 + 1, 2^24 - 1] units of u, its increment not a half-way tie, whose
// rounding would depend on the sum's parity); the first element that fails is added with a float add and the
// next window starts after it. Where failures are dense (a sum near zero, or crossing binades quickly), a
// stretch is summed in order by one thread.
constexpr int kSumThreads = 1024;
constexpr int kSumPer = 16;
constexpr int kSumWindow = kSumThreads * kSumPer;

__global__ void __launch_bounds__(kSumThreads) k_exact_sequential_sum(const float* __restrict__ fm, int nf,
                                                                      float* center) {
    const float* x = fm + (size_t)blockIdx.x * nf;
    constexpr int kStage = 4096;
    __shared__ long long wsum[32];
    __shared__ int wmin[32];
    __shared__ float stage[kStage];
    __shared__ float s_sh;
    __shared__ int k_sh, burst_sh, fail_sh, short_sh;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        s_sh = 0.0f;
        k_sh = 0;
        burst_sh = 0;
        short_sh = 0;
    }
    __syncthreads();
    while (true) {
        const float s = s_sh;
        const int k = k_sh;
        const int burst = burst_sh;
        __syncthreads();  // everyone has read the state
        if (k >= nf) break;
        int e = 0;
        bool par = burst == 0 && s != 0.0f && isfinite(s);
        if (par) {
            e = ilogbf(s);
            par = e >= -125 && e <= 126;
        }
        if (!par) {
            // in order, staged through shared memory: a burst after dense failures, 64 elements while the sum is
            // zero or subnormal, the rest when it is not finite (every later sum stays so)
            const int n = min(burst > 0 ? burst : (isfinite(s) ? 64 : nf - k), nf - k);
            float t = s;
            for (int c = 0; c < n; c += kStage) {
                const int m = min(kStage, n - c);
                for (int i = threadIdx.x; i < m; i += kSumThreads) stage[i] = x[k + c + i];
                __syncthreads();
                if (threadIdx.x == 0)
                    for (int i = 0; i < m; ++i) t += stage[i];
                __syncthreads();
            }
            if (threadIdx.x == 0) {
                s_sh = t;
                k_sh = k + n;
                burst_sh = 0;
            }
            __syncthreads();
            continue;
        }
        // integer arithmetic on the float bits (the fp64 pipe is too slow for this): s = S * u with u = 2^(e-23),
        // x / u = +-m * 2^(ex - e) for x's 24-bit significand m
        const unsigned sb = __float_as_uint(s);
        const long long S = (sb >> 31) ? -(long long)((sb & 0x7FFFFFu) | 0x800000u) : (long long)((sb & 0x7FFFFFu) | 0x800000u);
        const int base = k + threadIdx.x * kSumPer;
        const int wend = min(k + kSumWindow, nf);
        long long q[kSumPer];
        unsigned badm = 0;
        long long tsum = 0;
#pragma unroll
        for (int i = 0; i < kSumPer; ++i) {
            const int idx = base + i;
            q[i] = 0;
            if (idx < wend) {
                const unsigned b = __float_as_uint(x[idx]);
                const int bex = (int)((b >> 23) & 0xFFu);
                if (bex == 0xFF) {
                    badm |= 1u << i;  // inf or nan
                } else if ((b & 0x7FFFFFFFu) != 0u) {
                    const long long m = bex ? (long long)((b & 0x7FFFFFu) | 0x800000u) : (long long)(b & 0x7FFFFFu);
                    const int sh = (bex ? bex - 127 : -126) - e;  // x / u = m * 2^sh
                    long long mag;
                    if (sh >= 0) {
                        if (sh > 16) badm |= 1u << i;  // |x / u| >= 2^40: leaves the binade anyway
                        mag = sh > 16 ? 0 : m << sh;
                    } else if (-sh >= 25) {
                        mag = 0;  // |x / u| < 1/2
                    } else {
                        const int kk = -sh;
                        const long long rem = m & ((1ll << kk) - 1), half = 1ll << (kk - 1);
                        if (rem == half) badm |= 1u << i;  // a tie: rounds by the sum's parity
                        mag = (m >> kk) + (rem > half ? 1 : 0);
                    }
                    q[i] = (b >> 31) ? -mag : mag;
                }
            }
            tsum += q[i];
        }
        // block exclusive scan of the per-thread sums
        long long inc = tsum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            long long w = wsum[lane];
            long long wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long t = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += t;
            }
            wsum[lane] = wi - w;
        }
        __syncthreads();
        long long R = S + wsum[warp] + inc - tsum;
        const long long lo = s > 0.0f ? (1ll << 23) + 1 : -((1ll << 24) - 1);
        const long long hi = s > 0.0f ? (1ll << 24) - 1 : -((1ll << 23) + 1);
        int first = nf;
#pragma unroll
        for (int i = 0; i < kSumPer; ++i) {
            const int idx = base + i;
            if (idx < wend && first == nf) {
                R += q[i];
                if ((badm >> i & 1u) || R < lo || R > hi) first = idx;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
        if (lane == 0) wmin[warp] = first;
        __syncthreads();
        if (warp == 0) {
            int m = wmin[lane];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) fail_sh = m;
        }
        __syncthreads();
        const int f = min(fail_sh, wend);  // elements [k, f) are exact; f fails (or ends the window)
        // the owner of element f - 1 publishes the sum after it
        if (f > k && (f - 1 - k) / kSumPer == (int)threadIdx.x) {
            long long r = S + wsum[warp] + inc - tsum;
            for (int i = 0; i <= (f - 1 - k) % kSumPer; ++i) r += q[i];
            // r * u with 2^23 < |r| < 2^24: the float with r's significand and s's exponent
            s_sh = __uint_as_float((r < 0 ? 0x80000000u : 0u) | ((unsigned)(e + 127) << 23) |
                                   ((unsigned)(r < 0 ? -r : r) & 0x7FFFFFu));
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            if (f < wend) {  // the failing element: a float add in order
                s_sh = s_sh + x[f];
                k_sh = f + 1;
                // four windows in a row that advanced less than 32 elements: sum the next 1024 in order
                short_sh = (f - k < 32) ? short_sh + 1 : 0;
                if (short_sh >= 4) {
                    burst_sh = 1024;
                    short_sh = 0;
                }
            } else {
                k_sh = wend;
                short_sh = 0;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) center[blockIdx.x] = s_sh / (float)nf;
}

__global__ void k_center_points(const float* __restrict__ pts, int np, const float* __restrict__ center, float4* out,
                                unsigned* ext) {
    const float cx = center[0], cy = center[1], cz = center[2];
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int v = gtid(); v < np; v += gstride()) {
        const float x = pts[3 * v] - cx, y = pts[3 * v + 1] - cy, z = pts[3 * v + 2] - cz;
        out[v] = make_float4(x, y, z, 0.f);
        mn[0] = fminf(mn[0], x); mn[1] = fminf(mn[1], y); mn[2] = fminf(mn[2], z);
        mx[0] = fmaxf(mx[0], x); mx[1] = fmaxf(mx[1], y); mx[2] = fmaxf(mx[2], z);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d)
        for (int o = 16; o > 0; o >>= 1) {
            mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            unsigned a = __float_as_uint(mn[d]), b = __float_as_uint(mx[d]);
            a = (a & 0x80000000u) ? ~a : (a | 0x80000000u);
            b = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
            atomicMin(&ext[d], a);
            atomicMax(&ext[3 + d], b);
        }
    }
}

__device__ __forceinline__ float ord_dec(unsigned u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }

// scale = max(max(ex, ey), ez) of the centred points (pamo/__init__.py:126)
__global__ void k_extents(const unsigned* ext, float* scale) {
    if (threadIdx.x != 0) return;
    const float ex = ord_dec(ext[3]) - ord_dec(ext[0]);
    const float ey = ord_dec(ext[4]) - ord_dec(ext[1]);
    const float ez = ord_dec(ext[5]) - ord_dec(ext[2]);
    const float m = (ey > ex) ? ey : ex;
    *scale = (ez > m) ? ez : m;
}

// ================================================================== device-driven rounds
// The same steps as the host-sized launchers, with every size read from the device (LoopState, RoundCounters),
// so that one captured graph serves every round of a size class.

// *ls = *next; the round's counters as forward() sets them (a stuck round starts its undo list with the
// carried-over entries)
__global__ void k_round_begin(RoundCounters* rc, LoopState* ls, const LoopState* next) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const LoopState L = *next;
    *ls = L;
    RoundCounters z = {};
    z.n_pts = L.np;
    z.n_tris = L.nf;
    if (L.is_stuck) {
        z.first_undo = L.nu;
        z.n_vertices_undo = L.nu;
    }
    *rc = z;
}

// not stuck and undo vertices carried in: the invalid table is cleared (cusimp_free.cu:905-908)
__global__ void k_invalid_clear_dev(const LoopState* ls, unsigned char* invalid, int len) {
    if (ls->is_stuck || ls->nu == 0) return;
    for (int i = gtid(); i < len; i += gstride()) invalid[i] = 0;
}

// stuck: the undo list restarts from the carried vertices mapped through the previous map (:869-878);
// then the carried vertices are marked invalid (:880-889)
__global__ void k_undo_book_dev(const int* __restrict__ verts_undo, const LoopState* ls, int* tmp_undo, int* undo_list,
                                const int* __restrict__ pts_map, int map_len, unsigned char* invalid, int len) {
    const int n = ls->nu;
    const bool stuck = ls->is_stuck != 0;
    for (int a = gtid(); a < n; a += gstride()) {
        const int x = verts_undo[a];
        if (stuck) {
            tmp_undo[a] = x;
            undo_list[a] = (x >= 0 && x < map_len) ? pts_map[x] : 0;
        }
        if (x >= 0 && x < len) invalid[x] = 1;
    }
}

// the start of a device round (launch_round_prologue_dev)
__global__ void k_round_prologue_dev(const LoopState* ls, const RoundCounters* rc, const int* __restrict__ pts_map,
                                     int* pts_map_prev, const float4* __restrict__ pts_in, float4* pos, float4* orig_pos,
                                     int* occ, const int4* __restrict__ tri_in, int4* tri, int4* orig_tri, int* valence,
                                     int* cursor, int* vedges, int* vcursor, int* qflag) {
    const int nm = ls->np, np = rc->n_pts, nf = rc->n_tris;
    const int n = max(max(nm, np + 1), nf + 1);
    for (int i = gtid(); i < n; i += gstride()) {
        if (i < nm) pts_map_prev[i] = pts_map[i];
        if (i < np) {
            const float4 p = pts_in[i];
            pos[i] = p;
            orig_pos[i] = p;
            occ[i] = 1;
        } else if (i == np) {
            occ[np] = 0;
        }
        if (i <= np) valence[i] = cursor[i] = vedges[i] = vcursor[i] = 0;
        if (i < nf) {
            const int4 t = tri_in[i];
            tri[i] = t;
            orig_tri[i] = t;
        }
        if (i <= nf) qflag[i] = 0;
    }
}

__global__ void k_fill_u64_dev(const RoundCounters* rc, unsigned long long* p, unsigned long long v) {
    const int n = rc->n_pts + 1;
    for (int i = gtid(); i < n; i += gstride()) p[i] = v;
}

__global__ void k_zero_face_bytes_dev(const RoundCounters* rc, unsigned char* p) {
    const int n = rc->n_tris + 1;
    for (int i = gtid(); i < n; i += gstride()) p[i] = 0;
}

// After compaction: the next round's state (pamo/__init__.py:131-159: sizes, undo vertices, the no-progress
// count and is_stuck) computed from this round's start state; recomputing it after an undo pass is harmless.
__global__ void k_round_end(const RoundCounters* rc, const LoopState* ls, LoopState* next) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    LoopState L = *ls;
    const int nf = rc->n_tris_out;
    if (nf == L.nf) {
        L.count += 1;
    } else {
        L.count = 0;
        L.is_stuck = 0;
    }
    if (L.count >= 2) L.is_stuck = 1;
    L.np = rc->n_pts_out;
    L.nf = nf;
    L.nu = rc->n_vertices_undo;
    *next = L;
}

// the previous round's compaction map, kept for the undo passes of this round (the round's own compaction
// overwrites pts_map before an undo pass may follow); undo entries index it with this round's vertex ids (< np)
// undo vertices carried to the next round (the host loop's copy of the previous undo list)
__global__ void k_copy_undo_dev(const RoundCounters* rc, const int* __restrict__ src, int* dst, int cap) {
    const int n = min(rc->n_vertices_undo, cap);
    for (int i = gtid(); i < n; i += gstride()) dst[i] = src[i];
}

}  // namespace

// ================================================================== host launchers
Feistel make_feistel(unsigned long long m) {
    Feistel fb{};
    unsigned long long bits;
    if (m <= 16) {
        bits = 4;
    } else {
        bits = 0;
        unsigned long long t = m - 1;
        while (t) {
            ++bits;
            t >>= 1;
        }
    }
    fb.lbits = (uint32_t)(bits / 2);
    fb.rbits = (uint32_t)(bits - bits / 2);
    fb.lmask = (uint32_t)((1ull << fb.lbits) - 1);
    fb.rmask = (uint32_t)((1ull << fb.rbits) - 1);
    unsigned long long x = 1;  // minstd_rand, default seed
    for (int r = 0; r < 24; ++r) {
        x = (x * 48271ull) % 2147483647ull;
        fb.key[r] = (uint32_t)x;
    }
    fb.n = 1ull << bits;
    fb.m = m;
    return fb;
}

void launch_undo_bookkeeping(const int* verts_undo, int n_verts_undo, int is_stuck, int* tmp_undo, int* undo_list,
                             const int* pts_map, int pts_map_len, unsigned char* invalid, int invalid_len, cudaStream_t s) {
    if (is_stuck) {
        if (n_verts_undo > 0)
            k_undo_stuck<<<grid_for(n_verts_undo, kT), kT, 0, s>>>(verts_undo, n_verts_undo, tmp_undo, undo_list, pts_map,
                                                                   pts_map_len); note_launch();
    } else if (n_verts_undo != 0) {
        cudaMemsetAsync(invalid, 0, invalid_len, s);
    }
    if (n_verts_undo > 0)
        k_invalid_mark<<<grid_for(n_verts_undo, kT), kT, 0, s>>>(verts_undo, n_verts_undo, invalid, invalid_len); note_launch();
}

void launch_load_points(const float* pts, int n, float4* pos, float4* orig_pos, int* occ, cudaStream_t s) {
    k_load_points<<<grid_for(n, kT), kT, 0, s>>>(pts, n, pos, orig_pos, occ); note_launch();
}
void launch_load_points4(const float4* pts, int n, float4* pos, float4* orig_pos, int* occ, cudaStream_t s) {
    k_load_points4<<<grid_for(n, kT), kT, 0, s>>>(pts, n, pos, orig_pos, occ); note_launch();
}
void launch_load_tris(const int* tris, int n, int n_pts, int4* tri, RoundCounters* rc, cudaStream_t s) {
    k_load_tris<<<grid_for(n, kT), kT, 0, s>>>(tris, n, n_pts, tri, rc); note_launch();
}
void launch_load_tris4(const int4* tris, int n, int4* tri, cudaStream_t s) {
    k_copy4<<<grid_for(n, kT), kT, 0, s>>>(tris, tri, n); note_launch();
}
void launch_copy_tris(const int4* src, int4* dst, int n, cudaStream_t s) {
    k_copy4<<<grid_for(n, kT), kT, 0, s>>>(src, dst, n); note_launch();
}
void launch_shuffle_tris(const Feistel& fb, int* flags, int* scan_scratch, int4* src, int4* dst, int n, cudaStream_t s,
                         int* err) {
    (void)n;
    const int g = grid_for((long long)fb.n, kT);
    k_shuffle_flags<<<g, kT, 0, s>>>(fb, flags); note_launch();
    exclusive_scan(flags, flags, nullptr, (int)fb.n + 1, nullptr, scan_scratch, s, err, 0);
    k_shuffle_gather<<<g, kT, 0, s>>>(fb, flags, src, dst); note_launch();
}

void launch_face_counts(const int4* tri, const RoundCounters* rc, int n_tris_bound, int* valence, int* ecount,
                        int* vedges, cudaStream_t s, const float4* pos, float4* fgeo, bool plane_df) {
    k_face_counts<<<grid_for(n_tris_bound, kT), kT, 0, s>>>(tri, rc, valence, ecount, vedges, pos, fgeo,
                                                            plane_df ? 1 : 0);
    note_launch();
}
void launch_fill_adjacency(const int4* tri, const RoundCounters* rc, int n_tris_bound, const int* nt_off, int* cursor,
                           int* nt, const int* edge_off, int2* edges, const int* voff, int* vcursor, int* eorder,
                           cudaStream_t s) {
    k_fill_adjacency<<<grid_for(n_tris_bound, kT), kT, 0, s>>>(tri, rc, nt_off, cursor, nt, edge_off, edges, voff, vcursor,
                                                               eorder);
    note_launch();
}
void launch_sort_adjacency(const RoundCounters* rc, int n_pts_bound, const int* nt_off, int* nt, cudaStream_t s) {
    k_sort_adjacency<<<grid_for(n_pts_bound, kT), kT, 0, s>>>(rc, nt_off, nt); note_launch();
}
void launch_quadrics(const RoundCounters* rc, int n_pts_bound, const int* nt_off, const int* nt, const int4* tri,
                     const float4* fgeo, Quadric* q, int* nxt, int2* spc, cudaStream_t s, Quadric* qlo) {
    if (qlo) k_quadrics<true><<<grid_for(n_pts_bound, kT), kT, 0, s>>>(rc, nt_off, nt, tri, fgeo, q, nxt, spc, qlo);
    else k_quadrics<false><<<grid_for(n_pts_bound, kT), kT, 0, s>>>(rc, nt_off, nt, tri, fgeo, q, nxt, spc, nullptr);
    note_launch();
}
void launch_edge_cost_capacity(RoundCounters* rc, int* d_cap, uint32_t* edge_cost, int phys_len, cudaStream_t s) {
    k_edge_cost_capacity<<<1, 1, 0, s>>>(rc, d_cap); note_launch();
    k_edge_cost_zero<<<grid_for(phys_len, kT), kT, 0, s>>>(rc, edge_cost, phys_len); note_launch();
}
void launch_edge_cost(const RoundCounters* rc, int n_edges_bound, const int* eorder, const int2* edges, const int* nt_off,
                      const int* nt, const int4* tri, const float4* pos, const Quadric* q, const float4* fgeo,
                      const int* nxt, const int2* spc, const unsigned char* invalid, uint32_t* cost,
                      unsigned long long* vmin,
                      const float* d_scale, float tres, int is_stuck, cudaStream_t s, const int* is_stuck_dev, bool legacy,
                      bool device_pow, int mode, float* raw, float4* place, const Quadric* qlo) {
    const int g = grid_for(n_edges_bound, kT);
#define PAMO_COST_MODE(M, P, O)                                                                                      \
    k_edge_cost<false, P, false, M, O><<<g, kT, 0, s>>>(rc, eorder, edges, nt_off, nt, tri, pos, q, fgeo, nxt,       \
                                                        spc, invalid, cost, vmin, d_scale, tres, is_stuck, is_stuck_dev,  \
                                                        nullptr, nullptr, raw, place, qlo)
    if (!legacy && mode == 1) {
        if (raw || place) {
            if (device_pow) PAMO_COST_MODE(1, true, true);
            else PAMO_COST_MODE(1, false, true);
        } else {
            if (device_pow) PAMO_COST_MODE(1, true, false);
            else PAMO_COST_MODE(1, false, false);
        }
        note_launch();
        return;
    }
    if (!legacy && mode == 2) {
        if (device_pow) PAMO_COST_MODE(2, true, true);
        else PAMO_COST_MODE(2, false, true);
        note_launch();
        return;
    }
    if (raw || place) {  // the reference's arithmetic with the probe outputs
        if (device_pow) PAMO_COST_MODE(0, true, true);
        else PAMO_COST_MODE(0, false, true);
        note_launch();
        return;
    }
#undef PAMO_COST_MODE
    if (legacy) {
        if (device_pow)
            k_edge_cost<true, true, false><<<g, kT, 0, s>>>(rc, eorder, edges, nt_off, nt, tri, pos, q, fgeo, nxt, spc, invalid,
                                                            cost, vmin, d_scale, tres, 0, nullptr, nullptr, nullptr);
        else
            k_edge_cost<true, false, false><<<g, kT, 0, s>>>(rc, eorder, edges, nt_off, nt, tri, pos, q, fgeo, nxt, spc, invalid,
                                                             cost, vmin, d_scale, tres, 0, nullptr, nullptr, nullptr);
    } else if (device_pow) {
        k_edge_cost<false, true, false><<<g, kT, 0, s>>>(rc, eorder, edges, nt_off, nt, tri, pos, q, fgeo, nxt, spc, invalid,
                                                         cost, vmin, d_scale, tres, is_stuck, is_stuck_dev, nullptr,
                                                         nullptr);
    } else {
        k_edge_cost<false, false, false><<<g, kT, 0, s>>>(rc, eorder, edges, nt_off, nt, tri, pos, q, fgeo, nxt, spc, invalid,
                                                          cost, vmin, d_scale, tres, is_stuck, is_stuck_dev, nullptr,
                                                          nullptr);
    }
    note_launch();
}
void launch_edge_cost_batch(const RoundCounters* rc, int n_edges_bound, const int* eorder, const int2* edges,
                            const int* nt_off, const int* nt, const int4* tri, const float4* pos, const Quadric* q,
                            const float4* fgeo, const int* nxt, const int2* spc, const unsigned char* invalid,
                            uint32_t* cost,
                            unsigned long long* vmin, const float* mesh_scale, const int* mesh_stuck, const int* vmesh,
                            float tres, cudaStream_t s, bool device_pow) {
    const int g = grid_for(n_edges_bound, kT);
    if (device_pow)
        k_edge_cost<false, true, true><<<g, kT, 0, s>>>(rc, eorder, edges, nt_off, nt, tri, pos, q, fgeo, nxt, spc, invalid,
                                                        cost, vmin, mesh_scale, tres, 0, nullptr, vmesh, mesh_stuck);
    else
        k_edge_cost<false, false, true><<<g, kT, 0, s>>>(rc, eorder, edges, nt_off, nt, tri, pos, q, fgeo, nxt, spc, invalid,
                                                         cost, vmin, mesh_scale, tres, 0, nullptr, vmesh, mesh_stuck);
    note_launch();
}
void launch_face_keys(const RoundCounters* rc, int n_tris_bound, const int4* tri, const unsigned long long* vmin,
                      unsigned long long* fkey, cudaStream_t s) {
    k_face_keys<<<grid_for(n_tris_bound, kT), kT, 0, s>>>(rc, tri, vmin, fkey); note_launch();
}
void launch_collapse(RoundCounters* rc, int n_edges_bound, const int* eorder, const int2* edges, const uint32_t* cost,
                     uint32_t collapse_t, const unsigned long long* fkey, const int* nt_off, const int* nt, int4* tri,
                     const int4* orig_tri, float4* pos, const float4* orig_pos, int* occ, int* win, cudaStream_t s,
                     bool restore, const float4* place) {
    if (restore && place)
        k_collapse<true, true><<<grid_for(n_edges_bound, kT), kT, 0, s>>>(rc, eorder, edges, cost, collapse_t, fkey,
                                                                          nt_off, nt, tri, orig_tri, pos, orig_pos, occ,
                                                                          win, place);
    else if (restore)
        k_collapse<true><<<grid_for(n_edges_bound, kT), kT, 0, s>>>(rc, eorder, edges, cost, collapse_t, fkey, nt_off, nt,
                                                                    tri, orig_tri, pos, orig_pos, occ, win);
    else
        k_collapse<false><<<grid_for(n_edges_bound, kT), kT, 0, s>>>(rc, eorder, edges, cost, collapse_t, fkey, nt_off, nt,
                                                                     tri, orig_tri, pos, orig_pos, occ, win);
    note_launch();
}
void launch_compact_winners(const RoundCounters* rc, int n_edges_bound, const int* win_scan, int* collapsed,
                            cudaStream_t s) {
    k_compact_winners<<<grid_for(n_edges_bound, kT), kT, 0, s>>>(rc, win_scan, collapsed); note_launch();
}
void launch_remove_invalid(const RoundCounters* rc, int n_tris_bound, int4* tri, cudaStream_t s) {
    k_remove_invalid<<<grid_for(n_tris_bound, kT), kT, 0, s>>>(rc, tri); note_launch();
}
void launch_line_edges(RoundCounters* rc, int n_edges_bound, const int2* edges, const int* nt_off, const int* nt,
                       int4* tri, float4* pos, int* occ, int* line_buf, int line_cap, int* collapsed, cudaStream_t s) {
    (void)line_buf;
    k_line_detect<<<grid_for(n_edges_bound, kT), kT, 0, s>>>(rc, edges, pos); note_launch();
    k_line_apply<<<1, 32, 0, s>>>(rc, edges, nt_off, nt, tri, pos, occ, collapsed, line_cap); note_launch();
}
void launch_line_detect(RoundCounters* rc, int n_edges_bound, const int2* edges, const float4* pos, cudaStream_t s) {
    k_line_detect<<<grid_for(n_edges_bound, kT), kT, 0, s>>>(rc, edges, pos); note_launch();
}
void launch_mark_query(const RoundCounters* rc, int n_edges_bound, const int* collapsed, const int2* edges,
                       const int* nt_off, const int* nt, int* qflag, cudaStream_t s) {
    k_mark_query<<<grid_for(n_edges_bound, kT), kT, 0, s>>>(rc, collapsed, edges, nt_off, nt, qflag); note_launch();
}
void launch_compact_flags(const int* scan, int n_bound, const int* d_n, int* out_list, cudaStream_t s) {
    k_compact_flags<<<grid_for(n_bound, kT), kT, 0, s>>>(scan, d_n, out_list); note_launch();
}
void launch_undo_check(RoundCounters* rc, int n_edges_bound, const int* collapsed, const int2* edges, const int* nt_off,
                       const int* nt, const unsigned char* hit, int* uflag, cudaStream_t s) {
    k_undo_check<<<grid_for(n_edges_bound, kT), kT, 0, s>>>(rc, collapsed, edges, nt_off, nt, hit, uflag); note_launch();
}
void launch_undo_apply(RoundCounters* rc, int n_edges_bound, const int* collapsed, const int* uscan, const int2* edges,
                       const int* nt_off, const int* nt, int4* tri, const int4* orig_tri, float4* pos,
                       const float4* orig_pos, int* occ, int* tmp_undo, int* undo_list, const int* pts_map,
                       int list_cap, cudaStream_t s) {
    k_undo_apply<<<grid_for(n_edges_bound, kT), kT, 0, s>>>(rc, collapsed, uscan, edges, nt_off, nt, tri, orig_tri, pos,
                                                            orig_pos, occ, tmp_undo, undo_list, pts_map, list_cap, list_cap); note_launch();
    k_after_apply<<<1, 1, 0, s>>>(rc); note_launch();
}
void launch_after_check(RoundCounters* rc, cudaStream_t s) {
    k_after_check<<<1, 1, 0, s>>>(rc); note_launch();
}

void launch_live_flags(const RoundCounters* rc, int n_tris_bound, const int4* tri, int* flags, cudaStream_t s) {
    k_live_flags<<<grid_for(n_tris_bound, kT), kT, 0, s>>>(rc, tri, flags); note_launch();
}
void launch_compact_mesh(RoundCounters* rc, int n_pts_bound, int n_tris_bound, const float4* pos, const int* occ,
                         const int* pts_map, const int4* tri, const int* face_scan, float4* out_pos, int4* out_tri,
                         cudaStream_t s) {
    const int n = n_pts_bound > n_tris_bound ? n_pts_bound : n_tris_bound;
    k_compact_mesh<<<grid_for(n, kT), kT, 0, s>>>(rc, pos, occ, pts_map, tri, face_scan, out_pos, out_tri); note_launch();
}
void launch_export_round(const RoundCounters* rc, int n_pts, int n_tris, const float4* pos, const int4* tri,
                         const int* occ, const int* pts_map, const int* undo_list, float* verts, int* tris,
                         int* verts_occ, int* verts_map, int* verts_undo, int n_undo, cudaStream_t s) {
    (void)rc;
    const int n = n_pts > n_tris ? n_pts : n_tris;
    k_export_round<<<grid_for(n, kT), kT, 0, s>>>(n_pts, n_tris, pos, tri, occ, pts_map, undo_list, verts, tris, verts_occ,
                                                  verts_map, verts_undo, n_undo); note_launch();
}
void launch_export_mesh(int n_pts, int n_tris, const float4* pos, const int4* tri, const float* add, float* verts,
                        int* tris, cudaStream_t s) {
    const int n = n_pts > n_tris ? n_pts : n_tris;
    k_export_mesh<<<grid_for(n, kT), kT, 0, s>>>(n_pts, n_tris, pos, tri, add, verts, tris); note_launch();
}

void launch_center(const float* pts, const int* tris, int n_pts, int n_tris, float* face_mean, float* center,
                   float* d_scale, float4* pos_out, cudaStream_t s, bool centre) {
    // center[0..2] = tris_mean (zero when not centring); center[4..9] scratch (order-preserving extents)
    if (centre) {
        k_face_means<<<grid_for(n_tris, kT), kT, 0, s>>>(pts, tris, n_tris, face_mean); note_launch();
        k_exact_sequential_sum<<<3, kSumThreads, 0, s>>>(face_mean, n_tris, center); note_launch();
    } else {
        cudaMemsetAsync(center, 0, 4 * sizeof(float), s);
    }
    unsigned* ext = (unsigned*)(center + 4);
    cudaMemsetAsync(ext, 0xFF, 3 * sizeof(unsigned), s);
    cudaMemsetAsync(ext + 3, 0x00, 3 * sizeof(unsigned), s);
    k_center_points<<<grid_for(n_pts, kT), kT, 0, s>>>(pts, n_pts, center, pos_out, ext); note_launch();
    k_extents<<<1, 32, 0, s>>>(ext, d_scale); note_launch();
}

// ---- device-driven rounds ----
void launch_round_begin(RoundCounters* rc, LoopState* ls, const LoopState* next, cudaStream_t s) {
    k_round_begin<<<1, 32, 0, s>>>(rc, ls, next); note_launch();
}
void launch_undo_bookkeeping_dev(const int* verts_undo, const LoopState* ls, int n_undo_bound, int* tmp_undo,
                                 int* undo_list, const int* pts_map, int pts_map_len, unsigned char* invalid,
                                 int invalid_len, cudaStream_t s) {
    k_invalid_clear_dev<<<grid_for(invalid_len, kT), kT, 0, s>>>(ls, invalid, invalid_len); note_launch();
    k_undo_book_dev<<<grid_for(n_undo_bound, kT), kT, 0, s>>>(verts_undo, ls, tmp_undo, undo_list, pts_map, pts_map_len,
                                                             invalid, invalid_len); note_launch();
}
void launch_round_prologue_dev(const LoopState* ls, const RoundCounters* rc, int n_pts_bound, int n_tris_bound,
                               const int* pts_map, int* pts_map_prev, const float4* pts_in, float4* pos,
                               float4* orig_pos, int* occ, const int4* tri_in, int4* tri, int4* orig_tri, int* valence,
                               int* cursor, int* vedges, int* vcursor, int* qflag, cudaStream_t s) {
    const int n = (n_pts_bound > n_tris_bound ? n_pts_bound : n_tris_bound) + 1;
    k_round_prologue_dev<<<grid_for(n, kT), kT, 0, s>>>(ls, rc, pts_map, pts_map_prev, pts_in, pos, orig_pos, occ, tri_in,
                                                        tri, orig_tri, valence, cursor, vedges, vcursor, qflag);
    note_launch();
}
void launch_fill_u64_dev(const RoundCounters* rc, int n_pts_bound, unsigned long long* p, unsigned long long v,
                         cudaStream_t s) {
    k_fill_u64_dev<<<grid_for(n_pts_bound + 1, kT), kT, 0, s>>>(rc, p, v); note_launch();
}
void launch_zero_face_bytes_dev(const RoundCounters* rc, int n_tris_bound, unsigned char* p, cudaStream_t s) {
    k_zero_face_bytes_dev<<<grid_for(n_tris_bound + 1, kT), kT, 0, s>>>(rc, p); note_launch();
}
void launch_round_end(const RoundCounters* rc, const LoopState* ls, LoopState* next, const int* undo_list, int* undo_in,
                      int undo_cap, int n_undo_bound, cudaStream_t s) {
    k_round_end<<<1, 32, 0, s>>>(rc, ls, next); note_launch();
    k_copy_undo_dev<<<grid_for(n_undo_bound, kT), kT, 0, s>>>(rc, undo_list, undo_in, undo_cap); note_launch();
}

}  // namespace pamo
