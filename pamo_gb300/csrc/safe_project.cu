// Stage 3 (safe projection) on GB300: kernels and the Newton driver.
//
// Reference: simp_cuda/safe_project/src/pamo_safe_project/ — processing.py:23-106 (normalisation, step
// loop), system.py:167-272 (register_mesh), :411-470 (step), cg_solver.py:96-158 (Jacobi PCG),
// energy.py:195-211 (distance to GT), :346-468 (StVK), :590-706 (hinge), :887-948 (contacts, barrier, CCD),
// kernels/*.py (per-element formulas). The reference runs on a forked Warp that is not available, so the
// formulas below follow the reference's kernels; where the reference calls a fork-only routine
// (wp.spd_project_blocks) or Warp internals (BVH queries, mesh_query_point_no_sign) this file uses its own
// implementation of the same mathematical operation (stated at each place).
//
// All simulation arrays are float32 as in the reference. Energies and the CG dot products are reduced in a
// fixed order with compensated (two-sum) float accumulation, and the gradient, Hessian-diagonal and
// Hessian-vector scatters (float atomics in the reference) are per-corner slots summed per vertex in a fixed
// order, so the solve gives the same bits run after run.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include <cooperative_groups.h>

#include "../../include/pamo_gb300.h"
#include "safe_project.cuh"
#include "scan.cuh"

namespace pamo {

namespace {

constexpr int kT = 256;
constexpr int kRedBlocks = 256;
constexpr int kPartials = 4096;  // >= 2 x the largest cooperative grid
constexpr int kQT = 128;
constexpr int kStack = 64;

// ------------------------------------------------------------------ float3 helpers (Warp vec3 semantics)
struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float4 a) { return {a.x, a.y, a.z}; }
__device__ __forceinline__ float4 f4(F3 a) { return make_float4(a.x, a.y, a.z, 0.f); }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator-(F3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ F3 operator*(float s, F3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ F3 operator/(F3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ float length_sq(F3 a) { return dot(a, a); }
__device__ __forceinline__ float length(F3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ F3 normalize(F3 a) {  // Warp: zero vector when the length is 0
    const float l = length(a);
    return l > 0.f ? a / l : F3{0.f, 0.f, 0.f};
}
__device__ __forceinline__ F3 fmin3(F3 a, F3 b) { return {fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
__device__ __forceinline__ F3 fmax3(F3 a, F3 b) { return {fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
// Hinge Hessians are kept as the packed upper triangle of their symmetric top-left 9x9 part (45 floats, padded
// to 48): the reference's block_spd_project_kernel (utils_kernels.py:21-39) sets the fourth block row and
// column to minus the sums of the first three, so H v follows from that part alone (see hvp_elements).
constexpr int kHingeStride = 48;
__host__ __device__ constexpr int sym9(int i, int j) {
    return i <= j ? i * 9 - i * (i - 1) / 2 + (j - i) : j * 9 - j * (j - 1) / 2 + (i - j);
}

// Warp's step(x): 1 when x < 0, else 0
__device__ __forceinline__ float wstep(float x) { return x < 0.f ? 1.f : 0.f; }

// ------------------------------------------------------------------ distances (distance_kernels.py:8-30)
__device__ __forceinline__ float pt_distance(F3 x0, F3 x1, F3 x2, F3 x3) {
    return fabsf(dot(x0 - x1, normalize(cross(x2 - x1, x3 - x1))));
}
__device__ __forceinline__ float ee_distance(F3 x0, F3 x1, F3 x2, F3 x3) {
    return fabsf(dot(x0 - x2, normalize(cross(x1 - x0, x3 - x2))));
}
__device__ __forceinline__ float pe_distance(F3 x0, F3 x1, F3 x2) { return length(cross(x1 - x0, x2 - x0)) / length(x1 - x2); }
__device__ __forceinline__ float pp_distance(F3 x0, F3 x1) { return length(x1 - x0); }

enum PT { PT_PT = 0, PT_PP01 = 1, PT_PP02 = 2, PT_PE012 = 3, PT_PP03 = 4, PT_PE031 = 5, PT_PE023 = 6 };
enum EE { EE_PP02 = 0, EE_PP03 = 1, EE_PP12 = 2, EE_PP13 = 3, EE_PE023 = 4, EE_PE123 = 5, EE_PE201 = 6, EE_PE301 = 7,
          EE_EE = 8 };
enum Block { BLOCK_PT = 3, BLOCK_EE = 4 };

// pt_pair_classify (distance_kernels.py:72-225)
__device__ int pt_classify(F3 x0, F3 x1, F3 x2, F3 x3) {
    F3 x10 = x0 - x1;
    const F3 x12 = x2 - x1, x13 = x3 - x1;
    const float area_sq = length_sq(cross(x12, x13));
    if (area_sq <= 1e-6f * (length_sq(x12) * length_sq(x13)) || area_sq <= 1e-16f) {
        const float d1 = length(x10), d2 = length(x0 - x2), d3 = length(x0 - x3);
        if (d1 < d2) return d1 < d3 ? PT_PP01 : PT_PP03;
        return d2 < d3 ? PT_PP02 : PT_PP03;
    }
    const F3 n = normalize(cross(x12, x13));
    const F3 xp = x0 - dot(n, x10) * n;
    x10 = xp - x1;
    const F3 x20 = xp - x2, x30 = xp - x3;
    const float a00 = dot(x12, x12), a01 = dot(x12, x13), a11 = dot(x13, x13);
    const float b0 = dot(x10, x12), b1 = dot(x10, x13);
    const float det = a00 * a11 - a01 * a01;
    const float beta = b0 * a11 - b1 * a01;
    const float gamma = a00 * b1 - b0 * a01;
    const float alpha = det - beta - gamma;
    const float nneg = wstep(alpha) + wstep(beta) + wstep(gamma);
    if (nneg == 0.f) return PT_PT;
    if (nneg == 1.f) {
        if (alpha < 0.f) {
            const F3 x23 = x3 - x2, x20b = x0 - x2;
            const float dr = dot(x23, x20b);
            if (dr < 0.f) return PT_PP02;
            if (dr > dot(x23, x23)) return PT_PP03;
            return PT_PE023;
        } else if (beta < 0.f) {
            const F3 x31 = x1 - x3, x30b = x0 - x3;
            const float dr = dot(x31, x30b);
            if (dr < 0.f) return PT_PP03;
            if (dr > dot(x31, x31)) return PT_PP01;
            return PT_PE031;
        } else if (gamma < 0.f) {
            const float dr = dot(x12, x10);
            if (dr < 0.f) return PT_PP01;
            if (dr > dot(x12, x12)) return PT_PP02;
            return PT_PE012;
        }
        return -1;
    }
    if (alpha >= 0.f) {
        const float d12 = dot(x12, x10), d13 = dot(x13, x10);
        if (d12 > 0.f && d13 <= 0.f) return dot(x12, x20) > 0.f ? PT_PP02 : PT_PE012;
        if (d13 > 0.f && d12 <= 0.f) return dot(x13, x30) > 0.f ? PT_PP03 : PT_PE031;
        return PT_PP01;
    } else if (beta >= 0.f) {
        const F3 x23 = x3 - x2, x21 = x1 - x2;
        const float d23 = dot(x23, x20), d21 = dot(x21, x20);
        if (d23 > 0.f && d21 <= 0.f) return dot(x23, x30) > 0.f ? PT_PP03 : PT_PE023;
        if (d21 > 0.f && d23 <= 0.f) return dot(x21, x10) > 0.f ? PT_PP01 : PT_PE012;
        return PT_PP02;
    }
    const F3 x31 = x1 - x3, x32 = x2 - x3;
    const float d31 = dot(x31, x30), d32 = dot(x32, x30);
    if (d31 > 0.f && d32 <= 0.f) return dot(x31, x10) > 0.f ? PT_PP01 : PT_PE031;
    if (d32 > 0.f && d31 <= 0.f) return dot(x32, x20) > 0.f ? PT_PP02 : PT_PE023;
    return PT_PP03;
}

__device__ float pt_pair_distance(F3 x0, F3 x1, F3 x2, F3 x3, int t) {
    switch (t) {
        case PT_PT: return pt_distance(x0, x1, x2, x3);
        case PT_PP01: return pp_distance(x0, x1);
        case PT_PP02: return pp_distance(x0, x2);
        case PT_PE012: return pe_distance(x0, x1, x2);
        case PT_PP03: return pp_distance(x0, x3);
        case PT_PE031: return pe_distance(x0, x3, x1);
        case PT_PE023: return pe_distance(x0, x2, x3);
    }
    return 1e9f;
}

// ee_pair_classify (distance_kernels.py:300-418)
__device__ int ee_classify(F3 x0, F3 x1, F3 x2, F3 x3, float sin_thres) {
    const F3 e0 = x0 - x1, e1 = x2 - x3;
    const float e0_sq = dot(e0, e0), e1_sq = dot(e1, e1);
    const float a00 = e0_sq, a01 = -dot(e0, e1), a10 = dot(e0, e1), a11 = -e1_sq;
    const float b0 = dot(x3 - x1, e0), b1 = dot(x3 - x1, e1);
    const float mu0 = -(b0 * a11 - b1 * a01);
    const float mu1 = -(a00 * b1 - a10 * b0);
    const float detA = -(a00 * a11 - a01 * a10);
    const float l0_sq = length_sq(e0), l1_sq = length_sq(e1);
    const float edge_sin = length(cross(normalize(e0), normalize(e1)));
    if (mu0 >= 0.f && mu0 <= detA && mu1 >= 0.f && mu1 <= detA && edge_sin >= sin_thres && l0_sq > 1e-15f && l1_sq > 1e-15f)
        return EE_EE;
    float best = 1e9f;
    int type = -1;
    auto consider = [&](float d, int t) {
        if (d < best) {
            best = d;
            type = t;
        }
    };
    const float t0 = dot(x0 - x3, e1);
    if (t0 >= e1_sq) consider(pp_distance(x0, x2), EE_PP02);
    else if (t0 <= 0.f) consider(pp_distance(x0, x3), EE_PP03);
    else consider(pe_distance(x0, x2, x3), EE_PE023);
    const float t1 = dot(x1 - x3, e1);
    if (t1 >= e1_sq) consider(pp_distance(x1, x2), EE_PP12);
    else if (t1 <= 0.f) consider(pp_distance(x1, x3), EE_PP13);
    else consider(pe_distance(x1, x2, x3), EE_PE123);
    const float t2 = dot(x2 - x1, e0);
    if (t2 >= e0_sq) consider(pp_distance(x2, x0), EE_PP02);
    else if (t2 <= 0.f) consider(pp_distance(x2, x1), EE_PP12);
    else consider(pe_distance(x2, x0, x1), EE_PE201);
    const float t3 = dot(x3 - x1, e0);
    if (t3 >= e0_sq) consider(pp_distance(x3, x0), EE_PP03);
    else if (t3 <= 0.f) consider(pp_distance(x3, x1), EE_PP13);
    else consider(pe_distance(x3, x0, x1), EE_PE301);
    return type;
}

__device__ float ee_pair_distance(F3 x0, F3 x1, F3 x2, F3 x3, int t) {
    switch (t) {
        case EE_PP02: return pp_distance(x0, x2);
        case EE_PP03: return pp_distance(x0, x3);
        case EE_PP12: return pp_distance(x1, x2);
        case EE_PP13: return pp_distance(x1, x3);
        case EE_PE023: return pe_distance(x0, x2, x3);
        case EE_PE123: return pe_distance(x1, x2, x3);
        case EE_PE201: return pe_distance(x2, x0, x1);
        case EE_PE301: return pe_distance(x3, x0, x1);
        case EE_EE: return ee_distance(x0, x1, x2, x3);
    }
    return 1e9f;
}

// ------------------------------------------------------------------ distance gradients (own derivation)
// pp: d = |xa - xb|
__device__ __forceinline__ void pp_grad(F3 xa, F3 xb, int a, int b, F3* g) {
    const F3 u = normalize(xa - xb);
    g[a] = u;
    g[b] = -u;
}
// pe: distance from xa to the line (xb, xc); c = xb + t (xc - xb) the foot point, n = (xa - c)/|xa - c|
__device__ __forceinline__ void pe_grad(F3 xa, F3 xb, F3 xc, int a, int b, int c, F3* g) {
    const F3 e = xc - xb;
    const float ee = dot(e, e);
    const float t = ee > 0.f ? dot(xa - xb, e) / ee : 0.f;
    const F3 n = normalize(xa - (xb + t * e));
    g[a] = n;
    g[b] = -(1.0f - t) * n;
    g[c] = -t * n;
}
// pt: d = |n.(x0 - x1)|; the projection has barycentric weights (l1, l2, l3): dd/dx0 = s n, dd/dxi = -li s n
__device__ __forceinline__ void pt_grad(F3 x0, F3 x1, F3 x2, F3 x3, F3* g) {
    const F3 e1 = x2 - x1, e2 = x3 - x1;
    const F3 n = normalize(cross(e1, e2));
    const float sd = dot(n, x0 - x1);
    const F3 sn = (sd < 0.f ? -1.f : 1.f) * n;
    const F3 pr = x0 - sd * n - x1;
    const float a00 = dot(e1, e1), a01 = dot(e1, e2), a11 = dot(e2, e2);
    const float b0 = dot(pr, e1), b1 = dot(pr, e2);
    const float det = a00 * a11 - a01 * a01;
    const float l2 = det != 0.f ? (b0 * a11 - b1 * a01) / det : 0.f;
    const float l3 = det != 0.f ? (a00 * b1 - b0 * a01) / det : 0.f;
    const float l1 = 1.f - l2 - l3;
    g[0] = sn;
    g[1] = -l1 * sn;
    g[2] = -l2 * sn;
    g[3] = -l3 * sn;
}
// ee: d = |n.(c0 - c1)| with c0 = x0 + a (x1 - x0), c1 = x2 + b (x3 - x2) the closest points of the lines
__device__ __forceinline__ void ee_grad(F3 x0, F3 x1, F3 x2, F3 x3, F3* g) {
    const F3 d1 = x1 - x0, d2 = x3 - x2, r0 = x0 - x2;
    const F3 n = normalize(cross(d1, d2));
    const float sd = dot(n, r0);
    const F3 sn = (sd < 0.f ? -1.f : 1.f) * n;
    const float A = dot(d1, d1), B = dot(d1, d2), C = dot(d2, d2), D = dot(d1, r0), E = dot(d2, r0);
    const float den = A * C - B * B;
    const float a = den != 0.f ? (B * E - C * D) / den : 0.f;
    const float b = den != 0.f ? (A * E - B * D) / den : 0.f;
    g[0] = (1.f - a) * sn;
    g[1] = a * sn;
    g[2] = -(1.f - b) * sn;
    g[3] = -b * sn;
}

__device__ void pt_pair_grad(F3 x0, F3 x1, F3 x2, F3 x3, int t, F3* g) {
    g[0] = g[1] = g[2] = g[3] = F3{0.f, 0.f, 0.f};
    switch (t) {
        case PT_PT: pt_grad(x0, x1, x2, x3, g); break;
        case PT_PP01: pp_grad(x0, x1, 0, 1, g); break;
        case PT_PP02: pp_grad(x0, x2, 0, 2, g); break;
        case PT_PE012: pe_grad(x0, x1, x2, 0, 1, 2, g); break;
        case PT_PP03: pp_grad(x0, x3, 0, 3, g); break;
        case PT_PE031: pe_grad(x0, x3, x1, 0, 3, 1, g); break;
        case PT_PE023: pe_grad(x0, x2, x3, 0, 2, 3, g); break;
    }
}

__device__ void ee_pair_grad(F3 x0, F3 x1, F3 x2, F3 x3, int t, F3* g) {
    g[0] = g[1] = g[2] = g[3] = F3{0.f, 0.f, 0.f};
    switch (t) {
        case EE_PP02: pp_grad(x0, x2, 0, 2, g); break;
        case EE_PP03: pp_grad(x0, x3, 0, 3, g); break;
        case EE_PP12: pp_grad(x1, x2, 1, 2, g); break;
        case EE_PP13: pp_grad(x1, x3, 1, 3, g); break;
        case EE_PE023: pe_grad(x0, x2, x3, 0, 2, 3, g); break;
        case EE_PE123: pe_grad(x1, x2, x3, 1, 2, 3, g); break;
        case EE_PE201: pe_grad(x2, x0, x1, 2, 0, 1, g); break;
        case EE_PE301: pe_grad(x3, x0, x1, 3, 0, 1, g); break;
        case EE_EE: ee_grad(x0, x1, x2, x3, g); break;
    }
}

// IPC log-barrier and derivatives (collision_energy.py:8-28); Warp's select(c, a, b) returns a when c is false
__device__ __forceinline__ float barrier(float d, float dh) { return d >= dh ? 0.f : -(d - dh) * (d - dh) * logf(d / dh); }
__device__ __forceinline__ float barrier_d1(float d, float dh) {
    const float t = d - dh;
    return d >= dh ? 0.f : -2.0f * t * logf(d / dh) - t * t / d;
}
__device__ __forceinline__ float barrier_d2(float d, float dh) {
    return d >= dh ? 0.f : -2.0f * logf(d / dh) - 2.0f * (d - dh) / d - 1.0f + (dh * dh) / (d * d);
}

// ------------------------------------------------------------------ compensated reductions (deterministic)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
struct CSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        float t, e;
        two_sum(s, x, t, e);
        s = t;
        c += e;
    }
    __device__ __forceinline__ void merge(const CSum& o) {
        add(o.s);
        c += o.c;
    }
};

__device__ CSum block_reduce(CSum v) {
    __shared__ float ss[32], cc[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        CSum w;
        w.s = __shfl_down_sync(0xffffffffu, v.s, o);
        w.c = __shfl_down_sync(0xffffffffu, v.c, o);
        if (lane + o < 32) v.merge(w);
    }
    if (lane == 0) {
        ss[warp] = v.s;
        cc[warp] = v.c;
    }
    __syncthreads();
    CSum r;
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        if (lane < nw) {
            r.s = ss[lane];
            r.c = cc[lane];
        }
        for (int o = 16; o > 0; o >>= 1) {
            CSum w;
            w.s = __shfl_down_sync(0xffffffffu, r.s, o);
            w.c = __shfl_down_sync(0xffffffffu, r.c, o);
            if (lane + o < 32) r.merge(w);
        }
    }
    __syncthreads();
    return r;
}

// Ends a grid-wide compensated sum: every block stores its partial; the last block to arrive (counted in
// *counter) reduces the partials in block order, stores the result in *out (after copying the old value to
// *copy_prev when given) and resets the counter. The order of every addition is fixed by the grid shape,
// so the sum is deterministic. All blocks of the grid must call it.
__device__ void grid_sum_finish(CSum acc, float2* partial, int* counter, float* out, float* copy_prev) {
    __shared__ int last;
    CSum r = block_reduce(acc);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = make_float2(r.s, r.c);
        __threadfence();
        last = (atomicAdd(counter, 1) == (int)gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    CSum a;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        CSum t;
        t.s = __ldcg(&partial[b].x);
        t.c = __ldcg(&partial[b].y);
        a.merge(t);
    }
    CSum f = block_reduce(a);
    if (threadIdx.x == 0) {
        if (copy_prev) *copy_prev = *out;
        *out = f.s + f.c;
        *counter = 0;
    }
}

// ------------------------------------------------------------------ set-up kernels
// normalisation of processing.py:15-21: centre = mean of the GT vertices, scale = 1 / max extent (float64).
// Two passes with a fixed summation order: per-block sums, minima and maxima of contiguous chunks, then one
// block combines them in block order.
constexpr int kNormBlocks = 4 * 152;

__global__ void __launch_bounds__(kT) k_norm_partial(const double* __restrict__ gt, int n, double* part) {
    __shared__ double sh[9][kT];
    const long long chunk = ((long long)n + gridDim.x - 1) / gridDim.x;
    const long long lo = chunk * blockIdx.x, hi = min((long long)n, lo + chunk);
    double s[3] = {0, 0, 0}, mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x)
        for (int d = 0; d < 3; ++d) {
            const double x = gt[3 * i + d];
            s[d] += x;
            mn[d] = fmin(mn[d], x);
            mx[d] = fmax(mx[d], x);
        }
    for (int d = 0; d < 3; ++d) {
        sh[d][threadIdx.x] = s[d];
        sh[3 + d][threadIdx.x] = mn[d];
        sh[6 + d][threadIdx.x] = mx[d];
    }
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int d = 0; d < 3; ++d) {
                sh[d][threadIdx.x] += sh[d][threadIdx.x + o];
                sh[3 + d][threadIdx.x] = fmin(sh[3 + d][threadIdx.x], sh[3 + d][threadIdx.x + o]);
                sh[6 + d][threadIdx.x] = fmax(sh[6 + d][threadIdx.x], sh[6 + d][threadIdx.x + o]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 9) part[(size_t)blockIdx.x * 9 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void __launch_bounds__(kT) k_norm_final(const double* __restrict__ part, int nparts, int n, double* stats) {
    __shared__ double sh[9][kT];
    double s[3] = {0, 0, 0}, mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int b = threadIdx.x; b < nparts; b += blockDim.x)
        for (int d = 0; d < 3; ++d) {
            s[d] += part[(size_t)b * 9 + d];
            mn[d] = fmin(mn[d], part[(size_t)b * 9 + 3 + d]);
            mx[d] = fmax(mx[d], part[(size_t)b * 9 + 6 + d]);
        }
    for (int d = 0; d < 3; ++d) {
        sh[d][threadIdx.x] = s[d];
        sh[3 + d][threadIdx.x] = mn[d];
        sh[6 + d][threadIdx.x] = mx[d];
    }
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int d = 0; d < 3; ++d) {
                sh[d][threadIdx.x] += sh[d][threadIdx.x + o];
                sh[3 + d][threadIdx.x] = fmin(sh[3 + d][threadIdx.x], sh[3 + d][threadIdx.x + o]);
                sh[6 + d][threadIdx.x] = fmax(sh[6 + d][threadIdx.x], sh[6 + d][threadIdx.x + o]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double ext = 0;
        for (int d = 0; d < 3; ++d) ext = fmax(ext, sh[6 + d][0] - sh[3 + d][0]);
        const double scale = 1.0 / ext;
        for (int d = 0; d < 3; ++d) {
            const double c = sh[d][0] / (double)n;
            stats[d] = c;
            stats[4 + d] = -c * scale;  // t = -centre * scale
        }
        stats[3] = scale;
    }
}

// V * scale + t in float64 (numpy), stored as float32 (the simulation arrays)
template <typename T>
__global__ void k_normalize(const T* __restrict__ in, int n, const double* __restrict__ st, float4* out, float4* copy) {
    const double s = st[3];
    for (int i = gtid(); i < n; i += gstride()) {
        const float4 p = make_float4((float)((double)in[3 * i] * s + st[4]), (float)((double)in[3 * i + 1] * s + st[5]),
                                     (float)((double)in[3 * i + 2] * s + st[6]), 0.f);
        out[i] = p;
        if (copy) copy[i] = p;
    }
}

__global__ void k_denormalize(const float4* __restrict__ q, int n, const double* __restrict__ st, double* out) {
    const double s = st[3];
    for (int i = gtid(); i < n; i += gstride()) {
        const float4 p = q[i];
        out[3 * i] = ((double)p.x - st[4]) / s;
        out[3 * i + 1] = ((double)p.y - st[5]) / s;
        out[3 * i + 2] = ((double)p.z - st[6]) / s;
    }
}

// int32 rows of 3 -> int4; an index outside [0, n_points) sets *bad and the face becomes (0, 0, 0)
__global__ void k_tris4(const int* __restrict__ t, int n, int n_points, int4* out, int* bad) {
    for (int i = gtid(); i < n; i += gstride()) {
        int4 f = make_int4(t[3 * i], t[3 * i + 1], t[3 * i + 2], 0);
        if ((unsigned)f.x >= (unsigned)n_points || (unsigned)f.y >= (unsigned)n_points ||
            (unsigned)f.z >= (unsigned)n_points) {
            atomicOr(bad, 1);
            f = make_int4(0, 0, 0, 0);
        }
        out[i] = f;
    }
}

// The float64 normalised position of vertex i, as numpy forms it from the float32 input (V * scale + t).
struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 norm_pos(const double* __restrict__ pts, int i, const double* __restrict__ st) {
    const double s = st[3];
    return {(double)pts[3 * i] * s + st[4], (double)pts[3 * i + 1] * s + st[5], (double)pts[3 * i + 2] * s + st[6]};
}
__device__ __forceinline__ double dsq(D3 a, D3 b) {
    const double x = a.x - b.x, y = a.y - b.y, z = a.z - b.z;
    return (x * x + y * y) + z * z;
}

// Mixed Voronoi area per vertex (Meyer, Desbrun, Schroeder, Barr 2003) in the circumcentre form that
// igl::massmatrix(V, F, MASSMATRIX_TYPE_VORONOI) evaluates in float64 (system.py:223-225): corner cosines
// by the law of cosines, circumcentre barycentric weights cos_i * l_i normalised to sum 1, the vertex
// taking half of the two sub-triangles beside it; an obtuse corner takes half the area, the others a quarter.
// Each corner's part goes to its position in its vertex's range (inv_vs, the hinge positions staying zero);
// k_weights_f32 sums a vertex's range in float64 in order (deterministic), then rounds to float32 (the
// simulation's weights array).
__global__ void k_voronoi(const double* __restrict__ pts, const double* __restrict__ st, const int4* __restrict__ tri,
                          int nt, const int* __restrict__ inv_vs, double* wslot) {
    for (int f = gtid(); f < nt; f += gstride()) {
        const int4 t = tri[f];
        const D3 p[3] = {norm_pos(pts, t.x, st), norm_pos(pts, t.y, st), norm_pos(pts, t.z, st)};
        double l[3], l2[3];
        for (int k = 0; k < 3; ++k) {  // l[k]: edge opposite corner k
            l2[k] = dsq(p[(k + 1) % 3], p[(k + 2) % 3]);
            l[k] = sqrt(l2[k]);
        }
        // doublearea by Heron's formula on the sorted lengths (Kahan's stable arrangement)
        double a = l[0], b = l[1], c = l[2];
        if (a < b) { const double tt = a; a = b; b = tt; }
        if (b < c) { const double tt = b; b = c; c = tt; }
        if (a < b) { const double tt = a; a = b; b = tt; }
        double dblA = 0.5 * sqrt((a + (b + c)) * (c - (a - b)) * (c + (a - b)) * (a + (b - c)));
        if (dblA != dblA) dblA = 0.0;
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
        for (int k = 0; k < 3; ++k) wslot[inv_vs[3 * (size_t)f + k]] = quad[k];
    }
}

__global__ void k_weights_f32(const double* __restrict__ wslot, const int* __restrict__ vs_off, int n, float* w) {
    for (int i = gtid(); i < n; i += gstride()) {
        double acc = 0.0;
        for (int s = vs_off[i]; s < vs_off[i + 1]; ++s) acc += wslot[s];
        w[i] = (float)acc;
    }
}

// elastic_preprocess_kernel (elastic_energy.py:7-37)
__global__ void k_elastic_pre(const float4* __restrict__ xr, const int4* __restrict__ tri, int nt, float* area, float4* invDm) {
    for (int f = gtid(); f < nt; f += gstride()) {
        const int4 t = tri[f];
        const F3 x0 = f3(xr[t.x]), x1 = f3(xr[t.y]), x2 = f3(xr[t.z]);
        const F3 x01 = x1 - x0, x02 = x2 - x0;
        const float W = 0.5f * length(cross(x01, x02));
        const F3 b1 = normalize(x01);
        F3 b2 = x02 - dot(x02, b1) * b1;
        b2 = normalize(b2);
        const float a = dot(b1, x01), b = dot(b1, x02), c = dot(b2, x01), d = dot(b2, x02);
        // wp.inverse of a 2x2: adjugate times 1/det, the zero matrix when det == 0
        const float det = a * d - c * b;
        const float id = det != 0.f ? 1.0f / det : 0.f;
        area[f] = W;
        invDm[f] = make_float4(d * id, -b * id, -c * id, a * id);
    }
}

// compute_hinge_angle (hinge_energy.py:4-18)
__device__ __forceinline__ float hinge_angle(F3 x0, F3 x1, F3 x2, F3 x3) {
    const F3 e12 = normalize(x2 - x1);
    const F3 n1 = normalize(cross(e12, x0 - x1));
    const F3 n2 = normalize(cross(x3 - x1, e12));
    return atan2f(dot(cross(n1, n2), e12), dot(n1, n2));
}

__global__ void k_hinge_pre(const float4* __restrict__ xr, const int4* __restrict__ hinge, int nh, float2* rest) {
    for (int h = gtid(); h < nh; h += gstride()) {
        const int4 i = hinge[h];
        const F3 x0 = f3(xr[i.x]), x1 = f3(xr[i.y]), x2 = f3(xr[i.z]), x3 = f3(xr[i.w]);
        rest[h] = make_float2(hinge_angle(x0, x1, x2, x3), length(x1 - x2));
    }
}

// The do-nothing test of system.py:214-221: min over igl::internal_angles(V, F) (float64, law of cosines on
// squared edge lengths, acos without clamping) converted to degrees, compared with min_angle_thres. numpy's
// min propagates NaN (a zero-length edge, or an acos argument rounded past 1), and NaN <= thres is false, so
// one NaN angle anywhere disables the test. flag bit 0: some angle <= thres; bit 1: some angle is NaN.
__global__ void k_min_angle(const double* __restrict__ pts, const double* __restrict__ st, const int4* __restrict__ tri,
                            int nt, double thres_deg, int* flag) {
    for (int f = gtid(); f < nt; f += gstride()) {
        const int4 t = tri[f];
        const D3 p[3] = {norm_pos(pts, t.x, st), norm_pos(pts, t.y, st), norm_pos(pts, t.z, st)};
        double s[3];
        for (int k = 0; k < 3; ++k) s[k] = dsq(p[(k + 1) % 3], p[(k + 2) % 3]);  // opposite corner k
        for (int d = 0; d < 3; ++d) {
            const double s1 = s[d], s2 = s[(d + 1) % 3], s3 = s[(d + 2) % 3];
            const double ang = acos((s3 + s2 - s1) / (2. * sqrt(s3 * s2)));
            const double deg = ang * 180.0 / 3.141592653589793;
            if (deg != deg) atomicOr(flag, 2);
            else if (deg <= thres_deg) atomicOr(flag, 1);
        }
    }
}

// ------------------------------------------------------------------ closest point on the GT mesh
// Closest point of p on triangle (a, b, c): Ericson, Real-Time Collision Detection, 5.1.5
__device__ F3 closest_on_triangle(F3 p, F3 a, F3 b, F3 c) {
    const F3 ab = b - a, ac = c - a, ap = p - a;
    const float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.f && d2 <= 0.f) return a;
    const F3 bp = p - b;
    const float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.f && d4 <= d3) return b;
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) return a + (d1 / (d1 - d3)) * ab;
    const F3 cp = p - c;
    const float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.f && d5 <= d6) return c;
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) return a + (d2 / (d2 - d6)) * ac;
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) return b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b);
    const float den = 1.f / (va + vb + vc);
    return a + (vb * den) * ab + (vc * den) * ac;
}

__device__ __forceinline__ float box_dist_sq(F3 p, float4 lo, float4 hi) {
    const float dx = fmaxf(fmaxf(lo.x - p.x, 0.f), p.x - hi.x);
    const float dy = fmaxf(fmaxf(lo.y - p.y, 0.f), p.y - hi.y);
    const float dz = fmaxf(fmaxf(lo.z - p.z, 0.f), p.z - hi.z);
    return dx * dx + dy * dy + dz * dz;
}

// mesh_query_point_no_sign(gt, x, 1e9) + mesh_eval_position (geometry_kernels.py:81-93): nearest point of the
// GT surface by branch and bound over the GT LBVH (stack in shared memory, nearer child first)
__global__ void __launch_bounds__(kQT) k_closest_gt(const float4* __restrict__ q, int np, const int2* __restrict__ child,
                                                    const float4* __restrict__ nlo, const float4* __restrict__ nhi,
                                                    const float4* __restrict__ llo, const float4* __restrict__ lhi,
                                                    const int* __restrict__ leaf_face, const int4* __restrict__ gtri,
                                                    const float4* __restrict__ gpos, const RoundCounters* grc,
                                                    float4* target, int* status) {
    __shared__ int stack[kStack][kQT];
    const int nl = grc->n_live;
    for (int i = gtid(); i < np; i += gstride()) {
        const F3 p = f3(q[i]);
        float best = 1e18f;  // (max distance 1e9)^2
        F3 bp = p;
        auto leaf = [&](int li) {
            const int4 t = gtri[leaf_face[li]];
            const F3 c = closest_on_triangle(p, f3(gpos[t.x]), f3(gpos[t.y]), f3(gpos[t.z]));
            const float d = length_sq(c - p);
            if (d < best) {
                best = d;
                bp = c;
            }
        };
        if (nl == 1) leaf(0);
        if (nl >= 2) {
            int sp = 0, node = 0, guard = 0;
            while (true) {
                if (++guard > (1 << 22)) {
                    atomicOr(status, 2);
                    break;
                }
                const int2 c = child[node];
                int nxt[2];
                float nd[2];
                int nn = 0;
                for (int side = 0; side < 2; ++side) {
                    const int x = side ? c.y : c.x;
                    const float d = x < 0 ? box_dist_sq(p, llo[~x], lhi[~x]) : box_dist_sq(p, nlo[x], nhi[x]);
                    if (d >= best) continue;
                    if (x < 0) leaf(~x);
                    else {
                        nxt[nn] = x;
                        nd[nn] = d;
                        ++nn;
                    }
                }
                if (nn == 2) {
                    if (nd[1] < nd[0]) {
                        const int t = nxt[0]; nxt[0] = nxt[1]; nxt[1] = t;
                    }
                    if (sp >= kStack) {
                        atomicOr(status, 4);
                        break;
                    }
                    stack[sp++][threadIdx.x] = nxt[1];
                    node = nxt[0];
                } else if (nn == 1) {
                    node = nxt[0];
                } else {
                    bool found = false;
                    while (sp > 0) {
                        node = stack[--sp][threadIdx.x];
                        // re-test the stacked node against the current best
                        if (box_dist_sq(p, nlo[node], nhi[node]) < best) {
                            found = true;
                            break;
                        }
                    }
                    if (!found) break;
                }
            }
        }
        target[i] = f4(bp);
    }
}

// ------------------------------------------------------------------ contact detection (contact_detection.py:120-216)
// The reference queries its BVHs with boxes of half-width 2 radius + d_hat around every vertex and every edge
// and keeps the point-triangle and edge-edge pairs (no shared vertex; edge pairs with e0 < e1) whose
// classified distance is <= 2 radius + d_hat. The box query only filters candidates, so this build keeps a
// candidate list made with the half-width plus a skin, valid while no vertex moved more than half the skin
// (in any coordinate) since it was built, and re-evaluates the distance filter on it every iteration. The
// contact set is the reference's; the LBVH traversal runs only when the list is rebuilt.

// rebuild when some vertex moved more than half the skin since the lists were built
__global__ void k_disp_check(const float4* __restrict__ q, const float4* __restrict__ qref, int np, float half_skin,
                             SolverScalars* sc) {
    if (sc->abort) return;
    bool moved = false;
    for (int i = gtid(); i < np; i += gstride()) {
        const float4 a = q[i], b = qref[i];
        moved |= fmaxf(fabsf(a.x - b.x), fmaxf(fabsf(a.y - b.y), fabsf(a.z - b.z))) > half_skin;
    }
    if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) sc->rebuild = 1;
}

// LBVH traversal over the candidate pairs whose boxes overlap within reach (one thread per query, stack in
// shared memory, bounded), in two passes so that the list order is fixed: with qoff == nullptr each query's
// count goes to qcount[qi]; with the exclusive prefix sums of the counts in qoff, each query writes its pairs at
// qoff[qi], qoff[qi] + 1, ... in traversal order (the same pairs in the same order as the counting pass).
template <bool kEdges>
__global__ void __launch_bounds__(kQT) k_candidates(const float4* __restrict__ x, int n_query, const int4* __restrict__ elems,
                                                    const int2* __restrict__ child, const float4* __restrict__ nlo,
                                                    const float4* __restrict__ nhi, const float4* __restrict__ llo,
                                                    const float4* __restrict__ lhi, const int* __restrict__ leaf_id,
                                                    const RoundCounters* brc, float d_hat, float skin, int2* out,
                                                    int cap, int* qcount, const int* __restrict__ qoff,
                                                    SolverScalars* sc) {
    __shared__ int stack[kStack][kQT];
    if (sc->abort || !sc->rebuild) return;
    const float reach = 2.0f * sc->radius + d_hat + skin;
    const int nl = brc->n_live;
    for (int qi = gtid(); qi < n_query; qi += gstride()) {
        int cnt = 0;
        const int base = qoff ? qoff[qi] : 0;
        int i0, i1 = -1;
        F3 lo, hi;
        if (!kEdges) {
            i0 = qi;
            const F3 x0 = f3(x[i0]);
            lo = x0 - F3{reach, reach, reach};
            hi = x0 + F3{reach, reach, reach};
        } else {
            const int4 e = elems[qi];
            i0 = e.x;
            i1 = e.y;
            const F3 x0 = f3(x[i0]), x1 = f3(x[i1]);
            lo = fmin3(x0, x1) - F3{reach, reach, reach};
            hi = fmax3(x0, x1) + F3{reach, reach, reach};
        }
        const float4 qlo = make_float4(lo.x, lo.y, lo.z, 0.f), qhi = make_float4(hi.x, hi.y, hi.z, 0.f);
        auto overlap = [&](float4 a, float4 b) {
            return !(qhi.x < a.x || b.x < qlo.x || qhi.y < a.y || b.y < qlo.y || qhi.z < a.z || b.z < qlo.z);
        };
        auto leaf = [&](int li) {
            const int id = leaf_id[li];
            const int4 t = elems[id];
            if (!kEdges) {
                if (i0 == t.x || i0 == t.y || i0 == t.z) return;
            } else {
                if (!(qi < id)) return;
                if (i0 == t.x || i0 == t.y || i1 == t.x || i1 == t.y) return;
            }
            if (qoff) {
                const int at = base + cnt;
                if (at < cap) out[at] = make_int2(qi, id);
            }
            ++cnt;
        };
        if (nl == 1) {
            if (overlap(llo[0], lhi[0])) leaf(0);
            if (!qoff) qcount[qi] = cnt;
            continue;
        }
        if (nl < 1) {
            if (!qoff) qcount[qi] = 0;
            continue;
        }
        int sp = 0, node = 0, guard = 0;
        while (true) {
            if (++guard > (1 << 22)) {
                atomicOr(&sc->status, 2);
                break;
            }
            const int2 c = child[node];
            int nxt[2];
            int nn = 0;
            for (int side = 0; side < 2; ++side) {
                const int xx = side ? c.y : c.x;
                if (xx < 0) {
                    if (overlap(llo[~xx], lhi[~xx])) leaf(~xx);
                } else if (overlap(nlo[xx], nhi[xx])) {
                    nxt[nn++] = xx;
                }
            }
            if (nn == 2) {
                if (sp >= kStack) {
                    atomicOr(&sc->status, 4);
                    break;
                }
                stack[sp++][threadIdx.x] = nxt[1];
                node = nxt[0];
            } else if (nn == 1) {
                node = nxt[0];
            } else {
                if (sp == 0) break;
                node = stack[--sp][threadIdx.x];
            }
        }
        if (!qoff) qcount[qi] = cnt;
    }
}

// overflow of a candidate list: grow it and redo the iteration; otherwise the lists now hold positions q
__global__ void k_cand_done(const float4* __restrict__ q, float4* qref, int np, int cap_pt, int cap_ee,
                            SolverScalars* sc) {
    if (sc->abort || !sc->rebuild) return;
    if (sc->n_cand_pt > cap_pt || sc->n_cand_ee > cap_ee) {
        if (gtid() == 0) sc->abort = 3;
        return;
    }
    for (int i = gtid(); i < np; i += gstride()) qref[i] = q[i];
}

// the reference's distance filter on the candidates (detect_pt_contact_bvh_kernel, detect_ee_contact_bvh_kernel):
// candidate g (point-triangle pairs first, then edge-edge pairs) gets cflag[g] = 1 when it is a contact, with its
// vertex ids and type in cid[g] / cty[g]. The contacts are then listed in candidate order (k_contacts_scatter at
// the exclusive prefix sums of the flags), so the list, and every sum over it, is the same run after run.
__global__ void __launch_bounds__(kT) k_filter(const float4* __restrict__ x, const int2* __restrict__ cpt,
                                               const int2* __restrict__ cee, const int4* __restrict__ tri,
                                               const int4* __restrict__ edge4, float d_hat, float ee_thres,
                                               int* cflag, int4* cid, int2* cty, SolverScalars* sc) {
    if (sc->abort) return;
    const float thr = 2.0f * sc->radius + d_hat;
    const int npt = sc->n_cand_pt, nee = sc->n_cand_ee;
    if (gtid() == 0) sc->n_cand_all = npt + nee;
    for (int g = gtid(); g < npt + nee; g += gstride()) {
        int4 id;
        int block, ty;
        float d;
        if (g < npt) {
            const int2 c = cpt[g];
            const int4 t = tri[c.y];
            id = make_int4(c.x, t.x, t.y, t.z);
            const F3 x0 = f3(x[id.x]), x1 = f3(x[id.y]), x2 = f3(x[id.z]), x3 = f3(x[id.w]);
            ty = pt_classify(x0, x1, x2, x3);
            d = pt_pair_distance(x0, x1, x2, x3, ty);
            block = BLOCK_PT;
        } else {
            const int2 c = cee[g - npt];
            const int4 a = edge4[c.x], b = edge4[c.y];
            id = make_int4(a.x, a.y, b.x, b.y);
            const F3 x0 = f3(x[id.x]), x1 = f3(x[id.y]), x2 = f3(x[id.z]), x3 = f3(x[id.w]);
            ty = ee_classify(x0, x1, x2, x3, ee_thres);
            d = ee_pair_distance(x0, x1, x2, x3, ty);
            block = BLOCK_EE;
        }
        const int hit = d <= thr ? 1 : 0;
        cflag[g] = hit;
        if (hit) {
            cid[g] = id;
            cty[g] = make_int2(block, ty);
        }
    }
}

// Contact b = cpos[g] of candidate g (when it is one and fits), and the contacts of each vertex counted in ccnt
// (one per corner) for the vertex contact lists.
__global__ void __launch_bounds__(kT) k_contacts_scatter(const int* __restrict__ cflag, const int* __restrict__ cpos,
                                                         const int4* __restrict__ cid, const int2* __restrict__ cty,
                                                         int4* c_idx, int2* c_type, int* ccnt, SolverScalars* sc) {
    if (sc->abort) return;
    const int n = sc->n_cand_all;
    for (int g = gtid(); g < n; g += gstride()) {
        if (!cflag[g]) continue;
        const int b = cpos[g];
        const int4 id = cid[g];
        c_idx[b] = id;
        c_type[b] = cty[g];
        atomicAdd(&ccnt[id.x], 1);
        atomicAdd(&ccnt[id.y], 1);
        atomicAdd(&ccnt[id.z], 1);
        atomicAdd(&ccnt[id.w], 1);
    }
}

// The contact corners of each vertex in a fixed order: the codes 4b + k (contact b, corner k) are filled at the
// vertex offsets coff into ctmp (in the order the atomics come), then ranked within each vertex's range by one
// warp (ascending codes), which gives each corner its position cinv[4b + k] = coff[v] + rank. The per-corner parts
// of a contact are written at those positions, so each vertex's contact parts are contiguous and in code order.
__global__ void __launch_bounds__(kT) k_cvert_fill(const int4* __restrict__ c_idx, const int* __restrict__ coff,
                                                   int* ccur, int* ctmp, const SolverScalars* sc) {
    if (sc->abort) return;
    const int n = 4 * sc->n_contacts;
    for (int s = gtid(); s < n; s += gstride()) {
        const int4 id = c_idx[s >> 2];
        const int k = s & 3;
        const int v = k == 0 ? id.x : k == 1 ? id.y : k == 2 ? id.z : id.w;
        ctmp[coff[v] + atomicAdd(&ccur[v], 1)] = s;
    }
}

__global__ void __launch_bounds__(kT) k_cvert_rank(const int* __restrict__ coff, const int* __restrict__ ctmp,
                                                   int* cinv, int np, const SolverScalars* sc) {
    if (sc->abort) return;
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x / 32);
    for (long long v = gtid() / 32; v < np; v += warps) {
        const int a = coff[v], m = coff[v + 1] - a;
        for (int b0 = 0; b0 < m; b0 += 32) {
            const int x = b0 + lane < m ? ctmp[a + b0 + lane] : INT_MAX;
            int rank = 0;
            for (int c0 = 0; c0 < m; c0 += 32) {
                const int y = c0 + lane < m ? ctmp[a + c0 + lane] : INT_MAX;
                for (int j = 0; j < 32; ++j) rank += __shfl_sync(0xffffffffu, y, j) < x ? 1 : 0;
            }
            if (b0 + lane < m) cinv[x] = a + rank;  // the codes of a vertex are distinct
        }
    }
}

// Sum over vertex i's parts in src: its static parts (triangle corners and hinge slots, stored contiguously per
// vertex at [vs_off[i], vs_off[i + 1]) in ascending code order), then its contact parts at
// cbase + [coff[i], coff[i + 1]). The G lanes of a group (G a power of two, at most kGather) read them strided
// (lane k: parts k, k + G, ...) and the partial sums meet in a butterfly over the group, which gives every lane
// the same value (the same additions, each commutative). src_h (optional) is summed the same way into h. Called
// by whole warps with the same G (the shuffles); valid = false contributes zeros.
constexpr int kGather = 8;
struct VertexSlots {
    const int* vs_off;   // NP + 1 offsets of the static parts
    const int* coff;     // NP + 1 offsets of the contact parts
    const int* inv_vs;   // position of static code 3f + c (triangle corner) or 3 NT + 4h + a (hinge slot)
    const int* cinv;     // position (after cbase) of contact code 4b + k
    int cbase;           // 3 NT + 4 NH
};
// A vertex's two ranges as one sequence of m parts: [a, a + m1) then [ca, ca + m - m1); m = 0 for no vertex.
struct VRange {
    int a, m1, ca, m;
};
__device__ __forceinline__ VRange vertex_range(const VertexSlots& S, int i, bool valid) {
    VRange R{0, 0, 0, 0};
    if (valid) {
        R.a = S.vs_off[i];
        R.m1 = S.vs_off[i + 1] - R.a;
        const int c0 = S.coff[i];
        R.ca = S.cbase + c0;
        R.m = R.m1 + S.coff[i + 1] - c0;
    }
    return R;
}

__device__ __forceinline__ F3 gather_range(const float4* __restrict__ src, const float4* __restrict__ src_h, F3& h,
                                           const VRange& R, int lane, int G) {
    F3 acc = {0.f, 0.f, 0.f};
    h = F3{0.f, 0.f, 0.f};
    {
        // lane k takes parts k, k + G, ..., kBatch loads in flight at a time, added in sequence order
        constexpr int kBatch = 8;
        const int a = R.a, m1 = R.m1, ca = R.ca, m = R.m;
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int j0 = lane; j0 < m; j0 += kBatch * G) {
            float4 t[kBatch], th[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
                const int j = j0 + u * G;
                const int pos = j < m1 ? a + j : ca + (j - m1);
                t[u] = j < m ? src[pos] : zero;
                th[u] = (src_h && j < m) ? src_h[pos] : zero;
            }
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
                acc = acc + f3(t[u]);
                if (src_h) h = h + f3(th[u]);
            }
        }
    }
    for (int o = G / 2; o > 0; o >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
        if (src_h) {
            h.x += __shfl_xor_sync(0xffffffffu, h.x, o);
            h.y += __shfl_xor_sync(0xffffffffu, h.y, o);
            h.z += __shfl_xor_sync(0xffffffffu, h.z, o);
        }
    }
    return acc;
}

__device__ __forceinline__ F3 gather_slots(const float4* __restrict__ src, const float4* __restrict__ src_h, F3& h,
                                           const VertexSlots& S, int i, bool valid, int lane, int G) {
    return gather_range(src, src_h, h, vertex_range(S, i, valid), lane, G);
}

// The widest group (a power of two up to kGather) that still gives every vertex a group of its own when the grid
// has nthreads threads (one lane per vertex when the grid is smaller than the vertex count).
__host__ __device__ __forceinline__ int gather_width(long long nthreads, int np) {
    int G = kGather;
    while (G > 1 && nthreads / G < np) G >>= 1;
    return G;
}

// ------------------------------------------------------------------ energies
struct Mat2 {
    float a, b, c, d;  // [[a, b], [c, d]]
};
__device__ __forceinline__ Mat2 mmul(Mat2 x, Mat2 y) {
    return {x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d};
}
__device__ __forceinline__ Mat2 mtr(Mat2 x) { return {x.a, x.c, x.b, x.d}; }
__device__ __forceinline__ Mat2 madd(Mat2 x, Mat2 y) { return {x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d}; }
__device__ __forceinline__ Mat2 mscale(float s, Mat2 x) { return {s * x.a, s * x.b, s * x.c, s * x.d}; }
__device__ __forceinline__ float mtrace(Mat2 x) { return x.a + x.d; }

struct ElasticLocal {
    F3 b1, b2;
    Mat2 F, invDm;
    float W;
};
__device__ __forceinline__ ElasticLocal elastic_local(const float4* __restrict__ x, int4 t, float W, float4 inv) {
    ElasticLocal L;
    const F3 x0 = f3(x[t.x]), x1 = f3(x[t.y]), x2 = f3(x[t.z]);
    const F3 x01 = x1 - x0, x02 = x2 - x0;
    L.b1 = normalize(x01);
    L.b2 = normalize(x02 - dot(x02, L.b1) * L.b1);
    const Mat2 Ds = {dot(L.b1, x01), dot(L.b1, x02), dot(L.b2, x01), dot(L.b2, x02)};
    L.invDm = {inv.x, inv.y, inv.z, inv.w};
    L.F = mmul(Ds, L.invDm);
    L.W = W;
    return L;
}

}  // namespace

// Arguments of the energy kernels (declared in the header for Stage3::energy_args).
struct EnergyArgs {
    const float4* tgt;
    const float* w;
    float m2gt_k;
    int np;
    const int4* tri;
    const float* area;
    const float4* invDm;
    float mu, la;
    int nt;
    const int4* hinge;
    const float2* rest;
    float hinge_k;
    int nh;
    const int4* cidx;
    int2* ctype;
    float* cd;
    float kappa, d_hat, ee_thres;
};

namespace {

// Total energy at x (system.py:325-339): the four energies of the default set, one grid-stride pass over
// [vertices | triangles | hinges | contacts], summed with compensation in a fixed order into sc->energy.
// mesh2gt_pp_distance_energy_kernel (distance_energy.py:6-17), elastic_energy_kernel (elastic_energy.py:40-80),
// hinge_energy_kernel (hinge_energy.py:60-88), collision_energy_kernel (collision_energy.py:49-99: the contact
// is reclassified at x and its type and distance stored for the gradient).
// ls_n >= 1: the energy of line-search trial ls_n, skipped (like the trial itself, k_line_search) once an
// earlier trial was accepted: q and therefore the energy, distances and contact types are already those of the
// accepted trial. Every block reads the same flags: the last block writes sc->energy only after all have started.
// The energy terms of elements first, first + stride, ... of [vertices | triangles | hinges | contacts], summed
// with compensation in the thread.
__device__ __forceinline__ CSum energy_elements(const float4* __restrict__ x, const EnergyArgs& A, int nc, long long first,
                                                long long stride) {
    const long long e1 = A.np, e2 = e1 + A.nt, e3 = e2 + A.nh, total = e3 + nc;
    CSum acc;
    for (long long g = first; g < total; g += stride) {
        float e;
        if (g < e1) {
            const int i = (int)g;
            const float wi = A.w[i] * A.m2gt_k;
            e = 0.5f * length_sq(f3(x[i]) - f3(A.tgt[i])) * wi;
        } else if (g < e2) {
            const int f = (int)(g - e1);
            const ElasticLocal L = elastic_local(x, A.tri[f], A.area[f], A.invDm[f]);
            const Mat2 I = {1.f, 0.f, 0.f, 1.f};
            const Mat2 E = mscale(0.5f, madd(mmul(mtr(L.F), L.F), mscale(-1.f, I)));
            const float trE = mtrace(E);
            e = L.W * (A.mu * mtrace(mmul(E, mtr(E))) + 0.5f * A.la * trE * trE);
        } else if (g < e3) {
            const int h = (int)(g - e2);
            const int4 i = A.hinge[h];
            const float dth = hinge_angle(f3(x[i.x]), f3(x[i.y]), f3(x[i.z]), f3(x[i.w])) - A.rest[h].x;
            e = 0.5f * A.hinge_k * dth * dth * A.rest[h].y;
        } else {
            const int b = (int)(g - e3);
            const int4 i = A.cidx[b];
            const F3 x0 = f3(x[i.x]), x1 = f3(x[i.y]), x2 = f3(x[i.z]), x3 = f3(x[i.w]);
            int2 t = A.ctype[b];
            float d;
            if (t.x == BLOCK_PT) {
                t.y = pt_classify(x0, x1, x2, x3);
                d = pt_pair_distance(x0, x1, x2, x3, t.y);
            } else {
                t.y = ee_classify(x0, x1, x2, x3, A.ee_thres);
                d = ee_pair_distance(x0, x1, x2, x3, t.y);
            }
            A.ctype[b] = t;
            A.cd[b] = d;
            e = d < A.d_hat ? barrier(d, A.d_hat) * A.kappa : 0.f;
        }
        acc.add(e);
    }
    return acc;
}

__global__ void __launch_bounds__(kT) k_energy(const float4* __restrict__ x, EnergyArgs A, SolverScalars* sc,
                                               float2* partial, int ls_n) {
    if (sc->abort) return;
    if (ls_n > 0 && sc->energy < sc->energy_prev) return;
    const CSum acc = energy_elements(x, A, sc->n_contacts, gtid(), gstride());
    grid_sum_finish(acc, partial, &sc->red_count, &sc->energy, nullptr);
}

// ------------------------------------------------------------------ gradients and Hessian diagonal (coeff = -1)
// Each element writes its part of the gradient (and of the Hessian diagonal) per corner into the slot arrays
// gslot / hslot, at the corner's position in its vertex's range (inv_vs / cinv); k_gather_grad then sums each
// vertex's range in a fixed order (no float atomics, so the result is the same run after run).
__global__ void k_diff_elastic(const float4* __restrict__ x, const int4* __restrict__ tri, const float* __restrict__ area,
                               const float4* __restrict__ invDm, float mu, float la, float coeff, int nt, float4* gslot,
                               const int* __restrict__ inv_vs, const SolverScalars* sc) {
    if (sc->abort) return;
    for (int f = gtid(); f < nt; f += gstride()) {
        const int4 t = tri[f];
        const ElasticLocal L = elastic_local(x, t, area[f], invDm[f]);
        const Mat2 I = {1.f, 0.f, 0.f, 1.f};
        const Mat2 E = mscale(0.5f, madd(mmul(mtr(L.F), L.F), mscale(-1.f, I)));
        const float trE = mtrace(E);
        const Mat2 P = mmul(L.F, madd(mscale(2.f * mu, E), mscale(la * trE, I)));
        const Mat2 H = mmul(mscale(coeff * L.W, P), mtr(L.invDm));  // ((coeff W) P) invDm^T
        const F3 f1 = H.a * L.b1 + H.c * L.b2;
        const F3 f2 = H.b * L.b1 + H.d * L.b2;
        const int* at = inv_vs + 3 * (size_t)f;
        gslot[at[0]] = f4(-f1 - f2);
        gslot[at[1]] = f4(f1);
        gslot[at[2]] = f4(f2);
    }
}

struct M33 {
    float m[3][3];
};
__device__ __forceinline__ M33 outer(F3 a, F3 b) {
    const float A[3] = {a.x, a.y, a.z}, B[3] = {b.x, b.y, b.z};
    M33 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = A[i] * B[j];
    return r;
}
__device__ __forceinline__ M33 tr(M33 a) {
    M33 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i];
    return r;
}
__device__ __forceinline__ M33 add(M33 a, M33 b) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a.m[i][j] += b.m[i][j];
    return a;
}
__device__ __forceinline__ M33 sub(M33 a, M33 b) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a.m[i][j] -= b.m[i][j];
    return a;
}
__device__ __forceinline__ M33 scl(float s, M33 a) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a.m[i][j] *= s;
    return a;
}
__device__ __forceinline__ M33 sym(M33 a) { return add(a, tr(a)); }

// hinge_diff_kernel (hinge_energy.py:85-238): gradient, Hessian diagonal and the 4x4 blocks of 3x3
__global__ void k_diff_hinge(const float4* __restrict__ x, const int4* __restrict__ hinge, const float2* __restrict__ rest,
                             float k, float coeff, int nh, float* blocks, float4* gslot, float4* hslot,
                             const int* __restrict__ inv_h, const SolverScalars* sc) {
    if (sc->abort) return;
    for (int h = gtid(); h < nh; h += gstride()) {
        const int4 id = hinge[h];
        const F3 x0 = f3(x[id.x]), x1 = f3(x[id.y]), x2 = f3(x[id.z]), x3 = f3(x[id.w]);
        const float rest_angle = rest[h].x, rest_elen = rest[h].y;
        const F3 e0 = x2 - x1, e1 = x0 - x2, e2 = x0 - x1, e1_ = x3 - x2, e2_ = x3 - x1;
        const float e0_lensq = length_sq(e0);
        const float e0_len = sqrtf(e0_lensq), e1_len = length(e1), e2_len = length(e2), e1_len_ = length(e1_),
                    e2_len_ = length(e2_);
        const F3 e0u = normalize(e0), e1u = normalize(e1), e2u = normalize(e2), e1u_ = normalize(e1_), e2u_ = normalize(e2_);
        const float ca1 = dot(e2u, e0u), ca2 = -dot(e1u, e0u), ca1_ = dot(e2u_, e0u), ca2_ = -dot(e1u_, e0u);
        const float h0 = length(cross(e1, e2)) / e0_len, h1 = length(cross(e0, e2)) / e1_len, h2 = length(cross(e0, e1)) / e2_len;
        const float h0_ = length(cross(e1_, e2_)) / e0_len, h1_ = length(cross(e0, e2_)) / e1_len_,
                    h2_ = length(cross(e0, e1_)) / e2_len_;
        const F3 n = normalize(cross(e0, e2)), n_ = normalize(cross(e2_, e0));
        const float theta = atan2f(dot(cross(n, n_), e0) / e0_len, dot(n, n_));
        const float dE = k * (theta - rest_angle) * rest_elen;
        const float d2E = k * rest_elen;
        const F3 g1 = n * (ca2 / h1) + n_ * (ca2_ / h1_);
        const F3 g2 = n * (ca1 / h2) + n_ * (ca1_ / h2_);
        const F3 g0 = n * (-1.0f / h0);
        const F3 g3 = n_ * (-1.0f / h0_);
        const int* at = inv_h + 4 * (size_t)h;
        gslot[at[0]] = f4(dE * g0 * coeff);
        gslot[at[1]] = f4(dE * g1 * coeff);
        gslot[at[2]] = f4(dE * g2 * coeff);
        gslot[at[3]] = f4(dE * g3 * coeff);
        const F3 m0 = normalize(cross(e0, n)), m1 = normalize(cross(e1, n)), m2 = normalize(cross(n, e2));
        const F3 m0_ = normalize(cross(n_, e0)), m1_ = normalize(cross(n_, e1_)), m2_ = normalize(cross(e2_, n_));
        const M33 M0 = outer(n, m0), M1 = outer(n, m1), M2 = outer(n, m2);
        const M33 M0_ = outer(n_, m0_), M1_ = outer(n_, m1_), M2_ = outer(n_, m2_);
        const M33 N0 = scl(1.f / e0_lensq, M0), N0_ = scl(1.f / e0_lensq, M0_);
        const M33 P10 = scl(ca1 / (h1 * h0), tr(M0)), P11 = scl(ca1 / (h1 * h1), tr(M1)), P12 = scl(ca1 / (h1 * h2), tr(M2));
        const M33 P20 = scl(ca2 / (h2 * h0), tr(M0)), P21 = scl(ca2 / (h2 * h1), tr(M1)), P22 = scl(ca2 / (h2 * h2), tr(M2));
        const M33 P10_ = scl(ca1_ / (h1_ * h0_), tr(M0_)), P11_ = scl(ca1_ / (h1_ * h1_), tr(M1_)),
                  P12_ = scl(ca1_ / (h1_ * h2_), tr(M2_));
        const M33 P20_ = scl(ca2_ / (h2_ * h0_), tr(M0_)), P21_ = scl(ca2_ / (h2_ * h1_), tr(M1_)),
                  P22_ = scl(ca2_ / (h2_ * h2_), tr(M2_));
        const M33 Q0 = scl(1.f / (h0 * h0), M0), Q1 = scl(1.f / (h0 * h1), M1), Q2 = scl(1.f / (h0 * h2), M2);
        const M33 Q0_ = scl(1.f / (h0_ * h0_), M0_), Q1_ = scl(1.f / (h0_ * h1_), M1_), Q2_ = scl(1.f / (h0_ * h2_), M2_);
        M33 B[4][4];
        B[0][0] = add(scl(-dE, sym(Q0)), scl(d2E, outer(g0, g0)));
        B[3][3] = add(scl(-dE, sym(Q0_)), scl(d2E, outer(g3, g3)));
        B[1][1] = add(scl(dE, sub(add(sub(sym(P11), N0), sym(P11_)), N0_)), scl(d2E, outer(g1, g1)));
        B[2][2] = add(scl(dE, sub(add(sub(sym(P22), N0), sym(P22_)), N0_)), scl(d2E, outer(g2, g2)));
        B[1][0] = add(scl(dE, sub(P10, Q1)), scl(d2E, outer(g1, g0)));
        B[2][0] = add(scl(dE, sub(P20, Q2)), scl(d2E, outer(g2, g0)));
        B[1][3] = add(scl(dE, sub(P10_, Q1_)), scl(d2E, outer(g1, g3)));
        B[2][3] = add(scl(dE, sub(P20_, Q2_)), scl(d2E, outer(g2, g3)));
        B[1][2] = add(scl(dE, add(add(add(add(add(P12, tr(P21)), N0), P12_), tr(P21_)), N0_)), scl(d2E, outer(g1, g2)));
        B[0][3] = scl(d2E, outer(g0, g3));
        B[0][1] = tr(B[1][0]);
        B[0][2] = tr(B[2][0]);
        B[3][1] = tr(B[1][3]);
        B[3][2] = tr(B[2][3]);
        B[2][1] = tr(B[1][2]);
        B[3][0] = tr(B[0][3]);
        // the symmetric top-left 9x9 (blocks [0..2][0..2]) for the PSD projection
        float* out = blocks + (size_t)h * kHingeStride;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int b = a; b < 3; ++b)
#pragma unroll
                    for (int j = 0; j < 3; ++j)
                        if (b * 3 + j >= a * 3 + i) out[sym9(a * 3 + i, b * 3 + j)] = B[a][b].m[i][j];
        for (int a = 0; a < 4; ++a) hslot[at[a]] = f4(F3{B[a][a].m[0][0], B[a][a].m[1][1], B[a][a].m[2][2]});
    }
}

// block_spd_project_kernel (utils_kernels.py:21-39). The reference calls the fork-only
// wp.spd_project_blocks(3, block, it_max); here the 9x9 matrix of blocks [0..2][0..2] is made positive
// semi-definite by a cyclic Jacobi eigen-decomposition (it_max sweeps), clamping negative eigenvalues to
// zero; the fourth block row and column are then set from the first three as the reference does.
// Nine lanes per hinge (three hinges per warp; lanes 27-31 only take part in the warp barriers), lane k owning
// row k of A and of the eigenvector matrix V in shared memory. Each rotation (p, q) of the cyclic order is
// applied in two parallel halves, columns p and q of every row and then rows p and q of every column, which is
// the sequential update's order entry by entry, so the result is the one-thread-per-hinge sweep's bit for bit;
// the sweeps stay a loop with run-time (p, q) instead of a fully unrolled register version, whose code (tens
// of KB per sweep) streamed through the instruction cache with one warp per SM.
constexpr int kSpdWarps = 4;

__global__ void __launch_bounds__(32 * kSpdWarps) k_spd_project(float* blocks, int nh, int sweeps,
                                                                const SolverScalars* sc) {
    if (sc->abort) return;
    __shared__ float sA[kSpdWarps][3][81], sV[kSpdWarps][3][81];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = lane / 9;
    const bool owner = grp < 3;                 // lanes 27-31 read group 0's rows but never write
    const int g = owner ? grp : 0, k = owner ? lane - 9 * grp : 0;
    float* A = sA[warp][g];
    float* V = sV[warp][g];
    const long long warps = (long long)gridDim.x * kSpdWarps;
    for (long long base = ((long long)blockIdx.x * kSpdWarps + warp) * 3; base < nh; base += warps * 3) {
        const long long h = base + g;
        const bool live = owner && h < nh;
        float* B = blocks + (size_t)(live ? h : 0) * kHingeStride;
        if (live)
            for (int j = 0; j < 9; ++j) {
                A[9 * k + j] = B[sym9(k, j)];
                V[9 * k + j] = (k == j) ? 1.f : 0.f;
            }
        __syncwarp();
        for (int sw = 0; sw < sweeps; ++sw)
            for (int p = 0; p < 8; ++p)
                for (int q = p + 1; q < 9; ++q) {
                    const float apq = A[9 * p + q];
                    const bool rot = !(fabsf(apq) < 1e-30f);
                    // rotation angle by the fast (approximate) reciprocal and square-root instructions: the
                    // projection only needs an orthogonal rotation that shrinks the off-diagonal entry
                    const float th = __fdividef(A[9 * q + q] - A[9 * p + p], 2.f * apq);
                    const float r2 = fmaf(th, th, 1.f);
                    const float t = fabsf(th) > 1e18f ? __fdividef(0.5f, th)
                                                      : copysignf(__fdividef(1.f, fabsf(th) + r2 * rsqrtf(r2)), th);
                    const float c = rsqrtf(fmaf(t, t, 1.f)), sn = t * c;
                    const float akp = A[9 * k + p], akq = A[9 * k + q];
                    __syncwarp();  // the angle's entries are read before they change
                    if (live && rot) {
                        A[9 * k + p] = c * akp - sn * akq;
                        A[9 * k + q] = sn * akp + c * akq;
                    }
                    __syncwarp();
                    const float apk = A[9 * p + k], aqk = A[9 * q + k];
                    if (live && rot) {
                        A[9 * p + k] = c * apk - sn * aqk;
                        A[9 * q + k] = sn * apk + c * aqk;
                        const float vkp = V[9 * k + p], vkq = V[9 * k + q];
                        V[9 * k + p] = c * vkp - sn * vkq;
                        V[9 * k + q] = sn * vkp + c * vkq;
                    }
                    __syncwarp();
                }
        if (live) {
            float lam[9];
            for (int i = 0; i < 9; ++i) lam[i] = fmaxf(A[9 * i + i], 0.f);
            for (int j = k; j < 9; ++j) {
                float acc = 0.f;
                for (int i = 0; i < 9; ++i) acc += V[9 * k + i] * lam[i] * V[9 * j + i];
                B[sym9(k, j)] = acc;
            }
        }
        __syncwarp();  // the group's rows are read before the next hinge overwrites them
    }
}

// collision_diff_kernel (collision_energy.py:192-254)
__global__ void k_diff_contact(const float4* __restrict__ x, const int4* __restrict__ cidx, const int2* __restrict__ ctype,
                               const float* __restrict__ cd, const SolverScalars* sc, float kappa, float dh, float coeff,
                               float4* cdd, float4* gslot, float4* hslot, const int* __restrict__ cinv) {
    if (sc->abort) return;
    const int n = sc->n_contacts;
    for (int b = gtid(); b < n; b += gstride()) {
        const float d = cd[b];
        const int* at = cinv + 4 * (size_t)b;
        if (d >= dh) {  // no barrier term: zero parts
            const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int k = 0; k < 4; ++k) {
                gslot[at[k]] = zero;
                hslot[at[k]] = zero;
            }
            continue;
        }
        const int4 i = cidx[b];
        const F3 x0 = f3(x[i.x]), x1 = f3(x[i.y]), x2 = f3(x[i.z]), x3 = f3(x[i.w]);
        const int2 t = ctype[b];
        F3 g[4];
        if (t.x == BLOCK_PT) pt_pair_grad(x0, x1, x2, x3, t.y, g);
        else ee_pair_grad(x0, x1, x2, x3, t.y, g);
        const float ddc = barrier_d1(d, dh) * kappa * coeff;
        const float d2c = barrier_d2(d, dh) * kappa;
        for (int k = 0; k < 4; ++k) {
            cdd[4 * (size_t)b + k] = f4(g[k]);
            gslot[at[k]] = f4(g[k] * ddc);
            hslot[at[k]] = f4(d2c * F3{g[k].x * g[k].x, g[k].y * g[k].y, g[k].z * g[k].z});
        }
    }
}

// grad = the mesh-to-GT term (mesh2gt_pp_distance diff, distance_energy.py:20-33) plus the vertex's slots, hd
// the same for the Hessian diagonal; a group of kGather lanes per vertex.
__global__ void __launch_bounds__(kT) k_gather_grad(const float4* __restrict__ x, const float4* __restrict__ tgt,
                                                    const float* __restrict__ w, float stiff, float coeff, int np,
                                                    const float4* __restrict__ gslot, const float4* __restrict__ hslot,
                                                    VertexSlots S, float4* grad, float4* hd, const SolverScalars* sc) {
    if (sc->abort) return;
    const int G = gather_width((long long)gridDim.x * blockDim.x, np);
    const long long ngroups = (long long)gridDim.x * blockDim.x / G;
    const long long group = gtid() / G;
    const int lane = (int)(gtid() % G);
    const long long rounds = (np + ngroups - 1) / ngroups;
    for (long long k = 0; k < rounds; ++k) {
        const long long ii = group + k * ngroups;
        const bool valid = ii < np;
        const int i = valid ? (int)ii : 0;
        F3 h;
        const F3 g = gather_slots(gslot, hslot, h, S, i, valid, lane, G);
        if (valid && lane == 0) {
            const float wi = w[i] * stiff;
            grad[i] = f4((f3(x[i]) - f3(tgt[i])) * wi * coeff + g);
            hd[i] = f4(F3{wi, wi, wi} + h);
        }
    }
}

// ------------------------------------------------------------------ Jacobi PCG (cg_solver.py:46-158)
// Per CG iteration two phases, separated by grid barriers inside one cooperative kernel:
//   Hessian product: the search direction v = z + (z_r / z_r_last) v_prev is formed where it is read
//     (update_v_kernel, solver_kernels.py:26-35), each element writes its corners' parts of H v into the slot
//     array aslot (system.py:348-352: the hess_dx kernels of elastic_energy.py:151-220, hinge_energy.py:241-274
//     and the Gauss-Newton collision_hess_dx_kernel, collision_energy.py:379-409; the vertex term of
//     distance_energy.py:20-33 is added where Av is formed), and v.Av is summed per element (v_e . H_e v_e, which
//     equals v . Av), so no separate dot-product pass is needed;
//   p/r/z: Av_i = the vertex term plus the sum of vertex i's slots (gather_slots, a fixed order: the same result
//     run after run, where float atomics would add in the order the threads arrive), p += alpha v, r -= alpha Av
//     when v.Av > 1e-16, z = r / diag, z.r (update_p_r_z_compute_zr_kernel, solver_kernels.py:4-23).
struct HvpArgs {
    const float* w;
    float m2gt_k;
    int np;
    const int4* tri;
    const float* area;
    const float4* invDm;
    float mu, la;
    int nt;
    const int4* hinge;
    const float* blocks;
    int nh;
    const int4* cidx;
    const float* cd;
    const float4* cdd;
    float kappa, d_hat;
    float4* aslot;  // per-corner parts of H v (triangles, hinges, then contacts at S.cbase)
    VertexSlots S;
};

__device__ __forceinline__ F3 cg_dir(const float4* __restrict__ z, const float4* __restrict__ vprev, float s, int j) {
    return f3(z[j]) + s * f3(vprev[j]);
}

// The vertex ids of element g of hvp_elements (a triangle, hinge or contact; zeros for a vertex term or past
// the end). They do not change during a solve, so a thread loads those of its first element once.
__device__ __forceinline__ int4 element_ids(const HvpArgs& A, int nc, long long g) {
    const long long e1 = A.np, e2 = e1 + A.nt, e3 = e2 + A.nh, total = e3 + nc;
    if (g < e1 || g >= total) return make_int4(0, 0, 0, 0);
    if (g < e2) return A.tri[g - e1];
    if (g < e3) return A.hinge[g - e2];
    return A.cidx[g - e3];
}

// Where the corners' parts of element g go in A.aslot (unused entries zero; the vertex terms have none). Like the
// ids they are fixed during a solve, so a thread loads those of its first element once.
__device__ __forceinline__ int4 element_slots(const HvpArgs& A, int nc, long long g) {
    const long long e1 = A.np, e2 = e1 + A.nt, e3 = e2 + A.nh, total = e3 + nc;
    if (g < e1 || g >= total) return make_int4(0, 0, 0, 0);
    if (g < e2) {
        const int* at = A.S.inv_vs + 3 * (g - e1);
        return make_int4(at[0], at[1], at[2], 0);
    }
    if (g < e3) {
        const int* at = A.S.inv_vs + 3 * (size_t)A.nt + 4 * (g - e2);
        return make_int4(at[0], at[1], at[2], at[3]);
    }
    const int* at = A.S.cinv + 4 * (g - e3);
    return make_int4(A.S.cbase + at[0], A.S.cbase + at[1], A.S.cbase + at[2], A.S.cbase + at[3]);
}

// The corners' parts of H v over the elements gtid, gtid + stride, ... into A.aslot; returns this thread's part of
// v.Av. The direction is v = z + s v_prev, written to vout by the vertex terms. ids0 = element_ids(first),
// at0 = element_slots(first).
__device__ __forceinline__ CSum hvp_elements(const float4* __restrict__ x, const HvpArgs& A, const float4* __restrict__ z,
                                             const float4* __restrict__ vprev, float4* vout, float s, int nc,
                                             long long first, long long stride, int4 ids0, int4 at0) {
    const long long e1 = A.np, e2 = e1 + A.nt, e3 = e2 + A.nh, total = e3 + nc;
    CSum acc;
    for (long long g = first; g < total; g += stride) {
        const bool cached = g == first;
        if (g < e1) {
            const int i = (int)g;
            const F3 vi = cg_dir(z, vprev, s, i);
            vout[i] = f4(vi);
            const float wi = A.w[i] * A.m2gt_k;
            acc.add(dot(vi, vi * wi));
        } else if (g < e2) {
            const int f = (int)(g - e1);
            const int4 t = cached ? ids0 : A.tri[f];
            const ElasticLocal L = elastic_local(x, t, A.area[f], A.invDm[f]);
            const F3 v0 = cg_dir(z, vprev, s, t.x), v1 = cg_dir(z, vprev, s, t.y), v2 = cg_dir(z, vprev, s, t.z);
            const F3 dx01 = v1 - v0, dx02 = v2 - v0;
            const Mat2 dDs = {dot(L.b1, dx01), dot(L.b1, dx02), dot(L.b2, dx01), dot(L.b2, dx02)};
            const Mat2 dF = mmul(dDs, L.invDm);
            const Mat2 I = {1.f, 0.f, 0.f, 1.f};
            const Mat2 E = mscale(0.5f, madd(mmul(mtr(L.F), L.F), mscale(-1.f, I)));
            const float trE = mtrace(E);
            const Mat2 dE = mscale(0.5f, madd(mmul(mtr(dF), L.F), mmul(mtr(L.F), dF)));
            const float trdE = mtrace(dE);
            const Mat2 dP = madd(mmul(dF, madd(mscale(2.f * A.mu, E), mscale(A.la * trE, I))),
                                 mmul(L.F, madd(mscale(2.f * A.mu, dE), mscale(A.la * trdE, I))));
            const Mat2 dH = mmul(mscale(L.W, dP), mtr(L.invDm));
            const F3 df1 = dH.a * L.b1 + dH.c * L.b2;
            const F3 df2 = dH.b * L.b1 + dH.d * L.b2;
            const F3 df0 = -df1 - df2;
            const int4 at = cached ? at0 : element_slots(A, nc, g);
            A.aslot[at.x] = f4(df0);
            A.aslot[at.y] = f4(df1);
            A.aslot[at.z] = f4(df2);
            acc.add(dot(v0, df0) + dot(v1, df1) + dot(v2, df2));
        } else if (g < e3) {
            const int h = (int)(g - e2);
            const int4 id = cached ? ids0 : A.hinge[h];
            const int ids[4] = {id.x, id.y, id.z, id.w};
            // H v with the fourth block row/column minus the sums of the first three: for w_a = v_a - v_3,
            // (H v)_a = sum_b A_ab w_b (a < 3), (H v)_3 = -sum_a (H v)_a, and v.H v = w.A w
            const float4* B4 = reinterpret_cast<const float4*>(A.blocks + (size_t)h * kHingeStride);
            float Bm[kHingeStride];
#pragma unroll
            for (int k = 0; k < kHingeStride / 4; ++k) {
                const float4 b = B4[k];
                Bm[4 * k] = b.x; Bm[4 * k + 1] = b.y; Bm[4 * k + 2] = b.z; Bm[4 * k + 3] = b.w;
            }
            const F3 d3 = cg_dir(z, vprev, s, ids[3]);
            float w[9];
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const F3 wb = cg_dir(z, vprev, s, ids[b]) - d3;
                w[3 * b] = wb.x; w[3 * b + 1] = wb.y; w[3 * b + 2] = wb.z;
            }
            float u[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                float t = 0.f;
#pragma unroll
                for (int j = 0; j < 9; ++j) t += Bm[sym9(i, j)] * w[j];
                u[i] = t;
            }
            float vhv = 0.f;
            F3 sum = {0.f, 0.f, 0.f};
            const int4 at4 = cached ? at0 : element_slots(A, nc, g);
            const int at[4] = {at4.x, at4.y, at4.z, at4.w};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const F3 ua = {u[3 * a], u[3 * a + 1], u[3 * a + 2]};
                A.aslot[at[a]] = f4(ua);
                sum = sum + ua;
                vhv += w[3 * a] * ua.x + w[3 * a + 1] * ua.y + w[3 * a + 2] * ua.z;
            }
            A.aslot[at[3]] = f4(-sum);
            acc.add(vhv);
        } else {
            const int b = (int)(g - e3);
            const float dist = A.cd[b];
            float4* as = A.aslot;
            const int4 at4 = cached ? at0 : element_slots(A, nc, g);
            const int at[4] = {at4.x, at4.y, at4.z, at4.w};
            if (dist >= A.d_hat) {  // no barrier term: zero parts
                const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int k = 0; k < 4; ++k) as[at[k]] = zero;
                continue;
            }
            const float c = barrier_d2(dist, A.d_hat) * A.kappa;
            const int4 i = cached ? ids0 : A.cidx[b];
            const int ids[4] = {i.x, i.y, i.z, i.w};
            F3 gg[4];
            float sd = 0.f;
            for (int k = 0; k < 4; ++k) {
                gg[k] = f3(A.cdd[4 * (size_t)b + k]);
                sd += dot(gg[k], cg_dir(z, vprev, s, ids[k]));
            }
            for (int k = 0; k < 4; ++k) as[at[k]] = f4(gg[k] * (sd * c));
            acc.add(sd * sd * c);
        }
    }
    return acc;
}

// p = 0, r = grad, z = r / (diag + 1e-6) (compute_block_diag_inv_kernel), v_prev = 0; returns z.r part
__device__ __forceinline__ CSum cg_init_vertices(const float4* __restrict__ grad, const float4* __restrict__ hd, int np,
                                                 float4* p, float4* r, float4* z, float4* vprev, int first,
                                                 int stride) {
    CSum acc;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = first; i < np; i += stride) {
        const float4 g = grad[i], d = hd[i];
        p[i] = zero;
        r[i] = g;
        const float4 zz = make_float4(g.x / (d.x + 1e-6f), g.y / (d.y + 1e-6f), g.z / (d.z + 1e-6f), 0.f);
        z[i] = zz;
        vprev[i] = zero;
        acc.add(zz.x * g.x + zz.y * g.y + zz.z * g.z);
    }
    return acc;
}

// The p/r/z phase runs on groups of kGather lanes, group k of the grid taking vertices k, k + groups, ... (the same
// number of rounds in every warp, for the shuffles of gather_slots).
struct PrzLanes {
    int group, lane, groups, rounds, G;
};
__device__ __forceinline__ PrzLanes prz_lanes(int tid, int nthreads, int np) {
    PrzLanes L;
    L.G = gather_width(nthreads, np);
    L.group = tid / L.G;
    L.lane = tid % L.G;
    L.groups = nthreads / L.G;
    L.rounds = (np + L.groups - 1) / L.groups;
    return L;
}

// What the p/r/z phase reads for one vertex: v, p, r, diag and Av (the vertex term plus the gathered slots), all
// independent of v.Av, so that the first round's values are loaded before the block partials are summed.
struct PrzVertex {
    float4 v, p, r, d;
    F3 av;
};

__device__ __forceinline__ PrzVertex prz_load(const HvpArgs& A, const float4* __restrict__ v,
                                              const float4* __restrict__ hd, const float4* p, const float4* r,
                                              int i, bool valid, const PrzLanes& L, const VRange& R) {
    PrzVertex pv{};
    F3 unused;
    const F3 g = gather_range(A.aslot, nullptr, unused, R, L.lane, L.G);
    if (valid) {
        pv.v = v[i];
        pv.p = p[i];
        pv.r = r[i];
        pv.d = hd[i];
        pv.av = f3(pv.v) * (A.w[i] * A.m2gt_k) + g;
    }
    return pv;
}

// p += alpha v, r -= alpha Av when v.Av > 1e-16, z = r / diag; returns z.r part. `pre` holds the values of the
// group's first vertex, loaded before the block partials of v.Av were summed.
__device__ __forceinline__ CSum cg_prz_vertices(const HvpArgs& A, const float4* __restrict__ v,
                                                const float4* __restrict__ hd, float4* p, float4* r, float4* z,
                                                float zr, float vAv, const PrzLanes& L, const PrzVertex& pre) {
    const float alpha = zr / vAv;
    CSum acc;
    for (int k = 0; k < L.rounds; ++k) {
        const int i = L.group + k * L.groups;
        const bool valid = i < A.np;
        const PrzVertex pv = k == 0 ? pre : prz_load(A, v, hd, p, r, valid ? i : 0, valid, L,
                                                     vertex_range(A.S, valid ? i : 0, valid));
        if (!valid || L.lane != 0) continue;
        float4 ri = pv.r;
        if (vAv > 1e-16f) {
            float4 pi = pv.p;
            pi.x += alpha * pv.v.x; pi.y += alpha * pv.v.y; pi.z += alpha * pv.v.z;
            ri.x -= alpha * pv.av.x; ri.y -= alpha * pv.av.y; ri.z -= alpha * pv.av.z;
            p[i] = pi;
            r[i] = ri;
        }
        const float4 d = pv.d;
        const float4 zz = make_float4(ri.x / d.x, ri.y / d.y, ri.z / d.z, 0.f);
        z[i] = zz;
        acc.add(zz.x * ri.x + zz.y * ri.y + zz.z * ri.z);
    }
    return acc;
}

__device__ __forceinline__ unsigned ld_acquire(volatile unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Barrier across all blocks of a cooperative launch (co-residency guaranteed), sense-reversing on one counter
// that starts at zero: block 0 adds 2^31 - (gridDim.x - 1) and every other block adds 1, so the counter's top
// bit flips exactly when the last block arrives and its low 31 bits are zero again for the next barrier (no
// reset, nothing to do for the last arrival but its own add). Arrival is a release (the block's writes,
// ordered before it by the block barrier, become visible with it), the poll an acquire. The spin is bounded:
// on time-out it records kErrIterLimit in *status and lets the block go on (the host then reports the error).
// extra (0 outside tests) makes block 0 wait for that many arrivals beyond the grid, so that the wait runs out.
__device__ __forceinline__ void grid_barrier(unsigned* count, int* status, unsigned extra) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned inc = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1u) - extra : 1u;
        unsigned old;
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(count), "r"(inc) : "memory");
        long long spins = 0;
        while (((ld_acquire(count) ^ old) & 0x80000000u) == 0u) {
            // after a time-out anywhere in the grid every later wait gives up at once, so the kernel ends soon
            if ((spins & 255) == 255 && (*(volatile int*)status & kErrIterLimit)) break;
            if (++spins > (1ll << 22)) {
                atomicOr(status, kErrIterLimit);
                break;
            }
        }
    }
    __syncthreads();
}

// Sum of the per-block partials in block order, the same value in every block (after a barrier).
__device__ __forceinline__ float grid_partials_sum(const float2* partial) {
    __shared__ float result;
    CSum a;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        CSum t;
        t.s = __ldcg(&partial[b].x);
        t.c = __ldcg(&partial[b].y);
        a.merge(t);
    }
    CSum f = block_reduce(a);
    if (threadIdx.x == 0) result = f.s + f.c;
    __syncthreads();
    const float v = result;
    __syncthreads();
    return v;
}

__device__ __forceinline__ void store_partial(CSum acc, float2* partial) {
    CSum r = block_reduce(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = make_float2(r.s, r.c);
}

struct CgState {
    unsigned count;  // grid_barrier's counter, zeroed before each stage-3 run
};

// The same solve as two ordinary launches per iteration (cg_mode 7), for when a cooperative launch, which needs its
// whole grid resident at once, would wait for other streams' work to drain (many solves at a time on one GPU): each
// kernel is one phase of k_cg_solve with the same grid, threads and elements, and its block partials are summed by the
// last block in block order (grid_sum_finish) instead of by every block after a grid barrier, so the scalars and the
// iterates are the same. The scalars live in sc (z_r, z_r_last, v_A_v).
template <int kThreads>
__global__ void __launch_bounds__(kThreads) k_cg_start(const float4* __restrict__ grad, const float4* __restrict__ hd,
                                                       int np, float4* p, float4* r, float4* z, float4* v0,
                                                       SolverScalars* sc, float2* partial) {
    if (sc->abort) return;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
    grid_sum_finish(cg_init_vertices(grad, hd, np, p, r, z, v0, tid, nthreads), partial, &sc->red_count, &sc->z_r,
                    nullptr);
}

template <int kThreads>
__global__ void __launch_bounds__(kThreads) k_cg_product(const float4* __restrict__ x, HvpArgs A,
                                                         const float4* __restrict__ z, const float4* __restrict__ vin,
                                                         float4* vout, int it, SolverScalars* sc, float2* partial) {
    if (sc->abort) return;
    const int nc = sc->n_contacts;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
    const float s_dir = it == 0 ? 0.f : sc->z_r / sc->z_r_last;
    const int4 ids0 = element_ids(A, nc, tid);
    const int4 at0 = element_slots(A, nc, tid);
    grid_sum_finish(hvp_elements(x, A, z, vin, vout, s_dir, nc, tid, nthreads, ids0, at0), partial, &sc->red_count,
                    &sc->v_A_v, nullptr);
}

template <int kThreads>
__global__ void __launch_bounds__(kThreads) k_cg_update(HvpArgs A, const float4* __restrict__ v,
                                                        const float4* __restrict__ hd, float4* p, float4* r, float4* z,
                                                        SolverScalars* sc, float2* partial) {
    if (sc->abort) return;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
    const PrzLanes L = prz_lanes(tid, nthreads, A.np);
    const VRange R0 = vertex_range(A.S, L.group < A.np ? L.group : 0, L.group < A.np);
    const PrzVertex pre = prz_load(A, v, hd, p, r, L.group < A.np ? L.group : 0, L.group < A.np, L, R0);
    // read before any block can finish (the last block rewrites them after every block has arrived)
    const float zr = sc->z_r, vAv = sc->v_A_v;
    grid_sum_finish(cg_prz_vertices(A, v, hd, p, r, z, zr, vAv, L, pre), partial, &sc->red_count, &sc->z_r,
                    &sc->z_r_last);
}

// The whole Jacobi PCG solve (cg_solver.py:96-158, n_cg_iters iterations) as one cooperative kernel: each
// iteration is the Hessian product phase and the p/r/z phase, with a grid barrier after each. Every block
// forms the same totals (v.Av, z.r) from the block partials in block order.
template <int kThreads>
__global__ void __launch_bounds__(kThreads) k_cg_solve(const float4* __restrict__ x, HvpArgs A, const float4* __restrict__ grad,
                                                 const float4* __restrict__ hd, float4* p, float4* r, float4* z,
                                                 float4* v0, float4* v1, int n_iters, SolverScalars* sc,
                                                 float2* partial, CgState* bar) {
    if (sc->abort) return;
    const int nc = sc->n_contacts;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
    float2* part_a = partial;
    float2* part_b = partial + gridDim.x;
    const int4 ids0 = element_ids(A, nc, tid);
    const int4 at0 = element_slots(A, nc, tid);  // fixed for the whole solve
    const PrzLanes L = prz_lanes(tid, nthreads, A.np);
    const VRange R0 = vertex_range(A.S, L.group < A.np ? L.group : 0, L.group < A.np);  // the group's first vertex
    const unsigned extra = (unsigned)sc->barrier_extra;
    store_partial(cg_init_vertices(grad, hd, A.np, p, r, z, v0, tid, nthreads), part_a);
    grid_barrier(&bar->count, &sc->status, extra);
    float zr = grid_partials_sum(part_a), zr_last = zr;
    for (int it = 0; it < n_iters; ++it) {
        const float4* vin = (it & 1) ? v1 : v0;
        float4* vout = (it & 1) ? v0 : v1;
        const float s_dir = it == 0 ? 0.f : zr / zr_last;
        // partials alternate between two buffers phase by phase: a buffer is rewritten only after the next
        // barrier, which every block reaches after it has read that buffer
        store_partial(hvp_elements(x, A, z, vin, vout, s_dir, nc, tid, nthreads, ids0, at0), part_b);
        grid_barrier(&bar->count, &sc->status, extra);
        // the first vertex's loads and slot gather go out before the partials are summed (they do not depend on
        // v.Av)
        const PrzVertex pre = prz_load(A, vout, hd, p, r, L.group < A.np ? L.group : 0, L.group < A.np, L, R0);
        const float vAv = grid_partials_sum(part_b);
        store_partial(cg_prz_vertices(A, vout, hd, p, r, z, zr, vAv, L, pre), part_a);
        grid_barrier(&bar->count, &sc->status, extra);
        zr_last = zr;
        zr = grid_partials_sum(part_a);
        if (blockIdx.x == 0 && threadIdx.x == 0) sc->v_A_v = vAv;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->z_r = zr;
        sc->z_r_last = zr_last;
    }
}

// The line search (system.py:393-409 with line_search_kernel, solver_kernels.py:52-66) as one cooperative
// launch on k_energy's grid: trial n sets q = q0 + ccd_step 0.5^n p, its energy is summed as k_energy sums it
// (the same threads, block partials and order, so the same value), and the search stops at the first trial whose
// energy is below the energy before it. In place of n_trials launches of k_line_search and k_energy, most of
// which found an earlier trial accepted and returned at once.
__global__ void __launch_bounds__(kT) k_line_search_coop(const float4* __restrict__ q0, const float4* __restrict__ p,
                                                         float4* q, EnergyArgs A, int n_trials, SolverScalars* sc,
                                                         float2* partial, CgState* bar) {
    if (sc->abort) return;
    const int nc = sc->n_contacts;
    const float e_prev = sc->energy_prev, step = sc->ccd_step;
    const unsigned extra = (unsigned)sc->barrier_extra;
    float e = sc->energy;
    for (int n = 0; n < n_trials; ++n) {
        const float a = step * powf(0.5f, (float)n);
        for (int i = gtid(); i < A.np; i += gstride()) {
            const float4 a0 = q0[i], pi = p[i];
            q[i] = make_float4(a0.x + a * pi.x, a0.y + a * pi.y, a0.z + a * pi.z, 0.f);
        }
        grid_barrier(&bar->count, &sc->status, extra);
        // partials alternate between two buffers trial by trial (rewritten only after the next barrier)
        float2* part = partial + (size_t)(n & 1) * gridDim.x;
        store_partial(energy_elements(q, A, nc, gtid(), gstride()), part);
        grid_barrier(&bar->count, &sc->status, extra);
        e = grid_partials_sum(part);
        if (e < e_prev) break;  // the same total in every block
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->energy = e;
}

// The same solve inside one thread-block cluster (up to 16 CTAs): the barriers are the hardware cluster
// barrier and the block partials are exchanged through distributed shared memory instead of a grid-wide
// barrier through global memory. Selected with cg_mode 2.
constexpr int kClusterThreads = 1024;

__global__ void __launch_bounds__(kClusterThreads) k_cg_cluster(const float4* __restrict__ x, HvpArgs A,
                                                                const float4* __restrict__ grad,
                                                                const float4* __restrict__ hd, float4* p, float4* r,
                                                                float4* z, float4* v0, float4* v1,
                                                                int n_iters, SolverScalars* sc) {
    namespace cgr = cooperative_groups;
    cgr::cluster_group cl = cgr::this_cluster();
    __shared__ float2 slot[2];
    __shared__ float total;
    if (sc->abort) return;  // the same value in every CTA: the flag is written only by earlier kernels
    const int nc = sc->n_contacts;
    const unsigned nblk = cl.num_blocks();
    const int tid = (int)(cl.block_rank() * blockDim.x + threadIdx.x), nthreads = (int)(nblk * blockDim.x);
    int phase = 0;
    // cluster-wide compensated total, the same in every CTA (partials merged in rank order)
    auto cluster_total = [&](CSum acc) -> float {
        const int k = phase++ & 1;  // a slot is rewritten only after the next cluster barrier
        CSum br = block_reduce(acc);
        if (threadIdx.x == 0) slot[k] = make_float2(br.s, br.c);
        cl.sync();
        if (threadIdx.x < 32) {  // one remote read per lane, merged in rank order through shuffles
            const unsigned lane = threadIdx.x;
            const float2 t2 = lane < nblk ? *cl.map_shared_rank(&slot[k], lane) : make_float2(0.f, 0.f);
            CSum a;
            for (unsigned b = 0; b < nblk; ++b) {
                CSum t;
                t.s = __shfl_sync(0xffffffffu, t2.x, (int)b);
                t.c = __shfl_sync(0xffffffffu, t2.y, (int)b);
                a.merge(t);
            }
            if (lane == 0) total = a.s + a.c;
        }
        __syncthreads();
        const float v = total;
        __syncthreads();
        return v;
    };
    const int4 ids0 = element_ids(A, nc, tid);
    const int4 at0 = element_slots(A, nc, tid);
    const PrzLanes L = prz_lanes(tid, nthreads, A.np);
    const VRange R0 = vertex_range(A.S, L.group < A.np ? L.group : 0, L.group < A.np);  // the group's first vertex
    float zr = cluster_total(cg_init_vertices(grad, hd, A.np, p, r, z, v0, tid, nthreads)), zr_last = zr;
    float vAv = 0.f;
    for (int it = 0; it < n_iters; ++it) {
        const float4* vin = (it & 1) ? v1 : v0;
        float4* vout = (it & 1) ? v0 : v1;
        const float s_dir = it == 0 ? 0.f : zr / zr_last;
        vAv = cluster_total(hvp_elements(x, A, z, vin, vout, s_dir, nc, tid, nthreads, ids0, at0));
        const PrzVertex pre = prz_load(A, vout, hd, p, r, L.group < A.np ? L.group : 0, L.group < A.np, L, R0);
        const float zr_new = cluster_total(cg_prz_vertices(A, vout, hd, p, r, z, zr, vAv, L, pre));
        zr_last = zr;
        zr = zr_new;
    }
    if (cl.block_rank() == 0 && threadIdx.x == 0) {
        sc->v_A_v = vAv;
        sc->z_r = zr;
        sc->z_r_last = zr_last;
    }
    cl.sync();  // no CTA leaves while another may still read its shared memory
}

// ------------------------------------------------------------------ iteration bookkeeping
// Start of a Newton iteration (system.py:425-432): q_prev_newton = q; the per-vertex contact counts and fill
// cursors cleared.
__global__ void k_iter_begin(const float4* __restrict__ q, float4* qpn, int* ccnt, int* ccur, int np,
                             SolverScalars* sc) {
    if (sc->abort) return;
    for (int i = gtid(); i <= np; i += gstride()) {
        if (i < np) {
            qpn[i] = q[i];
            ccur[i] = 0;
        }
        ccnt[i] = 0;
    }
}

// After detection: the contact count, and the abort code when the list overflowed (energy.py:942-948 halves
// the radius when the count exceeds max_blocks; a count above this build's capacity grows the list instead).
__global__ void k_contacts_done(SolverScalars* sc, int cap, long long max_blocks) {
    if (sc->abort) return;
    const int raw = sc->n_contacts_raw;
    if ((long long)raw > max_blocks) {
        sc->abort = 2;
        return;
    }
    if (raw > cap) {
        sc->abort = 1;
        return;
    }
    sc->n_contacts = raw;
    sc->total_contacts += raw;
    if (raw > sc->max_contacts) sc->max_contacts = raw;
    if (sc->rebuild) sc->n_rebuilds += 1;
    sc->rebuild = 0;
}

// clamp_p_kernel (solver_kernels.py:68-85): keep |q_prev_newton + p - q_prev_detection| <= radius. Contacts are
// detected at the start of every Newton iteration, so q_prev_detection equals q_prev_newton.
__global__ void k_clamp_p(float4* p, const float4* __restrict__ qn, float radius, int np, const SolverScalars* sc) {
    if (sc->abort) return;
    for (int i = gtid(); i < np; i += gstride()) {
        const F3 pi = f3(p[i]), qni = f3(qn[i]);
        const F3 dq = qni + pi - qni;
        if (length(dq) > radius) p[i] = f4(normalize(dq) * radius + qni - qni);
    }
}

// _ccd (system.py:368-391) sets ccd_step = 1; _line_search (:393-409) keeps the energy before the search.
__global__ void k_before_ccd(SolverScalars* sc) {
    if (sc->abort) return;
    sc->ccd_step = 1.0f;
    sc->energy_prev = sc->energy;
}

// accd_kernel (ccd_kernels.py:9-111): additive CCD step bound per contact
// Contacts in the spread order (spread_first): the few heavy CCD contacts of a step land on as many SMs as there
// are active warps (the float64 pipe of one SM is what bounds the float64 CCD), not on the first blocks' SMs.
__global__ void k_accd(const float4* __restrict__ x, const float4* __restrict__ vel, const int4* __restrict__ cidx,
                       const int2* __restrict__ ctype, SolverScalars* sc, float slackness, float thickness, int max_iters,
                       float ee_thres) {
    if (sc->abort) return;
    const int n = sc->n_contacts;
    for (long long bb = spread_first(); bb < n; bb += spread_stride()) {
        const int b = (int)bb;
        const int4 id = cidx[b];
        F3 x0 = f3(x[id.x]), x1 = f3(x[id.y]), x2 = f3(x[id.z]), x3 = f3(x[id.w]);
        F3 v0 = f3(vel[id.x]), v1 = f3(vel[id.y]), v2 = f3(vel[id.z]), v3 = f3(vel[id.w]);
        const int type1 = ctype[b].x;
        const F3 va = (v0 + v1 + v2 + v3) / 4.0f;
        v0 = v0 - va; v1 = v1 - va; v2 = v2 - va; v3 = v3 - va;
        float lv;
        if (type1 == BLOCK_PT) lv = length(v0) + fmaxf(length(v1), fmaxf(length(v2), length(v3)));
        else lv = fmaxf(length(v0), length(v1)) + fmaxf(length(v2), length(v3));
        if (lv < 1e-12f) continue;
        auto dist = [&]() {
            if (type1 == BLOCK_PT) return pt_pair_distance(x0, x1, x2, x3, pt_classify(x0, x1, x2, x3));
            return ee_pair_distance(x0, x1, x2, x3, ee_classify(x0, x1, x2, x3, ee_thres));
        };
        float d = dist();
        float dsq = d * d;
        float dmt = fmaxf((dsq - thickness * thickness) / (sqrtf(dsq) + thickness), 0.f);
        const float gap = (1.0f - slackness) * dmt;
        float t = 0.f;
        float tl = slackness * dmt / lv;
        int it = 0;
        while (true) {
            x0 = x0 + tl * v0; x1 = x1 + tl * v1; x2 = x2 + tl * v2; x3 = x3 + tl * v3;
            d = dist();
            dsq = d * d;
            dmt = fmaxf((dsq - thickness * thickness) / (sqrtf(dsq) + thickness), 0.f);
            if ((it > 0 && dmt <= gap) || it >= max_iters) {
                atomicMin((int*)&sc->ccd_step, __float_as_int(t));  // t >= 0: int order = float order
                break;
            }
            t = t + tl;
            if (t > 1.0f) break;
            tl = 0.8f * dmt / lv;
            ++it;
        }
    }
}

// ------------------------------------------------------------------ CCD in a wider precision
// The precision mode's wide CCD roots: the additive CCD above with positions, step directions, the pair
// classification, the distances and the advancement in a wider real type R (Warp's kernels run it in float32):
// R = double (ccd_fp64 = 1), or R = WF, a double-float hi + lo pair built from FP32 operations only
// (ccd_fp64 = 2, the default): GB300 issues about one FP64 fused multiply-add per SM and clock against 128 in FP32,
// and the float64 CCD was throughput-bound on the FP64 pipe. The resulting step is rounded down to float, so that
// it never exceeds the wide time-of-impact bound. The template body performs, for R = double, the operations of the
// plain float64 code in the same order.
//
// WF: Dekker's double-length arithmetic (TwoSum, TwoProd with an explicit fused multiply-add), with the sloppy
// addition of Hida, Li and Bailey's double-double library: about 44 significant bits.
struct WF {
    float hi, lo;
};
__device__ __forceinline__ void wf_two_prod(float a, float b, float& p, float& e) {
    p = a * b;
    e = __fmaf_rn(a, b, -p);
}
__device__ __forceinline__ WF wf_fast(float a, float b) {  // |a| >= |b| or a == 0
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ WF operator+(WF a, WF b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    return wf_fast(s, e);
}
__device__ __forceinline__ WF operator-(WF a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ WF operator-(WF a, WF b) { return a + (-b); }
__device__ __forceinline__ WF operator*(WF a, WF b) {
    float p, e;
    wf_two_prod(a.hi, b.hi, p, e);
    e += a.hi * b.lo + a.lo * b.hi;
    return wf_fast(p, e);
}
__device__ __forceinline__ WF operator/(WF a, WF b) {
    const float q1 = a.hi / b.hi;
    float p, e;
    wf_two_prod(q1, b.hi, p, e);  // a - q1 b, to first order
    const float r = ((a.hi - p) - e + a.lo - q1 * b.lo);
    return wf_fast(q1, r / b.hi);
}
// comparisons of normalised pairs, false with a NaN as for double
__device__ __forceinline__ bool operator<(WF a, WF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(WF a, WF b) { return b < a; }
__device__ __forceinline__ bool operator<=(WF a, WF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }
__device__ __forceinline__ bool operator>=(WF a, WF b) { return b <= a; }
__device__ __forceinline__ bool operator==(WF a, WF b) { return a.hi == b.hi && a.lo == b.lo; }

// the real-type operations the template body uses, for double and for WF
template <class R> struct Real;
template <> struct Real<double> {
    __device__ static __forceinline__ double c(double v) { return v; }
    __device__ static __forceinline__ double of(float v) { return (double)v; }
    __device__ static __forceinline__ double sqrt_(double a) { return sqrt(a); }
    __device__ static __forceinline__ double abs_(double a) { return fabs(a); }
    __device__ static __forceinline__ double max_(double a, double b) { return fmax(a, b); }
    __device__ static __forceinline__ float floor_float(double a) { return __double2float_rd(a); }
};
template <> struct Real<WF> {
    // constants: hi = v rounded to float, lo = the rest (both folded at compile time for literal v)
    __device__ static __forceinline__ WF c(double v) { return {(float)v, (float)(v - (double)(float)v)}; }
    __device__ static __forceinline__ WF of(float v) { return {v, 0.0f}; }
    __device__ static __forceinline__ WF sqrt_(WF a) {
        if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
        const float r = sqrtf(a.hi);
        float p, e;
        wf_two_prod(r, r, p, e);
        return wf_fast(r, ((a.hi - p) - e + a.lo) / (2.0f * r));
    }
    __device__ static __forceinline__ WF abs_(WF a) { return a.hi < 0.0f ? -a : a; }
    __device__ static __forceinline__ WF max_(WF a, WF b) {  // fmax: a NaN operand gives the other
        if (a.hi != a.hi) return b;
        if (b.hi != b.hi) return a;
        return a < b ? b : a;
    }
    // the largest float not above hi + lo (|lo| <= ulp(hi) / 2)
    __device__ static __forceinline__ float floor_float(WF a) {
        return a.lo < 0.0f ? nextafterf(a.hi, -INFINITY) : a.hi;
    }
};

template <class R>
struct T3 {
    R x, y, z;
};
template <class R>
__device__ __forceinline__ T3<R> t3(float4 a) {
    return {Real<R>::of(a.x), Real<R>::of(a.y), Real<R>::of(a.z)};
}
template <class R>
__device__ __forceinline__ T3<R> operator+(T3<R> a, T3<R> b) {
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <class R>
__device__ __forceinline__ T3<R> operator-(T3<R> a, T3<R> b) {
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <class R>
__device__ __forceinline__ T3<R> operator*(R s, T3<R> a) {
    return {s * a.x, s * a.y, s * a.z};
}
template <class R>
__device__ __forceinline__ T3<R> operator/(T3<R> a, R s) {
    return {a.x / s, a.y / s, a.z / s};
}
template <class R>
__device__ __forceinline__ R dot(T3<R> a, T3<R> b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class R>
__device__ __forceinline__ T3<R> cross(T3<R> a, T3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R>
__device__ __forceinline__ R length_sq(T3<R> a) {
    return dot(a, a);
}
template <class R>
__device__ __forceinline__ R length(T3<R> a) {
    return Real<R>::sqrt_(dot(a, a));
}
template <class R>
__device__ __forceinline__ T3<R> normalize(T3<R> a) {
    const R l = length(a);
    const R zero = Real<R>::c(0.0);
    return l > zero ? a / l : T3<R>{zero, zero, zero};
}
template <class R>
__device__ __forceinline__ R wstep(R x) {
    return x < Real<R>::c(0.0) ? Real<R>::c(1.0) : Real<R>::c(0.0);
}
template <class R>
__device__ __forceinline__ R pt_distance(T3<R> x0, T3<R> x1, T3<R> x2, T3<R> x3) {
    return Real<R>::abs_(dot(x0 - x1, normalize(cross(x2 - x1, x3 - x1))));
}
template <class R>
__device__ __forceinline__ R ee_distance(T3<R> x0, T3<R> x1, T3<R> x2, T3<R> x3) {
    return Real<R>::abs_(dot(x0 - x2, normalize(cross(x1 - x0, x3 - x2))));
}
template <class R>
__device__ __forceinline__ R pe_distance(T3<R> x0, T3<R> x1, T3<R> x2) {
    return length(cross(x1 - x0, x2 - x0)) / length(x1 - x2);
}
template <class R>
__device__ __forceinline__ R pp_distance(T3<R> x0, T3<R> x1) {
    return length(x1 - x0);
}

template <class R>
__device__ int pt_classify(T3<R> x0, T3<R> x1, T3<R> x2, T3<R> x3) {
    typedef Real<R> K;
    const R zero = K::c(0.0);
    T3<R> x10 = x0 - x1;
    const T3<R> x12 = x2 - x1, x13 = x3 - x1;
    const R area_sq = length_sq(cross(x12, x13));
    if (area_sq <= K::c(1e-6) * (length_sq(x12) * length_sq(x13)) || area_sq <= K::c(1e-16)) {
        const R e1 = length(x10), e2 = length(x0 - x2), e3 = length(x0 - x3);
        if (e1 < e2) return e1 < e3 ? PT_PP01 : PT_PP03;
        return e2 < e3 ? PT_PP02 : PT_PP03;
    }
    const T3<R> n = normalize(cross(x12, x13));
    const T3<R> xp = x0 - dot(n, x10) * n;
    x10 = xp - x1;
    const T3<R> x20 = xp - x2, x30 = xp - x3;
    const R a00 = dot(x12, x12), a01 = dot(x12, x13), a11 = dot(x13, x13);
    const R b0 = dot(x10, x12), b1 = dot(x10, x13);
    const R det = a00 * a11 - a01 * a01;
    const R beta = b0 * a11 - b1 * a01;
    const R gamma = a00 * b1 - b0 * a01;
    const R alpha = det - beta - gamma;
    const R nneg = wstep(alpha) + wstep(beta) + wstep(gamma);
    if (nneg == zero) return PT_PT;
    if (nneg == K::c(1.0)) {
        if (alpha < zero) {
            const T3<R> x23 = x3 - x2, x20b = x0 - x2;
            const R dr = dot(x23, x20b);
            if (dr < zero) return PT_PP02;
            if (dr > dot(x23, x23)) return PT_PP03;
            return PT_PE023;
        } else if (beta < zero) {
            const T3<R> x31 = x1 - x3, x30b = x0 - x3;
            const R dr = dot(x31, x30b);
            if (dr < zero) return PT_PP03;
            if (dr > dot(x31, x31)) return PT_PP01;
            return PT_PE031;
        } else if (gamma < zero) {
            const R dr = dot(x12, x10);
            if (dr < zero) return PT_PP01;
            if (dr > dot(x12, x12)) return PT_PP02;
            return PT_PE012;
        }
        return -1;
    }
    if (alpha >= zero) {
        const R d12 = dot(x12, x10), d13 = dot(x13, x10);
        if (d12 > zero && d13 <= zero) return dot(x12, x20) > zero ? PT_PP02 : PT_PE012;
        if (d13 > zero && d12 <= zero) return dot(x13, x30) > zero ? PT_PP03 : PT_PE031;
        return PT_PP01;
    } else if (beta >= zero) {
        const T3<R> x23 = x3 - x2, x21 = x1 - x2;
        const R d23 = dot(x23, x20), d21 = dot(x21, x20);
        if (d23 > zero && d21 <= zero) return dot(x23, x30) > zero ? PT_PP03 : PT_PE023;
        if (d21 > zero && d23 <= zero) return dot(x21, x10) > zero ? PT_PP01 : PT_PE012;
        return PT_PP02;
    }
    const T3<R> x31 = x1 - x3, x32 = x2 - x3;
    const R d31 = dot(x31, x30), d32 = dot(x32, x30);
    if (d31 > zero && d32 <= zero) return dot(x31, x10) > zero ? PT_PP01 : PT_PE031;
    if (d32 > zero && d31 <= zero) return dot(x32, x20) > zero ? PT_PP02 : PT_PE023;
    return PT_PP03;
}

template <class R>
__device__ R pt_pair_distance(T3<R> x0, T3<R> x1, T3<R> x2, T3<R> x3, int t) {
    switch (t) {
        case PT_PT: return pt_distance(x0, x1, x2, x3);
        case PT_PP01: return pp_distance(x0, x1);
        case PT_PP02: return pp_distance(x0, x2);
        case PT_PE012: return pe_distance(x0, x1, x2);
        case PT_PP03: return pp_distance(x0, x3);
        case PT_PE031: return pe_distance(x0, x3, x1);
        case PT_PE023: return pe_distance(x0, x2, x3);
    }
    return Real<R>::c(1e9);
}

template <class R>
__device__ int ee_classify(T3<R> x0, T3<R> x1, T3<R> x2, T3<R> x3, R sin_thres) {
    typedef Real<R> K;
    const R zero = K::c(0.0);
    const T3<R> e0 = x0 - x1, e1 = x2 - x3;
    const R e0_sq = dot(e0, e0), e1_sq = dot(e1, e1);
    const R a00 = e0_sq, a01 = -dot(e0, e1), a10 = dot(e0, e1), a11 = -e1_sq;
    const R b0 = dot(x3 - x1, e0), b1 = dot(x3 - x1, e1);
    const R mu0 = -(b0 * a11 - b1 * a01);
    const R mu1 = -(a00 * b1 - a10 * b0);
    const R detA = -(a00 * a11 - a01 * a10);
    const R edge_sin = length(cross(normalize(e0), normalize(e1)));
    if (mu0 >= zero && mu0 <= detA && mu1 >= zero && mu1 <= detA && edge_sin >= sin_thres && e0_sq > K::c(1e-15) &&
        e1_sq > K::c(1e-15))
        return EE_EE;
    R best = K::c(1e9);
    int type = -1;
    auto consider = [&](R d, int t) {
        if (d < best) {
            best = d;
            type = t;
        }
    };
    const R t0 = dot(x0 - x3, e1);
    if (t0 >= e1_sq) consider(pp_distance(x0, x2), EE_PP02);
    else if (t0 <= zero) consider(pp_distance(x0, x3), EE_PP03);
    else consider(pe_distance(x0, x2, x3), EE_PE023);
    const R t1 = dot(x1 - x3, e1);
    if (t1 >= e1_sq) consider(pp_distance(x1, x2), EE_PP12);
    else if (t1 <= zero) consider(pp_distance(x1, x3), EE_PP13);
    else consider(pe_distance(x1, x2, x3), EE_PE123);
    const R t2 = dot(x2 - x1, e0);
    if (t2 >= e0_sq) consider(pp_distance(x2, x0), EE_PP02);
    else if (t2 <= zero) consider(pp_distance(x2, x1), EE_PP12);
    else consider(pe_distance(x2, x0, x1), EE_PE201);
    const R t3 = dot(x3 - x1, e0);
    if (t3 >= e0_sq) consider(pp_distance(x3, x0), EE_PP03);
    else if (t3 <= zero) consider(pp_distance(x3, x1), EE_PP13);
    else consider(pe_distance(x3, x0, x1), EE_PE301);
    return type;
}

template <class R>
__device__ R ee_pair_distance(T3<R> x0, T3<R> x1, T3<R> x2, T3<R> x3, int t) {
    switch (t) {
        case EE_PP02: return pp_distance(x0, x2);
        case EE_PP03: return pp_distance(x0, x3);
        case EE_PP12: return pp_distance(x1, x2);
        case EE_PP13: return pp_distance(x1, x3);
        case EE_PE023: return pe_distance(x0, x2, x3);
        case EE_PE123: return pe_distance(x1, x2, x3);
        case EE_PE201: return pe_distance(x2, x0, x1);
        case EE_PE301: return pe_distance(x3, x0, x1);
        case EE_EE: return ee_distance(x0, x1, x2, x3);
    }
    return Real<R>::c(1e9);
}

// slackness, thickness and ee_thres as R (the host passes their float values, widened)
template <class R>
__global__ void k_accd_wide(const float4* __restrict__ x, const float4* __restrict__ vel, const int4* __restrict__ cidx,
                            const int2* __restrict__ ctype, SolverScalars* sc, float slackness_f, float thickness_f,
                            int max_iters, float ee_thres_f) {
    typedef Real<R> K;
    if (sc->abort) return;
    const R slackness = K::of(slackness_f), thickness = K::of(thickness_f), ee_thres = K::of(ee_thres_f);
    const R zero = K::c(0.0), one = K::c(1.0);
    const int n = sc->n_contacts;
    for (long long bb = spread_first(); bb < n; bb += spread_stride()) {
        const int b = (int)bb;
        const int4 id = cidx[b];
        T3<R> x0 = t3<R>(x[id.x]), x1 = t3<R>(x[id.y]), x2 = t3<R>(x[id.z]), x3 = t3<R>(x[id.w]);
        T3<R> v0 = t3<R>(vel[id.x]), v1 = t3<R>(vel[id.y]), v2 = t3<R>(vel[id.z]), v3 = t3<R>(vel[id.w]);
        const int type1 = ctype[b].x;
        const T3<R> va = (v0 + v1 + v2 + v3) / K::c(4.0);
        v0 = v0 - va; v1 = v1 - va; v2 = v2 - va; v3 = v3 - va;
        R lv;
        if (type1 == BLOCK_PT) lv = length(v0) + K::max_(length(v1), K::max_(length(v2), length(v3)));
        else lv = K::max_(length(v0), length(v1)) + K::max_(length(v2), length(v3));
        if (lv < K::c(1e-12)) continue;
        auto dist = [&]() {
            if (type1 == BLOCK_PT) return pt_pair_distance(x0, x1, x2, x3, pt_classify(x0, x1, x2, x3));
            return ee_pair_distance(x0, x1, x2, x3, ee_classify(x0, x1, x2, x3, ee_thres));
        };
        R d = dist();
        R dsq = d * d;
        R dmt = K::max_((dsq - thickness * thickness) / (K::sqrt_(dsq) + thickness), zero);
        const R gap = (one - slackness) * dmt;
        R t = zero;
        R tl = slackness * dmt / lv;
        int it = 0;
        while (true) {
            x0 = x0 + tl * v0; x1 = x1 + tl * v1; x2 = x2 + tl * v2; x3 = x3 + tl * v3;
            d = dist();
            dsq = d * d;
            dmt = K::max_((dsq - thickness * thickness) / (K::sqrt_(dsq) + thickness), zero);
            if ((it > 0 && dmt <= gap) || it >= max_iters) {
                atomicMin((int*)&sc->ccd_step, __float_as_int(K::floor_float(t)));  // t >= 0: int order = float order
                break;
            }
            t = t + tl;
            if (t > one) break;
            tl = K::c(0.8) * dmt / lv;
            ++it;
        }
    }
}

// line_search_kernel (solver_kernels.py:52-66): q = q0 + ccd_step 0.5^n p unless a shorter step already
// lowered the energy
__global__ void k_line_search(const float4* __restrict__ q0, const float4* __restrict__ p, const SolverScalars* sc,
                              int n_halves, int np, float4* q) {
    if (sc->abort) return;
    if (n_halves > 0 && sc->energy < sc->energy_prev) return;
    const float a = sc->ccd_step * powf(0.5f, (float)n_halves);
    for (int i = gtid(); i < np; i += gstride()) {
        const float4 a0 = q0[i], pi = p[i];
        q[i] = make_float4(a0.x + a * pi.x, a0.y + a * pi.y, a0.z + a * pi.z, 0.f);
    }
}

__global__ void k_iter_end(SolverScalars* sc) {
    if (sc->abort) return;
    sc->iters_done += 1;
}

}  // namespace

// ================================================================== host driver
Stage3::~Stage3() { release(); }

// The size-dependent buffers come from the solver's own stream-ordered memory pool: freeing one is ordered after the
// solver's earlier work on its stream and waits for nothing else, where cudaFree would wait for the whole device (many
// solvers sharing a GPU, as in a server, would stall each other every time one of them grows a buffer).
int Stage3::dalloc(void** ptr, size_t bytes) {
    *ptr = nullptr;
    if (cudaMallocFromPoolAsync(ptr, std::max<size_t>(bytes, 16), pool, stream) != cudaSuccess) {
        *ptr = nullptr;
        return fail(PAMO_ERR_OOM, "cudaMallocFromPoolAsync");
    }
    return PAMO_OK;
}

void Stage3::dfree(void* ptr) {
    if (ptr) cudaFreeAsync(ptr, stream);
}

template <typename T>
int Stage3::grow(T*& ptr, size_t& cap, size_t n) {
    if (ptr && cap >= n) return PAMO_OK;
    drop_graph();
    dfree(ptr);
    ptr = nullptr;
    if (dalloc((void**)&ptr, std::max<size_t>(n, 1) * sizeof(T))) return PAMO_ERR_OOM;
    cap = n;
    return PAMO_OK;
}

void Stage3::drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    graph_kernels = 0;
}

void Stage3::release() {
    if (stream) cudaStreamSynchronize(stream);
    drop_graph();
    auto fp = [this](auto*& ptr) {  // pool buffers
        dfree(ptr);
        ptr = nullptr;
    };
    auto f = [](auto*& ptr) {  // the fixed-size buffers of the first call
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
    };
    fp(gt_pos); fp(gt_tri); fp(gt_bvh_mem); fp(q); fp(q_rest); fp(q_prev_newton); fp(p); fp(target);
    fp(grad); fp(hdiag); fp(r); fp(z); fp(v[0]); fp(v[1]); fp(vweight);
    fp(cand_cnt); fp(cand_off); fp(cflag); fp(cpos); fp(cid); fp(cty); fp(vs_off); fp(inv_vs); fp(c_cnt); fp(c_off);
    fp(c_cur); fp(c_tmp); fp(c_inv); fp(gslot); fp(hslot); fp(aslot); fp(scan_scratch);
    cap_cf = cap_vs = cap_vso = cap_slot = cap_cq = 0;
    fp(q_ref); fp(cand_pt); fp(cand_ee); fp(tri); fp(edge4); fp(el_area); fp(el_invDm);
    fp(hinge); fp(hinge_rest); fp(hinge_blocks); fp(c_idx); fp(c_type); fp(c_d); fp(c_dd); fp(tri_bvh_mem);
    fp(edge_bvh_mem);
    if (stream) cudaStreamSynchronize(stream);
    if (pool) cudaMemPoolDestroy(pool);
    pool = nullptr;
    f(gt_rc); f(tri_rc); f(edge_rc); f(sc); f(d_norm); f(cg_bar); f(partial);
    if (h_sc) cudaFreeHost(h_sc);
    h_sc = nullptr;
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    ev_in = ev_out = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
}

int Stage3::ensure(int np, int nt, int ne, int nh, int ngp, int ngt) {
    int rr;
    // first call: stream, pool, events and the fixed-size buffers; a failure part-way releases what was made, so
    // that the next call starts over
    if (!sc) {
        const int r0 = [&]() -> int {
            if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) return fail(PAMO_ERR_CUDA, "stream");
            {
                int dev0 = 0;
                cudaGetDevice(&dev0);
                cudaMemPoolProps props = {};
                props.allocType = cudaMemAllocationTypePinned;
                props.location.type = cudaMemLocationTypeDevice;
                props.location.id = dev0;
                if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) return fail(PAMO_ERR_CUDA, "memory pool");
                unsigned long long keep = ~0ull;  // freed memory stays in the pool for the next growth
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            }
            if (cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming) != cudaSuccess)
                return fail(PAMO_ERR_CUDA, "event");
            if (cudaMalloc((void**)&sc, sizeof(SolverScalars)) != cudaSuccess) return fail(PAMO_ERR_OOM, "cudaMalloc");
            if (cudaMallocHost((void**)&h_sc, sizeof(SolverScalars)) != cudaSuccess) return fail(PAMO_ERR_OOM, "cudaMallocHost");
            if (cudaMalloc((void**)&d_norm, (16 + 9 * kNormBlocks) * sizeof(double)) != cudaSuccess)
                return fail(PAMO_ERR_OOM, "cudaMalloc");
            if (cudaMalloc((void**)&partial, kPartials * sizeof(float2)) != cudaSuccess) return fail(PAMO_ERR_OOM, "cudaMalloc");
            if (cudaMalloc((void**)&cg_bar, 64) != cudaSuccess) return fail(PAMO_ERR_OOM, "cudaMalloc");
            cudaMemset(cg_bar, 0, 64);
            int dev = 0, nsm = 0, occ = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cg_solve<128>, 128, 0);
            coop_max_blocks = std::max(1, nsm * std::max(occ, 0));
            int occ_ls = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_ls, k_line_search_coop, kT, 0);
            ls_coop_max_blocks = nsm * std::max(occ_ls, 0);
            n_sm = std::max(1, nsm);
            // largest cluster the device runs k_cg_cluster with (16 needs the non-portable opt-in)
            cluster_size = 1;
            if (cudaFuncSetAttribute(k_cg_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(16);
                cfg.blockDim = dim3(kClusterThreads);
                int cs = 0;
                if (cudaOccupancyMaxPotentialClusterSize(&cs, k_cg_cluster, &cfg) == cudaSuccess) cluster_size = std::min(cs, 16);
            }
            cudaGetLastError();  // a refused attribute leaves the cooperative path in use
            if (cluster_size < 2) cluster_size = 1;
            if (cudaMalloc((void**)&gt_rc, sizeof(RoundCounters)) != cudaSuccess) return fail(PAMO_ERR_OOM, "cudaMalloc");
            if (cudaMalloc((void**)&tri_rc, sizeof(RoundCounters)) != cudaSuccess) return fail(PAMO_ERR_OOM, "cudaMalloc");
            if (cudaMalloc((void**)&edge_rc, sizeof(RoundCounters)) != cudaSuccess) return fail(PAMO_ERR_OOM, "cudaMalloc");
            return PAMO_OK;
        }();
        if (r0) {
            release();
            return r0;
        }
    }
    size_t c;
    if (cap_gp < (size_t)ngp + 2) {
        c = cap_gp;
        if ((rr = grow(gt_pos, c, (size_t)ngp + 2))) return rr;
        cap_gp = c;
    }
    if (cap_gt < (size_t)ngt + 2) {
        c = cap_gt;
        if ((rr = grow(gt_tri, c, (size_t)ngt + 2))) return rr;
        cap_gt = c;
    }
    if (gt_bvh_cap < (size_t)ngt + 2) {
        drop_graph();
        dfree(gt_bvh_mem);
        gt_bvh_mem = nullptr;
        if ((rr = dalloc((void**)&gt_bvh_mem, bvh_bytes(ngt + 2)))) return rr;
        bvh_carve(gt_bvh, ngt + 2, gt_bvh_mem, false);
        cudaMemsetAsync(gt_bvh.scan_scratch, 0, scan_scratch_ints() * sizeof(int), stream);
        gt_bvh_cap = (size_t)ngt + 2;
    }
    if (cap_v < (size_t)np + 2) {
        const size_t n = (size_t)np + 2;
        for (float4** b : {&q, &q_rest, &q_prev_newton, &q_ref, &p, &target, &grad, &hdiag, &r, &z, &v[0], &v[1]}) {
            c = cap_v;
            if ((rr = grow(*b, c, n))) return rr;
        }
        c = cap_v;
        if ((rr = grow(vweight, c, n))) return rr;
        cap_v = n;
    }
    if (cap_t < (size_t)nt + 2) {
        const size_t n = (size_t)nt + 2;
        c = cap_t;
        if ((rr = grow(tri, c, n))) return rr;
        c = cap_t;
        if ((rr = grow(el_area, c, n))) return rr;
        c = cap_t;
        if ((rr = grow(el_invDm, c, n))) return rr;
        cap_t = n;
        drop_graph();
        dfree(tri_bvh_mem);
        tri_bvh_mem = nullptr;
        if ((rr = dalloc((void**)&tri_bvh_mem, bvh_bytes((int)n)))) return rr;
        bvh_carve(tri_bvh, (int)n, tri_bvh_mem, false);
        cudaMemsetAsync(tri_bvh.scan_scratch, 0, scan_scratch_ints() * sizeof(int), stream);
        tri_bvh_cap = n;
    }
    if (cap_e < (size_t)ne + 2) {
        const size_t n = (size_t)ne + 2;
        c = cap_e;
        if ((rr = grow(edge4, c, n))) return rr;
        cap_e = n;
        drop_graph();
        dfree(edge_bvh_mem);
        edge_bvh_mem = nullptr;
        if ((rr = dalloc((void**)&edge_bvh_mem, bvh_bytes((int)n)))) return rr;
        bvh_carve(edge_bvh, (int)n, edge_bvh_mem, false);
        cudaMemsetAsync(edge_bvh.scan_scratch, 0, scan_scratch_ints() * sizeof(int), stream);
        edge_bvh_cap = n;
    }
    if (cap_h < (size_t)nh + 2) {
        const size_t n = (size_t)nh + 2;
        c = cap_h;
        if ((rr = grow(hinge, c, n))) return rr;
        c = cap_h;
        if ((rr = grow(hinge_rest, c, n))) return rr;
        c = cap_h;
        if ((rr = grow(hinge_blocks, c, n * kHingeStride))) return rr;
        cap_h = n;
    }
    return PAMO_OK;
}

int Stage3::ensure_contacts(size_t n) {
    if (cap_c >= n && c_idx) return PAMO_OK;
    size_t c;
    int rr;
    c = 0;
    drop_graph();
    dfree(c_idx); dfree(c_type); dfree(c_d); dfree(c_dd);
    c_idx = nullptr; c_type = nullptr; c_d = nullptr; c_dd = nullptr;
    if ((rr = grow(c_idx, c, n))) return rr;
    c = 0;
    if ((rr = grow(c_type, c, n))) return rr;
    c = 0;
    if ((rr = grow(c_d, c, n))) return rr;
    c = 0;
    if ((rr = grow(c_dd, c, 4 * n))) return rr;
    for (int** b : {&c_tmp, &c_inv}) {
        c = 0;
        dfree(*b);
        *b = nullptr;
        if ((rr = grow(*b, c, 4 * n))) return rr;
    }
    cap_c = n;
    drop_graph();
    return ensure_slots();
}

// The slot arrays (3 NT + 4 NH + 4 cap_c corners), the vertex lists' offsets and counts (NP + 2) and the scan
// scratch, for the current sizes.
int Stage3::ensure_slots() {
    int rr;
    size_t c;
    const size_t ns = (size_t)3 * NT + (size_t)4 * NH + (size_t)4 * cap_c;
    if (cap_slot < ns || !gslot) {
        for (float4** b : {&gslot, &hslot, &aslot}) {
            dfree(*b);
            *b = nullptr;
            c = 0;
            if ((rr = grow(*b, c, ns))) return rr;
        }
        cap_slot = ns;
    }
    const size_t nv = (size_t)NP + 2;
    if (cap_vso < nv || !vs_off) {
        for (int** b : {&vs_off, &c_cnt, &c_off, &c_cur}) {
            dfree(*b);
            *b = nullptr;
            c = 0;
            if ((rr = grow(*b, c, nv))) return rr;
        }
        cap_vso = nv;
    }
    const size_t nq = (size_t)NP + NE + 2;
    if (cap_cq < nq || !cand_cnt) {
        c = cap_cq;
        if ((rr = grow(cand_cnt, c, nq))) return rr;
        c = cap_cq;
        if ((rr = grow(cand_off, c, nq))) return rr;
        cap_cq = nq;
    }
    const size_t nl = (size_t)3 * NT + (size_t)4 * NH + 1;
    if (cap_vs < nl || !inv_vs) {
        c = cap_vs;
        if ((rr = grow(inv_vs, c, nl))) return rr;
        cap_vs = nl;
    }
    if (!scan_scratch) {
        c = 0;
        if ((rr = grow(scan_scratch, c, 2 * scan_scratch_ints()))) return rr;
        // both scratches start zeroed (a scan's tile counters live there), in stream order
        cudaMemsetAsync(scan_scratch, 0, 2 * scan_scratch_ints() * sizeof(int), stream);
    }
    return PAMO_OK;
}

int Stage3::ensure_candidates(size_t npt, size_t nee) {
    size_t c;
    int rr;
    if (cap_cpt < npt || !cand_pt) {
        c = cand_pt ? cap_cpt : 0;
        if ((rr = grow(cand_pt, c, npt))) return rr;
        cap_cpt = c;
    }
    if (cap_cee < nee || !cand_ee) {
        c = cand_ee ? cap_cee : 0;
        if ((rr = grow(cand_ee, c, nee))) return rr;
        cap_cee = c;
    }
    const size_t nf = cap_cpt + cap_cee + 1;
    if (cap_cf < nf || !cflag) {
        dfree(cflag); dfree(cpos); dfree(cid); dfree(cty);
        cflag = cpos = nullptr;
        cid = nullptr;
        cty = nullptr;
        c = 0;
        if ((rr = grow(cflag, c, nf))) return rr;
        c = 0;
        if ((rr = grow(cpos, c, nf))) return rr;
        c = 0;
        if ((rr = grow(cid, c, nf))) return rr;
        c = 0;
        if ((rr = grow(cty, c, nf))) return rr;
        cap_cf = nf;
    }
    return PAMO_OK;
}

EnergyArgs Stage3::energy_args() const {
    const Stage3Params& P = params;
    EnergyArgs A;
    A.tgt = target; A.w = vweight; A.m2gt_k = P.mesh2gt_dist_stiffness; A.np = NP;
    A.tri = tri; A.area = el_area; A.invDm = el_invDm;
    A.mu = P.elas_young_modulus / (2.f * (1.f + P.elas_poisson_ratio));
    A.la = P.elas_young_modulus * P.elas_poisson_ratio / ((1.f + P.elas_poisson_ratio) * (1.f - 2.f * P.elas_poisson_ratio));
    A.nt = NT; A.hinge = hinge; A.rest = hinge_rest; A.hinge_k = P.hinge_stiffness; A.nh = NH;
    A.cidx = c_idx; A.ctype = c_type; A.cd = c_d; A.kappa = P.coll_stiffness; A.d_hat = P.d_hat;
    A.ee_thres = P.ee_classify_thres;
    return A;
}

int Stage3::energy_grid() const {
    const long long total = (long long)NP + NT + NH + (long long)cap_c;
    return (int)std::min<long long>(kRedBlocks, (total + kT - 1) / kT);
}

void Stage3::launch_energy(const float4* x, int ls_n) {
    k_energy<<<energy_grid(), kT, 0, stream>>>(x, energy_args(), sc, partial, ls_n);
    note_launch();
}

void Stage3::newton_iteration() {
    cudaStream_t s = stream;
    const Stage3Params& P = params;
    const float mu = P.elas_young_modulus / (2.f * (1.f + P.elas_poisson_ratio));
    const float la = P.elas_young_modulus * P.elas_poisson_ratio / ((1.f + P.elas_poisson_ratio) * (1.f - 2.f * P.elas_poisson_ratio));
    const int gC = grid_for((long long)cap_c, kT);
    // q_prev_newton = q; contacts at q (system.py:425-432, _detect_contact :308-318 with refitted LBVHs)
    k_iter_begin<<<grid_for(NP + 1, kT), kT, 0, s>>>(q, q_prev_newton, c_cnt, c_cur, NP, sc);
    note_launch();
    const float skin = 2.0f * P.contact_detection_radius + P.d_hat;
    k_disp_check<<<grid_for(NP, kT), kT, 0, s>>>(q, q_ref, NP, 0.5f * skin, sc);
    note_launch();
    bvh_refit(tri_bvh, tri, q, tri_rc, NT, s, &sc->rebuild);
    bvh_refit(edge_bvh, edge4, q, edge_rc, NE, s, &sc->rebuild);
    // candidate lists in a fixed order: per-query counts, their prefix sums (the totals are the list lengths),
    // then each query's pairs at its offset (both passes only when the lists are rebuilt; the sums of unchanged
    // counts give the same offsets)
    int* cnt_pt = cand_cnt;
    int* cnt_ee = cand_cnt + NP;
    int* off_pt = cand_off;
    int* off_ee = cand_off + NP;
    k_candidates<false><<<grid_for(NP, kQT, 16), kQT, 0, s>>>(q, NP, tri, tri_bvh.child, tri_bvh.nlo, tri_bvh.nhi,
                                                             tri_bvh.llo, tri_bvh.lhi, tri_bvh.vals[0], tri_rc, P.d_hat,
                                                             skin, cand_pt, (int)cap_cpt, cnt_pt, nullptr, sc);
    note_launch();
    k_candidates<true><<<grid_for(NE, kQT, 16), kQT, 0, s>>>(q, NE, edge4, edge_bvh.child, edge_bvh.nlo, edge_bvh.nhi,
                                                            edge_bvh.llo, edge_bvh.lhi, edge_bvh.vals[0], edge_rc,
                                                            P.d_hat, skin, cand_ee, (int)cap_cee, cnt_ee, nullptr, sc);
    note_launch();
    {
        const size_t si = scan_scratch_ints();
        ScanJob jobs[2] = {{cnt_pt, off_pt, nullptr, NP, &sc->n_cand_pt, scan_scratch},
                           {cnt_ee, off_ee, nullptr, NE, &sc->n_cand_ee, scan_scratch + si}};
        exclusive_scans(jobs, 2, s, &sc->status, std::max(NP, NE));
        note_launch();
    }
    k_candidates<false><<<grid_for(NP, kQT, 16), kQT, 0, s>>>(q, NP, tri, tri_bvh.child, tri_bvh.nlo, tri_bvh.nhi,
                                                             tri_bvh.llo, tri_bvh.lhi, tri_bvh.vals[0], tri_rc, P.d_hat,
                                                             skin, cand_pt, (int)cap_cpt, cnt_pt, off_pt, sc);
    note_launch();
    k_candidates<true><<<grid_for(NE, kQT, 16), kQT, 0, s>>>(q, NE, edge4, edge_bvh.child, edge_bvh.nlo, edge_bvh.nhi,
                                                            edge_bvh.llo, edge_bvh.lhi, edge_bvh.vals[0], edge_rc,
                                                            P.d_hat, skin, cand_ee, (int)cap_cee, cnt_ee, off_ee, sc);
    note_launch();
    k_cand_done<<<grid_for(NP, kT), kT, 0, s>>>(q, q_ref, NP, (int)cap_cpt, (int)cap_cee, sc);
    note_launch();
    // contacts in candidate order: flags, their prefix sums (the total is the contact count), the list, then each
    // vertex's contact corners (counted, offsets, filled, sorted)
    const int cap = (int)std::min<size_t>(cap_c, (size_t)P.max_blocks);
    k_filter<<<grid_for((long long)(cap_cpt + cap_cee), kT), kT, 0, s>>>(q, cand_pt, cand_ee, tri, edge4, P.d_hat,
                                                                        P.ee_classify_thres, cflag, cid, cty, sc);
    note_launch();
    exclusive_scan(cflag, cpos, &sc->n_cand_all, 0, &sc->n_contacts_raw, scan_scratch, s, &sc->status,
                   (long long)(cap_cpt + cap_cee));
    note_launch();
    k_contacts_done<<<1, 1, 0, s>>>(sc, cap, P.max_blocks);
    note_launch();
    k_contacts_scatter<<<grid_for((long long)(cap_cpt + cap_cee), kT), kT, 0, s>>>(cflag, cpos, cid, cty, c_idx, c_type,
                                                                                  c_cnt, sc);
    note_launch();
    exclusive_scan(c_cnt, c_off, nullptr, NP + 1, nullptr, scan_scratch, s, &sc->status, NP + 1);
    note_launch();
    k_cvert_fill<<<grid_for(4ll * cap_c, kT), kT, 0, s>>>(c_idx, c_off, c_cur, c_tmp, sc);
    note_launch();
    k_cvert_rank<<<grid_for(32ll * NP, kT), kT, 0, s>>>(c_off, c_tmp, c_inv, NP, sc);
    note_launch();
    // energy, gradient (coeff -1), Hessian diagonal and hinge blocks (system.py:433-434): per-corner parts into
    // the slot arrays, then summed per vertex
    launch_energy(q);
    const size_t nt3 = (size_t)3 * NT, cbase = nt3 + (size_t)4 * NH;
    k_diff_elastic<<<grid_for(NT, kT), kT, 0, s>>>(q, tri, el_area, el_invDm, mu, la, -1.f, NT, gslot, inv_vs, sc);
    note_launch();
    if (NH) {
        k_diff_hinge<<<grid_for(NH, 128), 128, 0, s>>>(q, hinge, hinge_rest, P.hinge_stiffness, -1.f, NH, hinge_blocks,
                                                       gslot, hslot, inv_vs + nt3, sc);
        note_launch();
        k_spd_project<<<grid_for((NH + 3 * kSpdWarps - 1) / (3 * kSpdWarps), 1, 16), 32 * kSpdWarps, 0, s>>>(
            hinge_blocks, NH, P.spd_max_iters, sc);
        note_launch();
    }
    k_diff_contact<<<gC, kT, 0, s>>>(q, c_idx, c_type, c_d, sc, P.coll_stiffness, P.d_hat, -1.f, c_dd, gslot + cbase,
                                     hslot + cbase, c_inv);
    note_launch();
    VertexSlots S;
    S.vs_off = vs_off; S.coff = c_off; S.inv_vs = inv_vs; S.cinv = c_inv; S.cbase = (int)cbase;
    k_gather_grad<<<grid_for((long long)kGather * NP, kT), kT, 0, s>>>(q, target, vweight, P.mesh2gt_dist_stiffness,
                                                                      -1.f, NP, gslot, hslot, S, grad, hdiag, sc);
    note_launch();
    // Jacobi PCG (cg_solver.py:96-158)
    HvpArgs H;
    H.w = vweight; H.m2gt_k = P.mesh2gt_dist_stiffness; H.np = NP;
    H.tri = tri; H.area = el_area; H.invDm = el_invDm; H.mu = mu; H.la = la; H.nt = NT;
    H.hinge = hinge; H.blocks = hinge_blocks; H.nh = NH;
    H.cidx = c_idx; H.cd = c_d; H.cdd = c_dd; H.kappa = P.coll_stiffness; H.d_hat = P.d_hat;
    H.aslot = aslot; H.S = S;
    const long long elems_all = (long long)NP + NT + NH;
    // the cluster kernel measured slower than the grid-wide one on the 5k-face stage-2 output (fewer threads
    // per element pass), so it runs only when asked for
    const bool use_cluster = cluster_size > 1 && cg_mode == 2 && elems_all > 0;
    if (use_cluster) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cluster_size);
        cfg.blockDim = dim3(kClusterThreads);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cluster_size;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, k_cg_cluster, (const float4*)q, H, (const float4*)grad, (const float4*)hdiag, p, r, z,
                           v[0], v[1], P.n_cg_iters, sc);
        note_launch();
    } else if (cg_mode == 7) {
        // two ordinary launches per iteration (k_cg_solve's grid, 128 threads)
        const long long elems = (long long)NP + NT + NH;
        const int g = (int)std::max<long long>(1, std::min<long long>({(elems + 127) / 128, (long long)n_sm,
                                                                       (long long)kPartials / 2}));
        k_cg_start<128><<<g, 128, 0, s>>>(grad, hdiag, NP, p, r, z, v[0], sc, partial);
        note_launch();
        for (int it = 0; it < P.n_cg_iters; ++it) {
            float4* vin = (it & 1) ? v[1] : v[0];
            float4* vout = (it & 1) ? v[0] : v[1];
            k_cg_product<128><<<g, 128, 0, s>>>(q, H, z, vin, vout, it, sc, partial);
            note_launch();
            k_cg_update<128><<<g, 128, 0, s>>>(H, vout, hdiag, p, r, z, sc, partial);
            note_launch();
        }
    } else {
        // one cooperative launch: about one thread per element, at most one block per SM (cg_mode 0, 3, 4); or
        // at least one block per SM (5: 128 threads, 6: 64 threads, two blocks per SM)
        const int bt = cg_mode == 3 ? 256 : cg_mode == 4 ? 512 : cg_mode == 6 ? 64 : 128;
        const long long elems = (long long)NP + NT + NH;
        int g = (int)std::min<long long>((elems + bt - 1) / bt, (long long)n_sm);
        if (cg_mode == 5) g = (int)std::max<long long>((elems + bt - 1) / bt, (long long)n_sm);
        if (cg_mode == 6) g = (int)std::max<long long>((elems + bt - 1) / bt, 2ll * n_sm);
        g = std::max(1, std::min(g, std::min(coop_max_blocks, kPartials / 2)));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(g);
        cfg.blockDim = dim3(bt);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        CgState* bar = reinterpret_cast<CgState*>(cg_bar);
        if (bt == 64)
            cudaLaunchKernelEx(&cfg, k_cg_solve<64>, (const float4*)q, H, (const float4*)grad, (const float4*)hdiag, p, r,
                               z, v[0], v[1], P.n_cg_iters, sc, partial, bar);
        else if (bt == 512)
            cudaLaunchKernelEx(&cfg, k_cg_solve<512>, (const float4*)q, H, (const float4*)grad, (const float4*)hdiag, p, r,
                               z, v[0], v[1], P.n_cg_iters, sc, partial, bar);
        else if (bt == 256)
            cudaLaunchKernelEx(&cfg, k_cg_solve<256>, (const float4*)q, H, (const float4*)grad, (const float4*)hdiag, p, r,
                               z, v[0], v[1], P.n_cg_iters, sc, partial, bar);
        else
            cudaLaunchKernelEx(&cfg, k_cg_solve<128>, (const float4*)q, H, (const float4*)grad, (const float4*)hdiag, p, r,
                               z, v[0], v[1], P.n_cg_iters, sc, partial, bar);
        note_launch();
    }
    // step clamp, CCD, line search (system.py:441-459)
    k_clamp_p<<<grid_for(NP, kT), kT, 0, s>>>(p, q_prev_newton, P.contact_detection_radius, NP, sc);
    note_launch();
    k_before_ccd<<<1, 1, 0, s>>>(sc);
    note_launch();
    if (P.ccd_fp64 == 2)
        k_accd_wide<WF><<<gC, kT, 0, s>>>(q, p, c_idx, c_type, sc, P.ccd_slackness, P.ccd_thickness, P.ccd_max_iters,
                                          P.ee_classify_thres);
    else if (P.ccd_fp64)
        k_accd_wide<double><<<gC, kT, 0, s>>>(q, p, c_idx, c_type, sc, P.ccd_slackness, P.ccd_thickness,
                                              P.ccd_max_iters, P.ee_classify_thres);
    else
        k_accd<<<gC, kT, 0, s>>>(q, p, c_idx, c_type, sc, P.ccd_slackness, P.ccd_thickness, P.ccd_max_iters,
                                P.ee_classify_thres);
    note_launch();
    const int g_ls = energy_grid();
    if (ls_mode == 1 && P.n_line_search_iters > 0 && g_ls <= ls_coop_max_blocks && 2 * g_ls <= kPartials) {
        // the whole search in one cooperative launch on the energy's grid (co-residency checked at set-up)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(g_ls);
        cfg.blockDim = dim3(kT);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        CgState* ls_bar = reinterpret_cast<CgState*>(static_cast<char*>(cg_bar) + 32);
        cudaLaunchKernelEx(&cfg, k_line_search_coop, (const float4*)q_prev_newton, (const float4*)p, q, energy_args(),
                           P.n_line_search_iters, sc, partial, ls_bar);
        note_launch();
    } else {
        for (int n = 0; n < P.n_line_search_iters; ++n) {
            k_line_search<<<grid_for(NP, kT), kT, 0, s>>>(q_prev_newton, p, sc, n, NP, q);
            note_launch();
            launch_energy(q, n);
        }
    }
    k_iter_end<<<1, 1, 0, s>>>(sc);
    note_launch();
}

// Topology of one call, on the host.
// Edges: trimesh's edges_unique (the face edges with sorted endpoints, unique rows). For two int32 columns
// trimesh hashes a row (u, v) as u ^ (v << 32) and np.unique sorts the hashes, so the edges come ordered by
// (v, u); the same order is used here (it fixes which edge of an edge-edge pair is "first"). ukeys holds
// v * n_points + u per edge, ascending.
// Hinges: hinge_preprocess_slow_kernel (hinge_energy.py:21-57) pairs every directed edge (a, b), a < b, of a face
// t0 with every face t1 holding the edge as (b, a): hinge (opposite in t0, a, b, opposite in t1), in the order of
// t0's faces and corners, then of t1's faces and corners. Returns PAMO_ERR_INVALID_ARG for an index outside
// [0, n_points).
int stage3_topology(const int* hf, int n_points, int n_tris, std::vector<long long>& ukeys, std::vector<int4>& h4) {
    std::vector<std::pair<long long, int>> dkeys;  // directed edge (a * n + b) -> face * 3 + corner
    ukeys.clear();
    h4.clear();
    ukeys.reserve((size_t)3 * n_tris);
    dkeys.reserve((size_t)3 * n_tris);
    for (int f = 0; f < n_tris; ++f)
        for (int k = 0; k < 3; ++k) {
            const long long a = hf[3 * f + k], b = hf[3 * f + (k + 1) % 3];
            if (a < 0 || b < 0 || a >= n_points || b >= n_points) return PAMO_ERR_INVALID_ARG;
            ukeys.push_back(std::max(a, b) * n_points + std::min(a, b));
            dkeys.push_back({a * n_points + b, 3 * f + k});
        }
    std::sort(ukeys.begin(), ukeys.end());
    ukeys.erase(std::unique(ukeys.begin(), ukeys.end()), ukeys.end());
    std::sort(dkeys.begin(), dkeys.end());
    for (int f = 0; f < n_tris; ++f)
        for (int k = 0; k < 3; ++k) {
            const int a = hf[3 * f + k], b = hf[3 * f + (k + 1) % 3], c = hf[3 * f + (k + 2) % 3];
            if (!(a < b)) continue;
            const long long key = (long long)b * n_points + a;
            auto it = std::lower_bound(dkeys.begin(), dkeys.end(), std::make_pair(key, -1));
            for (; it != dkeys.end() && it->first == key; ++it) {
                const int f1 = it->second / 3, k1 = it->second % 3;
                h4.push_back(make_int4(c, a, b, hf[3 * f1 + (k1 + 2) % 3]));
            }
        }
    return PAMO_OK;
}

int Stage3::run(const double* gt_points, const int* gt_tris, int n_gt_points, int n_gt_tris, const double* points,
                const int* tris, int n_points, int n_tris, int n_iters, double* out_points, cudaStream_t caller) {
    int r = run_once(gt_points, gt_tris, n_gt_points, n_gt_tris, points, tris, n_points, n_tris, n_iters, out_points,
                     caller);
    if (r != PAMO_ERR_ITER_LIMIT || !barrier_gave_up) return r;
    const int cg = cg_mode, ls = ls_mode;
    cg_mode = 7;
    ls_mode = 0;
    r = run_once(gt_points, gt_tris, n_gt_points, n_gt_tris, points, tris, n_points, n_tris, n_iters, out_points, caller);
    cg_mode = cg;
    ls_mode = ls;
    stats.barrier_reruns = 1;
    return r;
}

int Stage3::run_once(const double* gt_points, const int* gt_tris, int n_gt_points, int n_gt_tris,
                     const double* points, const int* tris, int n_points, int n_tris, int n_iters, double* out_points,
                     cudaStream_t caller) {
    err.clear();
    stats = Stage3Stats{};
    barrier_gave_up = false;
    if (n_points < 3 || n_tris < 1 || n_gt_points < 3 || n_gt_tris < 1) return fail(PAMO_ERR_INVALID_ARG, "empty mesh");
    // topology on the host, once per call (stage3_topology)
    std::vector<int> hf((size_t)3 * n_tris);
    // on the caller's stream, after the work that produced the triangles there (a non-blocking stream does not
    // order with a copy on the legacy default stream)
    if (cudaMemcpyAsync(hf.data(), tris, hf.size() * sizeof(int), cudaMemcpyDeviceToHost, caller) != cudaSuccess ||
        cudaStreamSynchronize(caller) != cudaSuccess)
        return fail(PAMO_ERR_CUDA, "copy of the triangles");
    std::vector<long long> ukeys;
    std::vector<int4> h4;
    if (stage3_topology(hf.data(), n_points, n_tris, ukeys, h4)) return fail(PAMO_ERR_INVALID_ARG, "bad triangle index");
    NP = n_points;
    NT = n_tris;
    NE = (int)ukeys.size();
    NH = (int)h4.size();
    NGP = n_gt_points;
    NGT = n_gt_tris;
    stats.n_particles = NP;
    stats.n_triangles = NT;
    stats.n_edges = NE;
    stats.n_hinges = NH;
    int rr;
    drop_graph();  // kernel arguments of a captured iteration (sizes, coefficients) belong to one call
    if ((rr = ensure(NP, NT, NE, NH, NGP, NGT))) return rr;
    if ((rr = ensure_contacts(std::max<size_t>(std::max<size_t>(1 << 16, cap_c), (size_t)32 * (NP + NE))))) return rr;
    if ((rr = ensure_candidates(std::max<size_t>(1 << 16, (size_t)64 * NP), std::max<size_t>(1 << 16, (size_t)64 * NE))))
        return rr;
    if ((rr = ensure_slots())) return rr;
    {
        // the static parts' positions: each vertex's triangle corners (codes 3f + c) then hinge slots (3 NT + 4h + a)
        // contiguous at [off[v], off[v + 1]) in ascending code order; list[code] = its position
        std::vector<int> off((size_t)NP + 1, 0), list((size_t)3 * NT + (size_t)4 * NH);
        for (int k = 0; k < 3 * NT; ++k) off[hf[k] + 1]++;
        for (int h = 0; h < NH; ++h) {
            off[h4[h].x + 1]++; off[h4[h].y + 1]++; off[h4[h].z + 1]++; off[h4[h].w + 1]++;
        }
        for (int i = 0; i < NP; ++i) off[i + 1] += off[i];
        std::vector<int> cur(off.begin(), off.end() - 1);
        for (int k = 0; k < 3 * NT; ++k) list[k] = cur[hf[k]]++;  // codes visited ascending: each range sorted
        for (int h = 0; h < NH; ++h) {
            const int ids[4] = {h4[h].x, h4[h].y, h4[h].z, h4[h].w};
            for (int a = 0; a < 4; ++a) list[3 * NT + 4 * h + a] = cur[ids[a]]++;
        }
        vs_host_off.swap(off);
        vs_host_list.swap(list);
    }
    cudaStream_t s = stream;
    cudaMemsetAsync(cg_bar, 0, 64, s);  // the barrier counters of the PCG and of the line search
    cudaEventRecord(ev_in, caller);
    cudaStreamWaitEvent(s, ev_in, 0);
    std::vector<int4> e4(NE);
    for (int e = 0; e < NE; ++e) {
        const int u = (int)(ukeys[e] % n_points), w = (int)(ukeys[e] / n_points);
        e4[e] = make_int4(u, w, w, 0);
    }
    cudaMemcpyAsync(edge4, e4.data(), NE * sizeof(int4), cudaMemcpyHostToDevice, s);
    if (NH) cudaMemcpyAsync(hinge, h4.data(), NH * sizeof(int4), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(vs_off, vs_host_off.data(), vs_host_off.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    if (!vs_host_list.empty())
        cudaMemcpyAsync(inv_vs, vs_host_list.data(), vs_host_list.size() * sizeof(int), cudaMemcpyHostToDevice, s);

    // normalisation (processing.py:15-21, 57-59)
    k_norm_partial<<<kNormBlocks, kT, 0, s>>>(gt_points, NGP, d_norm + 16);
    note_launch();
    k_norm_final<<<1, kT, 0, s>>>(d_norm + 16, kNormBlocks, NGP, d_norm);
    note_launch();
    k_normalize<<<grid_for(NGP, kT), kT, 0, s>>>(gt_points, NGP, d_norm, gt_pos, nullptr);
    note_launch();
    std::memset(h_sc, 0, sizeof(SolverScalars));
    h_sc->radius = params.contact_detection_radius;
    h_sc->rebuild = 1;  // candidate lists are built in the first iteration
    h_sc->barrier_extra = test_barrier_extra;
    cudaMemcpyAsync(sc, h_sc, sizeof(SolverScalars), cudaMemcpyHostToDevice, s);
    k_tris4<<<grid_for(NGT, kT), kT, 0, s>>>(gt_tris, NGT, NGP, gt_tri, &sc->status);
    note_launch();
    k_normalize<<<grid_for(NP, kT), kT, 0, s>>>(points, NP, d_norm, q, q_rest);
    note_launch();
    k_tris4<<<grid_for(NT, kT), kT, 0, s>>>(tris, NT, NP, tri, &sc->status);
    note_launch();
    cudaMemcpyAsync(h_sc, sc, sizeof(SolverScalars), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return fail(PAMO_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    if (h_sc->status & 1) return fail(PAMO_ERR_INVALID_ARG, "GT triangle index out of range");
    // LBVHs: the GT mesh (static) and the simulated triangles and edges (refitted at every detection)
    {
        RoundCounters h{};
        h.n_pts = NGP;
        h.n_tris = NGT;
        cudaMemcpyAsync(gt_rc, &h, sizeof(h), cudaMemcpyHostToDevice, s);
        bvh_build(gt_bvh, gt_tri, gt_pos, gt_rc, NGT, s);
        h.n_pts = NP;
        h.n_tris = NT;
        cudaMemcpyAsync(tri_rc, &h, sizeof(h), cudaMemcpyHostToDevice, s);
        bvh_build(tri_bvh, tri, q, tri_rc, NT, s);
        h.n_tris = NE;
        cudaMemcpyAsync(edge_rc, &h, sizeof(h), cudaMemcpyHostToDevice, s);
        bvh_build(edge_bvh, edge4, q, edge_rc, NE, s);
    }
    // register_mesh preprocessing (system.py:167-272): Voronoi areas, elastic rest shape, hinge rest state,
    // minimum internal angle
    // scratch: 3 NT + 4 NH doubles in gslot, free until the first gradient
    double* wslot = reinterpret_cast<double*>(gslot);
    cudaMemsetAsync(wslot, 0, ((size_t)3 * NT + (size_t)4 * NH) * sizeof(double), s);
    // the triangle positions of hslot hold no Hessian part: zero for the whole call
    cudaMemsetAsync(hslot, 0, ((size_t)3 * NT + (size_t)4 * NH) * sizeof(float4), s);
    k_voronoi<<<grid_for(NT, kT), kT, 0, s>>>(points, d_norm, tri, NT, inv_vs, wslot);
    note_launch();
    k_weights_f32<<<grid_for(NP, kT), kT, 0, s>>>(wslot, vs_off, NP, vweight);
    note_launch();
    k_elastic_pre<<<grid_for(NT, kT), kT, 0, s>>>(q_rest, tri, NT, el_area, el_invDm);
    note_launch();
    if (NH) {
        k_hinge_pre<<<grid_for(NH, kT), kT, 0, s>>>(q_rest, hinge, NH, hinge_rest);
        note_launch();
    }
    k_min_angle<<<grid_for(NT, kT), kT, 0, s>>>(points, d_norm, tri, NT, (double)params.min_angle_thres, &sc->accepted);
    note_launch();
    cudaMemcpyAsync(h_sc, sc, sizeof(SolverScalars), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return fail(PAMO_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    stats.do_nothing = (h_sc->accepted == 1);  // some angle <= threshold and none NaN (system.py:214-221)

    if (!stats.do_nothing && n_iters > 0) {
        const int per_step = params.n_newton_iters;
        auto capture = [&]() -> int {
            drop_graph();
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                return fail(PAMO_ERR_CUDA, "stream capture");
            const long long l0 = launches_so_far();
            newton_iteration();
            graph_kernels = launches_so_far() - l0;
            note_launches(-graph_kernels);  // counted when the graph runs
            if (cudaStreamEndCapture(s, &g) != cudaSuccess || !g) return fail(PAMO_ERR_CUDA, "stream capture");
            const cudaError_t e = cudaGraphInstantiate(&graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                graph = nullptr;
                return fail(PAMO_ERR_CUDA, "graph instantiation");
            }
            return PAMO_OK;
        };
        int done = 0;
        for (int step = 0; step < n_iters; ++step) {
            ++stats.steps;
            // _update_vertex_target: closest points on the GT surface
            k_closest_gt<<<grid_for(NP, kQT, 16), kQT, 0, s>>>(q, NP, gt_bvh.child, gt_bvh.nlo, gt_bvh.nhi, gt_bvh.llo,
                                                              gt_bvh.lhi, gt_bvh.vals[0], gt_tri, gt_pos, gt_rc, target,
                                                              &sc->status);
            note_launch();
            const int goal = (step + 1) * per_step;
            for (int guard = 0;; ++guard) {
                if (guard > 64) return fail(PAMO_ERR_CAPACITY, "contact list did not settle");
                for (int k = done; k < goal; ++k) {
                    if (use_graph) {
                        if (!graph && (rr = capture())) return rr;
                        if (cudaGraphLaunch(graph, s) != cudaSuccess) return fail(PAMO_ERR_CUDA, "graph launch");
                        note_launches(graph_kernels);
                    } else {
                        newton_iteration();
                    }
                }
                cudaMemcpyAsync(h_sc, sc, sizeof(SolverScalars), cudaMemcpyDeviceToHost, s);
                if (cudaStreamSynchronize(s) != cudaSuccess)
                    return fail(PAMO_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
                done = h_sc->iters_done;
                // a grid barrier that gave up leaves this run's values undefined: stop here
                if (h_sc->status & kErrIterLimit) {
                    barrier_gave_up = true;
                    return fail(PAMO_ERR_ITER_LIMIT, "grid barrier of the PCG timed out");
                }
                if (h_sc->abort == 0) break;
                if (h_sc->abort == 2) {
                    // too many contacts: halve the detection radius and detect again (energy.py:942-948)
                    if (++stats.radius_halvings > 40) return fail(PAMO_ERR_CAPACITY, "contacts exceed max_blocks");
                    const float rad = h_sc->radius * 0.5f;
                    cudaMemcpyAsync(&sc->radius, &rad, sizeof(float), cudaMemcpyHostToDevice, s);
                } else if (h_sc->abort == 3) {
                    const size_t a = (size_t)h_sc->n_cand_pt, b = (size_t)h_sc->n_cand_ee;
                    if ((rr = ensure_candidates(a + a / 2 + 1024, b + b / 2 + 1024))) return rr;
                } else {
                    const size_t raw = (size_t)h_sc->n_contacts_raw;
                    if ((rr = ensure_contacts(raw + raw / 2 + 1024))) return rr;
                }
                cudaMemsetAsync(&sc->abort, 0, sizeof(int), s);
            }
        }
        stats.newton_iters = done;
    }
    k_denormalize<<<grid_for(NP, kT), kT, 0, s>>>(q, NP, d_norm, out_points);
    note_launch();
    cudaMemcpyAsync(h_sc, sc, sizeof(SolverScalars), cudaMemcpyDeviceToHost, s);
    cudaEventRecord(ev_out, s);
    cudaStreamWaitEvent(caller, ev_out, 0);
    if (cudaStreamSynchronize(s) != cudaSuccess) return fail(PAMO_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    if (h_sc->status & kErrIterLimit) {
        barrier_gave_up = true;
        return fail(PAMO_ERR_ITER_LIMIT, "grid barrier of the PCG timed out");
    }
    if (h_sc->status & 6) return fail(PAMO_ERR_ITER_LIMIT, "BVH traversal limit in stage 3");
    stats.last_energy = h_sc->energy;
    stats.max_contacts = h_sc->max_contacts;
    stats.total_contacts = h_sc->total_contacts;
    stats.candidate_rebuilds = h_sc->n_rebuilds;
    return PAMO_OK;
}

}  // namespace pamo

// ================================================================== C ABI
struct pamo_stage3 {
    int device = 0;
    pamo::Stage3 solver;
};

extern "C" {

int pamo_stage3_create(pamo_stage3** out, int device) {
    if (!out) return PAMO_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return PAMO_ERR_INVALID_ARG;
    pamo_stage3* s = new pamo_stage3();
    s->device = device;
    *out = s;
    return PAMO_OK;
}

int pamo_stage3_destroy(pamo_stage3* s) {
    if (!s) return PAMO_ERR_INVALID_ARG;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    delete s;
    cudaSetDevice(prev);
    return PAMO_OK;
}

const char* pamo_stage3_last_error(const pamo_stage3* s) { return s ? s->solver.err.c_str() : "null handle"; }

int pamo_stage3_set_param(pamo_stage3* s, const char* name, double value) {
    if (!s || !name) return PAMO_ERR_INVALID_ARG;
    pamo::Stage3Params& P = s->solver.params;
    const std::string n(name);
    if (n == "n_newton_iters") P.n_newton_iters = (int)value;
    else if (n == "n_cg_iters") P.n_cg_iters = (int)value;
    else if (n == "n_line_search_iters") P.n_line_search_iters = (int)value;
    else if (n == "d_hat") P.d_hat = (float)value;
    else if (n == "coll_stiffness") P.coll_stiffness = (float)value;
    else if (n == "contact_detection_radius") P.contact_detection_radius = (float)value;
    else if (n == "ee_classify_thres") P.ee_classify_thres = (float)value;
    else if (n == "ccd_slackness") P.ccd_slackness = (float)value;
    else if (n == "ccd_thickness") P.ccd_thickness = (float)value;
    else if (n == "ccd_max_iters") P.ccd_max_iters = (int)value;
    else if (n == "spd_max_iters") P.spd_max_iters = (int)value;
    else if (n == "elas_young_modulus") P.elas_young_modulus = (float)value;
    else if (n == "elas_poisson_ratio") P.elas_poisson_ratio = (float)value;
    else if (n == "hinge_stiffness") P.hinge_stiffness = (float)value;
    else if (n == "mesh2gt_dist_stiffness") P.mesh2gt_dist_stiffness = (float)value;
    else if (n == "min_angle_thres") P.min_angle_thres = (float)value;
    else if (n == "max_blocks") P.max_blocks = (long long)value;
    else if (n == "use_cuda_graph") s->solver.use_graph = value != 0.0;
    else if (n == "test_barrier_extra") s->solver.test_barrier_extra = (int)value;  // tests: grid barriers run out
    else if (n == "ccd_fp64") {  // 0 float32 (Warp's kernels), 1 float64, 2 double-float (default)
        if (value != 0.0 && value != 1.0 && value != 2.0) {
            s->solver.err = "ccd_fp64 is 0, 1 or 2";
            return PAMO_ERR_INVALID_ARG;
        }
        P.ccd_fp64 = (int)value;
    }
    else if (n == "ls_mode") s->solver.ls_mode = (int)value;  // 1 cooperative line search, 0 launches per trial
    else if (n == "cg_mode") s->solver.cg_mode = (int)value;  // 0/1 grid-cooperative (128), 2 cluster, 3 (256), 4 (512), 5 (128, >= 1 block per SM), 6 (64, >= 2 blocks per SM), 7 two ordinary launches per iteration
    else {
        s->solver.err = "unknown stage-3 parameter: " + n;
        return PAMO_ERR_INVALID_ARG;
    }
    return PAMO_OK;
}

int pamo_safe_project(pamo_stage3* s, const double* gt_points, const int32_t* gt_triangles, int32_t n_gt_points,
                      int32_t n_gt_triangles, const double* points, const int32_t* triangles, int32_t n_points,
                      int32_t n_triangles, int32_t n_iters, double* out_points, pamo_stream stream) {
    if (!s) return PAMO_ERR_INVALID_ARG;
    if (!gt_points || !gt_triangles || !points || !triangles || !out_points || n_iters < 0) {
        s->solver.err = "null pointer or negative n_iters";
        return PAMO_ERR_INVALID_ARG;
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    const int r = s->solver.run(gt_points, gt_triangles, n_gt_points, n_gt_triangles, points, triangles, n_points,
                                n_triangles, n_iters, out_points, (cudaStream_t)stream);
    cudaSetDevice(prev);
    return r;
}

int pamo_stage3_topology(const int32_t* triangles, int32_t n_points, int32_t n_triangles, int32_t* edges,
                         int32_t* n_edges, int32_t* hinges, int32_t hinge_capacity, int32_t* n_hinges) {
    if (!triangles || n_points < 1 || n_triangles < 1 || !edges || !n_edges || !n_hinges || hinge_capacity < 0 ||
        (hinge_capacity > 0 && !hinges))
        return PAMO_ERR_INVALID_ARG;
    std::vector<long long> ukeys;
    std::vector<int4> h4;
    const int r = pamo::stage3_topology(triangles, n_points, n_triangles, ukeys, h4);
    if (r) return r;
    for (size_t e = 0; e < ukeys.size(); ++e) {
        edges[2 * e] = (int32_t)(ukeys[e] % n_points);
        edges[2 * e + 1] = (int32_t)(ukeys[e] / n_points);
    }
    *n_edges = (int32_t)ukeys.size();
    *n_hinges = (int32_t)h4.size();
    if ((int64_t)h4.size() > hinge_capacity) return PAMO_ERR_CAPACITY;
    for (size_t h = 0; h < h4.size(); ++h) {
        hinges[4 * h] = h4[h].x;
        hinges[4 * h + 1] = h4[h].y;
        hinges[4 * h + 2] = h4[h].z;
        hinges[4 * h + 3] = h4[h].w;
    }
    return PAMO_OK;
}

int pamo_stage3_stats(const pamo_stage3* s, double* out, int32_t n) {
    if (!s || !out) return PAMO_ERR_INVALID_ARG;
    const pamo::Stage3Stats& t = s->solver.stats;
    const double v[13] = {(double)t.n_particles, (double)t.n_triangles, (double)t.n_edges, (double)t.n_hinges,
                          (double)t.steps, (double)t.newton_iters, (double)t.max_contacts, (double)t.radius_halvings,
                          (double)t.do_nothing, t.last_energy, (double)t.total_contacts, (double)t.candidate_rebuilds,
                          (double)t.barrier_reruns};
    for (int i = 0; i < n && i < 13; ++i) out[i] = v[i];
    return 13;
}

}  // extern "C"
