// Evaluation kernels of the reference's metrics module (simp_cuda/safe_project/src/pamo_safe_project/
// metrics.py:7-107): squared distances from points to a triangle mesh (the closest-point queries behind its
// Chamfer and Hausdorff distances) and the per-face minimum angles behind compute_min_angle and
// compute_bad_tri_ratio. Off the simplification path; inputs are float64 like the metrics' NumPy arrays.
//
// Point-to-mesh distance: the stage-2 LBVH built over float copies of the vertices, each box widened by a
// relative 2^-20 of its coordinates so that it bounds the float64 triangle; a branch-and-bound walk per point
// (nearest child first) with the exact float64 point-triangle distance at the leaves (Ericson, Real-Time
// Collision Detection, 5.1.5).
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/pamo_gb300.h"
#include "lbvh.cuh"
#include "pamo_common.cuh"

namespace {

using namespace pamo;

constexpr int kT = 256;
constexpr int kQT = 128;
constexpr int kStack = 64;

struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 dsub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 dadd(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 dmul(double s, D3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 dload(const double* v, int i) { return {v[3 * i], v[3 * i + 1], v[3 * i + 2]}; }

// closest point of triangle abc to p (region tests on the barycentric parameters)
__device__ D3 closest_point_triangle(D3 p, D3 a, D3 b, D3 c) {
    const D3 ab = dsub(b, a), ac = dsub(c, a), ap = dsub(p, a);
    const double d1 = ddot(ab, ap), d2 = ddot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) return a;
    const D3 bp = dsub(p, b);
    const double d3 = ddot(ab, bp), d4 = ddot(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) return b;
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) return dadd(a, dmul(d1 / (d1 - d3), ab));
    const D3 cp = dsub(p, c);
    const double d5 = ddot(ab, cp), d6 = ddot(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) return c;
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) return dadd(a, dmul(d2 / (d2 - d6), ac));
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0)
        return dadd(b, dmul((d4 - d3) / ((d4 - d3) + (d5 - d6)), dsub(c, b)));
    const double den = 1.0 / (va + vb + vc);
    return dadd(a, dadd(dmul(vb * den, ab), dmul(vc * den, ac)));
}

__global__ void k_to_float4(const double* __restrict__ v, int n, float4* out) {
    for (int i = gtid(); i < n; i += gstride())
        out[i] = make_float4((float)v[3 * i], (float)v[3 * i + 1], (float)v[3 * i + 2], 0.f);
}

__global__ void k_to_int4(const int* __restrict__ f, int n, int nv, int4* out, int* status) {
    for (int i = gtid(); i < n; i += gstride()) {
        const int a = f[3 * i], b = f[3 * i + 1], c = f[3 * i + 2];
        if (a < 0 || b < 0 || c < 0 || a >= nv || b >= nv || c >= nv) {
            atomicOr(status, kErrBadIndex);
            out[i] = make_int4(0, 0, 0, 0);
        } else {
            out[i] = make_int4(a, b, c, 0);
        }
    }
}

// squared distance from p to a box widened by a relative 2^-20 (so that it bounds the float64 geometry the
// float box was rounded from), as a lower bound for pruning
__device__ __forceinline__ double box_lower_bound(D3 p, float4 lo, float4 hi) {
    const double e = 9.5367431640625e-07;  // 2^-20
    auto axis = [&](double x, float l, float h) {
        const double dl = (double)l - e * fabs((double)l) - 1e-30, dh = (double)h + e * fabs((double)h) + 1e-30;
        return x < dl ? dl - x : (x > dh ? x - dh : 0.0);
    };
    const double dx = axis(p.x, lo.x, hi.x), dy = axis(p.y, lo.y, hi.y), dz = axis(p.z, lo.z, hi.z);
    return dx * dx + dy * dy + dz * dz;
}

__global__ void __launch_bounds__(kQT) k_point_mesh(const double* __restrict__ pts, int np, const double* __restrict__ V,
                                                    const int4* __restrict__ tri, const int2* __restrict__ child,
                                                    const float4* __restrict__ nlo, const float4* __restrict__ nhi,
                                                    const float4* __restrict__ llo, const float4* __restrict__ lhi,
                                                    const int* __restrict__ leaf_face, const RoundCounters* rc,
                                                    double* out_d2, int* out_face, int* status) {
    __shared__ int stack[kStack][kQT];
    const int nl = rc->n_live;
    for (int i = gtid(); i < np; i += gstride()) {
        const D3 p = dload(pts, i);
        double best = INFINITY;
        int bf = -1;
        auto leaf = [&](int li) {
            const int f = leaf_face[li];
            const int4 t = tri[f];
            const D3 c = closest_point_triangle(p, dload(V, t.x), dload(V, t.y), dload(V, t.z));
            const D3 d = dsub(c, p);
            const double d2 = ddot(d, d);
            if (d2 < best || (d2 == best && f < bf)) {
                best = d2;
                bf = f;
            }
        };
        if (nl == 1) leaf(0);
        if (nl >= 2) {
            int sp = 0, node = 0, guard = 0;
            while (true) {
                if (++guard > (1 << 22)) {
                    atomicOr(status, kErrIterLimit);
                    break;
                }
                const int2 c = child[node];
                int nxt[2];
                double nd[2];
                int nn = 0;
                for (int side = 0; side < 2; ++side) {
                    const int x = side ? c.y : c.x;
                    const double d = x < 0 ? box_lower_bound(p, llo[~x], lhi[~x]) : box_lower_bound(p, nlo[x], nhi[x]);
                    if (d > best) continue;
                    if (x < 0) leaf(~x);
                    else {
                        nxt[nn] = x;
                        nd[nn] = d;
                        ++nn;
                    }
                }
                if (nn == 2) {
                    if (nd[1] < nd[0]) {
                        const int t = nxt[0];
                        nxt[0] = nxt[1];
                        nxt[1] = t;
                    }
                    if (sp >= kStack) {
                        atomicOr(status, kErrStackOverflow);
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
                        if (box_lower_bound(p, nlo[node], nhi[node]) <= best) {
                            found = true;
                            break;
                        }
                    }
                    if (!found) break;
                }
            }
        }
        out_d2[i] = best;
        if (out_face) out_face[i] = bf;
    }
}

// Per face: the minimum angle of compute_min_angle_VF (edge vectors e_k = V[f_k] - V[f_(k+1)], the angle at each
// corner from -dot(e_k, e_(k-1)) / (|e_k| |e_(k-1)|) clipped to [-1, 1]) and of igl.internal_angles (law of
// cosines on the squared edge lengths), in radians; NaN for a face with a repeated index.
__global__ void k_face_min_angles(const double* __restrict__ V, const int* __restrict__ F, int nf, double* out_edge,
                                  double* out_igl) {
    for (int f = gtid(); f < nf; f += gstride()) {
        const int i0 = F[3 * f], i1 = F[3 * f + 1], i2 = F[3 * f + 2];
        if (i0 == i1 || i1 == i2 || i2 == i0) {
            if (out_edge) out_edge[f] = NAN;
            if (out_igl) out_igl[f] = NAN;
            continue;
        }
        const D3 p[3] = {dload(V, i0), dload(V, i1), dload(V, i2)};
        D3 e[3];
        double l[3];
        for (int k = 0; k < 3; ++k) {
            e[k] = dsub(p[k], p[(k + 1) % 3]);
            l[k] = sqrt(ddot(e[k], e[k]));
        }
        if (out_edge) {
            double m = INFINITY;
            for (int k = 0; k < 3; ++k) {
                const int km = (k + 2) % 3;
                double c = -ddot(e[k], e[km]) / (l[k] * l[km]);
                c = fmin(fmax(c, -1.0), 1.0);
                m = fmin(m, acos(c));
            }
            out_edge[f] = m;
        }
        if (out_igl) {
            // corner k is opposite the edge (k+1, k+2), whose squared length is |e_(k+1)|^2
            double m = INFINITY;
            for (int k = 0; k < 3; ++k) {
                const double a2 = l[(k + 1) % 3] * l[(k + 1) % 3];
                const double b = l[k], c = l[(k + 2) % 3];
                double x = (b * b + c * c - a2) / (2.0 * b * c);
                x = fmin(fmax(x, -1.0), 1.0);
                m = fmin(m, acos(x));
            }
            out_igl[f] = m;
        }
    }
}

int cuda_status(cudaError_t e) { return e == cudaSuccess ? PAMO_OK : PAMO_ERR_CUDA; }

}  // namespace

extern "C" {

int pamo_point_mesh_sqdist(const double* points, int32_t n_points, const double* vertices, int32_t n_vertices,
                           const int32_t* triangles, int32_t n_triangles, double* out_sqdist, int32_t* out_face,
                           pamo_stream stream) {
    if (!points || !vertices || !triangles || !out_sqdist || n_points < 0 || n_vertices < 1 || n_triangles < 1)
        return PAMO_ERR_INVALID_ARG;
    if (n_points == 0) return PAMO_OK;
    cudaStream_t s = (cudaStream_t)stream;
    float4* pos = nullptr;
    int4* tri = nullptr;
    RoundCounters* rc = nullptr;
    char* bvh_mem = nullptr;
    int r = PAMO_OK;
    if (cudaMalloc((void**)&pos, (size_t)n_vertices * sizeof(float4)) != cudaSuccess ||
        cudaMalloc((void**)&tri, ((size_t)n_triangles + 1) * sizeof(int4)) != cudaSuccess ||
        cudaMalloc((void**)&rc, sizeof(RoundCounters)) != cudaSuccess ||
        cudaMalloc((void**)&bvh_mem, bvh_bytes(n_triangles)) != cudaSuccess) {
        r = PAMO_ERR_OOM;
    }
    if (r == PAMO_OK) {
        BvhBuffers b;
        bvh_carve(b, n_triangles, bvh_mem);
        RoundCounters h{};
        h.n_pts = n_vertices;
        h.n_tris = n_triangles;
        cudaMemcpyAsync(rc, &h, sizeof(h), cudaMemcpyHostToDevice, s);
        k_to_float4<<<grid_for(n_vertices, kT), kT, 0, s>>>(vertices, n_vertices, pos);
        k_to_int4<<<grid_for(n_triangles, kT), kT, 0, s>>>(triangles, n_triangles, n_vertices, tri, &rc->status);
        note_launches(2);
        bvh_build(b, tri, pos, rc, n_triangles, s);
        k_point_mesh<<<grid_for(n_points, kQT, 16), kQT, 0, s>>>(points, n_points, vertices, tri, b.child, b.nlo, b.nhi,
                                                                b.llo, b.lhi, b.vals[0], rc, out_sqdist, out_face,
                                                                &rc->status);
        note_launch();
        r = cuda_status(cudaStreamSynchronize(s));
        if (r == PAMO_OK) {
            int st = 0;
            r = cuda_status(cudaMemcpy(&st, &rc->status, sizeof(int), cudaMemcpyDeviceToHost));
            if (r == PAMO_OK && (st & kErrBadIndex)) r = PAMO_ERR_INVALID_ARG;
            else if (r == PAMO_OK && st) r = PAMO_ERR_ITER_LIMIT;
        }
    }
    cudaFree(pos);
    cudaFree(tri);
    cudaFree(rc);
    cudaFree(bvh_mem);
    return r;
}

int pamo_face_min_angles(const double* vertices, const int32_t* triangles, int32_t n_triangles, double* out_edge_form,
                         double* out_igl_form, pamo_stream stream) {
    if (!vertices || !triangles || n_triangles < 0 || (!out_edge_form && !out_igl_form)) return PAMO_ERR_INVALID_ARG;
    if (n_triangles == 0) return PAMO_OK;
    cudaStream_t s = (cudaStream_t)stream;
    k_face_min_angles<<<grid_for(n_triangles, kT), kT, 0, s>>>(vertices, triangles, n_triangles, out_edge_form,
                                                               out_igl_form);
    note_launch();
    return cuda_status(cudaStreamSynchronize(s));
}

}  // extern "C"
