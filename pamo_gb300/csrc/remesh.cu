// Stage 1 of PaMO.run (simp_cuda/pamo/__init__.py:58-93): the input is normalised into the unit cube
// (preprocess_mesh), a narrow-band distance field of its triangles is sampled on an R^3 grid, shifted by 0.9
// voxel (`d - 0.9 / R`), and its zero set is extracted as a new mesh, mapped back with the reference's formula
// v = ((c + 0.5) / (R + 1) * margin - band) * tris_max + tris_min for a grid coordinate c. The reference calls
// two external libraries for this (torchcumesh2sdf.get_sdf and pdmc.DMC), which are absent; this file builds
// the same stage GB300-first:
//   * the distance field: voxels within the band of a triangle's box are marked (one pass over the
//     triangles), and each marked voxel takes its distance to the nearest triangle from an LBVH query; the rest
//     hold the band value;
//   * the sign: outside is the set of voxels farther than the iso value from the surface that a 6-connected
//     flood fill reaches from the grid boundary; everything else is inside, so open and self-intersecting
//     inputs give a closed shell;
//   * the surface: a dual extraction (one vertex per cell whose corners change sign, at the mean of the cell's
//     edge crossings; two triangles per grid edge with a sign change, joining the four cells around it,
//     oriented from inside to outside). Grid sample i lies at normalised coordinate (i + 0.5) / (R + 1).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/pamo_gb300.h"
#include "lbvh.cuh"
#include "pamo_common.cuh"
#include "scan.cuh"

namespace {

using namespace pamo;

constexpr int kT = 256;
constexpr int kQT = 128;
constexpr int kStack = 64;

__device__ __forceinline__ unsigned ord(float f) {  // order-preserving float -> uint
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord(unsigned u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u); }

// preprocess_mesh in float32: bounds of (p - mean) over the referenced corners
__global__ void k_corner_min(const float* __restrict__ pts, const int* __restrict__ tris, int nf, const float* mean,
                             unsigned* ext, int np, int* status) {
    float mn[3] = {INFINITY, INFINITY, INFINITY};
    for (int i = gtid(); i < 3 * nf; i += gstride()) {
        const int v = tris[i];
        if (v < 0 || v >= np) {
            atomicOr(status, kErrBadIndex);
            continue;
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) mn[d] = fminf(mn[d], pts[3 * v + d] - mean[d]);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (int o = 16; o > 0; o >>= 1) mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
        if ((threadIdx.x & 31) == 0) atomicMin(&ext[d], ord(mn[d]));
    }
}

__global__ void k_corner_max(const float* __restrict__ pts, const int* __restrict__ tris, int nf, const float* mean,
                             unsigned* ext, int np) {
    const float t0 = unord(ext[0]), t1 = unord(ext[1]), t2 = unord(ext[2]);
    float mx = -INFINITY;
    for (int i = gtid(); i < 3 * nf; i += gstride()) {
        const int v = tris[i];
        if (v < 0 || v >= np) continue;
        mx = fmaxf(mx, fmaxf((pts[3 * v] - mean[0]) - t0, fmaxf((pts[3 * v + 1] - mean[1]) - t1, (pts[3 * v + 2] - mean[2]) - t2)));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&ext[3], ord(mx));
}

// normalised vertices (tris = (tris / tris_max + band) / margin) and faces as int4
__global__ void k_normalise(const float* __restrict__ pts, int np, const int* __restrict__ tris, int nf,
                            const float* mean, const unsigned* ext, float band, float margin, float4* q, int4* tri) {
    const float t0 = unord(ext[0]), t1 = unord(ext[1]), t2 = unord(ext[2]), tmax = unord(ext[3]);
    for (int v = gtid(); v < np; v += gstride()) {
        const float x = ((pts[3 * v] - mean[0]) - t0) / tmax, y = ((pts[3 * v + 1] - mean[1]) - t1) / tmax,
                    z = ((pts[3 * v + 2] - mean[2]) - t2) / tmax;
        q[v] = make_float4((x + band) / margin, (y + band) / margin, (z + band) / margin, 0.f);
    }
    for (int f = gtid(); f < nf; f += gstride()) tri[f] = make_int4(tris[3 * f], tris[3 * f + 1], tris[3 * f + 2], 0);
}

__device__ __forceinline__ int cell_lo(float x, float band, int R) {  // first sample index >= x - band
    return max(0, (int)ceilf((x - band) * (float)(R + 1) - 0.5f));
}
__device__ __forceinline__ int cell_hi(float x, float band, int R) {  // last sample index <= x + band
    return min(R - 1, (int)floorf((x + band) * (float)(R + 1) - 0.5f));
}

// voxels within the band of a triangle's box
__global__ void k_mark_band(const float4* __restrict__ q, const int4* __restrict__ tri, int nf, int R, float band,
                            unsigned char* near) {
    for (int f = gtid(); f < nf; f += gstride()) {
        const int4 t = tri[f];
        const float4 a = q[t.x], b = q[t.y], c = q[t.z];
        const int x0 = cell_lo(fminf(a.x, fminf(b.x, c.x)), band, R), x1 = cell_hi(fmaxf(a.x, fmaxf(b.x, c.x)), band, R);
        const int y0 = cell_lo(fminf(a.y, fminf(b.y, c.y)), band, R), y1 = cell_hi(fmaxf(a.y, fmaxf(b.y, c.y)), band, R);
        const int z0 = cell_lo(fminf(a.z, fminf(b.z, c.z)), band, R), z1 = cell_hi(fmaxf(a.z, fmaxf(b.z, c.z)), band, R);
        for (int z = z0; z <= z1; ++z)
            for (int y = y0; y <= y1; ++y)
                for (int x = x0; x <= x1; ++x) near[((size_t)z * R + y) * R + x] = 1;
    }
}

struct P3f {
    float x, y, z;
};
__device__ __forceinline__ P3f psub(P3f a, P3f b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ float pdot(P3f a, P3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ P3f p3(float4 v) { return {v.x, v.y, v.z}; }

__device__ float point_tri_sq(P3f p, P3f a, P3f b, P3f c) {  // Ericson 5.1.5, squared distance
    const P3f ab = psub(b, a), ac = psub(c, a), ap = psub(p, a);
    const float d1 = pdot(ab, ap), d2 = pdot(ac, ap);
    P3f r;
    if (d1 <= 0.f && d2 <= 0.f) {
        r = a;
    } else {
        const P3f bp = psub(p, b);
        const float d3 = pdot(ab, bp), d4 = pdot(ac, bp);
        const float vc = d1 * d4 - d3 * d2;
        const P3f cp = psub(p, c);
        const float d5 = pdot(ab, cp), d6 = pdot(ac, cp);
        const float vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
        if (d3 >= 0.f && d4 <= d3) r = b;
        else if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
            const float v = d1 / (d1 - d3);
            r = {a.x + v * ab.x, a.y + v * ab.y, a.z + v * ab.z};
        } else if (d6 >= 0.f && d5 <= d6) r = c;
        else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
            const float w = d2 / (d2 - d6);
            r = {a.x + w * ac.x, a.y + w * ac.y, a.z + w * ac.z};
        } else if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
            const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
            r = {b.x + w * (c.x - b.x), b.y + w * (c.y - b.y), b.z + w * (c.z - b.z)};
        } else {
            const float den = 1.f / (va + vb + vc);
            const float v = vb * den, w = vc * den;
            r = {a.x + ab.x * v + ac.x * w, a.y + ab.y * v + ac.y * w, a.z + ab.z * v + ac.z * w};
        }
    }
    const P3f d = psub(r, p);
    return pdot(d, d);
}

__device__ __forceinline__ float box_sq(P3f p, float4 lo, float4 hi) {
    const float dx = fmaxf(fmaxf(lo.x - p.x, 0.f), p.x - hi.x), dy = fmaxf(fmaxf(lo.y - p.y, 0.f), p.y - hi.y),
                dz = fmaxf(fmaxf(lo.z - p.z, 0.f), p.z - hi.z);
    return dx * dx + dy * dy + dz * dz;
}

// distance of each marked voxel to the nearest triangle, capped at the band; unmarked voxels hold the band
__global__ void __launch_bounds__(kQT) k_udf(const unsigned char* __restrict__ near, int R, float band,
                                             const float4* __restrict__ q, const int4* __restrict__ tri,
                                             const int2* __restrict__ child, const float4* __restrict__ nlo,
                                             const float4* __restrict__ nhi, const float4* __restrict__ llo,
                                             const float4* __restrict__ lhi, const int* __restrict__ leaf_face,
                                             const RoundCounters* rc, float* udf, int* status) {
    __shared__ int stack[kStack][kQT];
    const long long n = (long long)R * R * R;
    const int nl = rc->n_live;
    const float inv = 1.0f / (float)(R + 1);
    for (long long i = gtid(); i < n; i += gstride()) {
        if (!near[i]) {
            udf[i] = band;
            continue;
        }
        const int x = (int)(i % R), y = (int)((i / R) % R), z = (int)(i / ((long long)R * R));
        const P3f p = {((float)x + 0.5f) * inv, ((float)y + 0.5f) * inv, ((float)z + 0.5f) * inv};
        float best = band * band;
        auto leaf = [&](int li) {
            const int4 t = tri[leaf_face[li]];
            best = fminf(best, point_tri_sq(p, p3(q[t.x]), p3(q[t.y]), p3(q[t.z])));
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
                int nn = 0;
                for (int side = 0; side < 2; ++side) {
                    const int xx = side ? c.y : c.x;
                    const float d = xx < 0 ? box_sq(p, llo[~xx], lhi[~xx]) : box_sq(p, nlo[xx], nhi[xx]);
                    if (d >= best) continue;
                    if (xx < 0) leaf(~xx);
                    else nxt[nn++] = xx;
                }
                if (nn == 2) {
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
                        if (box_sq(p, nlo[node], nhi[node]) < best) {
                            found = true;
                            break;
                        }
                    }
                    if (!found) break;
                }
            }
        }
        udf[i] = fminf(sqrtf(best), band);
    }
}

// outside flood fill: boundary voxels farther than iso start outside; a voxel farther than iso with an outside
// 6-neighbour becomes outside. In place (a voxel only ever turns 0 -> 1), repeated until nothing changes.
__global__ void k_fill_init(const float* __restrict__ udf, int R, float iso, unsigned char* out) {
    const long long n = (long long)R * R * R;
    for (long long i = gtid(); i < n; i += gstride()) {
        const int x = (int)(i % R), y = (int)((i / R) % R), z = (int)(i / ((long long)R * R));
        const bool border = x == 0 || y == 0 || z == 0 || x == R - 1 || y == R - 1 || z == R - 1;
        out[i] = (border && udf[i] > iso) ? 1 : 0;
    }
}

__global__ void k_fill_step(const float* __restrict__ udf, int R, float iso, unsigned char* out, int* changed) {
    const long long n = (long long)R * R * R;
    int ch = 0;
    for (long long i = gtid(); i < n; i += gstride()) {
        if (out[i] || !(udf[i] > iso)) continue;
        const int x = (int)(i % R), y = (int)((i / R) % R), z = (int)(i / ((long long)R * R));
        const long long RR = (long long)R * R;
        if ((x > 0 && out[i - 1]) || (x < R - 1 && out[i + 1]) || (y > 0 && out[i - R]) || (y < R - 1 && out[i + R]) ||
            (z > 0 && out[i - RR]) || (z < R - 1 && out[i + RR])) {
            out[i] = 1;
            ch = 1;
        }
    }
    if (__any_sync(0xffffffffu, ch) && (threadIdx.x & 31) == 0) *changed = 1;
}

// the extracted field: outside voxels udf - iso (> 0), the others -|udf - iso|
__device__ __forceinline__ float field_at(const float* udf, const unsigned char* out, float iso, long long i) {
    const float g = udf[i] - iso;
    return out[i] ? g : -fabsf(g);
}

// cells with a sign change: flag, then (after the scan) the vertex at the mean of the edge crossings
__global__ void k_cell_flags(const float* __restrict__ udf, const unsigned char* __restrict__ out, int R, float iso,
                             int* flag) {
    const int C = R - 1;
    const long long n = (long long)C * C * C;
    for (long long c = gtid(); c < n; c += gstride()) {
        const int x = (int)(c % C), y = (int)((c / C) % C), z = (int)(c / ((long long)C * C));
        int neg = 0;
        for (int k = 0; k < 8; ++k) {
            const long long i = ((long long)(z + (k >> 2)) * R + (y + ((k >> 1) & 1))) * R + (x + (k & 1));
            neg += field_at(udf, out, iso, i) < 0.f ? 1 : 0;
        }
        flag[c] = (neg > 0 && neg < 8) ? 1 : 0;
    }
    if (gtid() == 0) flag[n] = 0;
}

__constant__ int kEdgeCorners[12][2] = {{0, 1}, {2, 3}, {4, 5}, {6, 7}, {0, 2}, {1, 3}, {4, 6}, {5, 7},
                                        {0, 4}, {1, 5}, {2, 6}, {3, 7}};

__global__ void k_cell_vertices(const float* __restrict__ udf, const unsigned char* __restrict__ out, int R, float iso,
                                const int* __restrict__ scan, float band, float margin, const float* mean,
                                const unsigned* ext, float* verts) {
    const int C = R - 1;
    const long long n = (long long)C * C * C;
    const float t0 = unord(ext[0]), t1 = unord(ext[1]), t2 = unord(ext[2]), tmax = unord(ext[3]);
    for (long long c = gtid(); c < n; c += gstride()) {
        if (scan[c + 1] == scan[c]) continue;
        const int x = (int)(c % C), y = (int)((c / C) % C), z = (int)(c / ((long long)C * C));
        float v[8];
        for (int k = 0; k < 8; ++k)
            v[k] = field_at(udf, out, iso, ((long long)(z + (k >> 2)) * R + (y + ((k >> 1) & 1))) * R + (x + (k & 1)));
        float sx = 0.f, sy = 0.f, sz = 0.f;
        int m = 0;
        for (int e = 0; e < 12; ++e) {
            const int a = kEdgeCorners[e][0], b = kEdgeCorners[e][1];
            if ((v[a] < 0.f) == (v[b] < 0.f)) continue;
            const float t = v[a] / (v[a] - v[b]);
            sx += (float)(a & 1) + t * (float)((b & 1) - (a & 1));
            sy += (float)((a >> 1) & 1) + t * (float)(((b >> 1) & 1) - ((a >> 1) & 1));
            sz += (float)(a >> 2) + t * (float)((b >> 2) - (a >> 2));
            ++m;
        }
        const float cx = (float)x + sx / (float)m, cy = (float)y + sy / (float)m, cz = (float)z + sz / (float)m;
        // the reference's mapping back: ((c + 0.5) / (R + 1) * margin - band) * tris_max + tris_min
        const float k = 1.0f / (float)(R + 1);
        const long long o = 3 * (long long)scan[c];
        verts[o] = ((cx + 0.5f) * k * margin - band) * tmax + t0;
        verts[o + 1] = ((cy + 0.5f) * k * margin - band) * tmax + t1;
        verts[o + 2] = ((cz + 0.5f) * k * margin - band) * tmax + t2;
    }
}

// grid edges with a sign change whose four surrounding cells exist: two triangles each
__device__ __forceinline__ bool edge_quad(const float* udf, const unsigned char* out, int R, float iso, long long i,
                                          int axis, int x, int y, int z, bool& inside_low) {
    const int C = R - 1;
    const long long stride = axis == 0 ? 1 : (axis == 1 ? R : (long long)R * R);
    const int pos = axis == 0 ? x : (axis == 1 ? y : z);
    if (pos >= R - 1) return false;
    // the two other coordinates must allow cells on both sides
    const int u = axis == 0 ? y : (axis == 1 ? z : x), w = axis == 0 ? z : (axis == 1 ? x : y);
    if (u < 1 || w < 1 || u > C - 1 || w > C - 1) return false;
    const float a = field_at(udf, out, iso, i), b = field_at(udf, out, iso, i + stride);
    if ((a < 0.f) == (b < 0.f)) return false;
    inside_low = a < 0.f;
    return true;
}

__global__ void k_quad_flags(const float* __restrict__ udf, const unsigned char* __restrict__ out, int R, float iso,
                             int* qflag) {
    const long long n = (long long)R * R * R;
    for (long long i = gtid(); i < n; i += gstride()) {
        const int x = (int)(i % R), y = (int)((i / R) % R), z = (int)(i / ((long long)R * R));
        int cnt = 0;
        bool il;
        for (int axis = 0; axis < 3; ++axis) cnt += edge_quad(udf, out, R, iso, i, axis, x, y, z, il) ? 1 : 0;
        qflag[i] = cnt;
    }
    if (gtid() == 0) qflag[n] = 0;
}

__global__ void k_quads(const float* __restrict__ udf, const unsigned char* __restrict__ out, int R, float iso,
                        const int* __restrict__ qscan, const int* __restrict__ cscan, int* tris) {
    const int C = R - 1;
    const long long n = (long long)R * R * R;
    auto cell = [&](int cx, int cy, int cz) { return cscan[((long long)cz * C + cy) * C + cx]; };
    for (long long i = gtid(); i < n; i += gstride()) {
        if (qscan[i + 1] == qscan[i]) continue;
        const int x = (int)(i % R), y = (int)((i / R) % R), z = (int)(i / ((long long)R * R));
        long long o = 6 * (long long)qscan[i];
        for (int axis = 0; axis < 3; ++axis) {
            bool il;
            if (!edge_quad(udf, out, R, iso, i, axis, x, y, z, il)) continue;
            // the four cells around the edge, counter-clockwise about the axis direction
            int c00, c10, c11, c01;
            if (axis == 0) {  // plane (y, z)
                c00 = cell(x, y - 1, z - 1); c10 = cell(x, y, z - 1); c11 = cell(x, y, z); c01 = cell(x, y - 1, z);
            } else if (axis == 1) {  // plane (z, x)
                c00 = cell(x - 1, y, z - 1); c10 = cell(x - 1, y, z); c11 = cell(x, y, z); c01 = cell(x, y, z - 1);
            } else {  // plane (x, y)
                c00 = cell(x - 1, y - 1, z); c10 = cell(x, y - 1, z); c11 = cell(x, y, z); c01 = cell(x - 1, y, z);
            }
            // inside at the lower end: the surface faces the +axis direction, counter-clockwise seen from there
            if (il) {
                tris[o] = c00; tris[o + 1] = c10; tris[o + 2] = c11;
                tris[o + 3] = c00; tris[o + 4] = c11; tris[o + 5] = c01;
            } else {
                tris[o] = c00; tris[o + 1] = c11; tris[o + 2] = c10;
                tris[o + 3] = c00; tris[o + 4] = c01; tris[o + 5] = c11;
            }
            o += 6;
        }
    }
}

struct DBuf {
    void* p = nullptr;
    size_t n = 0;
    int grow(size_t bytes) {
        if (bytes <= n && p) return PAMO_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return PAMO_ERR_OOM;
        n = bytes;
        return PAMO_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

}  // namespace

struct pamo_remesher {
    int device = 0;
    DBuf q, tri, near, udf, outf, cflag, qflag, verts, tris, bvh, small, scratch;
    RoundCounters* rc = nullptr;
    int* h_small = nullptr;  // pinned: status, changed, vertex count, triangle count
    int nv = 0, nf = 0;
    void release() {
        for (DBuf* b : {&q, &tri, &near, &udf, &outf, &cflag, &qflag, &verts, &tris, &bvh, &small, &scratch}) b->release();
        if (rc) cudaFree(rc);
        if (h_small) cudaFreeHost(h_small);
        rc = nullptr;
        h_small = nullptr;
    }
};

extern "C" {

int pamo_remesher_create(pamo_remesher** out, int32_t device) {
    if (!out) return PAMO_ERR_INVALID_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return PAMO_ERR_INVALID_ARG;
    pamo_remesher* m = new pamo_remesher();
    m->device = device;
    if (cudaMalloc((void**)&m->rc, sizeof(RoundCounters)) != cudaSuccess ||
        cudaMallocHost((void**)&m->h_small, 16 * sizeof(int)) != cudaSuccess ||
        m->scratch.grow(scan_scratch_ints() * sizeof(int)) != PAMO_OK || scan_scratch_clear((int*)m->scratch.p)) {
        m->release();
        delete m;
        return PAMO_ERR_OOM;
    }
    *out = m;
    return PAMO_OK;
}

int pamo_remesher_destroy(pamo_remesher* m) {
    if (!m) return PAMO_ERR_INVALID_ARG;
    cudaSetDevice(m->device);
    cudaDeviceSynchronize();
    m->release();
    delete m;
    return PAMO_OK;
}

int pamo_remesh(pamo_remesher* m, const float* points, const int32_t* triangles, int32_t n_points, int32_t n_triangles,
                int32_t resolution, const float* mean3, int32_t* out_n_points, int32_t* out_n_triangles,
                pamo_stream stream) {
    if (!m || !points || !triangles || !mean3 || n_points < 1 || n_triangles < 1 || resolution < 4 ||
        resolution > 1024)
        return PAMO_ERR_INVALID_ARG;
    cudaSetDevice(m->device);
    cudaStream_t s = (cudaStream_t)stream;
    const int R = resolution;
    // the reference's Python floats (float64), applied to float32 arrays
    const float band = (float)(3.0 / R), margin = (float)(3.0 / R * 2.0 + 1.0), iso = (float)(0.9 / R);
    const long long NV = (long long)R * R * R, NC = (long long)(R - 1) * (R - 1) * (R - 1);
    if (NV >= (1ll << 31) - 2) return PAMO_ERR_CAPACITY;
    int r;
    if ((r = m->q.grow((size_t)n_points * sizeof(float4))) || (r = m->tri.grow(((size_t)n_triangles + 1) * sizeof(int4))) ||
        (r = m->near.grow(NV)) || (r = m->udf.grow(NV * sizeof(float))) || (r = m->outf.grow(NV)) ||
        (r = m->cflag.grow((NC + 1) * sizeof(int))) || (r = m->qflag.grow((NV + 1) * sizeof(int))) ||
        (r = m->bvh.grow(bvh_bytes(n_triangles))) || (r = m->small.grow(16 * sizeof(float) + 8 * sizeof(unsigned))))
        return r;
    BvhBuffers b;
    bvh_carve(b, n_triangles, (char*)m->bvh.p);
    float* d_mean = (float*)m->small.p;
    unsigned* ext = (unsigned*)((float*)m->small.p + 4);
    int* d_changed = (int*)((float*)m->small.p + 12);
    float4* q = (float4*)m->q.p;
    int4* tri = (int4*)m->tri.p;
    unsigned char* near = (unsigned char*)m->near.p;
    float* udf = (float*)m->udf.p;
    unsigned char* outf = (unsigned char*)m->outf.p;
    int* cflag = (int*)m->cflag.p;
    int* qflag = (int*)m->qflag.p;
    int* scratch = (int*)m->scratch.p;

    RoundCounters h{};
    h.n_pts = n_points;
    h.n_tris = n_triangles;
    std::memcpy(m->h_small + 4, mean3, 3 * sizeof(float));
    cudaMemcpyAsync(m->rc, &h, sizeof(h), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_mean, m->h_small + 4, 3 * sizeof(float), cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(ext, 0xFF, 3 * sizeof(unsigned), s);
    cudaMemsetAsync(ext + 3, 0x00, sizeof(unsigned), s);
    k_corner_min<<<grid_for(3ll * n_triangles, kT), kT, 0, s>>>(points, triangles, n_triangles, d_mean, ext, n_points,
                                                                &m->rc->status);
    k_corner_max<<<grid_for(3ll * n_triangles, kT), kT, 0, s>>>(points, triangles, n_triangles, d_mean, ext, n_points);
    k_normalise<<<grid_for(std::max(n_points, n_triangles), kT), kT, 0, s>>>(points, n_points, triangles, n_triangles,
                                                                           d_mean, ext, band, margin, q, tri);
    note_launches(3);
    // stop before touching the grid when an index was out of range
    cudaMemcpyAsync(m->h_small, &m->rc->status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return PAMO_ERR_CUDA;
    if (m->h_small[0] & kErrBadIndex) return PAMO_ERR_INVALID_ARG;

    bvh_build(b, tri, q, m->rc, n_triangles, s);
    cudaMemsetAsync(near, 0, NV, s);
    k_mark_band<<<grid_for(n_triangles, kT), kT, 0, s>>>(q, tri, n_triangles, R, band, near);
    k_udf<<<grid_for(NV, kQT, 16), kQT, 0, s>>>(near, R, band, q, tri, b.child, b.nlo, b.nhi, b.llo, b.lhi, b.vals[0],
                                               m->rc, udf, &m->rc->status);
    k_fill_init<<<grid_for(NV, kT), kT, 0, s>>>(udf, R, iso, outf);
    note_launches(3);
    // flood fill: batches of sweeps until a batch changes nothing (at most one sweep per voxel on a path)
    const int max_batches = (int)(NV / 16 + 2);
    for (int batch = 0; batch < max_batches; ++batch) {
        cudaMemsetAsync(d_changed, 0, sizeof(int), s);
        for (int k = 0; k < 16; ++k) k_fill_step<<<grid_for(NV, kT), kT, 0, s>>>(udf, R, iso, outf, d_changed);
        note_launches(16);
        cudaMemcpyAsync(m->h_small + 1, d_changed, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return PAMO_ERR_CUDA;
        if (m->h_small[1] == 0) break;
    }
    // cells with a sign change and their vertices
    k_cell_flags<<<grid_for(NC, kT), kT, 0, s>>>(udf, outf, R, iso, cflag);
    exclusive_scan(cflag, cflag, nullptr, (int)NC + 1, &m->rc->n_win, scratch, s, &m->rc->status);
    k_quad_flags<<<grid_for(NV, kT), kT, 0, s>>>(udf, outf, R, iso, qflag);
    exclusive_scan(qflag, qflag, nullptr, (int)NV + 1, &m->rc->n_query, scratch, s, &m->rc->status);
    note_launches(2);
    cudaMemcpyAsync(m->h_small + 2, &m->rc->n_win, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(m->h_small + 3, &m->rc->n_query, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(m->h_small, &m->rc->status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return PAMO_ERR_CUDA;
    if (m->h_small[0] & (kErrIterLimit | kErrStackOverflow)) return PAMO_ERR_ITER_LIMIT;
    m->nv = m->h_small[2];
    m->nf = 2 * m->h_small[3];
    if ((r = m->verts.grow(((size_t)m->nv + 1) * 3 * sizeof(float))) || (r = m->tris.grow(((size_t)m->nf + 1) * 3 * sizeof(int))))
        return r;
    k_cell_vertices<<<grid_for(NC, kT), kT, 0, s>>>(udf, outf, R, iso, cflag, band, margin, d_mean, ext,
                                                    (float*)m->verts.p);
    k_quads<<<grid_for(NV, kT), kT, 0, s>>>(udf, outf, R, iso, qflag, cflag, (int*)m->tris.p);
    note_launches(2);
    if (cudaStreamSynchronize(s) != cudaSuccess) return PAMO_ERR_CUDA;
    if (out_n_points) *out_n_points = m->nv;
    if (out_n_triangles) *out_n_triangles = m->nf;
    return PAMO_OK;
}

int pamo_remesh_result(pamo_remesher* m, float* verts, int32_t* tris, pamo_stream stream) {
    if (!m || !verts || !tris) return PAMO_ERR_INVALID_ARG;
    cudaSetDevice(m->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (m->nv) cudaMemcpyAsync(verts, m->verts.p, (size_t)m->nv * 3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (m->nf) cudaMemcpyAsync(tris, m->tris.p, (size_t)m->nf * 3 * sizeof(int), cudaMemcpyDeviceToDevice, s);
    return cudaStreamSynchronize(s) == cudaSuccess ? PAMO_OK : PAMO_ERR_CUDA;
}

}  // extern "C"
