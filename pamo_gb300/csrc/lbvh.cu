// LBVH over live faces: AABBs and scene bounds, 30-bit Morton codes of box centroids, an in-house stable
// LSD radix sort (8-bit digits, warp-match ranking), Karras (2012) topology with an index tie-break for
// equal codes, bottom-up boxes, and a per-face query that walks the tree with a stack in shared memory and
// runs the reference's pair test on every overlapping leaf.
//
// The tree only filters candidates: a (query f, hit g) pair is tested iff both faces are live, f != g and
// their closed boxes overlap (simp_cuda/src/bvh/query.cuh:8-133, aabb.cuh:154-162), which is the candidate
// set of the reference's global LBVH query.
#include <cstdint>
#include "lbvh.cuh"
#include "scan.cuh"
#include "tritri.cuh"

namespace pamo {

namespace {

constexpr int kSortTiles = 4 * kNumSM;
constexpr size_t kExactQueue = 1 << 20;  // pairs queued for the float64 pass (the rest are decided in place)
constexpr int kSortThreads = 256;
constexpr int kQueryThreads = 128;
constexpr int kStackDepth = 64;  // enough for any tree (depth <= 62 + 1)
constexpr int kShortStack = 24;  // first walk: deeper queries are handed to the second walk
constexpr int kPairChunk = 32;   // list slots a lane takes at a time
constexpr int kQueryBit = 1 << 30;  // set on a packed leaf's face id when the face is a query face

__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ unsigned expand10(unsigned v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// ---------------------------------------------------------------- boxes + scene bounds
__global__ void __launch_bounds__(256) k_boxes(const int4* __restrict__ tri, const float4* __restrict__ pos,
                                                const RoundCounters* rc, float4* box_lo, float4* box_hi, int* live,
                                                unsigned* scene, int all_faces) {
    const int n = rc->n_tris;
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int f = gtid(); f < n; f += gstride()) {
        int4 t = tri[f];
        int is_live = (t.x != -1);
        live[f] = all_faces ? 1 : is_live;
        if (!is_live) {
            if (all_faces) {  // an empty box: overlaps nothing
                box_lo[f] = make_float4(INFINITY, INFINITY, INFINITY, 0.f);
                box_hi[f] = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
            }
            continue;
        }
        float4 a = pos[t.x], b = pos[t.y], c = pos[t.z];
        float4 lo = make_float4(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)), 0.f);
        float4 hi = make_float4(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)), 0.f);
        box_lo[f] = lo;
        box_hi[f] = hi;
        mn[0] = fminf(mn[0], lo.x); mn[1] = fminf(mn[1], lo.y); mn[2] = fminf(mn[2], lo.z);
        mx[0] = fmaxf(mx[0], hi.x); mx[1] = fmaxf(mx[1], hi.y); mx[2] = fmaxf(mx[2], hi.z);
    }
    if (gtid() == 0) live[n] = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (mn[d] <= mx[d]) {
                atomicMin(&scene[d], f2ord(mn[d]));
                atomicMax(&scene[3 + d], f2ord(mx[d]));
            }
        }
    }
}

// ---------------------------------------------------------------- Morton codes of live faces
// fmesh (many meshes in one numbering): the key's top mesh_bits hold the face's mesh and the rest the top bits of its
// Morton code, so that the sort groups each mesh's faces and every Karras node under a mesh boundary covers one mesh
__global__ void __launch_bounds__(256) k_morton(const RoundCounters* rc, const int* live_scan, const float4* box_lo,
                                                 const float4* box_hi, const unsigned* scene, unsigned* keys, int* vals,
                                                 const int* __restrict__ fmesh, int mesh_bits) {
    const int n = rc->n_tris;
    float lo[3], ext[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        lo[d] = ord2f(scene[d]);
        float hi = ord2f(scene[3 + d]);
        ext[d] = hi - lo[d];
    }
    for (int f = gtid(); f < n; f += gstride()) {
        int i = live_scan[f];
        if (live_scan[f + 1] == i) continue;
        float4 a = box_lo[f], b = box_hi[f];
        float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        unsigned q[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float t = ext[d] > 0.f ? (c[d] - lo[d]) / ext[d] : 0.f;
            t = fminf(fmaxf(t * 1024.0f, 0.0f), 1023.0f);
            q[d] = (unsigned)t;
        }
        unsigned key = expand10(q[0]) * 4u + expand10(q[1]) * 2u + expand10(q[2]);
        if (fmesh) {
            const unsigned m = (unsigned)fmesh[f];
            key = mesh_bits <= 2 ? ((m << 30) | key) : ((m << (32 - mesh_bits)) | (key >> (mesh_bits - 2)));
        }
        keys[i] = key;
        vals[i] = f;
    }
}

// ---------------------------------------------------------------- stable LSD radix sort
__device__ __forceinline__ void sort_chunk(int n, int& lo, int& hi) {
    long long chunk = ((long long)n + gridDim.x - 1) / gridDim.x;
    chunk = (chunk + kSortThreads - 1) / kSortThreads * kSortThreads;
    long long a = chunk * blockIdx.x, b = a + chunk;
    lo = (int)(a < n ? a : n);
    hi = (int)(b < n ? b : n);
}

__global__ void __launch_bounds__(kSortThreads) k_rs_hist(const unsigned* __restrict__ keys, const int* d_n, int shift,
                                                          int* hist) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int lo, hi;
    sort_chunk(*d_n, lo, hi);
    for (int i = lo + threadIdx.x; i < hi; i += kSortThreads) atomicAdd(&h[(keys[i] >> shift) & 0xFF], 1);
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Each tile of 256 keys is ranked stably: lanes of a warp with the same digit find each other with
// __match_any_sync, warps are ordered through per-warp digit counts in shared memory.
__global__ void __launch_bounds__(kSortThreads) k_rs_scatter(const unsigned* __restrict__ kin, const int* __restrict__ vin,
                                                             unsigned* kout, int* vout, const int* d_n, int shift,
                                                             const int* hist) {
    constexpr int W = kSortThreads / 32;
    __shared__ int base[256];
    __shared__ int wcnt[W][256];
    __shared__ int tot[256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    base[threadIdx.x] = hist[threadIdx.x * gridDim.x + blockIdx.x];
    for (int w = 0; w < W; ++w) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    int lo, hi;
    sort_chunk(*d_n, lo, hi);
    for (int t0 = lo; t0 < hi; t0 += kSortThreads) {
        const int i = t0 + threadIdx.x;
        const bool valid = i < hi;
        unsigned key = valid ? kin[i] : 0u;
        int val = valid ? vin[i] : 0;
        const int dig = valid ? (int)((key >> shift) & 0xFF) : 256;
        const unsigned peers = __match_any_sync(0xffffffffu, dig);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) wcnt[warp][dig] = __popc(peers);
        __syncthreads();
        {
            int run = 0;
            for (int w = 0; w < W; ++w) {
                int c = wcnt[w][threadIdx.x];
                wcnt[w][threadIdx.x] = run;
                run += c;
            }
            tot[threadIdx.x] = run;
        }
        __syncthreads();
        if (valid) {
            const int dst = base[dig] + wcnt[warp][dig] + rank;
            kout[dst] = key;
            vout[dst] = val;
        }
        __syncthreads();
        base[threadIdx.x] += tot[threadIdx.x];
        for (int w = 0; w < W; ++w) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
    }
}

// ---------------------------------------------------------------- Karras topology
__device__ __forceinline__ int delta(const unsigned* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned a = k[i], b = k[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((unsigned)(i ^ j));
}

__global__ void __launch_bounds__(256) k_leaves(const RoundCounters* rc, const int* vals, const float4* box_lo,
                                                 const float4* box_hi, float4* llo, float4* lhi, int* visit, int* lparent) {
    const int n = rc->n_live;
    for (int i = gtid(); i < n; i += gstride()) {
        int f = vals[i];
        llo[i] = box_lo[f];
        lhi[i] = box_hi[f];
        if (i < n - 1) visit[i] = 0;
        if (n == 1) lparent[0] = -1;
    }
}

__global__ void __launch_bounds__(256) k_karras(const RoundCounters* rc, const unsigned* keys, int2* child, int* iparent,
                                                 int* lparent, int2* range) {
    const int n = rc->n_live;
    for (int i = gtid(); i < n - 1; i += gstride()) {
        const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
        const int dmin = delta(keys, n, i, i - d);
        int lmax = 2;
        while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        const int dnode = delta(keys, n, i, j);
        int s = 0;
        int t = l;
        do {
            t = (t + 1) >> 1;
            if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        const int gamma = i + s * d + (d < 0 ? -1 : 0);
        const int lo = min(i, j), hi = max(i, j);
        range[i] = make_int2(lo, hi);
        int left, right;
        if (lo == gamma) {
            left = ~gamma;
            lparent[gamma] = i;
        } else {
            left = gamma;
            iparent[gamma] = i;
        }
        if (hi == gamma + 1) {
            right = ~(gamma + 1);
            lparent[gamma + 1] = i;
        } else {
            right = gamma + 1;
            iparent[gamma + 1] = i;
        }
        child[i] = make_int2(left, right);
        if (i == 0) iparent[0] = -1;
    }
}

// Bottom-up boxes over tiles of kTileLeaves consecutive leaves, one thread per leaf. A Karras node covers a
// contiguous leaf range with its own index at one end, so every node whose range lies inside a tile has its
// index inside the tile too: those nodes count arrivals and keep their boxes in shared memory (the tile's leaf
// boxes are staged there as well). A chain that reaches a node whose range leaves the tile counts its arrival
// there in global memory (visit[], zeroed by the leaf kernels), with its own box in nlo/nhi; the second arrival
// queues the node (upq: count, then nodes) and stops, and k_bottom_up_upper finishes the nodes above the tiles,
// so a block never waits at its next tile for a chain climbing the upper tree. The second arrival at a node
// writes its packed record (kPack) and, with kNodes, its box to nlo/nhi. A node's range, children and parent are
// loaded together before its arrival count.
constexpr int kTileLeaves = 512;
constexpr int kTileThreads = kTileLeaves;

// Arrival counts of the bottom-up pass: a release add (the arriving child's box, stored before, becomes visible
// with the count) and an acquire-release add (the second arrival also sees the first child's box).
__device__ __forceinline__ int arrive_release(int* p) {
    int old;
    asm volatile("atom.release.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}
__device__ __forceinline__ int arrive_acq_rel(int* p) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

// The packed 64-byte record of node p (both children's boxes, child references, leaf face ids with the query bit).
__device__ __forceinline__ void write_packed(int p, int2 c, float4 alo, float4 ahi, float4 clo, float4 chi,
                                             const int* leaf_face, const int* qscan, float4* packed) {
    int fa = -1, fc = -1;
    if (c.x < 0) {
        fa = leaf_face[~c.x];
        if (qscan && fa >= 0 && qscan[fa + 1] != qscan[fa]) fa |= kQueryBit;
    }
    if (c.y < 0) {
        fc = leaf_face[~c.y];
        if (qscan && fc >= 0 && qscan[fc + 1] != qscan[fc]) fc |= kQueryBit;
    }
    float4* rec = packed + 4 * (size_t)p;
    alo.w = __int_as_float(c.x);
    ahi.w = __int_as_float(fa);
    clo.w = __int_as_float(c.y);
    chi.w = __int_as_float(fc);
    rec[0] = alo;
    rec[1] = ahi;
    rec[2] = clo;
    rec[3] = chi;
}

// From node p, both of whose children are done: its box from the children's boxes in global memory (and its
// packed record), then on to the parent as long as this is the parent's second arrival.
template <bool kPack>
__device__ void climb_from(RoundCounters* rc, int p, const int2* child, const int* iparent, const float4* llo,
                           const float4* lhi, float4* nlo, float4* nhi, int* visit, const int* leaf_face,
                           const int* qscan, float4* packed) {
    {
        int guard = 0;
        int2 c = child[p];
        int pp = iparent[p];
        while (p >= 0) {
            if (++guard > 4096) {
                atomicOr(&rc->status, kErrIterLimit);
                break;
            }
            float4 alo, ahi, clo, chi;
            if (c.x < 0) { alo = __ldcg(&llo[~c.x]); ahi = __ldcg(&lhi[~c.x]); }
            else { alo = __ldcg(&nlo[c.x]); ahi = __ldcg(&nhi[c.x]); }
            if (c.y < 0) { clo = __ldcg(&llo[~c.y]); chi = __ldcg(&lhi[~c.y]); }
            else { clo = __ldcg(&nlo[c.y]); chi = __ldcg(&nhi[c.y]); }
            const float4 blo = make_float4(fminf(alo.x, clo.x), fminf(alo.y, clo.y), fminf(alo.z, clo.z), 0.f);
            const float4 bhi = make_float4(fmaxf(ahi.x, chi.x), fmaxf(ahi.y, chi.y), fmaxf(ahi.z, chi.z), 0.f);
            __stcg(&nlo[p], blo);  // the parent's second arrival reads it
            __stcg(&nhi[p], bhi);
            if (kPack) write_packed(p, c, alo, ahi, clo, chi, leaf_face, qscan, packed);
            if (pp < 0) break;
            // the parent's topology is fixed: loaded before its arrival count, not after
            const int2 cn = child[pp];
            const int ppn = iparent[pp];
            if (arrive_acq_rel(&visit[pp]) == 0) break;
            p = pp;
            c = cn;
            pp = ppn;
        }
    }
}

template <bool kPack, bool kNodes>
__global__ void __launch_bounds__(kTileThreads, 3) k_bottom_up_tiles(RoundCounters* rc, const int2* child,
                                                                  const int* iparent, const int* lparent,
                                                                  const int2* range, const float4* llo,
                                                                  const float4* lhi, float4* nlo, float4* nhi, int* visit,
                                                                  const int* leaf_face, const int* qscan, float4* packed,
                                                                  int* meta_out, const int* active, int* upq) {
    __shared__ int svisit[kTileLeaves];
    __shared__ float4 slo[kTileLeaves], shi[kTileLeaves];    // internal nodes a .. b-2
    __shared__ float4 sllo[kTileLeaves], slhi[kTileLeaves];  // leaves a .. b-1
    if (active && *active == 0) return;
    const int n = rc->n_live;
    if (kPack && blockIdx.x == 0 && threadIdx.x == 0) meta_out[0] = n;
    // one tile per block (a single wave): a chain leaving its tile climbs on here, nothing waits for it; several
    // tiles per block: the nodes above the tiles are queued for k_bottom_up_upper
    const bool climb = (long long)gridDim.x * kTileLeaves >= n;
    // tiles in a block-stride loop: the leaf count is read on the device and may exceed the launch's bound
    for (int a = blockIdx.x * kTileLeaves; a < n; a += gridDim.x * kTileLeaves) {
        const int b = min(a + kTileLeaves, n);  // leaves [a, b)
        const int leaf = a + threadIdx.x;
        __syncthreads();  // the previous tile's shared state is no longer read
        svisit[threadIdx.x] = 0;
        float4 blo = make_float4(0.f, 0.f, 0.f, 0.f), bhi = blo;
        int p = -1;
        if (leaf < b) {
            blo = __ldcg(&llo[leaf]);
            bhi = __ldcg(&lhi[leaf]);
            sllo[threadIdx.x] = blo;
            slhi[threadIdx.x] = bhi;
            p = lparent[leaf];
        }
        __syncthreads();
        int ref = ~leaf;
        int guard = 0;
        while (p >= 0) {
            if (++guard > 4096) {
                atomicOr(&rc->status, kErrIterLimit);
                break;
            }
            const int2 rg = range[p];
            const int2 c = child[p];
            const int pp = iparent[p];
            if (!(rg.x >= a && rg.y < b)) {
                // leaving the tile: this child's box goes to global memory for the other child's chain; with
                // several tiles per block the second arrival queues p for k_bottom_up_upper instead of climbing
                // on, so that no chain through the upper tree holds this block at the next tile's barrier
                if (ref >= 0 && !kNodes) {
                    __stcg(&nlo[ref], blo);
                    __stcg(&nhi[ref], bhi);
                }
                if (!climb) {
                    if (arrive_release(&visit[p]) != 0) upq[1 + atomicAdd(upq, 1)] = p;
                } else if (arrive_acq_rel(&visit[p]) != 0) {
                    climb_from<kPack>(rc, p, child, iparent, llo, lhi, nlo, nhi, visit, leaf_face, qscan, packed);
                }
                break;
            }
            __threadfence_block();
            if (atomicAdd(&svisit[p - a], 1) == 0) break;
            __threadfence_block();
            // both children are in this tile
            float4 alo, ahi, clo, chi;
            if (c.x < 0) { alo = sllo[~c.x - a]; ahi = slhi[~c.x - a]; }
            else { alo = slo[c.x - a]; ahi = shi[c.x - a]; }
            if (c.y < 0) { clo = sllo[~c.y - a]; chi = slhi[~c.y - a]; }
            else { clo = slo[c.y - a]; chi = shi[c.y - a]; }
            blo = make_float4(fminf(alo.x, clo.x), fminf(alo.y, clo.y), fminf(alo.z, clo.z), 0.f);
            bhi = make_float4(fmaxf(ahi.x, chi.x), fmaxf(ahi.y, chi.y), fmaxf(ahi.z, chi.z), 0.f);
            slo[p - a] = blo;
            shi[p - a] = bhi;
            if (kNodes) {
                __stcg(&nlo[p], blo);
                __stcg(&nhi[p], bhi);
            }
            if (kPack) write_packed(p, c, alo, ahi, clo, chi, leaf_face, qscan, packed);
            ref = p;
            p = pp;
        }
    }
}

// The nodes above the tiles (their leaf ranges span two tiles or more): each queued node (both children done)
// takes its box from the children's boxes in global memory, and climbs on as the second arrival at each parent.
template <bool kPack, bool kNodes>
__global__ void __launch_bounds__(256) k_bottom_up_upper(RoundCounters* rc, const int2* child, const int* iparent,
                                                         const float4* llo, const float4* lhi, float4* nlo,
                                                         float4* nhi, int* visit, const int* leaf_face,
                                                         const int* qscan, float4* packed, const int* upq,
                                                         const int* active) {
    if (active && *active == 0) return;
    const int nq = upq[0];
    for (int k = gtid(); k < nq; k += gstride())
        climb_from<kPack>(rc, upq[1 + k], child, iparent, llo, lhi, nlo, nhi, visit, leaf_face, qscan, packed);
}

// blocks for k_bottom_up_tiles: a tile per block up to the resident count (the bound may be capped below the
// leaf count, which the block-stride loop covers)
inline int tile_grid(int n_bound) {
    int g = (n_bound + kTileLeaves - 1) / kTileLeaves;
    if (n_bound >= (1 << 19) && g < 3 * kNumSM) g = 3 * kNumSM;
    return g < 1 ? 1 : g;
}

// The whole bottom-up pass: the tiles, then the nodes above them.
template <bool kPack, bool kNodes>
void bottom_up(BvhBuffers& b, RoundCounters* rc, int n_bound, const int* leaf_face, const int* qscan, int* meta_out,
               const int* active, cudaStream_t s) {
    cudaMemsetAsync(b.upq, 0, sizeof(int), s);
    const int gT = tile_grid(n_bound);
    k_bottom_up_tiles<kPack, kNodes><<<gT, kTileThreads, 0, s>>>(rc, b.child, b.iparent, b.lparent, b.range, b.llo,
                                                                 b.lhi, b.nlo, b.nhi, b.visit, leaf_face, qscan,
                                                                 b.packed, meta_out, active, b.upq);
    note_launch();
    const int gU = std::max(1, std::min(gT, 4 * kNumSM));
    k_bottom_up_upper<kPack, kNodes><<<gU, 256, 0, s>>>(rc, b.child, b.iparent, b.llo, b.lhi, b.nlo, b.nhi, b.visit,
                                                        leaf_face, qscan, b.packed, b.upq, active);
    note_launch();
}

// ---------------------------------------------------------------- localized query
// 1. k_query_order: the query faces in leaf (Morton) order, so that neighbouring threads walk the same
//    part of the tree and test neighbouring faces.
// 2. k_traverse_list: one thread per query face walks the tree with a short stack in shared memory and emits
//    every overlapping leaf g as a candidate pair (f, g); a pair of two query faces is emitted only by the lower
//    face index. Queries that overflow the list or the stack walk again (k_traverse_redo) and decide in place.
// 3. k_pairs: one thread per candidate pair runs the reference's decision in both orders (float
//    certificates first, the fp64 path only for undecided pairs) and flags both faces when it holds.
__device__ __forceinline__ bool decide_pair(int f, int g, const int4* __restrict__ tri, const float4* __restrict__ pos,
                                            float eps, unsigned& exact) {
    const int4 qt = tri[f], gt = tri[g];
    // two or three shared vertex indices: no intersection in either order (pair_certainly_disjoint), decided
    // before the positions are loaded (edge-adjacent faces are about a quarter of the candidate pairs)
    const int shared = (qt.x == gt.x) + (qt.x == gt.y) + (qt.x == gt.z) + (qt.y == gt.x) + (qt.y == gt.y) +
                       (qt.y == gt.z) + (qt.z == gt.x) + (qt.z == gt.y) + (qt.z == gt.z);
    if (shared >= 2) return false;
    const float4 q0 = pos[qt.x], q1 = pos[qt.y], q2 = pos[qt.z];
    const float4 g0 = pos[gt.x], g1 = pos[gt.y], g2 = pos[gt.z];
    PairGeom ga, gb;
    pair_geom(g0, g1, g2, gt, q0, q1, q2, qt, ga);  // reference order: the hit is "current"
    pair_geom(q0, q1, q2, qt, g0, g1, g2, gt, gb);  // the order seen from g's own query
    const bool need_a = !pair_certainly_disjoint(ga);
    const bool need_b = !pair_certainly_disjoint(gb);
    if (!need_a && !need_b) return false;
    exact += (unsigned)need_a + (unsigned)need_b;
    return (need_a && pair_decide_exact(g0, g1, g2, gt, q0, q1, q2, qt, eps)) ||
           (need_b && pair_decide_exact(q0, q1, q2, qt, g0, g1, g2, gt, eps));
}

__global__ void __launch_bounds__(256) k_query_order(const RoundCounters* rc, const int* __restrict__ leaf_face,
                                                     const int* __restrict__ qscan, int* flags) {
    const int n = rc->n_live;
    for (int i = gtid(); i < n; i += gstride()) {
        const int f = leaf_face[i];
        flags[i] = (f >= 0 && qscan[f + 1] != qscan[f]) ? 1 : 0;  // f < 0: a leaf whose face is gone
    }
    if (gtid() == 0) flags[n] = 0;
}

__global__ void __launch_bounds__(256) k_query_gather(const RoundCounters* rc, const int* __restrict__ leaf_face,
                                                      const int* __restrict__ scan, int* qsorted) {
    const int n = rc->n_live;
    for (int i = gtid(); i < n; i += gstride())
        if (scan[i + 1] != scan[i]) qsorted[scan[i]] = leaf_face[i];
}

__device__ __forceinline__ bool box_overlap4(float4 qlo, float4 qhi, float4 lo, float4 hi) {
    return !(qhi.x < lo.x || hi.x < qlo.x || qhi.y < lo.y || hi.y < qlo.y || qhi.z < lo.z || hi.z < qlo.z);
}

// First walk: candidate pairs go to the pair list. The loop is flat: a thread whose query is done takes its
// next query in the same iteration in which the other lanes of its warp take their next node, so the lanes
// stay busy until the warp runs out of queries. From then on, a lane without work takes the bottom entry of the
// pending stack of a lane that has some (the subtree nearest the root, the largest), together with that lane's query
// face and box, so that a few long walks are shared by the warp instead of setting the launch's time. A walk whose
// pair does not fit the list, or whose deferred siblings do not fit the short stack, stops and marks its query in
// redo[] (counted in rc->pad[3]) for the second walk.
// With fmesh, a query walks only the subtree of its own mesh (mesh_root; < 0: the mesh has one leaf, no pair).
__device__ __forceinline__ int query_root(int f, const int* __restrict__ fmesh, const int* __restrict__ mesh_root) {
    return fmesh ? mesh_root[fmesh[f]] : 0;
}

// the lane of the r-th set bit of m (r < popc(m))
__device__ __forceinline__ int nth_lane(unsigned m, int r) {
    for (int k = 0; k < r; ++k) m &= m - 1u;
    return __ffs(m) - 1;
}

__global__ void __launch_bounds__(kQueryThreads) k_traverse_list(const float4* __restrict__ packed,
                                                                  const float4* __restrict__ box_lo,
                                                                  const float4* __restrict__ box_hi,
                                                                  const int* __restrict__ qsorted, int2* pairs_out,
                                                                  int pair_cap, RoundCounters* rc, int* redo,
                                                                  const int* __restrict__ fmesh,
                                                                  const int* __restrict__ mesh_root) {
    __shared__ int stack[kShortStack][kQueryThreads];
    int* n_list = &rc->pad[1];
    const int nq = rc->pad[2];
    const bool empty = rc->n_live < 2;
    unsigned long long npairs = 0;
    // each lane fills its own chunk of kPairChunk list slots, so that one atomic on the list length serves
    // many pairs (a single counter is an L2 hot spot); unused slots of a lane's last chunk are set to -1
    const int lane = threadIdx.x & 31;
    const unsigned lower = (1u << lane) - 1u;
    int cbase = -1, cused = kPairChunk;
    int qi = gtid() - gstride();  // this lane's query iterator
    int wq = -1;                  // the query of the current walk (the lane's own or a shared one)
    bool supply = true;           // this lane may still get queries of its own
    int f = 0, node = -1, sp = 0, bot = 0, guard = 0;  // pending entries: stack[bot .. sp)
    float4 qlo = make_float4(0.f, 0.f, 0.f, 0.f), qhi = qlo;
    while (true) {
        if (node < 0 && supply) {
            qi += gstride();
            if (qi >= nq) {
                supply = false;
            } else {
                redo[qi] = 0;
                if (!empty) {
                    f = qsorted[qi];
                    node = query_root(f, fmesh, mesh_root);
                    if (node >= 0) {
                        wq = qi;
                        qlo = box_lo[f];
                        qhi = box_hi[f];
                        sp = bot = 0;
                        guard = 0;
                    }
                }
            }
        }
        // sharing, once lanes are out of queries (every lane takes part: the shuffles need the whole warp)
        const bool idle = node < 0 && !supply;
        const unsigned I = __ballot_sync(0xffffffffu, idle);
        if (I == 0xffffffffu) break;
        const unsigned D = __ballot_sync(0xffffffffu, node >= 0 && sp > bot);
        if (I != 0u && D != 0u) {
            int partner = -1;
            if (idle) {
                const int r = __popc(I & lower);
                if (r < __popc(D)) partner = nth_lane(D, r);
            } else if ((D >> lane) & 1u) {
                const int r = __popc(D & lower);
                if (r < __popc(I)) partner = nth_lane(I, r);
            }
            int give = -1;
            if (!idle && partner >= 0) give = stack[bot++][threadIdx.x];
            const int src = (idle && partner >= 0) ? partner : lane;
            const int g_node = __shfl_sync(0xffffffffu, give, src);
            const int g_f = __shfl_sync(0xffffffffu, f, src);
            const int g_wq = __shfl_sync(0xffffffffu, wq, src);
            const float4 g_lo = make_float4(__shfl_sync(0xffffffffu, qlo.x, src), __shfl_sync(0xffffffffu, qlo.y, src),
                                            __shfl_sync(0xffffffffu, qlo.z, src), 0.f);
            const float4 g_hi = make_float4(__shfl_sync(0xffffffffu, qhi.x, src), __shfl_sync(0xffffffffu, qhi.y, src),
                                            __shfl_sync(0xffffffffu, qhi.z, src), 0.f);
            if (idle && partner >= 0) {
                node = g_node;
                f = g_f;
                wq = g_wq;
                qlo = g_lo;
                qhi = g_hi;
                sp = bot = 0;
                guard = 0;
            }
        }
        if (node < 0) continue;
        if (++guard > (1 << 22)) {
            atomicOr(&rc->status, kErrIterLimit);
            node = -1;
            continue;
        }
        const float4* rec = packed + 4 * (size_t)node;
        const float4 alo = __ldg(rec), ahi = __ldg(rec + 1), blo = __ldg(rec + 2), bhi = __ldg(rec + 3);
        int next[2];
        int nn = 0;
        bool abandon = false;
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const float4 lo = side ? blo : alo, hi = side ? bhi : ahi;
            if (!box_overlap4(qlo, qhi, lo, hi)) continue;
            const int x = __float_as_int(lo.w);
            if (x < 0) {
                const int graw = __float_as_int(hi.w);
                const int g = graw & ~kQueryBit;
                if (g == f) continue;
                if (g < f && (graw & kQueryBit)) continue;  // the lower query face owns the pair
                if (cused == kPairChunk) {
                    const unsigned am = __activemask();
                    const int leader = __ffs(am) - 1;
                    int b = 0;
                    if (lane == leader) b = atomicAdd(n_list, kPairChunk * __popc(am));
                    b = __shfl_sync(am, b, leader);
                    cbase = b + kPairChunk * __popc(am & lower);
                    cused = 0;
                }
                const int at = cbase + cused++;
                if (at < pair_cap) {
                    pairs_out[at] = make_int2(f, g);
                    ++npairs;
                } else {
                    abandon = true;
                }
            } else {
                next[nn++] = x;
            }
        }
        if (nn == 2) {
            if (sp >= kShortStack && bot > 0) {  // entries given away at the bottom: move the rest down
                for (int k = bot; k < sp; ++k) stack[k - bot][threadIdx.x] = stack[k][threadIdx.x];
                sp -= bot;
                bot = 0;
            }
            if (sp >= kShortStack) {
                abandon = true;
            } else {
                stack[sp++][threadIdx.x] = next[1];
                node = next[0];
            }
        } else if (nn == 1) {
            node = next[0];
        } else {
            node = sp > bot ? stack[--sp][threadIdx.x] : -1;
        }
        if (abandon) {
            redo[wq] = 1;
            atomicAdd(&rc->pad[3], 1);
            node = -1;
        }
    }
    if (cbase >= 0)
        for (int k = cused; k < kPairChunk && cbase + k < pair_cap; ++k) pairs_out[cbase + k] = make_int2(-1, -1);
    __syncwarp();
    for (int o = 16; o > 0; o >>= 1) npairs += __shfl_xor_sync(0xffffffffu, npairs, o);
    if (lane == 0 && npairs) atomicAdd(&rc->n_pairs, npairs);
}

// Second walk, only when the first marked queries: each marked query walks the whole tree again with a stack
// deep enough for any tree (the Karras split prefix grows by at least one of the 62 key bits per level) and
// decides every pair in place (pairs already listed are decided twice, which sets the same flags).
__global__ void __launch_bounds__(kQueryThreads) k_traverse_redo(const float4* __restrict__ packed,
                                                                  const float4* __restrict__ box_lo,
                                                                  const float4* __restrict__ box_hi,
                                                                  const int4* __restrict__ tri,
                                                                  const float4* __restrict__ pos,
                                                                  const int* __restrict__ qsorted, unsigned char* hit,
                                                                  RoundCounters* rc, float eps, const int* redo,
                                                                  const int* __restrict__ fmesh,
                                                                  const int* __restrict__ mesh_root) {
    __shared__ int stack[kStackDepth][kQueryThreads];
    if (rc->pad[3] == 0) return;
    const int nq = rc->pad[2];
    unsigned exact = 0;
    for (int qi = gtid(); qi < nq; qi += gstride()) {
        if (redo[qi] == 0) continue;
        const int f = qsorted[qi];
        int node = query_root(f, fmesh, mesh_root);
        if (node < 0) continue;
        const float4 qlo = box_lo[f], qhi = box_hi[f];
        int sp = 0;
        int guard = 0;
        while (true) {
            if (++guard > (1 << 22)) {
                atomicOr(&rc->status, kErrIterLimit);
                break;
            }
            const float4* rec = packed + 4 * (size_t)node;
            const float4 alo = __ldg(rec), ahi = __ldg(rec + 1), blo = __ldg(rec + 2), bhi = __ldg(rec + 3);
            int next[2];
            int nn = 0;
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const float4 lo = side ? blo : alo, hi = side ? bhi : ahi;
                if (!box_overlap4(qlo, qhi, lo, hi)) continue;
                const int x = __float_as_int(lo.w);
                if (x < 0) {
                    const int graw = __float_as_int(hi.w);
                    const int g = graw & ~kQueryBit;
                    if (g == f) continue;
                    if (g < f && (graw & kQueryBit)) continue;
                    if (decide_pair(f, g, tri, pos, eps, exact)) {
                        hit[f] = 1;
                        hit[g] = 1;
                    }
                } else {
                    next[nn++] = x;
                }
            }
            if (nn == 2) {
                if (sp >= kStackDepth) {
                    atomicOr(&rc->status, kErrStackOverflow);
                    break;
                }
                stack[sp++][threadIdx.x] = next[1];
                node = next[0];
            } else if (nn == 1) {
                node = next[0];
            } else {
                if (sp == 0) break;
                node = stack[--sp][threadIdx.x];
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) exact += __shfl_xor_sync(0xffffffffu, exact, o);
    if ((threadIdx.x & 31) == 0 && exact) atomicAdd(&rc->n_exact, (unsigned long long)exact);
}

// k_pairs decides every listed pair by the float certificates; each order of a pair they cannot decide (the float64
// path, a few pairs in a thousand) is queued in xq, and k_pairs_exact runs those one per thread spread over every SM
// (decided where they were listed, they clustered in a few warps and the float64 pipes of a few SMs set the time).
// An order that finds the queue full is decided in place. Either way it sets the same flags.
__global__ void __launch_bounds__(128, 8) k_pairs(const int4* __restrict__ tri, const float4* __restrict__ pos,
                                               const int2* __restrict__ pair_list, int pair_cap, unsigned char* hit,
                                               RoundCounters* rc, float eps, int4* xq, int xq_cap, int* xq_count) {
    const int n = min(rc->pad[1], pair_cap);
    unsigned exact = 0;
    for (int i = gtid(); i < n; i += gstride()) {
        const int2 pr = pair_list[i];
        if (pr.x < 0) continue;  // an unused slot of a chunk
        const int f = pr.x, g = pr.y;
        const int4 qt = tri[f], gt = tri[g];
        // two or three shared vertex indices: no intersection in either order (pair_certainly_disjoint), decided
        // before the positions are loaded (edge-adjacent faces are about a quarter of the candidate pairs)
        const int shared = (qt.x == gt.x) + (qt.x == gt.y) + (qt.x == gt.z) + (qt.y == gt.x) + (qt.y == gt.y) +
                           (qt.y == gt.z) + (qt.z == gt.x) + (qt.z == gt.y) + (qt.z == gt.z);
        if (shared >= 2) continue;
        const float4 q0 = pos[qt.x], q1 = pos[qt.y], q2 = pos[qt.z];
        const float4 g0 = pos[gt.x], g1 = pos[gt.y], g2 = pos[gt.z];
        PairGeom ga, gb;
        pair_geom(g0, g1, g2, gt, q0, q1, q2, qt, ga);  // reference order: the hit is "current"
        pair_geom(q0, q1, q2, qt, g0, g1, g2, gt, gb);  // the order seen from g's own query
        const bool need_a = !pair_certainly_disjoint(ga);
        const bool need_b = !pair_certainly_disjoint(gb);
        if (!need_a && !need_b) continue;
        exact += (unsigned)need_a + (unsigned)need_b;
        // one queue slot per order, taken for the whole warp by one atomic
        const unsigned am = __activemask();
        const int lane = threadIdx.x & 31, leader = __ffs(am) - 1;
        const unsigned ma = __ballot_sync(am, need_a), mb = __ballot_sync(am, need_b);
        int base = 0;
        if (lane == leader) base = atomicAdd(xq_count, __popc(ma) + __popc(mb));
        base = __shfl_sync(am, base, leader);
        const unsigned lower = (1u << lane) - 1u;
        const int at_a = base + __popc(ma & lower), at_b = base + __popc(ma) + __popc(mb & lower);
        bool h = false;
        if (need_a) {
            if (at_a < xq_cap) xq[at_a] = make_int4(f, g, 1, 0);
            else h = pair_decide_exact(g0, g1, g2, gt, q0, q1, q2, qt, eps);
        }
        if (need_b) {
            if (at_b < xq_cap) xq[at_b] = make_int4(f, g, 2, 0);
            else if (!h) h = pair_decide_exact(q0, q1, q2, qt, g0, g1, g2, gt, eps);
        }
        if (h) {
            hit[f] = 1;
            hit[g] = 1;
        }
    }
    for (int o = 16; o > 0; o >>= 1) exact += __shfl_xor_sync(0xffffffffu, exact, o);
    if ((threadIdx.x & 31) == 0 && exact) atomicAdd(&rc->n_exact, (unsigned long long)exact);
}

// The queued pairs, one per thread, consecutive pairs on different SMs (block-cyclic: item k goes to block
// k mod blocks).
__global__ void __launch_bounds__(64) k_pairs_exact(const int4* __restrict__ tri, const float4* __restrict__ pos,
                                                    const int4* __restrict__ xq, int xq_cap,
                                                    const int* __restrict__ xq_count, unsigned char* hit, float eps) {
    const int n = min(*xq_count, xq_cap);
    for (long long k = (long long)threadIdx.x * gridDim.x + blockIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int4 e = xq[k];
        const int f = e.x, g = e.y;
        const int4 qt = tri[f], gt = tri[g];
        const float4 q0 = pos[qt.x], q1 = pos[qt.y], q2 = pos[qt.z];
        const float4 g0 = pos[gt.x], g1 = pos[gt.y], g2 = pos[gt.z];
        const bool h = e.z == 1 ? pair_decide_exact(g0, g1, g2, gt, q0, q1, q2, qt, eps)
                                : pair_decide_exact(q0, q1, q2, qt, g0, g1, g2, gt, eps);
        if (h) {
            hit[f] = 1;
            hit[g] = 1;
        }
    }
}

// The subtree root of each mesh: its live faces are the leaves [live_scan[f0], live_scan[f0 + nf]) of a tree built
// with mesh keys; a Karras node has one end of its range at its own index, so the node covering exactly that range
// is internal node lo or hi. -1 for a mesh with fewer than two leaves.
__global__ void k_mesh_roots(const RoundCounters* rc, const int* __restrict__ live_scan, const int2* __restrict__ range,
                             const int* __restrict__ mesh_f0, const int* __restrict__ mesh_nf, const int* d_count,
                             int* root) {
    const int n = *d_count;
    const int n_live = rc->n_live;
    for (int m = gtid(); m < n; m += gstride()) {
        const int lo = live_scan[mesh_f0[m]], hi = live_scan[mesh_f0[m] + mesh_nf[m]] - 1;
        int r = -1;
        if (hi > lo && n_live >= 2) {
            const int2 a = range[lo];
            r = (a.x == lo && a.y == hi) ? lo : hi;
        }
        root[m] = r;
    }
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

size_t bvh_bytes(int cap) {
    size_t c = (size_t)cap + 1;
    size_t b = 0;
    b += 2 * align256(16 * c);              // box_lo / hi
    b += align256(4 * (c + 1));             // live_scan
    b += 2 * align256(4 * c);               // keys
    b += 2 * align256(4 * c);               // vals
    b += align256(4 * (256 * (size_t)kSortTiles + 1));
    b += align256(8 * c);                   // child
    b += align256(8 * c);                   // range
    b += 2 * align256(4 * c);               // iparent, lparent
    b += 4 * align256(16 * c);              // nlo nhi llo lhi
    b += align256(4 * c);                   // visit
    b += align256(4 * (c + 1));             // upq
    b += align256(16 * std::min<size_t>(c, kExactQueue) + 16);  // xq and its count
    b += align256(4 * 8);                   // scene
    b += align256(4 * scan_scratch_ints());
    b += align256(64 * c);                  // packed internal nodes
    b += align256(16);                      // meta
    return b;
}

void bvh_carve(BvhBuffers& b, int cap, char* base, bool clear_scan_scratch) {
    size_t c = (size_t)cap + 1;
    char* p = base;
    auto take = [&](size_t bytes) {
        char* r = p;
        p += align256(bytes);
        return r;
    };
    b.cap = cap;
    b.box_lo = (float4*)take(16 * c);
    b.box_hi = (float4*)take(16 * c);
    b.live_scan = (int*)take(4 * (c + 1));
    b.keys[0] = (unsigned*)take(4 * c);
    b.keys[1] = (unsigned*)take(4 * c);
    b.vals[0] = (int*)take(4 * c);
    b.vals[1] = (int*)take(4 * c);
    b.hist = (int*)take(4 * (256 * (size_t)kSortTiles + 1));
    b.child = (int2*)take(8 * c);
    b.range = (int2*)take(8 * c);
    b.iparent = (int*)take(4 * c);
    b.lparent = (int*)take(4 * c);
    b.nlo = (float4*)take(16 * c);
    b.nhi = (float4*)take(16 * c);
    b.llo = (float4*)take(16 * c);
    b.lhi = (float4*)take(16 * c);
    b.visit = (int*)take(4 * c);
    b.upq = (int*)take(4 * (c + 1));
    b.xq_cap = (int)std::min<size_t>(c, kExactQueue);
    b.xq = (int4*)take(16 * (size_t)b.xq_cap + 16);
    b.xq_count = reinterpret_cast<int*>(b.xq + b.xq_cap);
    b.scene = (unsigned*)take(4 * 8);
    b.scan_scratch = (int*)take(4 * scan_scratch_ints());
    b.packed = (float4*)take(64 * c);
    b.meta = (int*)take(16);
    if (clear_scan_scratch) scan_scratch_clear(b.scan_scratch);
}

void bvh_build(BvhBuffers& b, const int4* tri, const float4* pos, RoundCounters* rc, int n_tris_bound, cudaStream_t s,
               bool all_faces, const int* qscan, bool nodes, const BvhMeshes* meshes) {
    cudaMemsetAsync(b.scene, 0xFF, 3 * sizeof(unsigned), s);
    cudaMemsetAsync(b.scene + 3, 0x00, 3 * sizeof(unsigned), s);
    const int gF = grid_for(n_tris_bound, 256);
    k_boxes<<<gF, 256, 0, s>>>(tri, pos, rc, b.box_lo, b.box_hi, b.live_scan, b.scene, all_faces ? 1 : 0); note_launch();
    exclusive_scan(b.live_scan, b.live_scan, &rc->n_tris, 1, &rc->n_live, b.scan_scratch, s, &rc->status, n_tris_bound);
    k_morton<<<gF, 256, 0, s>>>(rc, b.live_scan, b.box_lo, b.box_hi, b.scene, b.keys[0], b.vals[0],
                                meshes ? meshes->fmesh : nullptr, meshes ? meshes->bits : 0); note_launch();
    // sort tiles from the launch's bound (about 2048 keys per tile; all kSortTiles from 2^19 on, where callers
    // cap their bounds); the histogram is
    // digit-major over the tiles, so its scan gives each tile's output offset per digit
    long long st = n_tris_bound >= (1 << 19) ? kSortTiles : ((long long)n_tris_bound + 2047) / 2048;
    const int sort_tiles = (int)(st < 1 ? 1 : (st > kSortTiles ? kSortTiles : st));
    for (int pass = 0; pass < 4; ++pass) {
        const int in = pass & 1, out = in ^ 1;
        k_rs_hist<<<sort_tiles, kSortThreads, 0, s>>>(b.keys[in], &rc->n_live, 8 * pass, b.hist); note_launch();
        exclusive_scan(b.hist, b.hist, nullptr, 256 * sort_tiles, nullptr, b.scan_scratch, s, &rc->status, 0);
        k_rs_scatter<<<sort_tiles, kSortThreads, 0, s>>>(b.keys[in], b.vals[in], b.keys[out], b.vals[out], &rc->n_live,
                                                         8 * pass, b.hist); note_launch();
    }
    k_leaves<<<gF, 256, 0, s>>>(rc, b.vals[0], b.box_lo, b.box_hi, b.llo, b.lhi, b.visit, b.lparent); note_launch();
    k_karras<<<gF, 256, 0, s>>>(rc, b.keys[0], b.child, b.iparent, b.lparent, b.range); note_launch();
    if (meshes) {
        k_mesh_roots<<<grid_for(meshes->count_bound, 256), 256, 0, s>>>(rc, b.live_scan, b.range, meshes->f0, meshes->nf,
                                                                          meshes->d_count, meshes->root);
        note_launch();
    }
    if (nodes) bottom_up<true, true>(b, rc, n_tris_bound, b.vals[0], qscan, b.meta, nullptr, s);
    else bottom_up<true, false>(b, rc, n_tris_bound, b.vals[0], qscan, b.meta, nullptr, s);
}

__global__ void __launch_bounds__(256) k_refit_leaves(const RoundCounters* rc, const int4* __restrict__ tri,
                                                      const float4* __restrict__ pos, const int* __restrict__ vals,
                                                      float4* llo, float4* lhi, int* visit, const int* active) {
    if (active && *active == 0) return;
    const int n = rc->n_live;
    for (int i = gtid(); i < n; i += gstride()) {
        const int4 t = tri[vals[i]];
        const float4 a = pos[t.x], b = pos[t.y], c = pos[t.z];
        llo[i] = make_float4(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)), 0.f);
        lhi[i] = make_float4(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)), 0.f);
        if (i < n - 1) visit[i] = 0;
    }
}

void bvh_refit(BvhBuffers& b, const int4* tri, const float4* pos, RoundCounters* rc, int n_tris_bound, cudaStream_t s,
               const int* active) {
    const int gF = grid_for(n_tris_bound, 256);
    k_refit_leaves<<<gF, 256, 0, s>>>(rc, tri, pos, b.vals[0], b.llo, b.lhi, b.visit, active); note_launch();
    bottom_up<false, true>(b, rc, n_tris_bound, nullptr, nullptr, nullptr, active, s);
}

__global__ void __launch_bounds__(256) k_reuse_leaves(RoundCounters* rc, const int4* __restrict__ tri,
                                                      const float4* __restrict__ box_lo, const float4* __restrict__ box_hi,
                                                      const int* __restrict__ new_ids, int* leaf_face, float4* llo,
                                                      float4* lhi, int* visit, const int* meta) {
    const int n = meta[0];
    if (gtid() == 0) rc->n_live = n;
    for (int i = gtid(); i < n; i += gstride()) {
        int f;
        if (new_ids) {
            f = new_ids[i];
            leaf_face[i] = f;
        } else {
            f = leaf_face[i];
        }
        if (f >= 0 && tri[f].x != -1) {
            llo[i] = box_lo[f];
            lhi[i] = box_hi[f];
        } else {
            llo[i] = make_float4(INFINITY, INFINITY, INFINITY, 0.f);
            lhi[i] = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
        }
        if (i < n - 1) visit[i] = 0;
    }
}

// next[i] = the leaf's face in the next numbering; reads the current ids only, so it can be repeated
__global__ void __launch_bounds__(256) k_remap_leaves(const int* meta, const int* __restrict__ fscan,
                                                      const int* __restrict__ leaf_face, int* next) {
    const int n = meta[0];
    for (int i = gtid(); i < n; i += gstride()) {
        const int f = leaf_face[i];
        next[i] = (f >= 0 && fscan[f + 1] != fscan[f]) ? fscan[f] : -1;
    }
}

void bvh_refit_faces(BvhBuffers& b, const int4* tri, const float4* pos, RoundCounters* rc, int n_tris_bound,
                     cudaStream_t s, bool next_round, const int* qscan) {
    const int gF = grid_for(n_tris_bound, 256);
    k_boxes<<<gF, 256, 0, s>>>(tri, pos, rc, b.box_lo, b.box_hi, b.live_scan, b.scene, 1); note_launch();
    k_reuse_leaves<<<gF, 256, 0, s>>>(rc, tri, b.box_lo, b.box_hi, next_round ? (const int*)b.keys[1] : nullptr,
                                      b.vals[0], b.llo, b.lhi, b.visit, b.meta); note_launch();
    bottom_up<true, false>(b, rc, n_tris_bound, b.vals[0], qscan, b.meta, nullptr, s);
}

void bvh_remap(BvhBuffers& b, const int* fscan, int n_tris_bound, cudaStream_t s) {
    k_remap_leaves<<<grid_for(n_tris_bound, 256), 256, 0, s>>>(b.meta, fscan, b.vals[0], (int*)b.keys[1]);
    note_launch();
}

void bvh_query(const BvhBuffers& b, const int4* tri, const float4* pos, const int* qlist, const int* qscan,
               unsigned char* hit, int2* pair_list, int pair_cap, RoundCounters* rc, int n_query_bound, float eps,
               cudaStream_t s, const int* fmesh, const int* mesh_root) {
    (void)qlist;
    cudaMemsetAsync(&rc->pad[1], 0, 3 * sizeof(int), s);  // list length, query count, redo count
    // query faces in leaf order (uses the sort's second buffers, free after the build)
    const int gF = grid_for(n_query_bound, 256);
    k_query_order<<<gF, 256, 0, s>>>(rc, b.vals[0], qscan, b.live_scan);
    note_launch();
    exclusive_scan(b.live_scan, b.live_scan, &rc->n_live, 1, &rc->pad[2], b.scan_scratch, s, &rc->status,
                   n_query_bound);
    k_query_gather<<<gF, 256, 0, s>>>(rc, b.vals[0], b.live_scan, b.vals[1]);
    note_launch();
    // b.visit (free between a tree's bottom-up passes) holds the per-query redo marks
    // a function-local static initialiser runs once even when worker threads query concurrently
    static const int blocks_per_sm = [] {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_traverse_list, kQueryThreads, 0) != cudaSuccess || nb < 1)
            nb = 4;
        return nb;
    }();
    k_traverse_list<<<grid_for(n_query_bound, kQueryThreads, blocks_per_sm), kQueryThreads, 0, s>>>(
        b.packed, b.box_lo, b.box_hi, b.vals[1], pair_list, pair_cap, rc, b.visit, fmesh, mesh_root);
    note_launch();
    cudaMemsetAsync(b.xq_count, 0, sizeof(int), s);
    k_pairs<<<grid_for((long long)pair_cap, 128, 16), 128, 0, s>>>(tri, pos, pair_list, pair_cap, hit, rc, eps, b.xq,
                                                                   b.xq_cap, b.xq_count);
    note_launch();
    k_pairs_exact<<<4 * kNumSM, 64, 0, s>>>(tri, pos, b.xq, b.xq_cap, b.xq_count, hit, eps);
    note_launch();
    k_traverse_redo<<<grid_for(n_query_bound, kQueryThreads, 4), kQueryThreads, 0, s>>>(
        b.packed, b.box_lo, b.box_hi, tri, pos, b.vals[1], hit, rc, eps, b.visit, fmesh, mesh_root);
    note_launch();
}

}  // namespace pamo
