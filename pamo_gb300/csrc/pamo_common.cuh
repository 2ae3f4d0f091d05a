// Shared device-side definitions of the PaMO stage-2 GB300 kernels.
//
// Layout in HBM: vertex positions float4 (x, y, z, 0) so every gather is one 128-bit load; faces int4
// (i, j, k, 0) with (-1, -1, -1) marking a removed face; edges int2 (u < v); per-vertex quadrics as three
// float4 holding the 10 distinct entries of the symmetric 4x4 matrix; vertex->face adjacency as CSR with
// each vertex's faces in ascending face order.
//
// All float arithmetic mirrors the reference's operation order (simp_cuda/src/cusimp_free.cu) and the file
// is compiled with --fmad=false, as the reference is, so products and sums round exactly as there.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pamo {

constexpr int kNumSM = 152;  // GB300: 2 dies x 76 SMs

// status bits written by device code (never trap)
enum : int {
    kErrNone = 0,
    kErrStackOverflow = 1 << 0,    // BVH traversal stack full
    kErrCapacity = 1 << 1,         // a fixed-capacity list overflowed
    kErrLineEdges = 1 << 2,        // too many coincident-endpoint edges for the ordered pass
    kErrIterLimit = 1 << 3,        // a bounded device loop ran out of iterations
    kErrBadIndex = 1 << 4,         // an input face references a vertex outside [0, n_points)
};

// Per-round counters kept in device memory so that the round loop needs no host reads.
struct RoundCounters {
    int n_pts;            // vertices of this round
    int n_tris;           // faces of this round
    int n_edges;          // unique edges
    int n_win;            // independent-set winners (regular collapses)
    int n_line;           // coincident-endpoint edges found after the collapse
    int n_collapsed;      // entries in the collapsed-edge list (winners, then line collapses)
    int n_considered;     // entries the undo check looks at
    int n_live;           // live faces in the BVH
    int n_query;          // faces whose intersections are tested
    int n_undo;           // undo edges found by the latest check
    int n_vertices_undo;  // length of the undo-vertex list
    int first_undo;       // first unmapped position of the undo-vertex list
    int passes;           // intersection checks run this round
    int n_pts_out;        // live vertices after the round
    int n_tris_out;       // live faces after the round
    int status;           // kErr* bits
    unsigned long long n_pairs;       // candidate pairs tested (diagnostic)
    unsigned long long n_exact;       // pairs that needed the FP64 path (diagnostic)
    int undo_per_pass[8];
    int pad[6];
};

// State of the PaMO.run loop kept on the device between rounds, so that a round can run without host input
// (pamo/__init__.py:131-159: sizes after compaction, undo vertices carried to the next call, the no-progress
// count and is_stuck).
struct LoopState {
    int np, nf;    // vertices and faces the round starts with
    int nu;        // undo vertices carried into the round
    int is_stuck;
    int count;     // rounds in a row without progress
    int pad[3];
};

struct Quadric {  // symmetric 4x4: a = (m00 m01 m02 m03), b = (m11 m12 m13 m22), c = (m23 m33 - -)
    float4 a, b, c;
};

__device__ __forceinline__ bool face_killed(int4 t) { return t.x == -1 && t.y == -1 && t.z == -1; }

// ---- Vertex<float> arithmetic of the reference (cusimp_free.h:31-97) ----
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float4 p) { return {p.x, p.y, p.z}; }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ float vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 vcross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float vnorm(V3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ V3 vdiv(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }

// min/max/clamp of cusimp_free.cu:29-34 (NaN maps to the upper bound)
__device__ __forceinline__ float rmin(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float rmax(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float rclamp(float x, float a, float b) { return rmin(rmax(a, x), b); }

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
    return __ldg(p);
}

// grid-stride helpers
__device__ __forceinline__ int gtid() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int gstride() { return gridDim.x * blockDim.x; }

// Item order that spreads heavy, clustered items over the SMs: a warp takes 32 consecutive items and
// consecutive warps are warp 0 of consecutive blocks, then warp 1, ... (the blocks of a grid are spread
// over the SMs first), so a run of heavy items lands on many SMs instead of the few blocks that hold it.
__device__ __forceinline__ long long spread_first() {
    return ((long long)(threadIdx.x >> 5) * gridDim.x + blockIdx.x) * 32 + (threadIdx.x & 31);
}
__device__ __forceinline__ long long spread_stride() { return (long long)gridDim.x * blockDim.x; }

// The quantised collapse threshold of forward() (cusimp_free.cu:923): clamp(threshold, 0, 10) / 10 * 2^32 as
// uint32, saturating (the reference's host conversion is undefined beyond the range; NaN clamps to the upper bound).
inline uint32_t collapse_threshold(float threshold) {
    constexpr float kRange = 10.0f;
    float t = threshold > 0.0f ? threshold : 0.0f;
    t = (t < kRange) ? t : kRange;
    if (threshold != threshold) t = kRange;
    const float f = t / kRange * 4294967296.0f;
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

// Host-side count of kernels this library has launched (for launch accounting in benchmarks).
void note_launch();
void note_launches(long long n);  // kernels run by a CUDA graph launch
long long launches_so_far();

inline int grid_for(long long n, int threads, int per_sm = 8) {
    long long g = (n + threads - 1) / threads;
    long long cap = (long long)kNumSM * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace pamo
