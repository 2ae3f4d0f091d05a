// Device-wide exclusive prefix sums whose element count may live in device memory, so that a round can
// be launched without reading sizes back to the host.
#pragma once
#include <cuda_runtime.h>

namespace pamo {

constexpr int kScanTiles = 4 * 152;

// scratch ints needed by exclusive_scan (8 header ints and a 64-bit status word per tile)
inline size_t scan_scratch_ints() { return 8 + 2 * (size_t)kScanTiles; }

// out[i] = sum_{j<i} in[i] for i in [0, n), n = (d_n ? *d_n : 0) + n_add. in == out is allowed.
// If d_total is given, *d_total = sum of all n inputs. Inputs are int32 counts (no overflow checks).
// The scratch must be all zero before the first scan (scan_scratch_clear, or zero-initialised static memory);
// every scan leaves it zero again. One scratch serves one stream at a time. A look-back that waits too long
// sets kErrIterLimit in *err (when given). n_bound >= 0: an upper bound of *d_n known when the launch is made,
// which sizes the grid (any value gives the same result; a low one only makes the tiles longer).
void exclusive_scan(const int* in, int* out, const int* d_n, int n_add, int* d_total, int* scratch,
                    cudaStream_t s, int* err = nullptr, long long n_bound = -1);

// Independent scans launched together (one launch instead of `count`): each job has the meaning of
// exclusive_scan's arguments and its own scratch; n_bound bounds every job's element count.
constexpr int kMaxScanJobs = 3;
struct ScanJob {
    const int* in;
    int* out;
    const int* d_n;
    int n_add;
    int* d_total;
    int* scratch;
};
void exclusive_scans(const ScanJob* jobs, int count, cudaStream_t s, int* err = nullptr, long long n_bound = -1);

// Zeroes a freshly allocated scan scratch (synchronous); returns nonzero on a CUDA error.
int scan_scratch_clear(int* scratch);

__device__ __forceinline__ int warp_inclusive_scan(int v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan (blockDim.x a multiple of 32, <= 1024); smem33 is 33 ints of shared memory.
// Every thread of the block must call it.
__device__ __forceinline__ int block_exclusive_scan(int v, int* total, int* smem33) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int inc = warp_inclusive_scan(v);
    __syncthreads();  // smem33 may still be read by a previous call
    if (lane == 31) smem33[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nw ? smem33[lane] : 0;
        int wi = warp_inclusive_scan(w);
        if (lane < nw) smem33[lane] = wi - w;
        if (lane == nw - 1) smem33[32] = wi;
    }
    __syncthreads();
    *total = smem33[32];
    return smem33[warp] + inc - v;
}

}  // namespace pamo
