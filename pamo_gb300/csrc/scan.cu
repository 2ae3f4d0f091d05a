// Three-phase exclusive scan over a fixed grid of tiles: per-tile sums, one-block scan of the tile sums,
// per-tile scan with carry. The tile count is fixed (4 per SM), the chunk each tile owns follows from the
// element count read on the device.
#include "pamo_common.cuh"
#include "scan.cuh"

#include <atomic>

namespace pamo {

static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

namespace {
constexpr int kThreads = 512;
constexpr int kItems = 4;

__device__ __forceinline__ void chunk_of(int n, int& lo, int& hi) {
    long long chunk = ((long long)n + kScanTiles - 1) / kScanTiles;
    chunk = (chunk + kItems - 1) / kItems * kItems;
    long long a = chunk * blockIdx.x, b = a + chunk;
    lo = (int)(a < n ? a : n);
    hi = (int)(b < n ? b : n);
}

__global__ void __launch_bounds__(kThreads) k_tile_sums(const int* in, const int* d_n, int n_add, int* tile_sums) {
    __shared__ int sm[33];
    const int n = (d_n ? *d_n : 0) + n_add;
    int lo, hi;
    chunk_of(n, lo, hi);
    int s = 0;
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) s += in[i];
    int tot;
    block_exclusive_scan(s, &tot, sm);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_tiles(int* tile_sums, int* d_total) {
    __shared__ int sm[33];
    int v = threadIdx.x < kScanTiles ? tile_sums[threadIdx.x] : 0;
    int tot;
    int ex = block_exclusive_scan(v, &tot, sm);
    if (threadIdx.x < kScanTiles) tile_sums[threadIdx.x] = ex;
    if (threadIdx.x == 0) {
        tile_sums[kScanTiles] = tot;
        if (d_total) *d_total = tot;
    }
}

__global__ void __launch_bounds__(kThreads) k_tile_scan(const int* in, int* out, const int* d_n, int n_add,
                                                        const int* tile_sums) {
    __shared__ int sm[33];
    const int n = (d_n ? *d_n : 0) + n_add;
    int lo, hi;
    chunk_of(n, lo, hi);
    int carry = tile_sums[blockIdx.x];
    for (int base = lo; base < hi; base += kThreads * kItems) {
        int idx = base + threadIdx.x * kItems;
        int v[kItems];
        int s = 0;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            v[k] = (idx + k < hi) ? in[idx + k] : 0;
            s += v[k];
        }
        int tot;
        int ex = block_exclusive_scan(s, &tot, sm);
        int run = carry + ex;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            if (idx + k < hi) out[idx + k] = run;
            run += v[k];
        }
        carry += tot;
    }
}
}  // namespace

void exclusive_scan(const int* in, int* out, const int* d_n, int n_add, int* d_total, int* scratch, cudaStream_t s) {
    k_tile_sums<<<kScanTiles, kThreads, 0, s>>>(in, d_n, n_add, scratch); note_launch();
    k_scan_tiles<<<1, 1024, 0, s>>>(scratch, d_total); note_launch();
    k_tile_scan<<<kScanTiles, kThreads, 0, s>>>(in, out, d_n, n_add, scratch); note_launch();
}

}  // namespace pamo
