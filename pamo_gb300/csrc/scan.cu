// Single-pass exclusive scan over a fixed grid of tiles (4 per SM) with decoupled look-back; the chunk each tile
// owns follows from the element count read on the device.
#include "pamo_common.cuh"
#include "scan.cuh"

#include <algorithm>
#include <atomic>

namespace pamo {

static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

namespace {
constexpr int kThreads = 512;
constexpr int kItems = 4;
constexpr int kPass = kThreads * kItems;  // elements one block handles per pass
constexpr long long kSpinLimit = 1ll << 22;

// scratch layout (ints): [0] next tile id, [1] finished blocks, [2] error bits, [3..7] unused, then one 64-bit
// status word per tile: flag << 32 | value, flag 1 = the tile's aggregate, 2 = its inclusive prefix
enum { kNext = 0, kDone = 1, kError = 2, kHeader = 8 };

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// chunk of tile t (of gridDim.x tiles): whole passes, at least one, tiles in element order
__device__ __forceinline__ void chunk_of(int n, int t, int& lo, int& hi) {
    long long chunk = ((long long)n + gridDim.x - 1) / gridDim.x;
    chunk = (chunk + kPass - 1) / kPass * kPass;
    long long a = chunk * t, b = a + chunk;
    lo = (int)(a < n ? a : n);
    hi = (int)(b < n ? b : n);
}

__device__ __forceinline__ void load4(const int* in, int idx, int hi, int v[kItems]) {
    if (idx + kItems <= hi && ((reinterpret_cast<uintptr_t>(in + idx) & 15) == 0)) {
        const int4 q = *reinterpret_cast<const int4*>(in + idx);
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
#pragma unroll
        for (int k = 0; k < kItems; ++k) v[k] = (idx + k < hi) ? in[idx + k] : 0;
    }
}

// Single-pass exclusive scan with decoupled look-back (Merrill and Garland, "Single-pass Parallel Prefix Scan
// with Decoupled Look-back", 2016). Tile ids come from an atomic counter in launch order, so a tile only ever
// waits for tiles whose blocks are already running; each tile publishes its aggregate before it looks back.
// The last block to finish clears the counters and status words for the next scan on the same scratch.
// Up to kMaxScanJobs independent scans in one launch: job blockIdx.y, each with its own scratch, so that
// their tiles never wait for one another.
struct ScanJobs {
    ScanJob j[kMaxScanJobs];
};

__global__ void __launch_bounds__(kThreads) k_scan(ScanJobs jobs, int* err) {
    const ScanJob& J = jobs.j[blockIdx.y];
    const int* in = J.in;
    int* out = J.out;
    const int* d_n = J.d_n;
    const int n_add = J.n_add;
    int* d_total = J.d_total;
    int* scratch = J.scratch;
    __shared__ int sm[33];
    __shared__ int s_tile, s_prefix;
    unsigned long long* status = reinterpret_cast<unsigned long long*>(scratch + kHeader);
    const int n = (d_n ? *d_n : 0) + n_add;
    if (threadIdx.x == 0) s_tile = atomicAdd(&scratch[kNext], 1);
    __syncthreads();
    const int t = s_tile;
    int lo, hi;
    chunk_of(n, t, lo, hi);
    if (lo < hi || (n == 0 && t == 0)) {
        // aggregate of the chunk
        int s = 0;
        for (int base = lo; base < hi; base += kPass) {
            int v[kItems];
            load4(in, base + threadIdx.x * kItems, hi, v);
#pragma unroll
            for (int k = 0; k < kItems; ++k) s += v[k];
        }
        int agg;
        block_exclusive_scan(s, &agg, sm);
        if (threadIdx.x == 0) {
            if (t == 0) st_release(&status[0], (2ull << 32) | (unsigned)agg);
            else st_release(&status[t], (1ull << 32) | (unsigned)agg);
        }
        // look-back over the predecessors, 32 at a time, nearest first
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            int excl = 0;
            if (t > 0) {
                int j = t - 1;
                long long spins = 0;
                while (true) {
                    const int idx = j - lane;
                    const unsigned long long w = idx >= 0 ? ld_acquire(&status[idx]) : (2ull << 32);
                    const unsigned flag = (unsigned)(w >> 32);
                    if (__any_sync(0xffffffffu, flag == 0)) {
                        if (++spins > kSpinLimit) {
                            if (lane == 0) {
                                atomicOr(&scratch[kError], kErrIterLimit);
                                if (err) atomicOr(err, kErrIterLimit);
                            }
                            break;
                        }
                        continue;
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, flag == 2);
                    const int first = m ? __ffs(m) - 1 : 32;
                    int v = lane <= first ? (int)(unsigned)w : 0;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    excl += v;
                    if (m) break;
                    j -= 32;
                }
                if (lane == 0) st_release(&status[t], (2ull << 32) | (unsigned)(excl + agg));
            }
            if (lane == 0) {
                s_prefix = excl;
                if (d_total && hi == n) *d_total = excl + agg;
            }
        }
        __syncthreads();
        int carry = s_prefix;
        for (int base = lo; base < hi; base += kPass) {
            const int idx = base + threadIdx.x * kItems;
            int v[kItems];
            load4(in, idx, hi, v);
            const int ts = v[0] + v[1] + v[2] + v[3];
            int tot;
            const int ex = block_exclusive_scan(ts, &tot, sm);
            int run = carry + ex;
            int o[kItems];
#pragma unroll
            for (int k = 0; k < kItems; ++k) {
                o[k] = run;
                run += v[k];
            }
            if (idx + kItems <= hi && ((reinterpret_cast<uintptr_t>(out + idx) & 15) == 0)) {
                *reinterpret_cast<int4*>(out + idx) = make_int4(o[0], o[1], o[2], o[3]);
            } else {
#pragma unroll
                for (int k = 0; k < kItems; ++k)
                    if (idx + k < hi) out[idx + k] = o[k];
            }
            carry += tot;
        }
    }
    // the last block out resets the scratch
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const int done = atomicAdd(&scratch[kDone], 1);
        s_tile = done == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (s_tile) {
        __threadfence();
        for (int i = threadIdx.x; i < kScanTiles; i += kThreads) status[i] = 0ull;
        if (threadIdx.x == 0) {
            scratch[kNext] = 0;
            scratch[kDone] = 0;
        }
    }
}
}  // namespace

void exclusive_scans(const ScanJob* jobs, int count, cudaStream_t s, int* err, long long n_bound) {
    if (count < 1 || count > kMaxScanJobs) return;
    ScanJobs all{};
    int n_add = 0;
    for (int k = 0; k < count; ++k) {
        all.j[k] = jobs[k];
        n_add = std::max(n_add, jobs[k].n_add);
    }
    int tiles = kScanTiles;
    if (n_bound >= 0 && n_bound < (1 << 19)) {  // callers cap their bounds at 2^19 (every grid full from there)
        const long long want = (n_bound + n_add + kPass - 1) / kPass;
        tiles = (int)(want < 1 ? 1 : (want > kScanTiles ? kScanTiles : want));
    }
    k_scan<<<dim3(tiles, count), kThreads, 0, s>>>(all, err); note_launch();
}

void exclusive_scan(const int* in, int* out, const int* d_n, int n_add, int* d_total, int* scratch, cudaStream_t s,
                    int* err, long long n_bound) {
    const ScanJob job{in, out, d_n, n_add, d_total, scratch};
    exclusive_scans(&job, 1, s, err, n_bound);
}

int scan_scratch_clear(int* scratch) {
    if (cudaMemset(scratch, 0, scan_scratch_ints() * sizeof(int)) != cudaSuccess) return 1;
    return cudaStreamSynchronize(0) == cudaSuccess ? 0 : 1;
}

}  // namespace pamo
