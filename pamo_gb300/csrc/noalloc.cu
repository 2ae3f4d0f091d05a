// Allocation-free variant of the whole-mesh self-intersection check (pamo_self_intersect_noalloc).
//
// Who needs it: callers that must not allocate device memory themselves or through a library — for example
// a host application that hands this library a fixed pool of device memory and forbids any other
// cudaMalloc/cudaFree (a renderer or game engine budgeting memory up front, a plug-in running inside such a
// host), or code that must not trigger an allocation that would synchronise the device in the middle of
// its own work. pamo_self_intersect needs a pamo_ctx, whose buffers come from cudaMalloc; this entry point
// needs none.
//
// How: all scratch of the check (copies of the mesh in the kernels' layout, the LBVH, the sort and scan
// scratch, the query list, the flags, the counters) lives in one file-scope __device__ array of
// kNoAllocBytes, carved the same way for every call. Every GPU that loads this library holds that array
// until the process exits. In host code the array's name is only a host-side stand-in, so its device
// address is looked up with cudaGetSymbolAddress, with the device current, on the first call made in each
// CUDA context, and passed to the kernels. A __device__ array has its own address in every context, so the
// address is cached per context, keyed on the context's process-unique id (cuCtxGetId): a host that runs its
// own context, or one that resets the device (cudaDeviceReset) and so gets a new primary context, gets a
// fresh lookup. Where the driver cannot report that id, the address is looked up on every call. The first
// call in a context should therefore come before any stream capture. All calls share the one array:
// everything that must start at zero is cleared at the start of each call, and calls that overlap on the GPU
// (concurrent streams, other host threads) race on it. Limits: at most kNoAllocMaxPoints points and
// kNoAllocMaxTriangles triangles per call; larger meshes are rejected with PAMO_ERR_CAPACITY before any GPU
// work. A CUDA error left pending by the caller's earlier work is reported as PAMO_ERR_CUDA before any GPU work
// and is not cleared. Once work is queued, every return synchronises the stream first, so no kernel of the
// call is still running on the shared array when it returns.
#include <cuda.h>  // CUcontext and the types of the two driver entry points (no link to the driver library)

#include <cstdint>
#include <mutex>

#include "../../include/pamo_gb300.h"
#include "lbvh.cuh"
#include "pamo_common.cuh"
#include "scan.cuh"
#include "simp_round.cuh"

namespace {

constexpr int kNoAllocMaxPoints = 65536;
constexpr int kNoAllocMaxTriangles = 65536;
constexpr size_t kNoAllocBytes = 24u << 20;  // 24 MiB
constexpr int kExactCap = 8 * kNoAllocMaxTriangles;
constexpr float kTriEps = 1e-3f;  // cusimp_free.cu:893

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kCachedContexts = 64;

std::mutex g_setup_mutex;
struct CachedAddress {
    unsigned long long ctx_id;  // 0 = empty slot
    unsigned char* ptr;
};
CachedAddress g_scratch_cache[kCachedContexts] = {};
int g_scratch_next = 0;

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

struct Layout {
    pamo::RoundCounters* rc;
    int* scan_scratch;
    float4* pos;
    float4* orig_pos;
    int* occ;
    int4* tri;
    int* qflag;
    int* qlist;
    unsigned char* hit;
    int2* exact;
    char* bvh;
    size_t end;
};

Layout carve(unsigned char* base) {
    Layout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base + off;
        off += up256(bytes);
        return p;
    };
    L.rc = (pamo::RoundCounters*)take(sizeof(pamo::RoundCounters));
    L.scan_scratch = (int*)take(pamo::scan_scratch_ints() * sizeof(int));
    L.pos = (float4*)take((kNoAllocMaxPoints + 2) * sizeof(float4));
    L.orig_pos = (float4*)take((kNoAllocMaxPoints + 2) * sizeof(float4));
    L.occ = (int*)take((kNoAllocMaxPoints + 2) * sizeof(int));
    L.tri = (int4*)take((kNoAllocMaxTriangles + 2) * sizeof(int4));
    L.qflag = (int*)take((kNoAllocMaxTriangles + 2) * sizeof(int));
    L.qlist = (int*)take((kNoAllocMaxTriangles + 2) * sizeof(int));
    L.hit = (unsigned char*)take(kNoAllocMaxTriangles + 2);
    L.exact = (int2*)take((size_t)kExactCap * sizeof(int2));
    L.bvh = (char*)take(pamo::bvh_bytes(kNoAllocMaxTriangles));
    L.end = off;
    return L;
}

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

// The process-unique id of the current context (cuCtxGetId), or 0 where no context is current yet or the
// driver cannot report it. The driver entry points are resolved through the runtime once.
unsigned long long current_context_id() {
    static PfnCtxGetCurrent get_current = nullptr;
    static PfnCtxGetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (PfnCtxGetCurrent)p;
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (PfnCtxGetId)p;
    });
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return 0;
    unsigned long long id = 0;
    return get_id(ctx, &id) == CUDA_SUCCESS ? id : 0;
}

// Device address of the scratch array in the current context: looked up once per context and cached by the
// context's id; looked up on every call where the id is unknown.
int scratch_on_current_device(unsigned char** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return PAMO_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long id = current_context_id();
    if (id != 0)
        for (const CachedAddress& c : g_scratch_cache)
            if (c.ctx_id == id) {
                *out = c.ptr;
                return PAMO_OK;
            }
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return PAMO_ERR_CUDA;
    id = current_context_id();  // the lookup made the device's primary context current if none was
    if (id != 0) {
        g_scratch_cache[g_scratch_next] = CachedAddress{id, (unsigned char*)p};
        g_scratch_next = (g_scratch_next + 1) % kCachedContexts;
    }
    *out = (unsigned char*)p;
    return PAMO_OK;
}

// counters of this call: zero, then the mesh sizes (no host staging buffer involved)
__global__ void k_noalloc_init(pamo::RoundCounters* rc, int n_points, int n_triangles) {
    int* w = (int*)rc;
    for (int i = threadIdx.x; i < (int)(sizeof(pamo::RoundCounters) / sizeof(int)); i += blockDim.x) w[i] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        rc->n_pts = n_points;
        rc->n_tris = n_triangles;
    }
}

}  // namespace

extern "C" int pamo_self_intersect_noalloc(const float* points, const int32_t* triangles, int32_t n_points,
                                           int32_t n_triangles, uint8_t* face_hit, pamo_stream stream) {
    if (!points || !triangles || !face_hit || n_points < 1 || n_triangles < 1) return PAMO_ERR_INVALID_ARG;
    if (n_points > kNoAllocMaxPoints || n_triangles > kNoAllocMaxTriangles) return PAMO_ERR_CAPACITY;
    if (cudaPeekAtLastError() != cudaSuccess) return PAMO_ERR_CUDA;  // the caller's pending error, left as is
    unsigned char* base = nullptr;
    int r = scratch_on_current_device(&base);
    if (r) return r;
    const Layout L = carve(base);
    if (L.end > kNoAllocBytes) return PAMO_ERR_CAPACITY;
    pamo::BvhBuffers bvh;
    pamo::bvh_carve(bvh, kNoAllocMaxTriangles, L.bvh, false);  // static memory: zero at load, kept zero by scans
    cudaStream_t s = (cudaStream_t)stream;

    // the counters and flags start from zero on every call (the array keeps the previous call's contents)
    k_noalloc_init<<<1, 64, 0, s>>>(L.rc, n_points, n_triangles);
    cudaMemsetAsync(L.hit, 0, n_triangles + 1, s);

    pamo::launch_load_points(points, n_points, L.pos, L.orig_pos, L.occ, s);
    pamo::launch_load_tris(triangles, n_triangles, n_points, L.tri, L.rc, s);
    pamo::launch_live_flags(L.rc, n_triangles, L.tri, L.qflag, s);
    pamo::exclusive_scan(L.qflag, L.qflag, &L.rc->n_tris, 1, &L.rc->n_query, L.scan_scratch, s, &L.rc->status,
                         n_triangles);
    pamo::launch_compact_flags(L.qflag, n_triangles, &L.rc->n_tris, L.qlist, s);
    pamo::bvh_build(bvh, L.tri, L.pos, L.rc, n_triangles, s, false, L.qflag, false);
    pamo::bvh_query(bvh, L.tri, L.pos, L.qlist, L.qflag, L.hit, L.exact, kExactCap, L.rc, n_triangles, kTriEps, s);
    cudaMemcpyAsync(face_hit, L.hit, n_triangles, cudaMemcpyDeviceToDevice, s);
    int status = 0;
    cudaMemcpyAsync(&status, &L.rc->status, sizeof(int), cudaMemcpyDeviceToHost, s);

    // whatever happened, nothing of this call may still run on the shared array when it returns
    const cudaError_t launched = cudaGetLastError();
    const cudaError_t finished = cudaStreamSynchronize(s);
    if (launched != cudaSuccess || finished != cudaSuccess) return PAMO_ERR_CUDA;
    if (status & pamo::kErrBadIndex) return PAMO_ERR_INVALID_ARG;
    if (status & (pamo::kErrStackOverflow | pamo::kErrIterLimit)) return PAMO_ERR_ITER_LIMIT;
    if (status & pamo::kErrCapacity) return PAMO_ERR_CAPACITY;
    return PAMO_OK;
}
