// Many meshes on one GPU: a pool of simplification workers, used two ways.
//
//   pamo_batch_*  : a batch of meshes concatenated in CSR form (vertex and face offsets per mesh) is simplified
//                   as a whole; every mesh runs the whole PaMO.run loop (simp_cuda/pamo/__init__.py:95-163)
//                   on a worker context, workers run concurrently on their own CUDA streams, and the results
//                   come back concatenated in CSR form.
//   pamo_server_* : a request loop. Requests (host arrays) queue in arrival order and are admitted while the
//                   device memory they are estimated to need fits a budget; an admitted request runs on the
//                   next free worker; finished results wait to be fetched.
//
// Each job starts from the state of a newly created context (pamo_ctx_reset), so a mesh gets the same result
// alone, in a batch or among other requests: the same kernels, state and arithmetic as pamo_simplify_device.
// Only the public C ABI of the library is used here.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pamo_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

// float32 -> float64, on the device (the request's input points, already there for stage 2, become the stage-3
// target without a host round trip)
__global__ void k_widen(const float* __restrict__ in, long long n, double* out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Worker {
    pamo_ctx* ctx = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
};

int make_workers(int device, int n, std::vector<Worker>& ws, std::string& err) {
    if (cudaSetDevice(device) != cudaSuccess) {
        err = "cudaSetDevice";
        return PAMO_ERR_CUDA;
    }
    ws.resize(n);
    for (auto& w : ws) {
        int r = pamo_ctx_create(&w.ctx, device);
        if (r) {
            err = "pamo_ctx_create";
            return r;
        }
        if (cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming) != cudaSuccess) {
            err = "stream or event creation";
            return PAMO_ERR_CUDA;
        }
    }
    return PAMO_OK;
}

void free_workers(int device, std::vector<Worker>& ws) {
    cudaSetDevice(device);
    for (auto& w : ws) {
        if (w.stream) cudaStreamSynchronize(w.stream);
        if (w.ctx) pamo_ctx_destroy(w.ctx);
        if (w.stream) cudaStreamDestroy(w.stream);
        if (w.done) cudaEventDestroy(w.done);
    }
    ws.clear();
}

// One whole simplification job on a worker: fresh state, the PaMO.run loop, result exported (centring undone)
// into out_points/out_tris (device, room for the input sizes).
int run_job(Worker& w, const float* points, const int32_t* tris, int32_t np, int32_t nt, double ratio, int32_t tolerance,
            float threshold, int32_t iter, int64_t min_verts, float* out_points, int32_t* out_tris, int32_t* onp,
            int32_t* ont, int32_t* rounds, std::string& err) {
    int r = pamo_ctx_reset(w.ctx, w.stream);
    if (!r) r = pamo_simplify_device(w.ctx, points, tris, np, nt, ratio, tolerance, threshold, iter, min_verts, onp, ont,
                                     rounds, w.stream);
    if (!r) r = pamo_simplify_result(w.ctx, out_points, out_tris, w.stream);
    if (r) err = pamo_ctx_last_error(w.ctx);
    return r;
}

}  // namespace

// ================================================================== batch
struct pamo_batch {
    int device = 0;
    std::vector<Worker> workers;
    std::string err;
    cudaEvent_t ev_in = nullptr;
    float* arena_p = nullptr;     // results at the input offsets, before compaction into the caller's buffers
    int32_t* arena_t = nullptr;
    size_t cap_p = 0, cap_t = 0;
    std::vector<int32_t> rounds;  // rounds per mesh of the last batch
};

extern "C" {

int pamo_batch_create(pamo_batch** out, int device, int32_t n_workers) {
    if (!out || n_workers < 1 || n_workers > 256) return PAMO_ERR_INVALID_ARG;
    *out = nullptr;
    auto* b = new pamo_batch();
    b->device = device;
    int r = make_workers(device, n_workers, b->workers, b->err);
    if (!r && cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming) != cudaSuccess) r = PAMO_ERR_CUDA;
    if (r) {
        free_workers(device, b->workers);
        delete b;
        return r;
    }
    *out = b;
    return PAMO_OK;
}

int pamo_batch_destroy(pamo_batch* b) {
    if (!b) return PAMO_ERR_INVALID_ARG;
    free_workers(b->device, b->workers);
    cudaSetDevice(b->device);
    if (b->ev_in) cudaEventDestroy(b->ev_in);
    cudaFree(b->arena_p);
    cudaFree(b->arena_t);
    delete b;
    return PAMO_OK;
}

const char* pamo_batch_last_error(const pamo_batch* b) { return b ? b->err.c_str() : "null batch"; }

int pamo_batch_simplify(pamo_batch* b, const float* points, const int32_t* triangles, const int64_t* vert_offsets,
                        const int64_t* face_offsets, int32_t n_meshes, const double* ratios, int32_t tolerance,
                        float threshold, int32_t iter, int64_t min_verts, float* out_points, int32_t* out_triangles,
                        int64_t* out_vert_offsets, int64_t* out_face_offsets, pamo_stream stream) {
    if (!b) return PAMO_ERR_INVALID_ARG;
    b->err.clear();
    if (n_meshes < 0 || (n_meshes > 0 && (!points || !triangles || !vert_offsets || !face_offsets || !ratios ||
                                          !out_points || !out_triangles || !out_vert_offsets || !out_face_offsets))) {
        b->err = "null pointer or negative mesh count";
        return PAMO_ERR_INVALID_ARG;
    }
    for (int m = 0; m < n_meshes; ++m)
        if (vert_offsets[m + 1] - vert_offsets[m] < 1 || face_offsets[m + 1] - face_offsets[m] < 1 ||
            vert_offsets[m + 1] - vert_offsets[m] > INT32_MAX || face_offsets[m + 1] - face_offsets[m] > INT32_MAX) {
            b->err = "mesh " + std::to_string(m) + " is empty or too large";
            return PAMO_ERR_INVALID_ARG;
        }
    cudaSetDevice(b->device);
    const size_t tv = n_meshes ? (size_t)vert_offsets[n_meshes] : 0, tf = n_meshes ? (size_t)face_offsets[n_meshes] : 0;
    if (tv * 3 > b->cap_p) {
        cudaFree(b->arena_p);
        b->arena_p = nullptr;
        if (cudaMalloc((void**)&b->arena_p, tv * 3 * sizeof(float)) != cudaSuccess) return PAMO_ERR_OOM;
        b->cap_p = tv * 3;
    }
    if (tf * 3 > b->cap_t) {
        cudaFree(b->arena_t);
        b->arena_t = nullptr;
        if (cudaMalloc((void**)&b->arena_t, tf * 3 * sizeof(int32_t)) != cudaSuccess) return PAMO_ERR_OOM;
        b->cap_t = tf * 3;
    }
    cudaStream_t caller = (cudaStream_t)stream;
    cudaEventRecord(b->ev_in, caller);  // inputs are ready in the caller's stream order
    // largest meshes first: the longest jobs start early, the short ones fill the gaps
    std::vector<int> order(n_meshes);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        return face_offsets[a + 1] - face_offsets[a] > face_offsets[c + 1] - face_offsets[c];
    });
    std::vector<int32_t> onp(n_meshes, 0), ont(n_meshes, 0);
    b->rounds.assign(n_meshes, 0);
    std::atomic<int> next{0};
    std::atomic<int> status{PAMO_OK};
    std::mutex err_mu;
    auto work = [&](Worker& w) {
        cudaSetDevice(b->device);
        cudaStreamWaitEvent(w.stream, b->ev_in, 0);
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= n_meshes || status.load() != PAMO_OK) break;
            const int m = order[k];
            const int64_t v0 = vert_offsets[m], f0 = face_offsets[m];
            std::string e;
            const int r = run_job(w, points + 3 * v0, triangles + 3 * f0, (int32_t)(vert_offsets[m + 1] - v0),
                                  (int32_t)(face_offsets[m + 1] - f0), ratios[m], tolerance, threshold, iter, min_verts,
                                  b->arena_p + 3 * v0, b->arena_t + 3 * f0, &onp[m], &ont[m], &b->rounds[m], e);
            if (r) {
                std::lock_guard<std::mutex> lock(err_mu);
                b->err = "mesh " + std::to_string(m) + ": " + e;
                status.store(r);
                break;
            }
        }
        cudaEventRecord(w.done, w.stream);
    };
    std::vector<std::thread> threads;
    for (size_t i = 1; i < b->workers.size(); ++i) threads.emplace_back(work, std::ref(b->workers[i]));
    work(b->workers[0]);
    for (auto& t : threads) t.join();
    if (status.load() != PAMO_OK) return status.load();
    // results in CSR form, packed in mesh order
    out_vert_offsets[0] = 0;
    out_face_offsets[0] = 0;
    for (int m = 0; m < n_meshes; ++m) {
        out_vert_offsets[m + 1] = out_vert_offsets[m] + onp[m];
        out_face_offsets[m + 1] = out_face_offsets[m] + ont[m];
    }
    for (auto& w : b->workers) cudaStreamWaitEvent(caller, w.done, 0);
    for (int m = 0; m < n_meshes; ++m) {
        cudaMemcpyAsync(out_points + 3 * out_vert_offsets[m], b->arena_p + 3 * vert_offsets[m],
                        (size_t)onp[m] * 3 * sizeof(float), cudaMemcpyDeviceToDevice, caller);
        cudaMemcpyAsync(out_triangles + 3 * out_face_offsets[m], b->arena_t + 3 * face_offsets[m],
                        (size_t)ont[m] * 3 * sizeof(int32_t), cudaMemcpyDeviceToDevice, caller);
    }
    if (cudaStreamSynchronize(caller) != cudaSuccess) {
        b->err = cudaGetErrorString(cudaGetLastError());
        return PAMO_ERR_CUDA;
    }
    return PAMO_OK;
}

int pamo_batch_rounds(const pamo_batch* b, int32_t* rounds, int32_t capacity) {
    if (!b || !rounds) return PAMO_ERR_INVALID_ARG;
    const int n = std::min<int>(capacity, (int)b->rounds.size());
    for (int i = 0; i < n; ++i) rounds[i] = b->rounds[i];
    return n;
}

}  // extern "C"

// ================================================================== server
namespace {

// Device bytes a job is taken to need while it runs: the working buffers a context allocates for its sizes
// (face and vertex arrays with the context's growth factor 1.2: about 700 B per face and 195 B per vertex, with
// the precision modes' arrays 740 and 255, rounded up to 780 and 330), its input and output copies, and 16 MiB of
// fixed-size scratch.
int64_t job_bytes(int64_t nv, int64_t nf) { return 780 * nf + 330 * nv + 2 * (12 * nv + 12 * nf) + (16ll << 20); }

// What stage 3 adds while it runs: the input as the float64 projection target and the stage-3 handle's buffers over
// it (its LBVH and per-face records, about 240 B per target face), plus 64 MiB for the small projected mesh.
int64_t stage3_bytes(int64_t nv, int64_t nf) { return 24 * nv + 240 * nf + (64ll << 20); }

struct Request {
    int64_t id = 0;
    std::vector<float> points;
    std::vector<int32_t> tris;
    double ratio = 0.001;
    int32_t tolerance = 4;
    float threshold = 1e-3f;
    bool stage3 = false;
    int64_t bytes = 0;
    Clock::time_point t_submit, t_admit, t_done;
    int status = PAMO_OK;
    std::string err;
    std::vector<float> out_points;
    std::vector<double> out_points64;  // stage 3: the projection's float64 positions
    std::vector<int32_t> out_tris;
    int32_t rounds = 0;
};

// What trimesh.Trimesh(V, F) does to the stage-2 output before the reference's stage 3 (simp_cuda/pamo/__init__.py:
// 166-172, trimesh 4.4.0 as pinned in env.yaml): faces touching a non-finite vertex are dropped, then referenced
// vertices whose coordinates agree after rounding to 8 decimals (round half to even, like numpy) are merged, keeping
// the first occurrence's coordinates, in order of first occurrence; unreferenced vertices are dropped.
void mesh_process(const std::vector<double>& V, const std::vector<int32_t>& F, std::vector<double>& Vo,
                  std::vector<int32_t>& Fo) {
    const size_t nv = V.size() / 3, nf = F.size() / 3;
    std::vector<int64_t> remap(nv, -1);
    size_t k = 0;
    for (size_t v = 0; v < nv; ++v)
        if (std::isfinite(V[3 * v]) && std::isfinite(V[3 * v + 1]) && std::isfinite(V[3 * v + 2])) remap[v] = (int64_t)k++;
    std::vector<int32_t> faces;
    faces.reserve(F.size());
    for (size_t f = 0; f < nf; ++f) {
        const int32_t a = F[3 * f], b = F[3 * f + 1], c = F[3 * f + 2];
        if (remap[a] < 0 || remap[b] < 0 || remap[c] < 0) continue;
        faces.push_back((int32_t)remap[a]);
        faces.push_back((int32_t)remap[b]);
        faces.push_back((int32_t)remap[c]);
    }
    std::vector<double> verts;
    verts.reserve(3 * k);
    for (size_t v = 0; v < nv; ++v)
        if (remap[v] >= 0) verts.insert(verts.end(), V.begin() + 3 * v, V.begin() + 3 * v + 3);
    std::vector<char> referenced(k, 0);
    for (int32_t x : faces) referenced[x] = 1;
    std::map<std::array<int64_t, 3>, int32_t> ids;
    std::vector<int32_t> inv(k, 0);
    Vo.clear();
    for (size_t v = 0; v < k; ++v) {
        if (!referenced[v]) continue;
        std::array<int64_t, 3> key;
        for (int d = 0; d < 3; ++d) key[d] = (int64_t)std::nearbyint(verts[3 * v + d] * 100000000.0);
        auto it = ids.find(key);
        if (it == ids.end()) {
            it = ids.emplace(key, (int32_t)(Vo.size() / 3)).first;
            Vo.insert(Vo.end(), verts.begin() + 3 * v, verts.begin() + 3 * v + 3);
        }
        inv[v] = it->second;
    }
    Fo.resize(faces.size());
    for (size_t i = 0; i < faces.size(); ++i) Fo[i] = inv[faces[i]];
}

}  // namespace

struct pamo_server {
    int device = 0;
    int64_t budget = 0;
    std::vector<Worker> workers;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;   // submitted, not admitted (arrival order)
    std::deque<std::shared_ptr<Request>> ready;   // admitted, waiting for a worker
    std::map<int64_t, std::shared_ptr<Request>> finished;
    std::deque<int64_t> finished_order;
    int64_t in_use = 0;  // bytes of admitted, unfinished requests
    int64_t max_in_use = 0, n_admitted = 0, n_finished = 0;
    int64_t next_id = 1;
    int64_t n_stage3_reruns = 0;  // stage-3 projections run again without cooperative kernels after a wait gave up
    bool stop = false;
    std::string err;
    // the workers' request buffers come from this stream-ordered pool (freed memory kept for the next growth): a
    // worker that grows a buffer waits for nothing but its own stream, where cudaFree would wait for the whole device
    // and stall every other worker
    cudaMemPool_t pool = nullptr;

    // admit queued requests in arrival order while they fit the budget (a request larger than the whole
    // budget is admitted alone, when nothing else runs)
    void admit_locked() {
        while (!queue.empty()) {
            auto& q = queue.front();
            if (in_use > 0 && in_use + q->bytes > budget) break;
            q->t_admit = Clock::now();
            in_use += q->bytes;
            max_in_use = std::max(max_in_use, in_use);
            ++n_admitted;
            ready.push_back(q);
            queue.pop_front();
        }
    }

    // grows a device buffer (elements of T) to at least n, in the order of the worker's stream st
    template <typename T>
    int ensure_dev(T*& p, size_t& cap, size_t n, cudaStream_t st) {
        if (n <= cap && p) return PAMO_OK;
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        cap = 0;
        if (cudaMallocFromPoolAsync((void**)&p, std::max<size_t>(n, 1) * sizeof(T), pool, st) != cudaSuccess) {
            p = nullptr;
            return PAMO_ERR_OOM;
        }
        cap = std::max<size_t>(n, 1);
        return PAMO_OK;
    }

    // stage 3 of a finished stage-2 job (simp_cuda/pamo/__init__.py:165-176): the stage-2 mesh through trimesh's
    // processing, then the projection onto the request's own input mesh; float64 positions
    int stage3_job(Worker& w, pamo_stage3*& s3, Request& q, const float* d_gt_points, const int32_t* d_gt_tris,
                   const float* d_res_p,
                   const int32_t* d_res_t, int32_t onp, int32_t ont, double*& gp, size_t& cgp, double*& sp,
                   size_t& csp, int32_t*& st, size_t& cst) {
        int r;
        if (!s3 && (r = pamo_stage3_create(&s3, device))) return r;
        std::vector<float> v2((size_t)onp * 3);
        std::vector<int32_t> f2((size_t)ont * 3);
        cudaMemcpyAsync(v2.data(), d_res_p, v2.size() * sizeof(float), cudaMemcpyDeviceToHost, w.stream);
        cudaMemcpyAsync(f2.data(), d_res_t, f2.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, w.stream);
        if (cudaStreamSynchronize(w.stream) != cudaSuccess) return PAMO_ERR_CUDA;
        std::vector<double> vd(v2.begin(), v2.end()), vm;
        std::vector<int32_t> fm;
        mesh_process(vd, f2, vm, fm);
        const size_t ngp = q.points.size() / 3, ngt = q.tris.size() / 3, nm = vm.size() / 3, nfm = fm.size() / 3;
        if (nm < 3 || nfm < 1) {  // nothing to project (the reference's stage 3 has no behaviour for an empty mesh)
            q.out_points64 = vm;
            q.out_tris = fm;
            q.out_points.assign(vm.begin(), vm.end());
            return PAMO_OK;
        }
        if ((r = ensure_dev(gp, cgp, 3 * ngp, w.stream)) ||
            (r = ensure_dev(sp, csp, 6 * std::max<size_t>(nm, 1), w.stream)) ||
            (r = ensure_dev(st, cst, 3 * std::max<size_t>(nfm, 1), w.stream)))
            return r;
        const long long ng = 3 * (long long)ngp;
        k_widen<<<(unsigned)std::min<long long>((ng + 255) / 256, 1024), 256, 0, w.stream>>>(d_gt_points, ng, gp);
        cudaMemcpyAsync(sp, vm.data(), vm.size() * sizeof(double), cudaMemcpyHostToDevice, w.stream);
        cudaMemcpyAsync(st, fm.data(), fm.size() * sizeof(int32_t), cudaMemcpyHostToDevice, w.stream);
        double* out = sp + 3 * nm;
        r = pamo_safe_project(s3, gp, d_gt_tris, (int32_t)ngp, (int32_t)ngt, sp, st, (int32_t)nm, (int32_t)nfm, 5, out,
                              w.stream);
        // the solver runs a projection again without cooperative kernels when a grid barrier gave up (other
        // workers' kernels on the GPU can keep a cooperative kernel's blocks from running at once)
        double st3[13] = {};
        if (pamo_stage3_stats(s3, st3, 13) >= 13 && st3[12] > 0.0) {
            std::lock_guard<std::mutex> lock(mu);
            ++n_stage3_reruns;
        }
        if (r) {
            q.err = pamo_stage3_last_error(s3);
            return r;
        }
        q.out_points64.resize(3 * nm);
        q.out_tris = fm;
        cudaMemcpyAsync(q.out_points64.data(), out, 3 * nm * sizeof(double), cudaMemcpyDeviceToHost, w.stream);
        if (cudaStreamSynchronize(w.stream) != cudaSuccess) return PAMO_ERR_CUDA;
        q.out_points.assign(q.out_points64.begin(), q.out_points64.end());
        return PAMO_OK;
    }

    void worker_loop(int i) {
        Worker& w = workers[i];
        cudaSetDevice(device);
        float* dp = nullptr;
        int32_t* dt = nullptr;
        size_t cp = 0, ct = 0;
        float* rp = nullptr;  // stage-2 result (the input copies stay the stage-3 target)
        int32_t* rt = nullptr;
        size_t crp = 0, crt = 0;
        double* gp = nullptr;
        double* sp = nullptr;
        int32_t* st = nullptr;
        size_t cgp = 0, csp = 0, cst = 0;
        pamo_stage3* s3 = nullptr;
        for (;;) {
            std::shared_ptr<Request> q;
            {
                std::unique_lock<std::mutex> lock(mu);
                cv_work.wait(lock, [&] { return stop || !ready.empty(); });
                if (stop && ready.empty()) break;
                q = ready.front();
                ready.pop_front();
            }
            const size_t np = q->points.size() / 3, nt = q->tris.size() / 3;
            int r = PAMO_OK;
            r = ensure_dev(dp, cp, np * 3, w.stream);
            if (!r) r = ensure_dev(dt, ct, nt * 3, w.stream);
            int32_t onp = 0, ont = 0;
            if (!r && q->stage3) {
                r = ensure_dev(rp, crp, np * 3, w.stream);
                if (!r) r = ensure_dev(rt, crt, nt * 3, w.stream);
            }
            if (!r) {
                cudaMemcpyAsync(dp, q->points.data(), np * 3 * sizeof(float), cudaMemcpyHostToDevice, w.stream);
                cudaMemcpyAsync(dt, q->tris.data(), nt * 3 * sizeof(int32_t), cudaMemcpyHostToDevice, w.stream);
                // without stage 3 the result is exported over the input copies (both at least as large)
                r = run_job(w, dp, dt, (int32_t)np, (int32_t)nt, q->ratio, q->tolerance, q->threshold, 1000000, 0,
                            q->stage3 ? rp : dp, q->stage3 ? rt : dt, &onp, &ont, &q->rounds, q->err);
            }
            if (!r && q->stage3) {
                r = stage3_job(w, s3, *q, dp, dt, rp, rt, onp, ont, gp, cgp, sp, csp, st, cst);
            } else if (!r) {
                q->out_points.resize((size_t)onp * 3);
                q->out_tris.resize((size_t)ont * 3);
                cudaMemcpyAsync(q->out_points.data(), dp, (size_t)onp * 3 * sizeof(float), cudaMemcpyDeviceToHost,
                                w.stream);
                cudaMemcpyAsync(q->out_tris.data(), dt, (size_t)ont * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                w.stream);
                if (cudaStreamSynchronize(w.stream) != cudaSuccess) {
                    r = PAMO_ERR_CUDA;
                    q->err = cudaGetErrorString(cudaGetLastError());
                }
            }
            q->status = r;
            q->t_done = Clock::now();
            {
                std::lock_guard<std::mutex> lock(mu);
                in_use -= q->bytes;
                ++n_finished;
                finished[q->id] = q;
                finished_order.push_back(q->id);
                admit_locked();
            }
            cv_work.notify_all();
            cv_done.notify_all();
        }
        for (void* b : {(void*)dp, (void*)dt, (void*)rp, (void*)rt, (void*)gp, (void*)sp, (void*)st})
            if (b) cudaFreeAsync(b, w.stream);
        cudaStreamSynchronize(w.stream);
        if (s3) pamo_stage3_destroy(s3);
    }
};

extern "C" {

int pamo_server_create(pamo_server** out, int device, int32_t n_workers, int64_t hbm_budget_bytes) {
    if (!out || n_workers < 1 || n_workers > 256 || hbm_budget_bytes <= 0) return PAMO_ERR_INVALID_ARG;
    *out = nullptr;
    auto* s = new pamo_server();
    s->device = device;
    s->budget = hbm_budget_bytes;
    int r = make_workers(device, n_workers, s->workers, s->err);
    if (!r) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess) {
            s->pool = nullptr;
            r = PAMO_ERR_CUDA;
        } else {
            unsigned long long keep = ~0ull;
            cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    if (r) {
        free_workers(device, s->workers);
        delete s;
        return r;
    }
    for (int i = 0; i < n_workers; ++i) s->threads.emplace_back(&pamo_server::worker_loop, s, i);
    *out = s;
    return PAMO_OK;
}

int pamo_server_destroy(pamo_server* s) {
    if (!s) return PAMO_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        s->queue.clear();  // not admitted: dropped
    }
    s->cv_work.notify_all();
    for (auto& t : s->threads) t.join();
    free_workers(s->device, s->workers);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return PAMO_OK;
}

int pamo_server_submit(pamo_server* s, const float* points, const int32_t* triangles, int32_t n_points,
                       int32_t n_triangles, double ratio, int32_t tolerance, float threshold, int64_t* request_id) {
    return pamo_server_submit_ex(s, points, triangles, n_points, n_triangles, ratio, tolerance, threshold, 0,
                                 request_id);
}

int pamo_server_submit_ex(pamo_server* s, const float* points, const int32_t* triangles, int32_t n_points,
                          int32_t n_triangles, double ratio, int32_t tolerance, float threshold, int32_t use_stage3,
                          int64_t* request_id) {
    if (!s || !points || !triangles || n_points < 1 || n_triangles < 1 || !request_id) return PAMO_ERR_INVALID_ARG;
    auto q = std::make_shared<Request>();
    q->stage3 = use_stage3 != 0;
    q->points.assign(points, points + 3 * (size_t)n_points);
    q->tris.assign(triangles, triangles + 3 * (size_t)n_triangles);
    q->ratio = ratio;
    q->tolerance = tolerance;
    q->threshold = threshold;
    q->bytes = job_bytes(n_points, n_triangles) + (q->stage3 ? stage3_bytes(n_points, n_triangles) : 0);
    q->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->stop) return PAMO_ERR_STATE;
        q->id = s->next_id++;
        *request_id = q->id;
        s->queue.push_back(q);
        s->admit_locked();
    }
    s->cv_work.notify_all();
    return PAMO_OK;
}

int pamo_server_wait(pamo_server* s, int32_t timeout_ms, int64_t* request_id, int32_t* status, int32_t* out_n_points,
                     int32_t* out_n_triangles, double* times_ms) {
    if (!s || !request_id) return PAMO_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lock(s->mu);
    if (!s->cv_done.wait_for(lock, std::chrono::milliseconds(std::max(0, timeout_ms)),
                             [&] { return !s->finished_order.empty(); }))
        return 0;
    const int64_t id = s->finished_order.front();
    s->finished_order.pop_front();
    const auto& q = s->finished[id];
    *request_id = id;
    if (status) *status = q->status;
    if (out_n_points) *out_n_points = (int32_t)(q->out_points.size() / 3);
    if (out_n_triangles) *out_n_triangles = (int32_t)(q->out_tris.size() / 3);
    if (times_ms) {
        times_ms[0] = ms_between(q->t_submit, q->t_admit);  // queued until admitted
        times_ms[1] = ms_between(q->t_admit, q->t_done);    // admitted until finished
        times_ms[2] = ms_between(q->t_submit, q->t_done);   // submitted until finished
    }
    return 1;
}

int pamo_server_fetch(pamo_server* s, int64_t request_id, float* points, int32_t* triangles) {
    if (!s) return PAMO_ERR_INVALID_ARG;
    std::shared_ptr<Request> q;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        auto it = s->finished.find(request_id);
        if (it == s->finished.end()) return PAMO_ERR_STATE;
        q = it->second;
        s->finished.erase(it);
    }
    if (q->status != PAMO_OK) {
        std::lock_guard<std::mutex> lock(s->mu);
        s->err = q->err;
        return q->status;
    }
    if (points) std::memcpy(points, q->out_points.data(), q->out_points.size() * sizeof(float));
    if (triangles) std::memcpy(triangles, q->out_tris.data(), q->out_tris.size() * sizeof(int32_t));
    return PAMO_OK;
}

int pamo_server_fetch_f64(pamo_server* s, int64_t request_id, double* points, int32_t* triangles) {
    if (!s) return PAMO_ERR_INVALID_ARG;
    std::shared_ptr<Request> q;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        auto it = s->finished.find(request_id);
        if (it == s->finished.end()) return PAMO_ERR_STATE;
        q = it->second;
        s->finished.erase(it);
    }
    if (q->status != PAMO_OK) {
        std::lock_guard<std::mutex> lock(s->mu);
        s->err = q->err;
        return q->status;
    }
    if (points) {
        if (!q->out_points64.empty()) std::memcpy(points, q->out_points64.data(), q->out_points64.size() * sizeof(double));
        else
            for (size_t i = 0; i < q->out_points.size(); ++i) points[i] = q->out_points[i];
    }
    if (triangles) std::memcpy(triangles, q->out_tris.data(), q->out_tris.size() * sizeof(int32_t));
    return PAMO_OK;
}

const char* pamo_server_last_error(const pamo_server* s) { return s ? s->err.c_str() : "null server"; }

int pamo_server_stats(pamo_server* s, int64_t* out, int32_t n) {
    if (!s || !out) return PAMO_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lock(s->mu);
    const int64_t v[7] = {s->in_use,   s->max_in_use, s->n_admitted,      s->n_finished, (int64_t)s->queue.size(),
                          s->budget, s->n_stage3_reruns};
    for (int i = 0; i < n && i < 7; ++i) out[i] = v[i];
    return 7;
}

int64_t pamo_server_job_bytes(int32_t n_points, int32_t n_triangles) { return job_bytes(n_points, n_triangles); }

int pamo_mesh_process(const double* points, int32_t n_points, const int32_t* triangles, int32_t n_triangles,
                      double* out_points, int32_t* out_n_points, int32_t* out_triangles, int32_t* out_n_triangles) {
    if (n_points < 0 || n_triangles < 0 || (n_points && !points) || (n_triangles && !triangles) || !out_n_points ||
        !out_n_triangles || (n_points && !out_points) || (n_triangles && !out_triangles))
        return PAMO_ERR_INVALID_ARG;
    for (int64_t i = 0; i < 3 * (int64_t)n_triangles; ++i)
        if (triangles[i] < 0 || triangles[i] >= n_points) return PAMO_ERR_INVALID_ARG;
    std::vector<double> V(points, points + 3 * (size_t)n_points), Vo;
    std::vector<int32_t> F(triangles, triangles + 3 * (size_t)n_triangles), Fo;
    mesh_process(V, F, Vo, Fo);
    std::copy(Vo.begin(), Vo.end(), out_points);
    std::copy(Fo.begin(), Fo.end(), out_triangles);
    *out_n_points = (int32_t)(Vo.size() / 3);
    *out_n_triangles = (int32_t)(Fo.size() / 3);
    return PAMO_OK;
}

}  // extern "C"
