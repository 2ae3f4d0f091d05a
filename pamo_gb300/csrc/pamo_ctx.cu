// Host driver of the PaMO stage-2 GB300 path and its C ABI (include/pamo_gb300.h).
//
// The context owns every device buffer (grow-only) and the state the reference keeps between forward()
// calls: the edge-cost buffer whose stale entries are read back in stuck rounds, the invalid-vertex table,
// the previous call's compaction map and the undo-vertex list (simp_cuda/src/cusimp_free.h:184-280). The
// reference's capacity policy (new capacity = n + n/5, fresh buffers read as zero) is kept for these
// buffers because it decides when their contents are reset.
#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/pamo_gb300.h"
#include "lbvh.cuh"
#include "pamo_common.cuh"
#include "scan.cuh"
#include "simp_round.cuh"

using namespace pamo;

namespace {

constexpr float kCostRange = 10.0f;
constexpr int kMaxExtraPasses = 5;  // cusimp_free.cu:1039
constexpr float kTriEps = 1e-3f;    // cusimp_free.cu:893

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;  // elements
    size_t bytes() const { return p ? n * sizeof(T) : 0; }
};


}  // namespace

// Phase timers (CUDA events on the context's stream), enabled with pamo_profile_enable.
enum Phase { kPhLoad, kPhAdj, kPhQuad, kPhCost, kPhCollapse, kPhMarks, kPhBvh, kPhQuery, kPhUndo, kPhCompact, kPhCenter,
             kNumPhases };

struct Profiler {
    bool on = false;
    cudaEvent_t ev[2 * kNumPhases] = {};
    bool pending[kNumPhases] = {};
    double ms[kNumPhases] = {};
    long long count[kNumPhases] = {};
    bool ready = false;
    void create() {
        if (ready) return;
        for (auto& e : ev) cudaEventCreate(&e);
        ready = true;
    }
    void destroy() {
        if (!ready) return;
        for (auto& e : ev) cudaEventDestroy(e);
        ready = false;
    }
    void begin(int p, cudaStream_t s) {
        if (!on) return;
        cudaEventRecord(ev[2 * p], s);
    }
    void end(int p, cudaStream_t s) {
        if (!on) return;
        cudaEventRecord(ev[2 * p + 1], s);
        pending[p] = true;
    }
    // called after a stream synchronisation
    void collect() {
        if (!on) return;
        for (int p = 0; p < kNumPhases; ++p)
            if (pending[p]) {
                float t = 0.f;
                cudaEventElapsedTime(&t, ev[2 * p], ev[2 * p + 1]);
                ms[p] += t;
                count[p] += 1;
                pending[p] = false;
            }
    }
};

struct pamo_ctx {
    int device = 0;
    Profiler prof;
    std::string err;
    cudaStream_t stream = nullptr;

    // ---- capacities ----
    size_t cap_v = 0;    // physical per-vertex capacity
    size_t cap_f = 0;    // physical per-face capacity
    size_t cap_ec = 0;   // physical edge-cost length
    size_t logical_pts = 0;  // reference's allocated_pts

    // ---- persistent reference state ----
    DevBuf<uint32_t> edge_cost;
    DevBuf<unsigned char> invalid;
    DevBuf<int> pts_map, undo_list, tmp_undo;
    DevBuf<int> pts_map_prev;  // device rounds: the previous round's map while this round's replaces pts_map
    int* d_ecap = nullptr;  // reference's allocated_edge_cost, kept on the device

    // ---- per-vertex working buffers ----
    DevBuf<float4> pos, orig_pos, pos_in, pos_out;
    DevBuf<int> occ, valence, cursor;
    DevBuf<int> vedges, vcursor;  // edges per lower endpoint (offsets) and fill cursors
    DevBuf<Quadric> quad;
    DevBuf<Quadric> quad_lo;  // precision modes: the quadrics' lo parts (q = quad + quad_lo in double-float)
    DevBuf<unsigned long long> vmin;
    DevBuf<int> undo_in;

    // ---- per-face ----
    DevBuf<int4> tri, orig_tri, tri_in, tri_out;
    DevBuf<int> ecount, qflag, qlist, fflags, nt, shuffle_flags;
    DevBuf<int> nxt;        // per CSR slot: the vertex after the ring's vertex in the slot's face
    DevBuf<int2> spc;       // per CSR slot: the vertex before it and its corner
    DevBuf<float4> fgeo;    // per face: a 64-byte ring record, then the planes (room for six float4 per face)
    DevBuf<unsigned long long> fkey;
    DevBuf<unsigned char> hit;
    BvhBuffers bvh;
    char* bvh_mem = nullptr;
    size_t bvh_cap = 0;

    // ---- per-edge ----
    DevBuf<int2> edges;
    DevBuf<int> win, collapsed, uflag;
    DevBuf<int> eorder;  // edge ids grouped by lower endpoint
    DevBuf<int2> exact_list;  // candidate pairs of the self-intersection check

    // ---- small ----
    RoundCounters* rc = nullptr;
    RoundCounters* h_rc = nullptr;  // pinned
    int* scan_scratch = nullptr;
    float* d_scale = nullptr;
    float* d_center = nullptr;  // [16]
    LoopState* d_ls = nullptr;  // [0] this round, [1] the next one
    cudaStream_t own_stream = nullptr;  // for callers on the legacy default stream (graphs need a capturable one)
    cudaEvent_t ev_join = nullptr;

    int ensure_own_stream() {
        if (own_stream) return PAMO_OK;
        if (cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming) != cudaSuccess)
            return fail(PAMO_ERR_CUDA, "stream creation");
        return PAMO_OK;
    }

    // captured device-driven rounds: (input buffer, face class, vertex class, kind) -> graph; dropped whenever
    // a buffer is reallocated (kernel arguments hold the buffer addresses)
    struct RoundGraph {
        cudaGraphExec_t exec = nullptr;
        long long kernels = 0;
    };
    std::map<std::tuple<const void*, int, int, int>, RoundGraph> graphs;
    bool use_graphs = true;     // device rounds as cached graphs
    bool device_rounds = true;  // rounds after the first from device-resident sizes (pamo_simplify_device)
    bool bvh_reuse = true;      // device rounds refit the LBVH carried from the previous round
    bool skinny_pow = false;    // 1: the skinny term squares with the device's pow(float, int), as the reference does
                                // (12x slower edge cost; every measured job is bit-identical with either form)
    int precision = 0;          // 0 the reference's arithmetic; 1 compensated sums; 2 compensated, optimal placement
    DevBuf<float4> place;       // precision 2: each edge's placement
    DevBuf<float> probe_raw;    // pamo_cost_probe: each edge's cost before quantisation
    int ensure_place(size_t n_edges) { return precision == 2 ? grow(place, n_edges) : PAMO_OK; }
    float4* place_ptr() { return precision == 2 ? place.p : nullptr; }
    int ensure_quad_lo() { return precision > 0 && cap_v ? grow(quad_lo, cap_v) : PAMO_OK; }
    Quadric* qlo_ptr() { return precision > 0 ? quad_lo.p : nullptr; }
    long long pair_cap_limit = 0;  // > 0: at most this many listed candidate pairs per check (tests the overflow path)

    int pair_cap() const {
        const long long n = (long long)exact_list.n;
        return (int)(pair_cap_limit > 0 && pair_cap_limit < n ? pair_cap_limit : n);
    }
    DevBuf<float> face_mean;
    float* h_pinned_f = nullptr;

    // ---- results of the last round / run ----
    bool have_round = false;
    int out_np = 0, out_nt = 0, out_nu = 0;
    RoundCounters last{};
    bool have_run = false;
    int run_np = 0, run_nt = 0;
    std::vector<int> faces_per_round;
    std::vector<double> round_ms;  // host wall time of each round of the last loop (rounds end with a sync)
    std::vector<double> round_gpu_ms;  // device time of each device round's graph launches (events around them)
    // edge-cost kernel timer: events recorded around every k_edge_cost launch (captured into the round graphs)
    bool time_cost = false;
    cudaEvent_t ev_c0 = nullptr, ev_c1 = nullptr;
    double cost_ms = 0.0;
    long long cost_n = 0;
    // recorded as event-record nodes when the stream is being captured into a round graph (the external flag is
    // valid only during a capture)
    void record_timer(cudaEvent_t ev, cudaStream_t s) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(s, &cs);
        if (cs == cudaStreamCaptureStatusActive) cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal);
        else cudaEventRecord(ev, s);
    }
    void cost_begin(cudaStream_t s) {
        if (time_cost) record_timer(ev_c0, s);
    }
    void cost_end(cudaStream_t s) {
        if (time_cost) record_timer(ev_c1, s);
    }
    // after the stream was synchronised: add the last edge-cost launch's duration
    void cost_note() {
        float t = 0.f;
        if (time_cost && cudaEventElapsedTime(&t, ev_c0, ev_c1) == cudaSuccess) {
            cost_ms += t;
            ++cost_n;
        }
    }
    cudaEvent_t ev_g0 = nullptr, ev_g1 = nullptr;
    bool time_rounds = false;  // option "time_rounds": timing events around the round graphs (off: events with
                               // timing on every launch cost concurrency between the streams of a worker pool)
    double cur_gpu_ms = 0.0;
    // totals over the rounds of the last pamo_simplify_device call
    long long tot[10] = {};

    int fail(int code, const char* fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }

    int check(cudaError_t e, const char* what) {
        if (e == cudaSuccess) return PAMO_OK;
        return fail(e == cudaErrorMemoryAllocation ? PAMO_ERR_OOM : PAMO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }

    void drop_graphs() {
        for (auto& kv : graphs)
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
    }

    template <typename T>
    int grow(DevBuf<T>& b, size_t n, bool keep = false, bool zero = false) {
        if (b.n >= n && b.p) return PAMO_OK;
        drop_graphs();
        T* p = nullptr;
        cudaError_t e = cudaMalloc((void**)&p, n * sizeof(T));
        if (e != cudaSuccess) return check(e, "cudaMalloc");
        if (zero) cudaMemsetAsync(p, 0, n * sizeof(T), stream);
        if (keep && b.p && b.n) cudaMemcpyAsync(p, b.p, b.n * sizeof(T), cudaMemcpyDeviceToDevice, stream);
        if (b.p) {
            cudaStreamSynchronize(stream);
            cudaFree(b.p);
        }
        b.p = p;
        b.n = n;
        return PAMO_OK;
    }

    int init() {
        int r;
        if ((r = check(cudaSetDevice(device), "cudaSetDevice"))) return r;
        if ((r = check(cudaMalloc((void**)&rc, sizeof(RoundCounters)), "cudaMalloc"))) return r;
        if ((r = check(cudaMallocHost((void**)&h_rc, sizeof(RoundCounters)), "cudaMallocHost"))) return r;
        if ((r = check(cudaMallocHost((void**)&h_pinned_f, 64 * sizeof(float)), "cudaMallocHost"))) return r;
        // one scratch per job of a combined scan launch (exclusive_scans)
        if ((r = check(cudaMalloc((void**)&scan_scratch, kMaxScanJobs * scan_scratch_ints() * sizeof(int)), "cudaMalloc")))
            return r;
        for (int k = 0; k < kMaxScanJobs; ++k)
            if (scan_scratch_clear(scan_scratch + k * scan_scratch_ints())) return check(cudaGetLastError(), "scan scratch");
        if ((r = check(cudaMalloc((void**)&d_ecap, sizeof(int)), "cudaMalloc"))) return r;
        if ((r = check(cudaMalloc((void**)&d_scale, sizeof(float)), "cudaMalloc"))) return r;
        if ((r = check(cudaMalloc((void**)&d_center, 16 * sizeof(float)), "cudaMalloc"))) return r;
        if ((r = check(cudaMalloc((void**)&d_ls, 2 * sizeof(LoopState)), "cudaMalloc"))) return r;
        cudaMemset(d_ecap, 0, sizeof(int));
        return PAMO_OK;
    }

    void release() {
        cudaSetDevice(device);
        cudaDeviceSynchronize();
        auto fr = [](auto& b) {
            if (b.p) cudaFree(b.p);
            b.p = nullptr;
            b.n = 0;
        };
        fr(edge_cost); fr(invalid); fr(pts_map); fr(pts_map_prev); fr(undo_list); fr(tmp_undo);
        fr(pos); fr(orig_pos); fr(pos_in); fr(pos_out); fr(occ); fr(valence); fr(cursor); fr(quad); fr(quad_lo); fr(vmin); fr(undo_in);
        fr(nxt); fr(spc); fr(fgeo); fr(tri); fr(orig_tri); fr(tri_in); fr(tri_out); fr(ecount); fr(qflag); fr(qlist); fr(fflags); fr(nt);
        fr(shuffle_flags); fr(fkey); fr(eorder); fr(vedges); fr(vcursor); fr(hit); fr(edges); fr(win); fr(collapsed); fr(uflag); fr(face_mean); fr(exact_list); fr(place); fr(probe_raw);
        if (bvh_mem) cudaFree(bvh_mem);
        bvh_mem = nullptr;
        prof.destroy();
        if (rc) cudaFree(rc);
        if (h_rc) cudaFreeHost(h_rc);
        if (h_pinned_f) cudaFreeHost(h_pinned_f);
        if (scan_scratch) cudaFree(scan_scratch);
        if (d_ecap) cudaFree(d_ecap);
        if (d_scale) cudaFree(d_scale);
        if (d_center) cudaFree(d_center);
        if (d_ls) cudaFree(d_ls);
        drop_graphs();
        if (ev_c0) cudaEventDestroy(ev_c0);
        if (ev_c1) cudaEventDestroy(ev_c1);
        ev_c0 = ev_c1 = nullptr;
        if (ev_g0) cudaEventDestroy(ev_g0);
        if (ev_g1) cudaEventDestroy(ev_g1);
        ev_g0 = ev_g1 = nullptr;
        if (own_stream) cudaStreamDestroy(own_stream);
        if (ev_join) cudaEventDestroy(ev_join);
        own_stream = nullptr;
        ev_join = nullptr;
        rc = nullptr;
    }

    // Reference allocation semantics for the per-vertex state (cusimp_free.cu:47-85): when n exceeds the
    // capacity the buffers are replaced by fresh (zero) ones of n + n/5 + 1 entries.
    int ensure_pts_state(size_t n) {
        if (n <= logical_pts && pts_map.p) return PAMO_OK;
        logical_pts = n + n / 5;
        const size_t len = logical_pts + 1;
        int r;
        // the reference allocates new (here: zero-filled) buffers; a large enough one is cleared in place
        auto fresh = [&](auto& b) {
            if (b.p && b.n >= len) {
                cudaMemsetAsync(b.p, 0, b.n * sizeof(*b.p), stream);
                return (int)PAMO_OK;
            }
            if (b.p) {
                cudaStreamSynchronize(stream);
                cudaFree(b.p);
                b.p = nullptr;
                b.n = 0;
            }
            return grow(b, len, false, true);
        };
        if ((r = fresh(invalid))) return r;
        if ((r = fresh(pts_map))) return r;
        if ((r = fresh(undo_list))) return r;
        if ((r = fresh(tmp_undo))) return r;
        if ((r = grow(pts_map_prev, len))) return r;
        return PAMO_OK;
    }

    // State as in a newly created context (a new CUSimp_Free in the reference): no logical capacities, and
    // the buffers the reference reads before writing zeroed when they are next sized. Buffers are kept.
    void reset_state(cudaStream_t s) {
        stream = s;
        logical_pts = 0;
        cudaMemsetAsync(d_ecap, 0, sizeof(int), s);
        if (edge_cost.p) cudaMemsetAsync(edge_cost.p, 0, edge_cost.n * sizeof(uint32_t), s);
        have_round = false;
        have_run = false;
    }

    size_t device_bytes() const {
        size_t b = 0;
        b += pos.bytes() + orig_pos.bytes() + pos_in.bytes() + pos_out.bytes() + occ.bytes() + valence.bytes() +
             cursor.bytes() + vedges.bytes() + vcursor.bytes() + quad.bytes() + quad_lo.bytes() + vmin.bytes() +
             undo_in.bytes();
        b += nxt.bytes() + spc.bytes() + fgeo.bytes();
        b += tri.bytes() + orig_tri.bytes() + tri_in.bytes() + tri_out.bytes() + ecount.bytes() + qflag.bytes() +
             qlist.bytes() + fflags.bytes() + nt.bytes() + shuffle_flags.bytes() + fkey.bytes() + hit.bytes() +
             edges.bytes() + win.bytes() + collapsed.bytes() + uflag.bytes() + eorder.bytes() + exact_list.bytes() +
             face_mean.bytes();
        b += edge_cost.bytes() + invalid.bytes() + pts_map.bytes() + pts_map_prev.bytes() + undo_list.bytes() +
             tmp_undo.bytes();
        b += bvh_cap ? bvh_bytes((int)bvh_cap) : 0;
        return b;
    }

    int ensure_vertex_buffers(size_t n) {
        const size_t c = n + 2;
        if (c <= cap_v && pos.p) return PAMO_OK;
        const size_t nc = c + c / 5;
        int r;
        if ((r = grow(pos, nc)) || (r = grow(orig_pos, nc)) || (r = grow(pos_out, nc)) || (r = grow(occ, nc + 1)) ||
            (r = grow(valence, nc + 1)) || (r = grow(cursor, nc)) || (r = grow(vedges, nc + 1)) || (r = grow(vcursor, nc)) || (r = grow(quad, nc)) || (r = grow(vmin, nc)) ||
            (r = grow(pos_in, nc)))
            return r;
        cap_v = nc;
        return ensure_quad_lo();
    }

    int ensure_face_buffers(size_t n) {
        if (n >= (size_t)(1 << 30) - 8) return fail(PAMO_ERR_CAPACITY, "more than 2^30 faces");
        const size_t c = n + 2;
        if (c <= cap_f && tri.p) return PAMO_OK;
        const size_t nc = c + c / 5;
        int r;
        if ((r = grow(tri, nc)) || (r = grow(orig_tri, nc)) || (r = grow(tri_in, nc)) || (r = grow(tri_out, nc)) ||
            (r = grow(ecount, nc + 1)) || (r = grow(qflag, nc + 1)) || (r = grow(qlist, nc)) || (r = grow(fflags, nc + 1)) ||
            (r = grow(nt, 3 * nc)) || (r = grow(nxt, 3 * nc)) || (r = grow(spc, 3 * nc)) || (r = grow(fgeo, 6 * nc)) || (r = grow(shuffle_flags, 2 * nc + 40)) || (r = grow(fkey, nc)) || (r = grow(hit, nc)) ||
            (r = grow(eorder, 2 * nc)) ||
            (r = grow(edges, 2 * nc)) || (r = grow(win, 2 * nc + 1)) || (r = grow(collapsed, 2 * nc)) ||
            (r = grow(uflag, 2 * nc + 1)) || (r = grow(face_mean, 3 * nc)) ||
            (r = grow(exact_list, std::max<size_t>(1 << 20, 16 * nc))))
            return r;
        // edge costs keep their stale contents when the physical buffer grows
        if ((r = grow(edge_cost, 2 * nc + 2 * nc / 5 + 2, true, true))) return r;
        if ((r = ensure_place(2 * nc))) return r;
        if (bvh_cap < nc) {
            drop_graphs();
            if (bvh_mem) {
                cudaStreamSynchronize(stream);
                cudaFree(bvh_mem);
                bvh_mem = nullptr;
            }
            cudaError_t e = cudaMalloc((void**)&bvh_mem, bvh_bytes((int)nc));
            if (e != cudaSuccess) return check(e, "cudaMalloc(bvh)");
            bvh_carve(bvh, (int)nc, bvh_mem);
            bvh_cap = nc;
        }
        cap_f = nc;
        return PAMO_OK;
    }

    // One round of the legacy simplifier CUSimp::forward (cusimp.cu:587-720): the cost without the penalty
    // factor and with the ring length counted twice, no invalid table, stuck mode, face clean-up,
    // self-intersection check or undo; the compaction map over n_pts + 1 entries.
    int legacy_round(const float* pts3, const int* tris3, int nP, int nT, float threshold, int init) {
        cudaStream_t s = stream;
        int r;
        if ((r = ensure_vertex_buffers(nP)) || (r = ensure_face_buffers(nT)) || (r = ensure_pts_state(nP))) return r;
        std::memset(h_rc, 0, sizeof(RoundCounters));
        h_rc->n_pts = nP;
        h_rc->n_tris = nT;
        cudaMemcpyAsync(rc, h_rc, sizeof(RoundCounters), cudaMemcpyHostToDevice, s);
        const uint32_t collapse_t = collapse_threshold(threshold);
        launch_load_points(pts3, nP, pos.p, orig_pos.p, occ.p, s);
        int4* tri_src = init ? tri_in.p : tri.p;
        launch_load_tris(tris3, nT, nP, tri_src, rc, s);
        if (init) {
            Feistel fb = make_feistel((unsigned long long)nT);
            if (nT > 0) launch_shuffle_tris(fb, shuffle_flags.p, scan_scratch, tri_src, tri.p, nT, s, &rc->status);
        }
        cudaMemsetAsync(valence.p, 0, (nP + 1) * sizeof(int), s);
        cudaMemsetAsync(cursor.p, 0, (nP + 1) * sizeof(int), s);
        cudaMemsetAsync(vedges.p, 0, (nP + 1) * sizeof(int), s);
        cudaMemsetAsync(vcursor.p, 0, (nP + 1) * sizeof(int), s);
        launch_face_counts(tri.p, rc, nT, valence.p, ecount.p, vedges.p, s, pos.p, fgeo.p);
        scan_adjacency_counts(s, std::max(nP, nT));
        launch_fill_adjacency(tri.p, rc, nT, valence.p, cursor.p, nt.p, ecount.p, edges.p, vedges.p, vcursor.p, eorder.p, s);
        launch_sort_adjacency(rc, nP, valence.p, nt.p, s);
        const int* nt_off = valence.p;
        const int eb = 2 * nT;
        launch_quadrics(rc, nP, nt_off, nt.p, tri.p, fgeo.p, quad.p, nxt.p, spc.p, s);
        launch_edge_cost_capacity(rc, d_ecap, edge_cost.p, (int)edge_cost.n, s);
        cudaMemsetAsync(vmin.p, 0xFF, (nP + 1) * sizeof(unsigned long long), s);
        launch_edge_cost(rc, eb, eorder.p, edges.p, nt_off, nt.p, tri.p, pos.p, quad.p, fgeo.p, nxt.p, spc.p, invalid.p, edge_cost.p, vmin.p,
                         d_scale, threshold, 0, s, nullptr, true, skinny_pow);
        launch_face_keys(rc, nT, tri.p, vmin.p, fkey.p, s);
        launch_collapse(rc, eb, eorder.p, edges.p, edge_cost.p, collapse_t, fkey.p, nt_off, nt.p, tri.p, orig_tri.p, pos.p,
                        orig_pos.p, occ.p, win.p, s, false);
        exclusive_scan(occ.p, pts_map.p, &rc->n_pts, 1, nullptr, scan_scratch, s, &rc->status, nP);
        if ((r = read_counters())) return r;
        if ((r = status_to_error(h_rc->status))) return r;
        last = *h_rc;
        last.n_vertices_undo = 0;
        return PAMO_OK;
    }

    // pamo_cost_probe: one round up to the edge costs (no shuffle, no collapse) with the given precision mode; the
    // edges, their costs before quantisation and their placements stay in edges / probe_raw / place.
    int probe(const float* pts3, const int* tris3, int nP, int nT, float threshold, int mode) {
        cudaStream_t s = stream;
        const int keep = precision;
        precision = mode;
        int r;
        if ((r = ensure_vertex_buffers(nP)) || (r = ensure_face_buffers(nT)) || (r = ensure_pts_state(nP)) ||
            (r = grow(probe_raw, 2 * cap_f)) || (r = grow(place, 2 * cap_f)) || (mode > 0 && (r = grow(quad_lo, cap_v)))) {
            precision = keep;
            return r;
        }
        std::memset(h_rc, 0, sizeof(RoundCounters));
        h_rc->n_pts = nP;
        h_rc->n_tris = nT;
        cudaMemcpyAsync(rc, h_rc, sizeof(RoundCounters), cudaMemcpyHostToDevice, s);
        launch_load_points(pts3, nP, pos.p, orig_pos.p, occ.p, s);
        launch_load_tris(tris3, nT, nP, tri.p, rc, s);
        cudaMemsetAsync(valence.p, 0, (nP + 1) * sizeof(int), s);
        cudaMemsetAsync(cursor.p, 0, (nP + 1) * sizeof(int), s);
        cudaMemsetAsync(vedges.p, 0, (nP + 1) * sizeof(int), s);
        cudaMemsetAsync(vcursor.p, 0, (nP + 1) * sizeof(int), s);
        cudaMemsetAsync(invalid.p, 0, invalid.n, s);
        launch_face_counts(tri.p, rc, nT, valence.p, ecount.p, vedges.p, s, pos.p, fgeo.p, mode > 0);
        scan_adjacency_counts(s, std::max(nP, nT));
        launch_fill_adjacency(tri.p, rc, nT, valence.p, cursor.p, nt.p, ecount.p, edges.p, vedges.p, vcursor.p, eorder.p, s);
        launch_sort_adjacency(rc, nP, valence.p, nt.p, s);
        Quadric* qlo = mode > 0 ? quad_lo.p : nullptr;
        launch_quadrics(rc, nP, valence.p, nt.p, tri.p, fgeo.p, quad.p, nxt.p, spc.p, s, qlo);
        cudaMemsetAsync(vmin.p, 0xFF, (nP + 1) * sizeof(unsigned long long), s);
        cudaMemsetAsync(probe_raw.p, 0xFF, probe_raw.n * sizeof(float), s);  // NaN where no cost is computed
        launch_edge_cost(rc, 2 * nT, eorder.p, edges.p, valence.p, nt.p, tri.p, pos.p, quad.p, fgeo.p, nxt.p, spc.p, invalid.p,
                         edge_cost.p, vmin.p, d_scale, threshold, 0, s, nullptr, false, skinny_pow, mode, probe_raw.p,
                         place.p, qlo);
        precision = keep;
        if ((r = read_counters())) return r;
        return status_to_error(h_rc->status);
    }

    // Host copy of the counters (synchronises the stream).
    int read_counters() {
        int r;
        if ((r = check(cudaGetLastError(), "kernel launch"))) return r;
        cudaMemcpyAsync(h_rc, rc, sizeof(RoundCounters), cudaMemcpyDeviceToHost, stream);
        r = check(cudaStreamSynchronize(stream), "round");
        prof.collect();
        return r;
    }

    // One device-driven round (the rounds after the first in pamo_simplify_device): every size and flag comes
    // from d_ls and rc, and nPb/nTb only bound the grids, so the same launches serve every round of a size
    // class and can be captured as a graph. kind 0 / 2: the whole round, with the compaction and the next
    // round's state computed as if no undo pass follows, building the LBVH afresh (0) or refitting the one
    // carried from the previous round (2); kind 1: one more undo pass (cusimp_free.cu:1016-1040), then the
    // compaction and next state again. The same kernels and order as round() plus the compaction of
    // simplify_loop; the LBVH only filters candidate pairs, so building or refitting gives the same pairs.
    void round_dev(int kind, int nPb, int nTb, float threshold) {
        cudaStream_t s = stream;
        const int* nt_off = valence.p;
        const int eb = 2 * nTb;
        const int list_cap = (int)undo_list.n;
        const uint32_t collapse_t = collapse_threshold(threshold);
        if (kind != 1) {
            launch_round_begin(rc, d_ls, d_ls + 1, s);
            launch_undo_bookkeeping_dev(undo_in.p, d_ls, list_cap, tmp_undo.p, undo_list.p, pts_map.p, (int)pts_map.n,
                                        invalid.p, (int)invalid.n, s);
            launch_round_prologue_dev(d_ls, rc, nPb, nTb, pts_map.p, pts_map_prev.p, pos_in.p, pos.p, orig_pos.p, occ.p,
                                      tri_in.p, tri.p, orig_tri.p, valence.p, cursor.p, vedges.p, vcursor.p, qflag.p, s);
            launch_face_counts(tri.p, rc, nTb, valence.p, ecount.p, vedges.p, s, pos.p, fgeo.p, precision > 0);
            scan_adjacency_counts(s, std::max(nPb, nTb));
            launch_fill_adjacency(tri.p, rc, nTb, valence.p, cursor.p, nt.p, ecount.p, edges.p, vedges.p, vcursor.p,
                                  eorder.p, s);
            launch_sort_adjacency(rc, nPb, valence.p, nt.p, s);
            launch_quadrics(rc, nPb, nt_off, nt.p, tri.p, fgeo.p, quad.p, nxt.p, spc.p, s, qlo_ptr());
            launch_edge_cost_capacity(rc, d_ecap, edge_cost.p, (int)edge_cost.n, s);
            launch_fill_u64_dev(rc, nPb, vmin.p, ~0ull, s);
            cost_begin(s);
            launch_edge_cost(rc, eb, eorder.p, edges.p, nt_off, nt.p, tri.p, pos.p, quad.p, fgeo.p, nxt.p, spc.p, invalid.p, edge_cost.p,
                             vmin.p, d_scale, threshold, 0, s, &d_ls->is_stuck, false, skinny_pow, precision, nullptr,
                             place_ptr(), qlo_ptr());
            cost_end(s);
            launch_face_keys(rc, nTb, tri.p, vmin.p, fkey.p, s);
            launch_collapse(rc, eb, eorder.p, edges.p, edge_cost.p, collapse_t, fkey.p, nt_off, nt.p, tri.p, orig_tri.p,
                            pos.p, orig_pos.p, occ.p, win.p, s, true, place_ptr());
            exclusive_scan(win.p, win.p, &rc->n_edges, 1, &rc->n_win, scan_scratch, s, &rc->status, eb);
            launch_compact_winners(rc, eb, win.p, collapsed.p, s);
            launch_remove_invalid(rc, nTb, tri.p, s);
            launch_line_edges(rc, eb, edges.p, nt_off, nt.p, tri.p, pos.p, occ.p, nullptr, (int)collapsed.n,
                              collapsed.p, s);
            launch_mark_query(rc, eb, collapsed.p, edges.p, nt_off, nt.p, qflag.p, s);
            exclusive_scan(qflag.p, qflag.p, &rc->n_tris, 1, &rc->n_query, scan_scratch, s, &rc->status, nTb);
            launch_compact_flags(qflag.p, nTb, &rc->n_tris, qlist.p, s);
        } else {
            launch_undo_apply(rc, eb, collapsed.p, uflag.p, edges.p, nt_off, nt.p, tri.p, orig_tri.p, pos.p, orig_pos.p,
                              occ.p, tmp_undo.p, undo_list.p, pts_map_prev.p, list_cap, s);
        }
        // intersection check; the LBVH spans every face slot of the round and is refitted when reused
        launch_zero_face_bytes_dev(rc, nTb, hit.p, s);
        if (kind == 0) bvh_build(bvh, tri.p, pos.p, rc, nTb, s, true, qflag.p, false);
        else bvh_refit_faces(bvh, tri.p, pos.p, rc, nTb, s, kind == 2, qflag.p);
        bvh_query(bvh, tri.p, pos.p, qlist.p, qflag.p, hit.p, exact_list.p, pair_cap(), rc, nTb, kTriEps, s);
        launch_undo_check(rc, eb, collapsed.p, edges.p, nt_off, nt.p, hit.p, uflag.p, s);
        exclusive_scan(uflag.p, uflag.p, &rc->n_considered, 1, &rc->n_undo, scan_scratch, s, &rc->status, eb);
        launch_after_check(rc, s);
        // compaction map (cusimp_free.cu:1042-1045), compaction (pamo/__init__.py:136-140), next round's state
        launch_live_flags(rc, nTb, tri.p, fflags.p, s);
        scan_compaction_maps(s, std::max(nPb, nTb));
        launch_compact_mesh(rc, nPb, nTb, pos.p, occ.p, pts_map.p, tri.p, fflags.p, pos_out.p, tri_out.p, s);
        bvh_remap(bvh, fflags.p, nTb, s);  // the tree's leaves in the next round's face numbering
        launch_round_end(rc, d_ls, d_ls + 1, undo_list.p, undo_in.p, (int)std::min(undo_in.n, undo_list.n), list_cap, s);
    }

    // Vertex valences, per-face edge counts (their total is the edge count) and per-vertex edge counts, scanned
    // by one launch (three independent scans, each on its own scratch).
    void scan_adjacency_counts(cudaStream_t s, long long bound) {
        const size_t sz = scan_scratch_ints();
        const ScanJob jobs[3] = {{valence.p, valence.p, &rc->n_pts, 1, nullptr, scan_scratch},
                                 {ecount.p, ecount.p, &rc->n_tris, 1, &rc->n_edges, scan_scratch + sz},
                                 {vedges.p, vedges.p, &rc->n_pts, 1, nullptr, scan_scratch + 2 * sz}};
        exclusive_scans(jobs, 3, s, &rc->status, bound);
    }

    // The vertex compaction map (occ -> pts_map) and the live-face offsets, scanned by one launch.
    void scan_compaction_maps(cudaStream_t s, long long bound) {
        const size_t sz = scan_scratch_ints();
        const ScanJob jobs[2] = {{occ.p, pts_map.p, &rc->n_pts, 1, nullptr, scan_scratch},
                                 {fflags.p, fflags.p, &rc->n_tris, 1, nullptr, scan_scratch + sz}};
        exclusive_scans(jobs, 2, s, &rc->status, bound);
    }

    // Enqueue round_dev through a cached graph of its size class (or directly when graphs are off or the
    // phase timers are on).
    int run_round_dev(int kind, int np, int nf, float threshold) {
        // size class: the next power of two from 1024 up to 2^19; every grid is at its cap from 2^19 elements on,
        // and all loops are grid-stride over the device sizes
        auto cls = [](int n) {
            int b = 1024;
            while (b < n && b < (1 << 19)) b <<= 1;
            return b;
        };
        const int nPb = cls(np), nTb = cls(nf);
        if (!use_graphs || prof.on) {
            round_dev(kind, nPb, nTb, threshold);
            return check(cudaGetLastError(), "kernel launch");
        }
        int tbits;
        std::memcpy(&tbits, &threshold, sizeof(int));
        const auto key = std::make_tuple((const void*)pos_in.p, nTb * 4 + kind, nPb, tbits);
        auto it = graphs.find(key);
        if (it == graphs.end()) {
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                return fail(PAMO_ERR_CUDA, "stream capture");
            const long long l0 = launches_so_far();
            round_dev(kind, nPb, nTb, threshold);
            RoundGraph rg;
            rg.kernels = launches_so_far() - l0;
            note_launches(-rg.kernels);  // counted when the graph runs
            if (cudaStreamEndCapture(stream, &g) != cudaSuccess || !g) return fail(PAMO_ERR_CUDA, "stream capture");
            const cudaError_t e = cudaGraphInstantiate(&rg.exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail(PAMO_ERR_CUDA, "graph instantiation");
            it = graphs.emplace(key, rg).first;
        }
        if (time_rounds && !ev_g0) {
            cudaEventCreate(&ev_g0);
            cudaEventCreate(&ev_g1);
        }
        if (time_rounds) cudaEventRecord(ev_g0, stream);
        if (cudaGraphLaunch(it->second.exec, stream) != cudaSuccess) return fail(PAMO_ERR_CUDA, "graph launch");
        if (time_rounds) cudaEventRecord(ev_g1, stream);
        note_launches(it->second.kernels);
        return PAMO_OK;
    }

    // device time of the graph launched last (call after the stream has been synchronised)
    void note_graph_time() {
        float ms = 0.f;
        if (time_rounds && ev_g0 && cudaEventElapsedTime(&ms, ev_g0, ev_g1) == cudaSuccess) cur_gpu_ms += ms;
    }

    int status_to_error(int bits) {
        if (bits & kErrBadIndex) return fail(PAMO_ERR_INVALID_ARG, "a triangle references a vertex outside [0, n_points)");
        if (bits & kErrStackOverflow) return fail(PAMO_ERR_ITER_LIMIT, "BVH traversal stack overflow");
        if (bits & kErrIterLimit) return fail(PAMO_ERR_ITER_LIMIT, "a bounded device loop hit its iteration limit");
        if (bits & kErrCapacity) return fail(PAMO_ERR_CAPACITY, "the undo-vertex list overflowed its capacity");
        return PAMO_OK;
    }

    // One forward() round. Points come either as AoS float [n,3] (pts3) or float4 (pts4); faces as AoS int
    // [m,3] (tris3, validated) or int4 (tris4). `shuffle` applies the reference's init shuffle.
    int round(const float* pts3, const float4* pts4, const int* tris3, const int4* tris4, const int* verts_undo, int nU,
              int nP, int nT, float threshold, int is_stuck, int init, bool operator_mode) {
        cudaStream_t s = stream;
        int r;
        if ((r = ensure_vertex_buffers(nP)) || (r = ensure_face_buffers(nT))) return r;
        if (is_stuck && nU > 0) {
            if (!pts_map.p) return fail(PAMO_ERR_STATE, "a stuck round needs a previous round on this context");
            if ((size_t)nU > undo_list.n) return fail(PAMO_ERR_CAPACITY, "verts_undo longer than the undo list");
        }

        // counters; a stuck round starts its undo list with the carried-over entries
        std::memset(h_rc, 0, sizeof(RoundCounters));
        h_rc->n_pts = nP;
        h_rc->n_tris = nT;
        if (is_stuck) {
            h_rc->first_undo = nU;
            h_rc->n_vertices_undo = nU;
        }
        cudaMemcpyAsync(rc, h_rc, sizeof(RoundCounters), cudaMemcpyHostToDevice, s);

        // undo-list bookkeeping with the previous call's map (cusimp_free.cu:895-918)
        launch_undo_bookkeeping(verts_undo, nU, is_stuck, tmp_undo.p, undo_list.p, pts_map.p, (int)pts_map.n, invalid.p,
                                (int)invalid.n, s);
        if ((r = ensure_pts_state(nP))) return r;

        const uint32_t collapse_t = collapse_threshold(threshold);

        // inputs
        prof.begin(kPhLoad, s);
        if (pts3) launch_load_points(pts3, nP, pos.p, orig_pos.p, occ.p, s);
        else launch_load_points4(pts4, nP, pos.p, orig_pos.p, occ.p, s);
        int4* tri_src = init ? tri_in.p : tri.p;
        if (tris3) launch_load_tris(tris3, nT, nP, tri_src, rc, s);
        else if (tri_src != tris4) launch_load_tris4(tris4, nT, tri_src, s);
        if (init) {
            Feistel fb = make_feistel((unsigned long long)nT);
            if (nT > 0) launch_shuffle_tris(fb, shuffle_flags.p, scan_scratch, tri_src, tri.p, nT, s, &rc->status);
        }
        launch_copy_tris(tri.p, orig_tri.p, nT, s);
        prof.end(kPhLoad, s);

        // adjacency
        prof.begin(kPhAdj, s);
        cudaMemsetAsync(valence.p, 0, (nP + 1) * sizeof(int), s);
        cudaMemsetAsync(cursor.p, 0, (nP + 1) * sizeof(int), s);
        cudaMemsetAsync(vedges.p, 0, (nP + 1) * sizeof(int), s);
        cudaMemsetAsync(vcursor.p, 0, (nP + 1) * sizeof(int), s);
        launch_face_counts(tri.p, rc, nT, valence.p, ecount.p, vedges.p, s, pos.p, fgeo.p, precision > 0);
        scan_adjacency_counts(s, std::max(nP, nT));
        launch_fill_adjacency(tri.p, rc, nT, valence.p, cursor.p, nt.p, ecount.p, edges.p, vedges.p, vcursor.p, eorder.p, s);
        launch_sort_adjacency(rc, nP, valence.p, nt.p, s);
        const int* nt_off = valence.p;
        const int eb = 2 * nT;
        prof.end(kPhAdj, s);

        // cost and selection
        prof.begin(kPhQuad, s);
        launch_quadrics(rc, nP, nt_off, nt.p, tri.p, fgeo.p, quad.p, nxt.p, spc.p, s, qlo_ptr());
        prof.end(kPhQuad, s);
        launch_edge_cost_capacity(rc, d_ecap, edge_cost.p, (int)edge_cost.n, s);
        cudaMemsetAsync(vmin.p, 0xFF, (nP + 1) * sizeof(unsigned long long), s);
        prof.begin(kPhCost, s);
        cost_begin(s);
        launch_edge_cost(rc, eb, eorder.p, edges.p, nt_off, nt.p, tri.p, pos.p, quad.p, fgeo.p, nxt.p, spc.p, invalid.p, edge_cost.p, vmin.p,
                         d_scale, threshold, is_stuck, s, nullptr, false, skinny_pow, precision, nullptr, place_ptr(),
                         qlo_ptr());
        cost_end(s);
        prof.end(kPhCost, s);
        prof.begin(kPhCollapse, s);
        launch_face_keys(rc, nT, tri.p, vmin.p, fkey.p, s);
        launch_collapse(rc, eb, eorder.p, edges.p, edge_cost.p, collapse_t, fkey.p, nt_off, nt.p, tri.p, orig_tri.p, pos.p,
                        orig_pos.p, occ.p, win.p, s, true, place_ptr());
        exclusive_scan(win.p, win.p, &rc->n_edges, 1, &rc->n_win, scan_scratch, s, &rc->status, eb);
        launch_compact_winners(rc, eb, win.p, collapsed.p, s);
        prof.end(kPhCollapse, s);
        prof.begin(kPhMarks, s);
        launch_remove_invalid(rc, nT, tri.p, s);
        launch_line_edges(rc, eb, edges.p, nt_off, nt.p, tri.p, pos.p, occ.p, nullptr, (int)collapsed.n, collapsed.p, s);

        // faces whose intersections decide the undo: rings of the considered collapsed edges
        cudaMemsetAsync(qflag.p, 0, (nT + 1) * sizeof(int), s);
        launch_mark_query(rc, eb, collapsed.p, edges.p, nt_off, nt.p, qflag.p, s);
        exclusive_scan(qflag.p, qflag.p, &rc->n_tris, 1, &rc->n_query, scan_scratch, s, &rc->status, nT);
        launch_compact_flags(qflag.p, nT, &rc->n_tris, qlist.p, s);
        prof.end(kPhMarks, s);

        // self-intersection check and undo passes (cusimp_free.cu:1014-1040)
        const int list_cap = (int)undo_list.n;
        auto check_pass = [&]() {
            cudaMemsetAsync(hit.p, 0, nT + 1, s);
            prof.begin(kPhBvh, s);
            bvh_build(bvh, tri.p, pos.p, rc, nT, s, false, qflag.p, false);
            prof.end(kPhBvh, s);
            prof.begin(kPhQuery, s);
            bvh_query(bvh, tri.p, pos.p, qlist.p, qflag.p, hit.p, exact_list.p, pair_cap(), rc, nT, kTriEps, s);
            prof.end(kPhQuery, s);
            launch_undo_check(rc, eb, collapsed.p, edges.p, nt_off, nt.p, hit.p, uflag.p, s);
            exclusive_scan(uflag.p, uflag.p, &rc->n_considered, 1, &rc->n_undo, scan_scratch, s, &rc->status, eb);
            launch_after_check(rc, s);
        };
        check_pass();
        if ((r = read_counters())) return r;
        cost_note();
        int extra = 0;
        while (h_rc->n_undo != 0) {
            ++extra;
            launch_undo_apply(rc, eb, collapsed.p, uflag.p, edges.p, nt_off, nt.p, tri.p, orig_tri.p, pos.p, orig_pos.p,
                              occ.p, tmp_undo.p, undo_list.p, pts_map.p, list_cap, s);
            check_pass();
            if ((r = read_counters())) return r;
            if (extra == kMaxExtraPasses) break;
        }

        // compaction map (cusimp_free.cu:1042-1045)
        exclusive_scan(occ.p, pts_map.p, &rc->n_pts, 1, nullptr, scan_scratch, s, &rc->status, nP);
        (void)operator_mode;
        if ((r = read_counters())) return r;
        if ((r = status_to_error(h_rc->status))) return r;
        if ((size_t)h_rc->n_vertices_undo > undo_list.n)
            return fail(PAMO_ERR_CAPACITY, "undo-vertex list longer than its capacity");
        last = *h_rc;
        return PAMO_OK;
    }
};

// =====================================================================================================
extern "C" {

const char* pamo_status_string(int status) {
    switch (status) {
        case PAMO_OK: return "ok";
        case PAMO_ERR_INVALID_ARG: return "invalid argument";
        case PAMO_ERR_OOM: return "out of device memory";
        case PAMO_ERR_CAPACITY: return "capacity exceeded";
        case PAMO_ERR_ITER_LIMIT: return "iteration limit";
        case PAMO_ERR_CUDA: return "CUDA error";
        case PAMO_ERR_STATE: return "invalid call order";
        default: return "unknown status";
    }
}

int pamo_ctx_create(pamo_ctx** out, int device) {
    if (!out) return PAMO_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return PAMO_ERR_INVALID_ARG;
    pamo_ctx* c = new pamo_ctx();
    c->device = device;
    int r = c->init();
    if (r) {
        c->release();
        delete c;
        return r;
    }
    *out = c;
    return PAMO_OK;
}

int pamo_ctx_destroy(pamo_ctx* ctx) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    ctx->release();
    delete ctx;
    return PAMO_OK;
}

const char* pamo_ctx_last_error(const pamo_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int pamo_ctx_reset(pamo_ctx* ctx, pamo_stream stream) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    ctx->err.clear();
    ctx->reset_state((cudaStream_t)stream);
    return ctx->check(cudaGetLastError(), "reset");
}

int64_t pamo_ctx_device_bytes(const pamo_ctx* ctx) { return ctx ? (int64_t)ctx->device_bytes() : -1; }

int pamo_ctx_set_option(pamo_ctx* ctx, const char* name, int64_t value) {
    if (!ctx || !name) return PAMO_ERR_INVALID_ARG;
    const std::string n(name);
    if (n == "graphs") ctx->use_graphs = value != 0;
    else if (n == "device_rounds") ctx->device_rounds = value != 0;
    else if (n == "bvh_reuse") ctx->bvh_reuse = value != 0;
    else if (n == "skinny_pow") {
        ctx->skinny_pow = value != 0;
        ctx->drop_graphs();
    } else if (n == "precision") {
        if (value < 0 || value > 2) return ctx->fail(PAMO_ERR_INVALID_ARG, "precision is 0, 1 or 2");
        ctx->precision = (int)value;
        ctx->drop_graphs();
        if (ctx->cap_f) {
            const int r = ctx->ensure_place(2 * ctx->cap_f);
            if (r) return r;
        }
        const int r = ctx->ensure_quad_lo();
        if (r) return r;
    }
    else if (n == "time_rounds") ctx->time_rounds = value != 0;
    else if (n == "time_edge_cost") {
        ctx->time_cost = value != 0;
        if (ctx->time_cost && !ctx->ev_c0) {
            cudaSetDevice(ctx->device);
            cudaEventCreate(&ctx->ev_c0);
            cudaEventCreate(&ctx->ev_c1);
        }
        ctx->cost_ms = 0.0;
        ctx->cost_n = 0;
        ctx->drop_graphs();
    } else if (n == "pair_cap") {
        ctx->pair_cap_limit = value;
        ctx->drop_graphs();
    } else return ctx->fail(PAMO_ERR_INVALID_ARG, "unknown option %s", name);
    return PAMO_OK;
}

int pamo_forward_round(pamo_ctx* ctx, const float* points, const int32_t* triangles, const int32_t* verts_undo,
                       int32_t n_verts_undo, int32_t n_points, int32_t n_triangles, float scale, float threshold,
                       int32_t is_stuck, int32_t init, pamo_stream stream) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    ctx->err.clear();
    // a round on zero faces is valid (the reference's loop makes one after a mesh has lost all its faces)
    if (n_points < 1 || n_triangles < 0 || !points || (n_triangles > 0 && !triangles) || n_verts_undo < 0 ||
        (n_verts_undo > 0 && !verts_undo))
        return ctx->fail(PAMO_ERR_INVALID_ARG, "invalid sizes or null pointers");
    cudaSetDevice(ctx->device);
    ctx->stream = (cudaStream_t)stream;
    ctx->have_round = false;
    ctx->h_pinned_f[0] = scale;
    cudaMemcpyAsync(ctx->d_scale, ctx->h_pinned_f, sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
    int r = ctx->round(points, nullptr, triangles, nullptr, verts_undo, n_verts_undo, n_points, n_triangles, threshold,
                       is_stuck, init, true);
    if (r) return r;
    ctx->have_round = true;
    ctx->out_np = n_points;
    ctx->out_nt = n_triangles;
    ctx->out_nu = ctx->last.n_vertices_undo;
    return PAMO_OK;
}

int pamo_legacy_round(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                      int32_t n_triangles, float scale, float threshold, int32_t init, pamo_stream stream) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    ctx->err.clear();
    if (n_points < 1 || n_triangles < 0 || !points || (n_triangles > 0 && !triangles))
        return ctx->fail(PAMO_ERR_INVALID_ARG, "invalid sizes or null pointers");
    cudaSetDevice(ctx->device);
    ctx->stream = (cudaStream_t)stream;
    ctx->have_round = false;
    ctx->h_pinned_f[0] = scale;
    cudaMemcpyAsync(ctx->d_scale, ctx->h_pinned_f, sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
    int r = ctx->legacy_round(points, triangles, n_points, n_triangles, threshold, init);
    if (r) return r;
    ctx->have_round = true;
    ctx->out_np = n_points;
    ctx->out_nt = n_triangles;
    ctx->out_nu = 0;
    return PAMO_OK;
}

int pamo_cost_probe(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                    int32_t n_triangles, float scale, float threshold, int32_t precision, int32_t* out_edges,
                    float* out_cost, float* out_place, int32_t capacity, int32_t* n_edges, pamo_stream stream) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    ctx->err.clear();
    if (n_points < 1 || n_triangles < 1 || !points || !triangles || !n_edges || precision < 0 || precision > 2)
        return ctx->fail(PAMO_ERR_INVALID_ARG, "invalid sizes, mode or null pointers");
    cudaSetDevice(ctx->device);
    ctx->stream = (cudaStream_t)stream;
    ctx->have_round = false;
    ctx->h_pinned_f[0] = scale;
    cudaMemcpyAsync(ctx->d_scale, ctx->h_pinned_f, sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
    int r = ctx->probe(points, triangles, n_points, n_triangles, threshold, precision);
    if (r) return r;
    const int ne = ctx->h_rc->n_edges;
    *n_edges = ne;
    if (capacity < ne) return capacity == 0 ? PAMO_OK : ctx->fail(PAMO_ERR_CAPACITY, "room for %d edges needed", ne);
    cudaStream_t s = ctx->stream;
    if (out_edges) cudaMemcpy2DAsync(out_edges, 2 * sizeof(int32_t), ctx->edges.p, sizeof(int2), 2 * sizeof(int32_t), ne,
                                     cudaMemcpyDeviceToDevice, s);
    if (out_cost) cudaMemcpyAsync(out_cost, ctx->probe_raw.p, ne * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (out_place) cudaMemcpy2DAsync(out_place, 3 * sizeof(float), ctx->place.p, sizeof(float4), 3 * sizeof(float), ne,
                                     cudaMemcpyDeviceToDevice, s);
    return ctx->check(cudaStreamSynchronize(s), "cost probe");
}

int pamo_round_sizes(const pamo_ctx* ctx, int32_t* n_points, int32_t* n_triangles, int32_t* n_verts_undo) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    if (!ctx->have_round) return PAMO_ERR_STATE;
    if (n_points) *n_points = ctx->out_np;
    if (n_triangles) *n_triangles = ctx->out_nt;
    if (n_verts_undo) *n_verts_undo = ctx->out_nu;
    return PAMO_OK;
}

int pamo_round_outputs(pamo_ctx* ctx, float* verts, int32_t* tris, int32_t* verts_occ, int32_t* verts_map,
                       int32_t* verts_undo, pamo_stream stream) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    if (!ctx->have_round) return ctx->fail(PAMO_ERR_STATE, "no round has run");
    if (!verts || (!tris && ctx->out_nt > 0)) return ctx->fail(PAMO_ERR_INVALID_ARG, "verts and tris are required");
    cudaSetDevice(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    launch_export_round(ctx->rc, ctx->out_np, ctx->out_nt, ctx->pos.p, ctx->tri.p, ctx->occ.p, ctx->pts_map.p,
                        ctx->undo_list.p, verts, tris, verts_occ, verts_map, verts_undo, ctx->out_nu, s);
    return ctx->check(cudaGetLastError(), "export");
}

int pamo_round_stats(const pamo_ctx* ctx, int64_t* out, int32_t n) {
    if (!ctx || !out) return PAMO_ERR_INVALID_ARG;
    const RoundCounters& c = ctx->last;
    int64_t v[18] = {c.n_edges, c.n_win, c.n_collapsed, c.n_considered, c.n_query, c.passes, c.n_vertices_undo,
                     c.status, (int64_t)c.n_pairs, (int64_t)c.n_exact};
    for (int i = 0; i < 8; ++i) v[10 + i] = c.undo_per_pass[i];
    for (int i = 0; i < n && i < 18; ++i) out[i] = v[i];
    return PAMO_OK;
}

}  // extern "C"

namespace {

// The round loop shared by PaMO.run (simp_cuda/pamo/__init__.py:95-163: centring, stop at the target face
// count or at 10 faces) and the Blender entry point (pamo_blender/cusimpinterface.cu:57-161: no centring,
// no target, stop only after `tolerance` rounds without progress).
struct LoopOptions {
    long long target = -1;  // stop when faces <= target (negative: never)
    bool stop_small = true; // stop when faces <= 10
    bool centre = true;     // subtract tris_mean first
    bool tolerance_ge = false;  // stop when count >= tolerance (Blender) instead of count == tolerance (PaMO.run)
};

int simplify_loop_on(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                     int32_t n_triangles, const LoopOptions& opt, int32_t tolerance, float threshold, int32_t iter,
                     int32_t* out_n_points, int32_t* out_n_triangles, int32_t* out_rounds, cudaStream_t s);

// Graphs cannot be captured on the legacy default stream: the loop then runs on the context's own stream,
// ordered after the caller's work and before the caller's next work by events.
int simplify_loop(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points, int32_t n_triangles,
                  const LoopOptions& opt, int32_t tolerance, float threshold, int32_t iter, int32_t* out_n_points,
                  int32_t* out_n_triangles, int32_t* out_rounds, cudaStream_t s) {
    if (s != nullptr && s != cudaStreamLegacy)
        return simplify_loop_on(ctx, points, triangles, n_points, n_triangles, opt, tolerance, threshold, iter,
                                out_n_points, out_n_triangles, out_rounds, s);
    int r;
    if ((r = ctx->ensure_own_stream())) return r;
    cudaEventRecord(ctx->ev_join, s);
    cudaStreamWaitEvent(ctx->own_stream, ctx->ev_join, 0);
    r = simplify_loop_on(ctx, points, triangles, n_points, n_triangles, opt, tolerance, threshold, iter, out_n_points,
                         out_n_triangles, out_rounds, ctx->own_stream);
    cudaEventRecord(ctx->ev_join, ctx->own_stream);
    cudaStreamWaitEvent(s, ctx->ev_join, 0);
    ctx->stream = s;
    return r;
}

int simplify_loop_on(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                     int32_t n_triangles, const LoopOptions& opt, int32_t tolerance, float threshold, int32_t iter,
                     int32_t* out_n_points, int32_t* out_n_triangles, int32_t* out_rounds, cudaStream_t s) {
    ctx->stream = s;
    ctx->have_run = false;
    ctx->faces_per_round.clear();
    ctx->round_ms.clear();
    ctx->round_gpu_ms.clear();
    ctx->cur_gpu_ms = 0.0;
    auto t_round = std::chrono::steady_clock::now();
    for (auto& t : ctx->tot) t = 0;
    int r;
    if ((r = ctx->ensure_vertex_buffers(n_points)) || (r = ctx->ensure_face_buffers(n_triangles))) return r;

    // centring and scale on the device, with numpy's float32 summation order
    ctx->prof.begin(kPhCenter, s);
    launch_center(points, triangles, n_points, n_triangles, ctx->face_mean.p, ctx->d_center, ctx->d_scale,
                  ctx->pos_in.p, s, opt.centre);
    ctx->prof.end(kPhCenter, s);

    int np = n_points, nf = n_triangles;
    int nu = 0;
    int count = 0, stuck = 0, init = 1, rounds = 0;
    // rounds after the first run from device-resident sizes and state (optionally as cached graphs); with the
    // phase timers on, every round takes the host-sized path that times each phase
    const bool dev_rounds = ctx->device_rounds && !ctx->prof.on;
    int tree_leaves = 0;  // leaves of the LBVH carried between device rounds (0: none)
    if (dev_rounds) {
        LoopState L = {};
        L.np = n_points;
        L.nf = n_triangles;
        cudaMemcpyAsync(ctx->d_ls, &L, sizeof(L), cudaMemcpyHostToDevice, s);
    }
    for (int it = 0; it < iter; ++it) {
        const int nf_prev = nf;
        if (!dev_rounds || init) {
            if (nu > 0) cudaMemcpyAsync(ctx->undo_in.p, ctx->undo_list.p, nu * sizeof(int), cudaMemcpyDeviceToDevice, s);
            if (init) r = ctx->round(nullptr, ctx->pos_in.p, triangles, nullptr, ctx->undo_in.p, nu, np, nf, threshold,
                                     stuck, init, false);
            else r = ctx->round(nullptr, ctx->pos_in.p, nullptr, ctx->tri_in.p, ctx->undo_in.p, nu, np, nf, threshold,
                                stuck, init, false);
            if (r) return r;
            nu = ctx->last.n_vertices_undo;
            // the device rounds copy the undo list into undo_in themselves: size it once for the whole list
            if ((r = ctx->grow(ctx->undo_in, dev_rounds ? std::max((size_t)nu + 1, ctx->undo_list.n) : (size_t)nu + 1)))
                return r;
            // compaction (pamo/__init__.py:136-140)
            ctx->prof.begin(kPhCompact, s);
            launch_live_flags(ctx->rc, nf, ctx->tri.p, ctx->fflags.p, s);
            exclusive_scan(ctx->fflags.p, ctx->fflags.p, &ctx->rc->n_tris, 1, nullptr, ctx->scan_scratch, s, &ctx->rc->status,
                           nf);
            launch_compact_mesh(ctx->rc, np, nf, ctx->pos.p, ctx->occ.p, ctx->pts_map.p, ctx->tri.p, ctx->fflags.p,
                                ctx->pos_out.p, ctx->tri_out.p, s);
            ctx->prof.end(kPhCompact, s);
            if (dev_rounds)
                launch_round_end(ctx->rc, ctx->d_ls, ctx->d_ls + 1, ctx->undo_list.p, ctx->undo_in.p,
                                 (int)std::min(ctx->undo_in.n, ctx->undo_list.n), (int)ctx->undo_list.n, s);
            if ((r = ctx->read_counters())) return r;
        } else {
            // rebuild the LBVH when a quarter of its leaves lost their faces, else refit the carried one
            const bool rebuild = !ctx->bvh_reuse || tree_leaves == 0 || (long long)nf * 4 < (long long)tree_leaves * 3;
            if (rebuild) tree_leaves = nf;
            ctx->cur_gpu_ms = 0.0;
            if ((r = ctx->run_round_dev(rebuild ? 0 : 2, np, nf, threshold))) return r;
            if ((r = ctx->read_counters())) return r;
            ctx->note_graph_time();
            ctx->cost_note();
            int extra = 0;
            while (ctx->h_rc->n_undo != 0) {  // cusimp_free.cu:1016-1040
                ++extra;
                if ((r = ctx->run_round_dev(1, np, nf, threshold))) return r;
                if ((r = ctx->read_counters())) return r;
                ctx->note_graph_time();
                if (extra == kMaxExtraPasses) break;
            }
            if ((r = ctx->status_to_error(ctx->h_rc->status))) return r;
            if ((size_t)ctx->h_rc->n_vertices_undo > ctx->undo_list.n)
                return ctx->fail(PAMO_ERR_CAPACITY, "undo-vertex list longer than its capacity");
            ctx->last = *ctx->h_rc;
            ctx->have_round = true;
        }
        ++rounds;
        init = 0;
        {
            const RoundCounters& c = ctx->last;
            long long* t = ctx->tot;
            t[0] += c.n_pts; t[1] += c.n_tris; t[2] += c.n_edges; t[3] += c.n_win;
            t[4] += (long long)c.n_query * c.passes; t[5] += (long long)c.n_pairs; t[6] += (long long)c.n_exact;
            t[7] += c.passes; t[8] += (long long)c.n_live * c.passes; t[9] += c.n_collapsed;
        }
        np = ctx->h_rc->n_pts_out;
        nf = ctx->h_rc->n_tris_out;
        std::swap(ctx->pos_in, ctx->pos_out);
        std::swap(ctx->tri_in, ctx->tri_out);
        ctx->faces_per_round.push_back(nf);
        {
            const auto t_now = std::chrono::steady_clock::now();
            ctx->round_ms.push_back(std::chrono::duration<double, std::milli>(t_now - t_round).count());
            ctx->round_gpu_ms.push_back(ctx->cur_gpu_ms);
            ctx->cur_gpu_ms = 0.0;
            t_round = t_now;
        }
        if ((opt.target >= 0 && nf <= opt.target) || (opt.stop_small && nf <= 10)) break;
        if (nf == nf_prev) {
            count++;
        } else {
            count = 0;
            stuck = 0;
        }
        if (count >= 2) stuck = 1;
        if (opt.tolerance_ge ? count >= tolerance : count == tolerance) break;
    }
    ctx->run_np = np;
    ctx->run_nt = nf;
    ctx->have_run = true;
    if (out_n_points) *out_n_points = np;
    if (out_n_triangles) *out_n_triangles = nf;
    if (out_rounds) *out_rounds = rounds;
    return PAMO_OK;
}

std::mutex g_blender_mu;
pamo_ctx* g_blender_ctx[64] = {};  // one context per device, kept like the reference's static CUSimp_Free

}  // namespace

extern "C" {

int pamo_simplify_device(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                         int32_t n_triangles, double ratio, int32_t tolerance, float threshold, int32_t iter,
                         int64_t min_verts, int32_t* out_n_points, int32_t* out_n_triangles, int32_t* out_rounds,
                         pamo_stream stream) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    ctx->err.clear();
    if (n_points < 1 || n_triangles < 1 || !points || !triangles)
        return ctx->fail(PAMO_ERR_INVALID_ARG, "invalid sizes or null pointers");
    cudaSetDevice(ctx->device);
    LoopOptions opt;
    // target_faces = max(int(ratio * F), min_verts) (pamo/__init__.py:97)
    opt.target = std::max((long long)(ratio * (double)n_triangles), (long long)min_verts);
    return simplify_loop(ctx, points, triangles, n_points, n_triangles, opt, tolerance, threshold, iter, out_n_points,
                         out_n_triangles, out_rounds, (cudaStream_t)stream);
}

int pamo_simplify_device_target(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                                int32_t n_triangles, int64_t target_faces, int32_t tolerance, float threshold,
                                int32_t iter, int32_t centre, int32_t* out_n_points, int32_t* out_n_triangles,
                                int32_t* out_rounds, pamo_stream stream) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    ctx->err.clear();
    if (n_points < 1 || n_triangles < 1 || !points || !triangles)
        return ctx->fail(PAMO_ERR_INVALID_ARG, "invalid sizes or null pointers");
    cudaSetDevice(ctx->device);
    LoopOptions opt;
    opt.target = (long long)target_faces;
    opt.centre = centre != 0;
    return simplify_loop(ctx, points, triangles, n_points, n_triangles, opt, tolerance, threshold, iter, out_n_points,
                         out_n_triangles, out_rounds, (cudaStream_t)stream);
}

int pamo_simplify(float* in_verts, int* in_tris, float* out_verts, int* out_tris, int* in_out_nv_ni, float threshold) {
    if (!in_verts || !in_tris || !out_verts || !out_tris || !in_out_nv_ni) return PAMO_ERR_INVALID_ARG;
    const int nv = in_out_nv_ni[0], nt = in_out_nv_ni[1];
    if (nv < 1 || nt < 1) return PAMO_ERR_INVALID_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return PAMO_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_blender_mu);
    pamo_ctx*& ctx = g_blender_ctx[dev];
    int r;
    if (!ctx && (r = pamo_ctx_create(&ctx, dev))) return r;
    ctx->err.clear();
    float* d_v = nullptr;
    int* d_t = nullptr;
    if (cudaMalloc((void**)&d_v, (size_t)nv * 3 * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void**)&d_t, (size_t)nt * 3 * sizeof(int)) != cudaSuccess) {
        cudaFree(d_v);
        cudaFree(d_t);
        return ctx->fail(PAMO_ERR_OOM, "cudaMalloc");
    }
    cudaStream_t s = nullptr;
    cudaMemcpyAsync(d_v, in_verts, (size_t)nv * 3 * sizeof(float), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_t, in_tris, (size_t)nt * 3 * sizeof(int), cudaMemcpyHostToDevice, s);
    LoopOptions opt;
    opt.target = -1;
    opt.stop_small = false;
    opt.centre = false;
    opt.tolerance_ge = true;
    int onv = 0, ont = 0, rounds = 0;
    r = simplify_loop(ctx, d_v, d_t, nv, nt, opt, 4, threshold, 1000000, &onv, &ont, &rounds, s);
    if (!r) {
        // the result is written over the input device copies (both are at least as large)
        launch_export_mesh(ctx->run_np, ctx->run_nt, ctx->pos_in.p, ctx->tri_in.p, ctx->d_center, d_v, d_t, s);
        cudaMemcpyAsync(out_verts, d_v, (size_t)onv * 3 * sizeof(float), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(out_tris, d_t, (size_t)ont * 3 * sizeof(int), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) r = ctx->fail(PAMO_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
        else {
            in_out_nv_ni[0] = onv;
            in_out_nv_ni[1] = ont;
        }
    }
    cudaFree(d_v);
    cudaFree(d_t);
    return r;
}

int pamo_simplify_result(pamo_ctx* ctx, float* verts, int32_t* tris, pamo_stream stream) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    if (!ctx->have_run) return ctx->fail(PAMO_ERR_STATE, "no simplification has run");
    if (!verts || (!tris && ctx->out_nt > 0)) return ctx->fail(PAMO_ERR_INVALID_ARG, "verts and tris are required");
    cudaSetDevice(ctx->device);
    launch_export_mesh(ctx->run_np, ctx->run_nt, ctx->pos_in.p, ctx->tri_in.p, ctx->d_center, verts, tris,
                       (cudaStream_t)stream);
    return ctx->check(cudaGetLastError(), "export");
}

int pamo_tris_mean(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                   int32_t n_triangles, float* out3, pamo_stream stream) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    ctx->err.clear();
    if (n_points < 1 || n_triangles < 1 || !points || !triangles || !out3)
        return ctx->fail(PAMO_ERR_INVALID_ARG, "invalid sizes or null pointers");
    cudaSetDevice(ctx->device);
    ctx->stream = (cudaStream_t)stream;
    int r;
    if ((r = ctx->ensure_vertex_buffers(n_points)) || (r = ctx->ensure_face_buffers(n_triangles))) return r;
    launch_center(points, triangles, n_points, n_triangles, ctx->face_mean.p, ctx->d_center, ctx->d_scale,
                  ctx->pos_out.p, ctx->stream, true);
    cudaMemcpyAsync(ctx->h_pinned_f, ctx->d_center, 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if ((r = ctx->check(cudaStreamSynchronize(ctx->stream), "tris_mean"))) return r;
    for (int d = 0; d < 3; ++d) out3[d] = ctx->h_pinned_f[d];
    return PAMO_OK;
}

int pamo_self_intersect(pamo_ctx* ctx, const float* points, const int32_t* triangles, int32_t n_points,
                        int32_t n_triangles, uint8_t* face_hit, pamo_stream stream) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    ctx->err.clear();
    if (n_points < 1 || n_triangles < 1 || !points || !triangles || !face_hit)
        return ctx->fail(PAMO_ERR_INVALID_ARG, "invalid sizes or null pointers");
    cudaSetDevice(ctx->device);
    ctx->stream = (cudaStream_t)stream;
    cudaStream_t s = ctx->stream;
    int r;
    if ((r = ctx->ensure_vertex_buffers(n_points)) || (r = ctx->ensure_face_buffers(n_triangles))) return r;
    RoundCounters* h = ctx->h_rc;
    std::memset(h, 0, sizeof(RoundCounters));
    h->n_pts = n_points;
    h->n_tris = n_triangles;
    cudaMemcpyAsync(ctx->rc, h, sizeof(RoundCounters), cudaMemcpyHostToDevice, s);
    launch_load_points(points, n_points, ctx->pos.p, ctx->orig_pos.p, ctx->occ.p, s);
    launch_load_tris(triangles, n_triangles, n_points, ctx->tri.p, ctx->rc, s);
    // every live face queries
    launch_live_flags(ctx->rc, n_triangles, ctx->tri.p, ctx->qflag.p, s);
    exclusive_scan(ctx->qflag.p, ctx->qflag.p, &ctx->rc->n_tris, 1, &ctx->rc->n_query, ctx->scan_scratch, s,
                   &ctx->rc->status, n_triangles);
    launch_compact_flags(ctx->qflag.p, n_triangles, &ctx->rc->n_tris, ctx->qlist.p, s);
    cudaMemsetAsync(ctx->hit.p, 0, n_triangles + 1, s);
    bvh_build(ctx->bvh, ctx->tri.p, ctx->pos.p, ctx->rc, n_triangles, s, false, ctx->qflag.p, false);
    bvh_query(ctx->bvh, ctx->tri.p, ctx->pos.p, ctx->qlist.p, ctx->qflag.p, ctx->hit.p, ctx->exact_list.p,
              ctx->pair_cap(), ctx->rc, n_triangles, kTriEps, s);
    cudaMemcpyAsync(face_hit, ctx->hit.p, n_triangles, cudaMemcpyDeviceToDevice, s);
    if ((r = ctx->read_counters())) return r;
    return ctx->status_to_error(ctx->h_rc->status);
}

int pamo_profile_enable(pamo_ctx* ctx, int32_t enable) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (enable) ctx->prof.create();
    ctx->prof.on = enable != 0;
    for (int p = 0; p < kNumPhases; ++p) {
        ctx->prof.ms[p] = 0.0;
        ctx->prof.count[p] = 0;
        ctx->prof.pending[p] = false;
    }
    return PAMO_OK;
}

int pamo_profile_read(const pamo_ctx* ctx, double* ms, int64_t* counts, int32_t n) {
    if (!ctx) return PAMO_ERR_INVALID_ARG;
    for (int p = 0; p < n && p < kNumPhases; ++p) {
        if (ms) ms[p] = ctx->prof.ms[p];
        if (counts) counts[p] = ctx->prof.count[p];
    }
    return kNumPhases;
}

int pamo_run_totals(const pamo_ctx* ctx, int64_t* out, int32_t n) {
    if (!ctx || !out) return PAMO_ERR_INVALID_ARG;
    for (int i = 0; i < n && i < 10; ++i) out[i] = ctx->tot[i];
    return 10;
}

int64_t pamo_launch_count(void) { return launches_so_far(); }

int pamo_simplify_round_ms(const pamo_ctx* ctx, double* ms, int32_t capacity) {
    if (!ctx || !ms) return PAMO_ERR_INVALID_ARG;
    const int n = std::min<int>(capacity, (int)ctx->round_ms.size());
    for (int i = 0; i < n; ++i) ms[i] = ctx->round_ms[i];
    return n;
}

int pamo_kernel_time(pamo_ctx* ctx, double* ms, int64_t* launches, int32_t reset) {
    if (!ctx || !ms || !launches) return PAMO_ERR_INVALID_ARG;
    *ms = ctx->cost_ms;
    *launches = ctx->cost_n;
    if (reset) {
        ctx->cost_ms = 0.0;
        ctx->cost_n = 0;
    }
    return PAMO_OK;
}

int pamo_simplify_round_gpu_ms(const pamo_ctx* ctx, double* ms, int32_t capacity) {
    if (!ctx || !ms) return PAMO_ERR_INVALID_ARG;
    const int n = std::min<int>(capacity, (int)ctx->round_gpu_ms.size());
    for (int i = 0; i < n; ++i) ms[i] = ctx->round_gpu_ms[i];
    return n;
}

int pamo_simplify_round_faces(const pamo_ctx* ctx, int32_t* faces_per_round, int32_t capacity) {
    if (!ctx || !faces_per_round) return PAMO_ERR_INVALID_ARG;
    for (int i = 0; i < capacity && i < (int)ctx->faces_per_round.size(); ++i) faces_per_round[i] = ctx->faces_per_round[i];
    return PAMO_OK;
}

}  // extern "C"
