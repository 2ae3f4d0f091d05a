// Batched stage-2 rounds: many meshes concatenated in CSR form (per-mesh vertex and face offsets) run the PaMO.run
// loop (simp_cuda/pamo/__init__.py:95-163) together, every round being one pass of the round's kernels over all live
// meshes (CUSimp_Free::forward, simp_cuda/src/cusimp_free.cu:891-1048, once per mesh).
//
// Layout: the round's working arrays hold every live mesh in one vertex and one face numbering (mesh k of the round
// owns vertices [v0_k, v0_k + np_k) and faces [f0_k, f0_k + nf_k), faces index vertices globally). Kernels that act
// per element (adjacency, quadrics, cost, keys, collapse, clean-up, undo check) run unchanged over the whole batch:
// rings never leave a mesh. A mesh's edges are numbered by the same face scan as alone, offset by its first edge,
// so key ties break as alone. The state the reference carries between forward calls and indexes with a mesh's own
// numbering (stale edge costs, the invalid-vertex table, the previous compaction map, the undo lists: Q1-Q3) lives
// in fixed regions per mesh, gathered into the global numbering before the kernels that read it and scattered back
// after. The LBVH keeps each mesh in its own subtree (mesh index in the top key bits) and each query walks only its
// mesh's subtree. Lists whose order the reference fixes per mesh (winners, then coincident-edge collapses; undo
// vertices) are assembled per mesh. Undo passes run while any mesh still needs one, each mesh for at most five.
// Loop control (target, no-progress count, is_stuck, tolerance) is per mesh; a finished mesh is written to the
// results and leaves the next round's arrays.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pamo_gb300.h"
#include "lbvh.cuh"
#include "pamo_common.cuh"
#include "round_ops.cuh"
#include "scan.cuh"
#include "simp_round.cuh"

namespace pamo {
namespace {

constexpr int kT = 256;
constexpr int kCtlThreads = 1024;
constexpr float kTriEpsB = 1e-3f;  // cusimp_free.cu:893
constexpr int kMaxExtra = 5;      // extra undo passes per round (cusimp_free.cu:1039)

// One mesh of a batch.
struct BatchMesh {
    // fixed for the job
    long long target;  // stop when faces <= target: max(int(ratio * F0), min_verts)
    int tolerance, iter;
    int lp;            // per-vertex state length: the reference's allocated_pts + 1 (V0 + V0/5 + 1)
    int ecap;          // edge-cost region length
    long long vreg;    // offset of the per-vertex state regions
    long long ereg;    // offset of the edge-cost region
    long long res_v0, res_f0;  // where the result goes in the result arrays (the input offsets)
    // loop state (pamo/__init__.py:128-158)
    int np, nf, nu, is_stuck, count, rounds, done;
    // this round
    int v0, f0, e0, ne;  // offsets in the round's numbering
    int nwin, w0, nline, l0, ncons, c0;
    int passes, extra, first_undo, n_vertices_undo, n_undo, checking, apply;
    int np_out, nf_out, nv0_next, nf0_next;
};

// Small control block read by the host after a round.
struct BatchCtl {
    int n_slots;        // live meshes this round
    int n_next;         // meshes running the next round
    int any_apply;      // some mesh takes an undo pass
    int status;
    long long v_next, f_next;  // vertices and faces of the next round
    long long results_v, results_f;
    int n_lines;        // coincident-endpoint collapses this round
    int pad[5];
};

__device__ __forceinline__ int bx_chunk(int n, int t, int& lo) {
    const int per = (n + kCtlThreads - 1) / kCtlThreads;
    lo = min(n, t * per);
    return min(n, lo + per) - lo;
}

// ---------------------------------------------------------------- round set-up (one block)
// Live meshes get slots in mesh order; their vertex and face offsets are prefix sums of their sizes; the global
// counters start as forward() sets them.
__global__ void __launch_bounds__(kCtlThreads) kb_round_begin(BatchMesh* mesh, int n_meshes, int* slot_mesh,
                                                              int* slot_v0, int* slot_np, int* slot_f0, int* slot_nf,
                                                              int* slot_stuck, float* slot_scale,
                                                              const float* mesh_scale, RoundCounters* rc,
                                                              BatchCtl* ctl) {
    __shared__ int sm[33];
    int lo;
    const int cnt = bx_chunk(n_meshes, threadIdx.x, lo);
    int live = 0, sv = 0, sf = 0;
    for (int i = lo; i < lo + cnt; ++i)
        if (!mesh[i].done) {
            ++live;
            sv += mesh[i].np;
            sf += mesh[i].nf;
        }
    int tl, tv, tf;
    int k = block_exclusive_scan(live, &tl, sm);
    int v0 = block_exclusive_scan(sv, &tv, sm);
    int f0 = block_exclusive_scan(sf, &tf, sm);
    for (int i = lo; i < lo + cnt; ++i) {
        BatchMesh& M = mesh[i];
        if (M.done) continue;
        M.v0 = v0;
        M.f0 = f0;
        M.nwin = M.nline = M.ncons = M.passes = M.extra = M.n_undo = M.apply = 0;
        M.checking = 1;
        M.first_undo = M.is_stuck ? M.nu : 0;
        M.n_vertices_undo = M.is_stuck ? M.nu : 0;
        slot_mesh[k] = i;
        slot_v0[k] = v0;
        slot_np[k] = M.np;
        slot_f0[k] = f0;
        slot_nf[k] = M.nf;
        slot_stuck[k] = M.is_stuck;
        slot_scale[k] = mesh_scale[i];
        ++k;
        v0 += M.np;
        f0 += M.nf;
    }
    if (threadIdx.x == 0) {
        RoundCounters z = {};
        z.n_pts = tv;
        z.n_tris = tf;
        *rc = z;
        ctl->n_slots = tl;
        ctl->any_apply = 0;
        ctl->n_lines = 0;
    }
}

// vertex and face -> slot
__global__ void kb_fill_slots(const BatchCtl* ctl, const int* slot_v0, const int* slot_np, const int* slot_f0,
                              const int* slot_nf, int* vmesh, int* fmesh) {
    for (int k = blockIdx.x; k < ctl->n_slots; k += gridDim.x) {
        const int v0 = slot_v0[k], np = slot_np[k], f0 = slot_f0[k], nf = slot_nf[k];
        for (int i = threadIdx.x; i < np; i += blockDim.x) vmesh[v0 + i] = k;
        for (int i = threadIdx.x; i < nf; i += blockDim.x) fmesh[f0 + i] = k;
    }
}

// undo bookkeeping of forward() per mesh (cusimp_free.cu:895-918): not stuck with undo vertices carried in: the
// invalid table is cleared; stuck: the undo list restarts from the carried vertices mapped through the previous
// map; then the carried vertices are marked invalid
__global__ void kb_undo_book(const BatchCtl* ctl, const int* slot_mesh, const BatchMesh* mesh, const int* undo_in,
                             int* tmp_undo, int* undo_list, const int* map, unsigned char* invalid) {
    for (int k = blockIdx.x; k < ctl->n_slots; k += gridDim.x) {
        const BatchMesh& M = mesh[slot_mesh[k]];
        const long long r = M.vreg;
        if (!M.is_stuck && M.nu != 0)
            for (int i = threadIdx.x; i < M.lp; i += blockDim.x) invalid[r + i] = 0;
        __syncthreads();
        for (int a = threadIdx.x; a < M.nu; a += blockDim.x) {
            const int x = undo_in[r + a];
            if (M.is_stuck) {
                tmp_undo[r + a] = x;
                undo_list[r + a] = (x >= 0 && x < M.lp) ? map[r + x] : 0;
            }
            if (x >= 0 && x < M.lp) invalid[r + x] = 1;
        }
        __syncthreads();
    }
}

// each mesh's edges: [e0, e0 + ne) of the round's edge numbering (from the scanned per-face edge counts)
__global__ void kb_slot_edges(const BatchCtl* ctl, const int* slot_mesh, BatchMesh* mesh, const int* ecount_scan,
                              RoundCounters* rc) {
    for (int k = gtid(); k < ctl->n_slots; k += gstride()) {
        BatchMesh& M = mesh[slot_mesh[k]];
        M.e0 = ecount_scan[M.f0];
        M.ne = ecount_scan[M.f0 + M.nf] - M.e0;
        if (M.ne > M.ecap) atomicOr(&rc->status, kErrCapacity);
    }
}

// the per-mesh state into the round's numbering: stale edge costs (Q1) and the invalid-vertex table (Q2)
__global__ void kb_gather(const RoundCounters* rc, const int* slot_mesh, const BatchMesh* mesh, const int* vmesh,
                          const int2* edges, const uint32_t* ecost_reg, const unsigned char* invalid_reg,
                          uint32_t* cost, unsigned char* invalid) {
    const int ne = rc->n_edges, np = rc->n_pts;
    const int n = max(ne, np);
    for (int i = gtid(); i < n; i += gstride()) {
        if (i < ne) {
            const BatchMesh& M = mesh[slot_mesh[vmesh[edges[i].x]]];
            const int l = i - M.e0;
            cost[i] = l < M.ecap ? ecost_reg[M.ereg + l] : 0u;
        }
        if (i < np) {
            const BatchMesh& M = mesh[slot_mesh[vmesh[i]]];
            const int l = i - M.v0;
            invalid[i] = l < M.lp ? invalid_reg[M.vreg + l] : 0;
        }
    }
}

__global__ void kb_scatter_costs(const RoundCounters* rc, const int* slot_mesh, const BatchMesh* mesh, const int* vmesh,
                                 const int2* edges, const uint32_t* cost, uint32_t* ecost_reg) {
    const int ne = rc->n_edges;
    for (int i = gtid(); i < ne; i += gstride()) {
        const BatchMesh& M = mesh[slot_mesh[vmesh[edges[i].x]]];
        const int l = i - M.e0;
        if (l < M.ecap) ecost_reg[M.ereg + l] = cost[i];
    }
}

// remove_line_edge_collapse (cusimp_free.cu:234-274) in edge order by one thread when any coincident edge exists;
// the collapses are listed in edge order (meshes in order) and counted per mesh
__global__ void kb_line_apply(RoundCounters* rc, BatchCtl* ctl, const int* slot_mesh, BatchMesh* mesh,
                              const int* vmesh, const int2* __restrict__ edges, const int* __restrict__ nt_off,
                              const int* __restrict__ nt, int4* tri, float4* pos, int* occ, int* lines, int cap) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int k = 0;
    if (rc->n_line > 0) {
        const int n = rc->n_edges;
        for (int e = 0; e < n; ++e) {
            const int2 ed = edges[e];
            const float4 p = pos[ed.x], q = pos[ed.y];
            if (!(p.x == q.x && p.y == q.y && p.z == q.z)) continue;
            if (k >= cap) {
                atomicOr(&rc->status, kErrCapacity);
                break;
            }
            lines[k++] = e;
            mesh[slot_mesh[vmesh[ed.x]]].nline += 1;
            pos[ed.y] = make_float4(0.f, 0.f, 0.f, 0.f);
            occ[ed.y] = 0;
            rewire(ed.x, ed.y, nt_off, nt, tri);
        }
    }
    ctl->n_lines = k;
}

// per mesh: winners [w0, w0 + nwin) of the winner list, coincident-edge collapses [l0, l0 + nline) of the line list,
// and the collapsed edges the undo check considers: the first min(k, roundup(h, 512)) of the h winners and k - h
// line collapses (the check's grid is sized from h before the line collapses are appended, :1007-1016)
__global__ void __launch_bounds__(kCtlThreads) kb_considered(const BatchCtl* ctl, const int* slot_mesh,
                                                             BatchMesh* mesh, const int* win_scan, RoundCounters* rc) {
    __shared__ int sm[33];
    const int n = ctl->n_slots;
    int lo;
    const int cnt = bx_chunk(n, threadIdx.x, lo);
    int sl = 0, sc = 0;
    for (int k = lo; k < lo + cnt; ++k) {
        BatchMesh& M = mesh[slot_mesh[k]];
        M.w0 = win_scan[M.e0];
        M.nwin = win_scan[M.e0 + M.ne] - M.w0;
        const int h = M.nwin, kk = h + M.nline;
        const int roundup = ((h + 511) / 512) * 512;
        M.ncons = (h == 0) ? 0 : (kk < roundup ? kk : roundup);
        sl += M.nline;
        sc += M.ncons;
    }
    int tl, tc;
    int l0 = block_exclusive_scan(sl, &tl, sm);
    int c0 = block_exclusive_scan(sc, &tc, sm);
    for (int k = lo; k < lo + cnt; ++k) {
        BatchMesh& M = mesh[slot_mesh[k]];
        M.l0 = l0;
        M.c0 = c0;
        l0 += M.nline;
        c0 += M.ncons;
    }
    if (threadIdx.x == 0) rc->n_considered = tc;
}

__global__ void kb_considered_fill(const BatchCtl* ctl, const int* slot_mesh, const BatchMesh* mesh,
                                   const int* winners, const int* lines, int* considered) {
    for (int k = blockIdx.x; k < ctl->n_slots; k += gridDim.x) {
        const BatchMesh& M = mesh[slot_mesh[k]];
        for (int i = threadIdx.x; i < M.ncons; i += blockDim.x)
            considered[M.c0 + i] = i < M.nwin ? winners[M.w0 + i] : lines[M.l0 + i - M.nwin];
    }
}

// after an intersection check, per mesh that was checked: its undo edges, the undo-vertex count, and whether it
// takes another pass (fewer than five extra passes so far, :1024-1040)
__global__ void kb_after_check(BatchCtl* ctl, const int* slot_mesh, BatchMesh* mesh, const int* uscan) {
    int any = 0;
    for (int k = gtid(); k < ctl->n_slots; k += gstride()) {
        BatchMesh& M = mesh[slot_mesh[k]];
        if (!M.checking) {
            M.n_undo = 0;
            M.apply = 0;
            continue;
        }
        M.n_undo = uscan[M.c0 + M.ncons] - uscan[M.c0];
        M.passes += 1;
        M.n_vertices_undo += 2 * M.n_undo;
        M.apply = (M.n_undo != 0 && M.extra < kMaxExtra) ? 1 : 0;
        any |= M.apply;
    }
    if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(&ctl->any_apply, 1);
}

// undo_collapse_kernel + rearrange_index_of_undo_vertices (:829-878) for the meshes that take a pass: the undo
// vertices go to the mesh's lists in its own numbering, mapped through its previous compaction map (Q3)
__global__ void kb_undo_apply(const RoundCounters* rc, const int* slot_mesh, const BatchMesh* mesh, const int* vmesh,
                              const int* __restrict__ considered, const int* __restrict__ uscan,
                              const int2* __restrict__ edges, const int* __restrict__ nt_off,
                              const int* __restrict__ nt, int4* tri, const int4* __restrict__ orig_tri, float4* pos,
                              const float4* __restrict__ orig_pos, int* occ, int* tmp_undo, int* undo_list,
                              const int* __restrict__ map, int* status) {
    const int n = rc->n_considered;
    for (int c = gtid(); c < n; c += gstride()) {
        if (uscan[c + 1] == uscan[c]) continue;
        const int2 ed = edges[considered[c]];
        const BatchMesh& M = mesh[slot_mesh[vmesh[ed.x]]];
        if (!M.apply) continue;
        const int a = uscan[c] - uscan[M.c0];
        const int u = ed.x, v = ed.y;
        occ[v] = 1;
        pos[u] = orig_pos[u];
        pos[v] = orig_pos[v];
        restore_ring(u, nt_off, nt, tri, orig_tri);
        restore_ring(v, nt_off, nt, tri, orig_tri);
        const int ul = u - M.v0, vl = v - M.v0;
        if (M.first_undo + 2 * a + 1 < M.lp) {
            tmp_undo[M.vreg + 2 * a] = ul;
            tmp_undo[M.vreg + 2 * a + 1] = vl;
            undo_list[M.vreg + M.first_undo + 2 * a] = ul < M.lp ? map[M.vreg + ul] : 0;
            undo_list[M.vreg + M.first_undo + 2 * a + 1] = vl < M.lp ? map[M.vreg + vl] : 0;
        } else {
            atomicOr(status, kErrCapacity);
        }
    }
}

__global__ void kb_after_apply(BatchCtl* ctl, const int* slot_mesh, BatchMesh* mesh) {
    for (int k = gtid(); k < ctl->n_slots; k += gstride()) {
        BatchMesh& M = mesh[slot_mesh[k]];
        M.checking = M.apply;
        if (M.apply) {
            M.first_undo += 2 * M.n_undo;
            M.extra += 1;
        }
    }
    if (gtid() == 0) ctl->any_apply = 0;
}

// after the checks: each mesh's sizes after compaction and the loop update of PaMO.run (:141-158); the meshes that
// go on get the next round's offsets (prefix sums in mesh order)
__global__ void __launch_bounds__(kCtlThreads) kb_round_end(BatchCtl* ctl, const int* slot_mesh, BatchMesh* mesh,
                                                            const int* vscan, const int* fscan, RoundCounters* rc) {
    __shared__ int sm[33];
    const int n = ctl->n_slots;
    int lo;
    const int cnt = bx_chunk(n, threadIdx.x, lo);
    int cont = 0, sv = 0, sf = 0;
    for (int k = lo; k < lo + cnt; ++k) {
        BatchMesh& M = mesh[slot_mesh[k]];
        M.np_out = vscan[M.v0 + M.np] - vscan[M.v0];
        M.nf_out = fscan[M.f0 + M.nf] - fscan[M.f0];
        if (M.n_vertices_undo > M.lp) atomicOr(&rc->status, kErrCapacity);
        M.rounds += 1;
        const int nf_prev = M.nf;
        bool done = M.nf_out <= M.target || M.nf_out <= 10;
        if (!done) {
            if (M.nf_out == nf_prev) {
                M.count += 1;
            } else {
                M.count = 0;
                M.is_stuck = 0;
            }
            if (M.count >= 2) M.is_stuck = 1;
            if (M.count == M.tolerance) done = true;
        }
        if (M.rounds >= M.iter) done = true;
        M.done = done ? 1 : 0;
        if (!done) {
            ++cont;
            sv += M.np_out;
            sf += M.nf_out;
        }
    }
    int tc, tv, tf;
    int c0 = block_exclusive_scan(cont, &tc, sm);
    int v0 = block_exclusive_scan(sv, &tv, sm);
    int f0 = block_exclusive_scan(sf, &tf, sm);
    (void)c0;
    for (int k = lo; k < lo + cnt; ++k) {
        BatchMesh& M = mesh[slot_mesh[k]];
        if (M.done) continue;
        M.nv0_next = v0;
        M.nf0_next = f0;
        v0 += M.np_out;
        f0 += M.nf_out;
    }
    if (threadIdx.x == 0) {
        ctl->n_next = tc;
        ctl->v_next = tv;
        ctl->f_next = tf;
        ctl->status = rc->status;
    }
}

// compaction (pamo/__init__.py:136-140) of every mesh: the mesh's compaction map (its own numbering, n_pts + 1
// entries) kept for the next round (Q3); a finished mesh goes to the results with its mean added back (:161), the
// others to the next round's arrays in the next round's numbering
__global__ void kb_compact(const RoundCounters* rc, const int* slot_mesh, BatchMesh* mesh, const int* vmesh,
                           const int* fmesh, const float4* __restrict__ pos, const int* __restrict__ occ,
                           const int* __restrict__ vscan, const int4* __restrict__ tri, const int* __restrict__ fscan,
                           int* map, const float4* __restrict__ mean, float4* next_pos, int4* next_tri, float4* res_pos,
                           int4* res_tri) {
    const int np = rc->n_pts, nf = rc->n_tris;
    const int n = max(np, nf);
    for (int i = gtid(); i < n; i += gstride()) {
        if (i < np) {
            const int mi = slot_mesh[vmesh[i]];
            const BatchMesh& M = mesh[mi];
            const int l = i - M.v0;
            const int base = vscan[M.v0];
            const int ln = vscan[i] - base;
            map[M.vreg + l] = ln;
            if (l == M.np - 1) map[M.vreg + M.np] = vscan[M.v0 + M.np] - base;
            if (occ[i]) {
                const float4 p = pos[i];
                if (M.done) {
                    const float4 c = mean[mi];
                    res_pos[M.res_v0 + ln] = make_float4(p.x + c.x, p.y + c.y, p.z + c.z, 0.f);
                } else {
                    next_pos[M.nv0_next + ln] = p;
                }
            }
        }
        if (i < nf && fscan[i + 1] != fscan[i]) {
            const BatchMesh& M = mesh[slot_mesh[fmesh[i]]];
            const int lf = fscan[i] - fscan[M.f0];
            const int base = vscan[M.v0];
            const int4 t = tri[i];
            const int a = vscan[t.x] - base, b = vscan[t.y] - base, c = vscan[t.z] - base;
            if (M.done) res_tri[M.res_f0 + lf] = make_int4(a, b, c, 0);
            else next_tri[M.nf0_next + lf] = make_int4(a + M.nv0_next, b + M.nv0_next, c + M.nv0_next, 0);
        }
    }
}

// the undo vertices each mesh carries into its next round (the host loop's verts_undo)
__global__ void kb_carry_undo(const BatchCtl* ctl, const int* slot_mesh, BatchMesh* mesh, const int* undo_list,
                              int* undo_in) {
    for (int k = blockIdx.x; k < ctl->n_slots; k += gridDim.x) {
        BatchMesh& M = mesh[slot_mesh[k]];
        const int nu = min(M.n_vertices_undo, M.lp);
        for (int i = threadIdx.x; i < nu; i += blockDim.x) undo_in[M.vreg + i] = undo_list[M.vreg + i];
        __syncthreads();
        if (threadIdx.x == 0) {
            M.nu = nu;
            M.np = M.np_out;
            M.nf = M.nf_out;
        }
    }
}

// ---------------------------------------------------------------- job set-up and results
__global__ void kb_offset_faces(int4* tri, const long long* foff, const long long* voff, int n_meshes, int n_faces) {
    for (int f = gtid(); f < n_faces; f += gstride()) {
        int lo = 0, hi = n_meshes - 1;  // the mesh m with foff[m] <= f < foff[m + 1]
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (foff[mid] <= f) lo = mid;
            else hi = mid - 1;
        }
        int4 t = tri[f];
        if (t.x >= 0) {
            const int o = (int)voff[lo];
            t.x += o;
            t.y += o;
            t.z += o;
        }
        tri[f] = t;
    }
}

__global__ void kb_pack_results(const BatchMesh* mesh, int n_meshes, const long long* out_voff,
                                const long long* out_foff, const float4* __restrict__ res_pos,
                                const int4* __restrict__ res_tri, float* out_points, int* out_tris) {
    for (int m = blockIdx.x; m < n_meshes; m += gridDim.x) {
        const BatchMesh& M = mesh[m];
        const int nv = (int)(out_voff[m + 1] - out_voff[m]), nf = (int)(out_foff[m + 1] - out_foff[m]);
        for (int i = threadIdx.x; i < nv; i += blockDim.x) {
            const float4 p = res_pos[M.res_v0 + i];
            float* o = out_points + 3 * (out_voff[m] + i);
            o[0] = p.x;
            o[1] = p.y;
            o[2] = p.z;
        }
        for (int i = threadIdx.x; i < nf; i += blockDim.x) {
            const int4 t = res_tri[M.res_f0 + i];
            int* o = out_tris + 3 * (out_foff[m] + i);
            o[0] = t.x;
            o[1] = t.y;
            o[2] = t.z;
        }
    }
}

__global__ void kb_mean_table(const float* centre16, int n_meshes, float4* mean) {
    for (int m = gtid(); m < n_meshes; m += gstride())
        mean[m] = make_float4(centre16[16 * m], centre16[16 * m + 1], centre16[16 * m + 2], 0.f);
}

template <typename T>
struct Buf {
    T* p = nullptr;
    size_t n = 0;
};

}  // namespace
}  // namespace pamo

using namespace pamo;

struct pamo_csr {
    int device = 0;
    std::string err;
    cudaStream_t stream = nullptr;
    bool skinny_pow = false;  // as pamo_ctx's option of the same name

    // per vertex / face / edge of a round
    Buf<float4> pos, orig_pos, pos_in, pos_next, res_pos;
    Buf<int> occ, valence, cursor, vedges, vcursor, vmesh, vscan;
    Buf<Quadric> quad;
    Buf<unsigned long long> vmin;
    Buf<unsigned char> invalid;
    Buf<int4> tri, orig_tri, tri_in, tri_next, res_tri, tri_load;
    Buf<int> ecount, qflag, qlist, fflags, nt, nxt, fmesh, shuffle_flags;
    Buf<int2> spc;
    Buf<float4> fgeo;
    Buf<float> face_mean;
    Buf<unsigned long long> fkey;
    Buf<unsigned char> hit;
    Buf<int2> edges, exact_list;
    Buf<int> eorder, win, winners, lines, considered, uflag;
    Buf<uint32_t> cost;
    BvhBuffers bvh;
    char* bvh_mem = nullptr;
    size_t bvh_cap = 0;
    // per mesh regions and tables
    Buf<int> map_reg, undo_list_reg, tmp_undo_reg, undo_in_reg;
    Buf<unsigned char> invalid_reg;
    Buf<uint32_t> ecost_reg;
    Buf<BatchMesh> mesh;
    Buf<int> slot_mesh, slot_v0, slot_np, slot_f0, slot_nf, slot_stuck, mesh_root;
    Buf<float> slot_scale, mesh_scale, centre;
    Buf<float4> mean;
    Buf<long long> dev_voff, dev_foff, dev_out_voff, dev_out_foff;
    RoundCounters* rc = nullptr;
    BatchCtl* ctl = nullptr;
    BatchCtl* h_ctl = nullptr;
    LoopState* zero_ls = nullptr;
    int* scan_scratch = nullptr;
    std::vector<int> rounds;
    std::vector<BatchMesh> h_mesh;

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
    template <typename T>
    int grow(Buf<T>& b, size_t n, bool zero = false) {
        if (b.p && b.n >= n) {
            if (zero) cudaMemsetAsync(b.p, 0, n * sizeof(T), stream);
            return PAMO_OK;
        }
        if (b.p) {
            cudaStreamSynchronize(stream);
            cudaFree(b.p);
            b.p = nullptr;
            b.n = 0;
        }
        cudaError_t e = cudaMalloc((void**)&b.p, std::max<size_t>(n, 1) * sizeof(T));
        if (e != cudaSuccess) return check(e, "cudaMalloc");
        b.n = std::max<size_t>(n, 1);
        if (zero) cudaMemsetAsync(b.p, 0, b.n * sizeof(T), stream);
        return PAMO_OK;
    }
    template <typename T>
    static void release(Buf<T>& b) {
        if (b.p) cudaFree(b.p);
        b.p = nullptr;
        b.n = 0;
    }

    int init() {
        int r;
        if ((r = check(cudaSetDevice(device), "cudaSetDevice"))) return r;
        if ((r = check(cudaMalloc((void**)&rc, sizeof(RoundCounters)), "cudaMalloc"))) return r;
        if ((r = check(cudaMalloc((void**)&ctl, sizeof(BatchCtl)), "cudaMalloc"))) return r;
        if ((r = check(cudaMallocHost((void**)&h_ctl, sizeof(BatchCtl)), "cudaMallocHost"))) return r;
        if ((r = check(cudaMalloc((void**)&zero_ls, sizeof(LoopState)), "cudaMalloc"))) return r;
        cudaMemset(zero_ls, 0, sizeof(LoopState));
        if ((r = check(cudaMalloc((void**)&scan_scratch, kMaxScanJobs * scan_scratch_ints() * sizeof(int)), "cudaMalloc")))
            return r;
        for (int k = 0; k < kMaxScanJobs; ++k)
            if (scan_scratch_clear(scan_scratch + k * scan_scratch_ints())) return check(cudaGetLastError(), "scan scratch");
        return PAMO_OK;
    }

    void destroy() {
        cudaSetDevice(device);
        cudaDeviceSynchronize();
        release(pos); release(orig_pos); release(pos_in); release(pos_next); release(res_pos);
        release(occ); release(valence); release(cursor); release(vedges); release(vcursor); release(vmesh);
        release(vscan); release(quad); release(vmin); release(invalid); release(tri); release(orig_tri);
        release(tri_in); release(tri_next); release(res_tri); release(tri_load); release(ecount); release(qflag);
        release(qlist); release(fflags); release(nt); release(nxt); release(spc); release(fmesh); release(shuffle_flags);
        release(fgeo); release(face_mean); release(fkey); release(hit); release(edges); release(exact_list);
        release(eorder); release(win); release(winners); release(lines); release(considered); release(uflag);
        release(cost); release(map_reg); release(undo_list_reg); release(tmp_undo_reg); release(undo_in_reg);
        release(invalid_reg); release(ecost_reg); release(mesh); release(slot_mesh); release(slot_v0);
        release(slot_np); release(slot_f0); release(slot_nf); release(slot_stuck); release(mesh_root);
        release(slot_scale); release(mesh_scale); release(centre); release(mean); release(dev_voff);
        release(dev_foff); release(dev_out_voff); release(dev_out_foff);
        if (bvh_mem) cudaFree(bvh_mem);
        bvh_mem = nullptr;
        if (rc) cudaFree(rc);
        if (ctl) cudaFree(ctl);
        if (h_ctl) cudaFreeHost(h_ctl);
        if (zero_ls) cudaFree(zero_ls);
        if (scan_scratch) cudaFree(scan_scratch);
        rc = nullptr;
    }

    int ensure(long long V, long long F, int M, long long vstate, long long estate) {
        const size_t vc = (size_t)V + 2, fc = (size_t)F + 2, ec = 3 * (size_t)F + 3;
        int r;
        if ((r = grow(pos, vc)) || (r = grow(orig_pos, vc)) || (r = grow(pos_in, vc)) || (r = grow(pos_next, vc)) ||
            (r = grow(res_pos, vc)) || (r = grow(occ, vc + 1)) || (r = grow(valence, vc + 1)) ||
            (r = grow(cursor, vc + 1)) || (r = grow(vedges, vc + 1)) || (r = grow(vcursor, vc + 1)) ||
            (r = grow(vmesh, vc)) || (r = grow(vscan, vc + 1)) || (r = grow(quad, vc)) || (r = grow(vmin, vc + 1)) ||
            (r = grow(invalid, vc)))
            return r;
        if ((r = grow(tri, fc)) || (r = grow(orig_tri, fc)) || (r = grow(tri_in, fc)) || (r = grow(tri_next, fc)) ||
            (r = grow(res_tri, fc)) || (r = grow(tri_load, fc)) || (r = grow(ecount, fc + 1)) ||
            (r = grow(qflag, fc + 1)) || (r = grow(qlist, fc)) || (r = grow(fflags, fc + 1)) || (r = grow(nt, 3 * fc)) ||
            (r = grow(nxt, 3 * fc)) || (r = grow(spc, 3 * fc)) || (r = grow(fmesh, fc)) || (r = grow(shuffle_flags, 2 * fc + 40)) ||
            (r = grow(fgeo, 6 * fc)) || (r = grow(face_mean, 3 * fc)) || (r = grow(fkey, fc)) || (r = grow(hit, fc + 1)))
            return r;
        if ((r = grow(edges, ec)) || (r = grow(eorder, ec)) || (r = grow(win, ec + 1)) || (r = grow(winners, ec)) ||
            (r = grow(lines, ec)) || (r = grow(considered, ec)) || (r = grow(uflag, ec + 1)) || (r = grow(cost, ec)) ||
            (r = grow(exact_list, std::max<size_t>(1 << 20, 16 * fc))))
            return r;
        if ((r = grow(map_reg, vstate, true)) || (r = grow(undo_list_reg, vstate, true)) ||
            (r = grow(tmp_undo_reg, vstate, true)) || (r = grow(undo_in_reg, vstate, true)) ||
            (r = grow(invalid_reg, vstate, true)) || (r = grow(ecost_reg, estate, true)))
            return r;
        const size_t mc = (size_t)M + 1;
        if ((r = grow(mesh, mc)) || (r = grow(slot_mesh, mc)) || (r = grow(slot_v0, mc)) || (r = grow(slot_np, mc)) ||
            (r = grow(slot_f0, mc)) || (r = grow(slot_nf, mc)) || (r = grow(slot_stuck, mc)) ||
            (r = grow(mesh_root, mc)) || (r = grow(slot_scale, mc)) || (r = grow(mesh_scale, mc)) ||
            (r = grow(centre, 16 * mc)) || (r = grow(mean, mc)) || (r = grow(dev_voff, mc + 1)) ||
            (r = grow(dev_foff, mc + 1)) || (r = grow(dev_out_voff, mc + 1)) || (r = grow(dev_out_foff, mc + 1)))
            return r;
        if (bvh_cap < fc) {
            if (bvh_mem) {
                cudaStreamSynchronize(stream);
                cudaFree(bvh_mem);
                bvh_mem = nullptr;
            }
            cudaError_t e = cudaMalloc((void**)&bvh_mem, bvh_bytes((int)fc));
            if (e != cudaSuccess) return check(e, "cudaMalloc(bvh)");
            bvh_carve(bvh, (int)fc, bvh_mem);
            bvh_cap = fc;
        }
        return PAMO_OK;
    }

    int read_ctl() {
        int r;
        if ((r = check(cudaGetLastError(), "kernel launch"))) return r;
        cudaMemcpyAsync(h_ctl, ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, stream);
        return check(cudaStreamSynchronize(stream), "batched round");
    }

    int status_error(int bits) {
        if (bits & kErrBadIndex) return fail(PAMO_ERR_INVALID_ARG, "a triangle references a vertex outside its mesh");
        if (bits & kErrStackOverflow) return fail(PAMO_ERR_ITER_LIMIT, "BVH traversal stack overflow");
        if (bits & kErrIterLimit) return fail(PAMO_ERR_ITER_LIMIT, "a bounded device loop hit its iteration limit");
        if (bits & kErrCapacity) return fail(PAMO_ERR_CAPACITY, "a per-mesh list overflowed its capacity");
        return PAMO_OK;
    }

    // one intersection check over the meshes being checked, then their undo counts (kb_after_check)
    void check_pass(int Vb, int Fb, int Eb, int M, const BvhMeshes& bm) {
        cudaStream_t s = stream;
        launch_zero_face_bytes_dev(rc, Fb, hit.p, s);
        bvh_build(bvh, tri.p, pos.p, rc, Fb, s, false, qflag.p, false, &bm);
        bvh_query(bvh, tri.p, pos.p, qlist.p, qflag.p, hit.p, exact_list.p, (int)exact_list.n, rc, Fb, kTriEpsB, s,
                  fmesh.p, mesh_root.p);
        launch_undo_check(rc, Eb, considered.p, edges.p, valence.p, nt.p, hit.p, uflag.p, s);
        exclusive_scan(uflag.p, uflag.p, &rc->n_considered, 1, &rc->n_undo, scan_scratch, s, &rc->status, Eb);
        kb_after_check<<<1, kCtlThreads, 0, s>>>(ctl, slot_mesh.p, mesh.p, uflag.p); note_launch();
        (void)Vb;
        (void)M;
    }

    // one round of every live mesh; Vb, Fb bound the round's vertices and faces
    int round(int M, int Vb, int Fb, float threshold) {
        cudaStream_t s = stream;
        const int Eb = 3 * Fb;
        const uint32_t collapse_t = collapse_threshold(threshold);
        const int gM = std::max(1, std::min(M, 4096));
        kb_round_begin<<<1, kCtlThreads, 0, s>>>(mesh.p, M, slot_mesh.p, slot_v0.p, slot_np.p, slot_f0.p, slot_nf.p,
                                                 slot_stuck.p, slot_scale.p, mesh_scale.p, rc, ctl); note_launch();
        kb_fill_slots<<<gM, kT, 0, s>>>(ctl, slot_v0.p, slot_np.p, slot_f0.p, slot_nf.p, vmesh.p, fmesh.p); note_launch();
        kb_undo_book<<<gM, kT, 0, s>>>(ctl, slot_mesh.p, mesh.p, undo_in_reg.p, tmp_undo_reg.p, undo_list_reg.p,
                                       map_reg.p, invalid_reg.p); note_launch();
        launch_round_prologue_dev(zero_ls, rc, Vb, Fb, nullptr, nullptr, pos_in.p, pos.p, orig_pos.p, occ.p, tri_in.p,
                                  tri.p, orig_tri.p, valence.p, cursor.p, vedges.p, vcursor.p, qflag.p, s);
        // adjacency, quadrics (per element: rings never leave a mesh)
        launch_face_counts(tri.p, rc, Fb, valence.p, ecount.p, vedges.p, s, pos.p, fgeo.p);
        {
            const size_t sz = scan_scratch_ints();
            const ScanJob jobs[3] = {{valence.p, valence.p, &rc->n_pts, 1, nullptr, scan_scratch},
                                     {ecount.p, ecount.p, &rc->n_tris, 1, &rc->n_edges, scan_scratch + sz},
                                     {vedges.p, vedges.p, &rc->n_pts, 1, nullptr, scan_scratch + 2 * sz}};
            exclusive_scans(jobs, 3, s, &rc->status, std::max(Vb, Fb));
        }
        launch_fill_adjacency(tri.p, rc, Fb, valence.p, cursor.p, nt.p, ecount.p, edges.p, vedges.p, vcursor.p,
                              eorder.p, s);
        launch_sort_adjacency(rc, Vb, valence.p, nt.p, s);
        const int* nt_off = valence.p;
        launch_quadrics(rc, Vb, nt_off, nt.p, tri.p, fgeo.p, quad.p, nxt.p, spc.p, s);
        // cost with each mesh's stale costs and invalid table, then the costs back to the meshes' regions
        kb_slot_edges<<<gM, kT, 0, s>>>(ctl, slot_mesh.p, mesh.p, ecount.p, rc); note_launch();
        kb_gather<<<grid_for(std::max(Eb, Vb), kT), kT, 0, s>>>(rc, slot_mesh.p, mesh.p, vmesh.p, edges.p, ecost_reg.p,
                                                               invalid_reg.p, cost.p, invalid.p); note_launch();
        launch_fill_u64_dev(rc, Vb, vmin.p, ~0ull, s);
        launch_edge_cost_batch(rc, Eb, eorder.p, edges.p, nt_off, nt.p, tri.p, pos.p, quad.p, fgeo.p, nxt.p, spc.p, invalid.p,
                               cost.p, vmin.p, slot_scale.p, slot_stuck.p, vmesh.p, threshold, s, skinny_pow);
        kb_scatter_costs<<<grid_for(Eb, kT), kT, 0, s>>>(rc, slot_mesh.p, mesh.p, vmesh.p, edges.p, cost.p, ecost_reg.p);
        note_launch();
        // selection and collapse
        launch_face_keys(rc, Fb, tri.p, vmin.p, fkey.p, s);
        launch_collapse(rc, Eb, eorder.p, edges.p, cost.p, collapse_t, fkey.p, nt_off, nt.p, tri.p, orig_tri.p, pos.p,
                        orig_pos.p, occ.p, win.p, s);
        exclusive_scan(win.p, win.p, &rc->n_edges, 1, &rc->n_win, scan_scratch, s, &rc->status, Eb);
        launch_compact_winners(rc, Eb, win.p, winners.p, s);
        launch_remove_invalid(rc, Fb, tri.p, s);
        launch_line_detect(rc, Eb, edges.p, pos.p, s);
        kb_line_apply<<<1, 32, 0, s>>>(rc, ctl, slot_mesh.p, mesh.p, vmesh.p, edges.p, nt_off, nt.p, tri.p, pos.p, occ.p,
                                       lines.p, (int)lines.n); note_launch();
        kb_considered<<<1, kCtlThreads, 0, s>>>(ctl, slot_mesh.p, mesh.p, win.p, rc); note_launch();
        kb_considered_fill<<<gM, kT, 0, s>>>(ctl, slot_mesh.p, mesh.p, winners.p, lines.p, considered.p); note_launch();
        // faces whose intersections decide the undo: rings of the considered collapsed edges
        launch_mark_query(rc, Eb, considered.p, edges.p, nt_off, nt.p, qflag.p, s);
        exclusive_scan(qflag.p, qflag.p, &rc->n_tris, 1, &rc->n_query, scan_scratch, s, &rc->status, Fb);
        launch_compact_flags(qflag.p, Fb, &rc->n_tris, qlist.p, s);
        // intersection checks and undo passes (cusimp_free.cu:1014-1040), per mesh
        BvhMeshes bm;
        bm.fmesh = fmesh.p;
        int bits = 1;
        while ((1 << bits) < M && bits < 16) ++bits;
        bm.bits = bits;
        bm.f0 = slot_f0.p;
        bm.nf = slot_nf.p;
        bm.d_count = &ctl->n_slots;
        bm.count_bound = M;
        bm.root = mesh_root.p;
        check_pass(Vb, Fb, Eb, M, bm);
        int r;
        if ((r = read_ctl())) return r;
        while (h_ctl->any_apply) {
            kb_undo_apply<<<grid_for(Eb, kT), kT, 0, s>>>(rc, slot_mesh.p, mesh.p, vmesh.p, considered.p, uflag.p,
                                                          edges.p, nt_off, nt.p, tri.p, orig_tri.p, pos.p, orig_pos.p,
                                                          occ.p, tmp_undo_reg.p, undo_list_reg.p, map_reg.p, &rc->status);
            note_launch();
            kb_after_apply<<<1, kCtlThreads, 0, s>>>(ctl, slot_mesh.p, mesh.p); note_launch();
            check_pass(Vb, Fb, Eb, M, bm);
            if ((r = read_ctl())) return r;
        }
        // compaction maps, loop update, compaction
        launch_live_flags(rc, Fb, tri.p, fflags.p, s);
        {
            const size_t sz = scan_scratch_ints();
            const ScanJob jobs[2] = {{occ.p, vscan.p, &rc->n_pts, 1, nullptr, scan_scratch},
                                     {fflags.p, fflags.p, &rc->n_tris, 1, nullptr, scan_scratch + sz}};
            exclusive_scans(jobs, 2, s, &rc->status, std::max(Vb, Fb));
        }
        kb_round_end<<<1, kCtlThreads, 0, s>>>(ctl, slot_mesh.p, mesh.p, vscan.p, fflags.p, rc); note_launch();
        kb_compact<<<grid_for(std::max(Vb, Fb), kT), kT, 0, s>>>(rc, slot_mesh.p, mesh.p, vmesh.p, fmesh.p, pos.p, occ.p,
                                                                 vscan.p, tri.p, fflags.p, map_reg.p, mean.p,
                                                                 pos_next.p, tri_next.p, res_pos.p, res_tri.p);
        note_launch();
        kb_carry_undo<<<gM, kT, 0, s>>>(ctl, slot_mesh.p, mesh.p, undo_list_reg.p, undo_in_reg.p); note_launch();
        if ((r = read_ctl())) return r;
        if ((r = status_error(h_ctl->status))) return r;
        std::swap(pos_in, pos_next);
        std::swap(tri_in, tri_next);
        return PAMO_OK;
    }

    int simplify(const float* points, const int32_t* triangles, const int64_t* voff, const int64_t* foff, int M,
                 const double* ratios, int tolerance, float threshold, int iter, int64_t min_verts, float* out_points,
                 int32_t* out_tris, int64_t* out_voff, int64_t* out_foff) {
        cudaStream_t s = stream;
        err.clear();
        if (M < 1 || M > 65536) return fail(PAMO_ERR_INVALID_ARG, "1 to 65536 meshes per batch");
        const long long V = voff[M], F = foff[M];
        if (V > (1ll << 30) || F > (1ll << 29)) return fail(PAMO_ERR_CAPACITY, "batch larger than 2^29 faces");
        h_mesh.assign(M, BatchMesh{});
        long long vstate = 0, estate = 0;
        for (int m = 0; m < M; ++m) {
            const long long nv = voff[m + 1] - voff[m], nf = foff[m + 1] - foff[m];
            if (nv < 0 || nf < 0) return fail(PAMO_ERR_INVALID_ARG, "offsets must not decrease");
            BatchMesh& B = h_mesh[m];
            B.target = std::max((long long)(ratios[m] * (double)nf), (long long)min_verts);
            B.tolerance = tolerance;
            B.iter = iter;
            B.lp = (int)(nv + nv / 5 + 1);
            B.ecap = (int)(3 * nf + 1);
            B.vreg = vstate;
            B.ereg = estate;
            B.res_v0 = voff[m];
            B.res_f0 = foff[m];
            B.np = (int)nv;
            B.nf = (int)nf;
            B.done = (iter <= 0) ? 1 : 0;
            vstate += B.lp + 1;
            estate += B.ecap + 1;
        }
        int r;
        if ((r = ensure(V, F, M, vstate, estate))) return r;
        cudaMemcpyAsync(mesh.p, h_mesh.data(), M * sizeof(BatchMesh), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dev_voff.p, voff, (M + 1) * sizeof(long long), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dev_foff.p, foff, (M + 1) * sizeof(long long), cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(rc, 0, sizeof(RoundCounters), s);
        // per mesh: centring and scale (numpy's order), validation, the first round's shuffle
        for (int m = 0; m < M; ++m) {
            const int nv = (int)(voff[m + 1] - voff[m]), nf = (int)(foff[m + 1] - foff[m]);
            if (nv > 0 && nf > 0)
                launch_center(points + 3 * voff[m], triangles + 3 * foff[m], nv, nf, face_mean.p, centre.p + 16 * m,
                              mesh_scale.p + m, pos_in.p + voff[m], s, true);
            else
                cudaMemsetAsync(centre.p + 16 * m, 0, 16 * sizeof(float), s);
            if (nf > 0) {
                launch_load_tris(triangles + 3 * foff[m], nf, nv, tri_load.p + foff[m], rc, s);
                Feistel fb = make_feistel((unsigned long long)nf);
                launch_shuffle_tris(fb, shuffle_flags.p, scan_scratch, tri_load.p + foff[m], tri_in.p + foff[m], nf, s,
                                    &rc->status);
            }
        }
        kb_offset_faces<<<grid_for(F, kT), kT, 0, s>>>(tri_in.p, dev_foff.p, dev_voff.p, M, (int)F); note_launch();
        kb_mean_table<<<grid_for(M, kT), kT, 0, s>>>(centre.p, M, mean.p); note_launch();
        {
            int st = 0;
            cudaMemcpyAsync(&st, &rc->status, sizeof(int), cudaMemcpyDeviceToHost, s);
            if ((r = check(cudaStreamSynchronize(s), "batch set-up"))) return r;
            if ((r = status_error(st))) return r;
        }
        rounds.assign(M, 0);
        long long Vr = V, Fr = F;
        for (int it = 0;; ++it) {
            auto cls = [](long long n) {  // grid bound: next power of two, from 1024
                long long b = 1024;
                while (b < n && b < (1ll << 30)) b <<= 1;
                return (int)b;
            };
            if ((r = round(M, cls(Vr), cls(Fr), threshold))) return r;
            if (h_ctl->n_next == 0) break;
            Vr = h_ctl->v_next;
            Fr = h_ctl->f_next;
            if (it > iter + 4) return fail(PAMO_ERR_ITER_LIMIT, "batch did not finish");
        }
        // results, packed in mesh order
        cudaMemcpyAsync(h_mesh.data(), mesh.p, M * sizeof(BatchMesh), cudaMemcpyDeviceToHost, s);
        if ((r = check(cudaStreamSynchronize(s), "batch results"))) return r;
        out_voff[0] = 0;
        out_foff[0] = 0;
        for (int m = 0; m < M; ++m) {
            out_voff[m + 1] = out_voff[m] + h_mesh[m].np_out;
            out_foff[m + 1] = out_foff[m] + h_mesh[m].nf_out;
            rounds[m] = h_mesh[m].rounds;
        }
        cudaMemcpyAsync(dev_out_voff.p, out_voff, (M + 1) * sizeof(long long), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dev_out_foff.p, out_foff, (M + 1) * sizeof(long long), cudaMemcpyHostToDevice, s);
        kb_pack_results<<<std::max(1, std::min(M, 4096)), kT, 0, s>>>(mesh.p, M, dev_out_voff.p, dev_out_foff.p,
                                                                       res_pos.p, res_tri.p, out_points, out_tris);
        note_launch();
        return check(cudaStreamSynchronize(s), "batch results");
    }
};

extern "C" {

int pamo_csr_create(pamo_csr** out, int device) {
    if (!out) return PAMO_ERR_INVALID_ARG;
    auto* b = new pamo_csr();
    b->device = device;
    const int r = b->init();
    if (r) {
        b->destroy();
        delete b;
        return r;
    }
    *out = b;
    return PAMO_OK;
}

int pamo_csr_destroy(pamo_csr* b) {
    if (!b) return PAMO_ERR_INVALID_ARG;
    b->destroy();
    delete b;
    return PAMO_OK;
}

const char* pamo_csr_last_error(const pamo_csr* b) { return b ? b->err.c_str() : "null batch"; }

int pamo_csr_set_option(pamo_csr* b, const char* name, int64_t value) {
    if (!b || !name) return PAMO_ERR_INVALID_ARG;
    if (std::string(name) == "skinny_pow") b->skinny_pow = value != 0;
    else return b->fail(PAMO_ERR_INVALID_ARG, "unknown option %s", name);
    return PAMO_OK;
}

int pamo_csr_simplify(pamo_csr* b, const float* points, const int32_t* triangles, const int64_t* vert_offsets,
                      const int64_t* face_offsets, int32_t n_meshes, const double* ratios, int32_t tolerance,
                      float threshold, int32_t iter, int64_t min_verts, float* out_points, int32_t* out_triangles,
                      int64_t* out_vert_offsets, int64_t* out_face_offsets, pamo_stream stream) {
    if (!b || !points || !triangles || !vert_offsets || !face_offsets || !ratios || !out_points || !out_triangles ||
        !out_vert_offsets || !out_face_offsets)
        return PAMO_ERR_INVALID_ARG;
    if (cudaSetDevice(b->device) != cudaSuccess) return PAMO_ERR_CUDA;
    b->stream = (cudaStream_t)stream;
    return b->simplify(points, triangles, vert_offsets, face_offsets, n_meshes, ratios, tolerance, threshold, iter,
                       min_verts, out_points, out_triangles, out_vert_offsets, out_face_offsets);
}

int pamo_csr_rounds(const pamo_csr* b, int32_t* rounds, int32_t capacity) {
    if (!b || (!rounds && capacity > 0)) return PAMO_ERR_INVALID_ARG;
    const int n = std::min<int>(capacity, (int)b->rounds.size());
    for (int i = 0; i < n; ++i) rounds[i] = b->rounds[i];
    return n;
}

}  // extern "C"
