// Kernels of one stage-2 collapse round (host launchers). Every count is read from RoundCounters in device
// memory; the *_bound arguments only size the grids.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "pamo_common.cuh"

namespace pamo {

struct Feistel {  // thrust::shuffle's bijection parameters for m elements
    uint32_t key[24];
    uint32_t lbits, rbits, lmask, rmask;
    unsigned long long n;  // 2^bits
    unsigned long long m;
};
Feistel make_feistel(unsigned long long m);

// ---- set-up of a round ----
void launch_undo_bookkeeping(const int* verts_undo, int n_verts_undo, int is_stuck, int* tmp_undo, int* undo_list,
                             const int* pts_map, int pts_map_len, unsigned char* invalid, int invalid_len, cudaStream_t s);
void launch_load_points(const float* pts, int n, float4* pos, float4* orig_pos, int* occ, cudaStream_t s);
void launch_load_points4(const float4* pts, int n, float4* pos, float4* orig_pos, int* occ, cudaStream_t s);
void launch_load_tris(const int* tris, int n, int n_pts, int4* tri, RoundCounters* rc, cudaStream_t s);
void launch_load_tris4(const int4* tris, int n, int4* tri, cudaStream_t s);
void launch_shuffle_tris(const Feistel& fb, int* flags, int* scan_scratch, int4* tmp, int4* tri, int n, cudaStream_t s,
                         int* err = nullptr);
void launch_copy_tris(const int4* src, int4* dst, int n, cudaStream_t s);

// ---- adjacency ----
// with fgeo: also the per-face geometry the rings read (from pos; room for six float4 per face): a 64-byte record per
// face (fgeo[4f .. 4f + 3]: edge lengths, normal, corner positions), then the planes after all n faces' records, one
// float4 per face (fgeo[4n + f]) or, with plane_df (precision mode), a double-float pair (fgeo[4n + 2f], +1)
void launch_face_counts(const int4* tri, const RoundCounters* rc, int n_tris_bound, int* valence, int* ecount,
                        int* vedges, cudaStream_t s, const float4* pos = nullptr, float4* fgeo = nullptr,
                        bool plane_df = false);
void launch_fill_adjacency(const int4* tri, const RoundCounters* rc, int n_tris_bound, const int* nt_off, int* cursor,
                           int* nt, const int* edge_off, int2* edges, const int* voff, int* vcursor, int* eorder,
                           cudaStream_t s);
void launch_sort_adjacency(const RoundCounters* rc, int n_pts_bound, const int* nt_off, int* nt, cudaStream_t s);

// ---- cost, selection, collapse ----
// qlo (precision mode; needs the plane_df planes): each quadric as a double-float sum, hi parts to q, lo to qlo
// nxt, spc: per ring slot, the vertex after the ring's vertex in the slot's face and (the vertex before it, its corner)
void launch_quadrics(const RoundCounters* rc, int n_pts_bound, const int* nt_off, const int* nt, const int4* tri,
                     const float4* fgeo, Quadric* q, int* nxt, int2* spc, cudaStream_t s, Quadric* qlo = nullptr);
void launch_edge_cost_capacity(RoundCounters* rc, int* d_cap, uint32_t* edge_cost, int phys_len, cudaStream_t s);
// mode: 0 the reference's arithmetic; precision mode 1 (double-float quadrics q + qlo, compensated sums) or 2 (as 1,
// placement at the quadric's minimiser, written to place[e]). raw (optional): each edge's cost before clamp and quantisation (NaN where
// none is computed); place (optional, required by mode 2): each edge's placement.
void launch_edge_cost(const RoundCounters* rc, int n_edges_bound, const int* eorder, const int2* edges, const int* nt_off,
                      const int* nt, const int4* tri, const float4* pos, const Quadric* q, const float4* fgeo,
                      const int* nxt, const int2* spc, const unsigned char* invalid, uint32_t* cost,
                      unsigned long long* vmin,
                      const float* d_scale, float tres, int is_stuck, cudaStream_t s, const int* is_stuck_dev = nullptr,
                      bool legacy = false, bool device_pow = false, int mode = 0, float* raw = nullptr,
                      float4* place = nullptr, const Quadric* qlo = nullptr);
// The edge cost of many meshes in one vertex numbering: the scale and is_stuck of each edge's mesh (vmesh of its
// lower vertex) come from mesh_scale and mesh_stuck.
void launch_edge_cost_batch(const RoundCounters* rc, int n_edges_bound, const int* eorder, const int2* edges,
                            const int* nt_off, const int* nt, const int4* tri, const float4* pos, const Quadric* q,
                            const float4* fgeo, const int* nxt, const int2* spc, const unsigned char* invalid,
                            uint32_t* cost,
                            unsigned long long* vmin, const float* mesh_scale, const int* mesh_stuck, const int* vmesh,
                            float tres, cudaStream_t s, bool device_pow = false);
void launch_face_keys(const RoundCounters* rc, int n_tris_bound, const int4* tri, const unsigned long long* vmin,
                      unsigned long long* fkey, cudaStream_t s);
void launch_collapse(RoundCounters* rc, int n_edges_bound, const int* eorder, const int2* edges, const uint32_t* cost,
                     uint32_t collapse_t, const unsigned long long* fkey, const int* nt_off, const int* nt, int4* tri,
                     const int4* orig_tri, float4* pos, const float4* orig_pos, int* occ, int* win, cudaStream_t s,
                     bool restore = true, const float4* place = nullptr);
void launch_compact_winners(const RoundCounters* rc, int n_edges_bound, const int* win_scan, int* collapsed,
                            cudaStream_t s);
void launch_remove_invalid(const RoundCounters* rc, int n_tris_bound, int4* tri, cudaStream_t s);
void launch_line_edges(RoundCounters* rc, int n_edges_bound, const int2* edges, const int* nt_off, const int* nt,
                       int4* tri, float4* pos, int* occ, int* line_buf, int line_cap, int* collapsed, cudaStream_t s);

// ---- self-intersection rollback ----
// counts coincident-endpoint edges into rc->n_line (the first half of launch_line_edges)
void launch_line_detect(RoundCounters* rc, int n_edges_bound, const int2* edges, const float4* pos, cudaStream_t s);
void launch_mark_query(const RoundCounters* rc, int n_edges_bound, const int* collapsed, const int2* edges,
                       const int* nt_off, const int* nt, int* qflag, cudaStream_t s);
void launch_compact_flags(const int* scan, int n_bound, const int* d_n, int* out_list, cudaStream_t s);
void launch_undo_check(RoundCounters* rc, int n_edges_bound, const int* collapsed, const int2* edges, const int* nt_off,
                       const int* nt, const unsigned char* hit, int* uflag, cudaStream_t s);
void launch_undo_apply(RoundCounters* rc, int n_edges_bound, const int* collapsed, const int* uscan, const int2* edges,
                       const int* nt_off, const int* nt, int4* tri, const int4* orig_tri, float4* pos,
                       const float4* orig_pos, int* occ, int* tmp_undo, int* undo_list, const int* pts_map,
                       int list_cap, cudaStream_t s);

// ---- outputs ----
void launch_live_flags(const RoundCounters* rc, int n_tris_bound, const int4* tri, int* flags, cudaStream_t s);
void launch_compact_mesh(RoundCounters* rc, int n_pts_bound, int n_tris_bound, const float4* pos, const int* occ,
                         const int* pts_map, const int4* tri, const int* face_scan, float4* out_pos, int4* out_tri,
                         cudaStream_t s);
void launch_export_round(const RoundCounters* rc, int n_pts, int n_tris, const float4* pos, const int4* tri,
                         const int* occ, const int* pts_map, const int* undo_list, float* verts, int* tris,
                         int* verts_occ, int* verts_map, int* verts_undo, int n_undo, cudaStream_t s);
void launch_export_mesh(int n_pts, int n_tris, const float4* pos, const int4* tri, const float* add, float* verts,
                        int* tris, cudaStream_t s);

// ---- whole-loop helpers ----
void launch_center(const float* pts, const int* tris, int n_pts, int n_tris, float* face_mean, float* center,
                   float* d_scale, float4* pos_out, cudaStream_t s,
                   bool centre = true);
void launch_after_check(RoundCounters* rc, cudaStream_t s);

// ---- device-driven rounds: sizes from LoopState / RoundCounters, host values only bound the grids ----
void launch_round_begin(RoundCounters* rc, LoopState* ls, const LoopState* next, cudaStream_t s);
void launch_undo_bookkeeping_dev(const int* verts_undo, const LoopState* ls, int n_undo_bound, int* tmp_undo,
                                 int* undo_list, const int* pts_map, int pts_map_len, unsigned char* invalid,
                                 int invalid_len, cudaStream_t s);
// Start of a device round, after the undo bookkeeping, in one launch: pts_map_prev[0, ls->np) = pts_map (the
// previous round's map, read by this round's undo passes); pos = orig_pos = the round's points, occ = 1 and
// occ[n_pts] = 0; tri = orig_tri = the round's faces; valence, cursor, vedges, vcursor = 0 over n_pts + 1 entries;
// qflag = 0 over n_tris + 1 entries.
void launch_round_prologue_dev(const LoopState* ls, const RoundCounters* rc, int n_pts_bound, int n_tris_bound,
                               const int* pts_map, int* pts_map_prev, const float4* pts_in, float4* pos,
                               float4* orig_pos, int* occ, const int4* tri_in, int4* tri, int4* orig_tri, int* valence,
                               int* cursor, int* vedges, int* vcursor, int* qflag, cudaStream_t s);
void launch_fill_u64_dev(const RoundCounters* rc, int n_pts_bound, unsigned long long* p, unsigned long long v,
                         cudaStream_t s);
void launch_zero_face_bytes_dev(const RoundCounters* rc, int n_tris_bound, unsigned char* p, cudaStream_t s);
void launch_round_end(const RoundCounters* rc, const LoopState* ls, LoopState* next, const int* undo_list, int* undo_in,
                      int undo_cap, int n_undo_bound, cudaStream_t s);

}  // namespace pamo
