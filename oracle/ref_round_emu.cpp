// The reference's stage-2 round (simp_cuda/src/cusimp_free.cu with its LBVH headers, simp_cuda/src/bvh/), compiled
// for the host under the emulation in oracle/ref_emu and exported with a C interface for the fixture generator
// tests/golden/make_ref_round_golden.py. oracle/build_ref.py rewrites only the launch syntax (and the device's
// saturating float->uint32 cost conversion, cusimp_free.cu:584) into oracle/_ref/emu_src/ and builds this file into
// oracle/_ref/libref_round_emu.so. Test infrastructure only: it pins the oracle's restatement of the round to the
// reference's own kernels; nothing of it is part of the product or travels as source.
#include "emu_prelude.h"

#include "cusimp_free.cu"

using cusimp_free::CUSimp_Free;
using cusimp_free::Triangle;
using cusimp_free::Vertex;

extern "C" {

// like the pybind operator's constructor (simp_cuda/src/pybind.cpp:19): all buffers unallocated
void* ref_create() { return new CUSimp_Free(); }

void ref_destroy(void* h) { delete static_cast<CUSimp_Free*>(h); }

// one CUDSP_Free.forward call (pybind.cpp:52-72): inputs are host arrays here
void ref_forward(void* h, const float* pts, const int* tris, const int* undo, int n_undo, int n_pts, int n_tris,
                 float scale, float threshold, int is_stuck, int init) {
    auto* sp = static_cast<CUSimp_Free*>(h);
    sp->forward(reinterpret_cast<Vertex<float>*>(const_cast<float*>(pts)),
                reinterpret_cast<Triangle<int>*>(const_cast<int*>(tris)), const_cast<int*>(undo), n_undo, n_pts,
                n_tris, scale, threshold, is_stuck != 0, init != 0);
}

// n_pts, n_tris, n_vertices_undo, collapsed edges, edges
void ref_counts(void* h, long long* out) {
    auto* sp = static_cast<CUSimp_Free*>(h);
    out[0] = sp->n_pts;
    out[1] = sp->n_tris;
    out[2] = sp->n_vertices_undo;
    out[3] = sp->n_collapsed ? *sp->n_collapsed : 0;
    out[4] = sp->n_edges;
}

// the five outputs the pybind operator clones (pybind.cpp:74-100)
void ref_outputs(void* h, float* verts, int* tris, int* occ, int* vmap, int* undo) {
    auto* sp = static_cast<CUSimp_Free*>(h);
    std::memcpy(verts, sp->points, sizeof(float) * 3 * sp->n_pts);
    std::memcpy(tris, sp->triangles, sizeof(int) * 3 * sp->n_tris);
    std::memcpy(occ, sp->pts_occ, sizeof(int) * sp->n_pts);
    std::memcpy(vmap, sp->pts_map, sizeof(int) * sp->n_pts);
    if (sp->n_vertices_undo > 0) std::memcpy(undo, sp->vertices_undo_list, sizeof(int) * sp->n_vertices_undo);
}

// the collapsed edges of the last forward, as (u, v) pairs in the order the collapse kernel listed them
void ref_collapsed(void* h, int* uv) {
    auto* sp = static_cast<CUSimp_Free*>(h);
    const int n = sp->n_collapsed ? *sp->n_collapsed : 0;
    for (int i = 0; i < n; ++i) {
        const auto e = sp->edges[sp->collapsed_edge_idx[i]];
        uv[2 * i] = e.u;
        uv[2 * i + 1] = e.v;
    }
}

// the quantised edge costs and edges of the last forward
void ref_edges(void* h, int* uv, unsigned* cost) {
    auto* sp = static_cast<CUSimp_Free*>(h);
    for (int i = 0; i < sp->n_edges; ++i) {
        uv[2 * i] = sp->edges[i].u;
        uv[2 * i + 1] = sp->edges[i].v;
        cost[i] = sp->original_edge_cost[i];
    }
}
}
