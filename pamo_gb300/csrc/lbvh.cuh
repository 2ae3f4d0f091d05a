// Morton-code LBVH over the live faces and the localized self-intersection query of one collapse round.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>
#include "pamo_common.cuh"

namespace pamo {

struct BvhBuffers {
    int cap = 0;                       // face capacity
    float4* box_lo = nullptr;          // per face AABB (by face id)
    float4* box_hi = nullptr;
    int* live_scan = nullptr;          // exclusive scan of live flags [cap + 1]
    unsigned* keys[2] = {nullptr, nullptr};  // Morton codes, sort ping-pong
    int* vals[2] = {nullptr, nullptr};       // face ids, sort ping-pong
    int* hist = nullptr;               // radix histograms [256 * kSortTiles + 1]
    int2* child = nullptr;             // internal node children; v < 0 encodes leaf ~v
    int2* range = nullptr;             // internal node leaf range [lo, hi] (the node index is one end)
    int* iparent = nullptr;            // parent of internal node
    int* lparent = nullptr;            // parent of leaf
    float4* nlo = nullptr;             // internal node boxes
    float4* nhi = nullptr;
    float4* llo = nullptr;             // leaf boxes in sorted order
    float4* lhi = nullptr;
    int* visit = nullptr;              // bottom-up arrival counters
    int* upq = nullptr;                // [0] count, then the nodes above the tiles queued by the bottom-up pass
    int4* xq = nullptr;                // candidate pairs for the float64 pass (f, g, orders) and their count
    int* xq_count = nullptr;
    int xq_cap = 0;
    unsigned* scene = nullptr;         // scene bounds as order-preserving uints (6)
    // internal nodes packed for traversal, 64 B each: {lo_a, hi_a, lo_b, hi_b} with the boxes of both children;
    // lo.w = child reference (>= 0 internal node, < 0 leaf ~i), hi.w = the leaf's face id (or -1), as int bits
    float4* packed = nullptr;
    int* scan_scratch = nullptr;
    int* meta = nullptr;               // [0]: leaves of the current tree (kept across refits)
};

// Many meshes in one face numbering (faces of mesh m: [f0[m], f0[m] + nf[m]), meshes in face order): the tree keeps
// each mesh in its own subtree (its mesh index in the top `bits` key bits, 1 <= bits <= 16) and writes each mesh's
// subtree root to root[m] (-1 below two live faces); d_count meshes, at most count_bound.
struct BvhMeshes {
    const int* fmesh = nullptr;  // mesh of each face
    int bits = 0;
    const int* f0 = nullptr;
    const int* nf = nullptr;
    const int* d_count = nullptr;
    int count_bound = 0;
    int* root = nullptr;
};

size_t bvh_bytes(int cap);
// Lays the buffers out from base; clear_scan_scratch zeroes the tree's scan scratch (synchronous), which
// memory that is not zero-initialised needs before its first build.
void bvh_carve(BvhBuffers& b, int cap, char* base, bool clear_scan_scratch = true);

// Builds the LBVH over faces with tri[f].x != -1 (count from rc->n_tris); writes rc->n_live. With all_faces,
// every face slot below rc->n_tris is a leaf and a removed face has an empty box, so that the tree can be
// refitted after faces are removed or restored (bvh_refit_faces) and carried to the next round (bvh_remap).
// qscan (exclusive scan of the query flags, or null) marks the query faces in the packed leaves for bvh_query.
// nodes: also keep the internal node boxes nlo/nhi for every node (the traversals of the projection stage read
// them); the packed records that bvh_query reads are always written.
void bvh_build(BvhBuffers& b, const int4* tri, const float4* pos, RoundCounters* rc, int n_tris_bound, cudaStream_t s,
               bool all_faces = false, const int* qscan = nullptr, bool nodes = true,
               const BvhMeshes* meshes = nullptr);

// New boxes for the leaves of a tree built with all_faces (a removed face, or a leaf whose face is gone, gets an
// empty box that overlaps nothing); sets rc->n_live to the tree's leaf count. next_round: first take the leaf
// face ids bvh_remap computed for this round's numbering.
void bvh_refit_faces(BvhBuffers& b, const int4* tri, const float4* pos, RoundCounters* rc, int n_tris_bound,
                     cudaStream_t s, bool next_round, const int* qscan = nullptr);

// After a compaction with exclusive scan fscan of the kept faces: the leaves' face ids in the new numbering
// (-1 for faces not kept), kept aside until bvh_refit_faces(next_round = true); repeating it is harmless.
void bvh_remap(BvhBuffers& b, const int* fscan, int n_tris_bound, cudaStream_t s);

// Recomputes the leaf and node boxes of a tree built by bvh_build over the same faces after the positions
// moved (same topology and leaf order; the tree may bound more loosely than a rebuilt one). With `active`,
// the kernels do nothing unless *active != 0 (a device flag, so the call can sit in a captured graph).
void bvh_refit(BvhBuffers& b, const int4* tri, const float4* pos, RoundCounters* rc, int n_tris_bound, cudaStream_t s,
               const int* active = nullptr);

// For every face in the query list that is still live: hit[f] = 1 iff some live face g != f with an
// overlapping closed AABB makes the reference's pair test true in either order. Query faces are taken
// as the faces f with qscan[f + 1] != qscan[f] (qscan: exclusive scan of the query flags), visited in leaf
// order. The tree must have been built or refitted with the same qscan (face ids below 2^30). Candidate pairs
// go through pair_list (capacity pair_cap; queries beyond it decide their pairs in place).
// qlist is unused (kept for callers that hold one).
// With fmesh and mesh_root (from a bvh_build with BvhMeshes), each query walks only its own mesh's subtree, so
// pairs never join two meshes.
void bvh_query(const BvhBuffers& b, const int4* tri, const float4* pos, const int* qlist, const int* qscan,
               unsigned char* hit, int2* pair_list, int pair_cap, RoundCounters* rc, int n_query_bound, float eps,
               cudaStream_t s, const int* fmesh = nullptr, const int* mesh_root = nullptr);

}  // namespace pamo
