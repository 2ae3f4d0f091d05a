// The reference's legacy stage-2 round without rollback (simp_cuda/src/cusimp.cu, class cusimp::CUSimp), compiled
// for the host under the emulation in oracle/ref_emu like oracle/ref_round_emu.cpp, with the same kind of C
// interface for tests/golden/make_ref_round_golden.py. Test infrastructure only.
#include "emu_prelude.h"

#include "cusimp.cu"

extern "C" {

// like the pybind operator's constructor (simp_cuda/src/pybind.cpp:116-121): all buffers unallocated
void* ref_legacy_create() { return new cusimp::CUSimp(); }

void ref_legacy_destroy(void* h) { delete static_cast<cusimp::CUSimp*>(h); }

// one CUDSP.forward call (pybind.cpp:140-158): inputs are host arrays here
void ref_legacy_forward(void* h, const float* pts, const int* tris, int n_pts, int n_tris, float scale,
                        float threshold, int init) {
    auto* sp = static_cast<cusimp::CUSimp*>(h);
    sp->forward(reinterpret_cast<cusimp::Vertex<float>*>(const_cast<float*>(pts)),
                reinterpret_cast<cusimp::Triangle<int>*>(const_cast<int*>(tris)), n_pts, n_tris, scale, threshold,
                init != 0);
}

// n_pts, n_tris
void ref_legacy_counts(void* h, long long* out) {
    auto* sp = static_cast<cusimp::CUSimp*>(h);
    out[0] = sp->n_pts;
    out[1] = sp->n_tris;
}

// the four outputs the pybind operator clones (pybind.cpp:160-180)
void ref_legacy_outputs(void* h, float* verts, int* tris, int* occ, int* vmap) {
    auto* sp = static_cast<cusimp::CUSimp*>(h);
    std::memcpy(verts, sp->points, sizeof(float) * 3 * sp->n_pts);
    std::memcpy(tris, sp->triangles, sizeof(int) * 3 * sp->n_tris);
    std::memcpy(occ, sp->pts_occ, sizeof(int) * sp->n_pts);
    std::memcpy(vmap, sp->pts_map, sizeof(int) * sp->n_pts);
}
}
