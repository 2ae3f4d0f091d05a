// Ring operations of a collapse round shared by the single-mesh and the batched kernels.
#pragma once
#include "pamo_common.cuh"

namespace pamo {

// collapse of (u, v) onto u in the faces of both rings (cusimp_free.cu:676-730, 245-273): faces holding both die,
// v becomes u in the others
__device__ __forceinline__ void rewire(int u, int v, const int* __restrict__ nt_off, const int* __restrict__ nt, int4* tri) {
    for (int s = nt_off[u]; s < nt_off[u + 1]; ++s) {
        const int f = nt[s];
        const int4 t = tri[f];
        if (t.x == v || t.y == v || t.z == v) tri[f] = make_int4(-1, -1, -1, 0);
    }
    for (int s = nt_off[v]; s < nt_off[v + 1]; ++s) {
        const int f = nt[s];
        int4 t = tri[f];
        if (t.x == u || t.y == u || t.z == u) t = make_int4(-1, -1, -1, 0);
        else if (t.x == v) t.x = u;
        else if (t.y == v) t.y = u;
        else if (t.z == v) t.z = u;
        tri[f] = t;
    }
}

// the faces of w's ring from the round's snapshot (cusimp_free.cu:849-866)
__device__ __forceinline__ void restore_ring(int w, const int* __restrict__ nt_off, const int* __restrict__ nt, int4* tri,
                                             const int4* __restrict__ orig_tri) {
    for (int s = nt_off[w]; s < nt_off[w + 1]; ++s) {
        const int f = nt[s];
        tri[f] = orig_tri[f];
    }
}

}  // namespace pamo
