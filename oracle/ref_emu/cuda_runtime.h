// Host emulation of the small part of the CUDA runtime that the reference's stage-2 round uses
// (simp_cuda/src/cusimp_free.cu, simp_cuda/src/bvh/*.cuh), so that its own kernels can be compiled by g++ and
// run on the CPU as the pin of the oracle. Test infrastructure only (oracle/_ref), never part of the product.
//
// Semantics:
//  * device memory is host memory; every allocation carries a zeroed 256-byte guard in front, so the
//    reference's read of the vertex before the array for removed faces (self_intersect.cuh:164-170) reads
//    zeros instead of leaving the allocation; fresh allocations are zeroed (the state a new process sees);
//  * a kernel launch runs its threads one after another in (block, thread) order: one of the interleavings a
//    GPU may produce. The reference's kernels use neither shared memory nor warp operations, so each thread
//    can run to completion before the next starts; atomics are then plain read-modify-writes;
//  * float -> uint32 conversions that the device performs with cvt.rzi.u32.f32 saturate (PTX ISA, cvt:
//    float-to-integer conversions clamp to the destination range, NaN gives 0); device_f2u32 does the same.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>

#include "vector_types.h"

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

typedef int cudaError_t;
enum : int { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice,
                      cudaMemcpyDefault };
typedef void* cudaStream_t;

namespace emu {
constexpr size_t kGuard = 256;

inline void* alloc(size_t n) {
    unsigned char* p = static_cast<unsigned char*>(std::calloc(1, n + kGuard));
    return p ? p + kGuard : nullptr;
}
inline void release(void* p) {
    if (p) std::free(static_cast<unsigned char*>(p) - kGuard);
}

// cvt.rzi.u32.f32: round toward zero, clamp to [0, 2^32 - 1], NaN -> 0
inline uint32_t device_f2u32(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return static_cast<uint32_t>(x);
}

template <class T>
struct same {
    using type = T;
};
template <class T>
using same_t = typename same<T>::type;  // keeps the value operands of the atomics out of deduction, like CUDA's overloads

inline uint3 threadIdx_v, blockIdx_v;
inline dim3 blockDim_v, gridDim_v;

template <class F>
struct Launch {
    F fn;
    dim3 grid, block;
    Launch(F f, dim3 g, dim3 b) : fn(f), grid(g), block(b) {}
    template <class... A>
    void operator()(A&&... a) const {
        gridDim_v = grid;
        blockDim_v = block;
        for (unsigned bz = 0; bz < grid.z; ++bz)
            for (unsigned by = 0; by < grid.y; ++by)
                for (unsigned bx = 0; bx < grid.x; ++bx)
                    for (unsigned tz = 0; tz < block.z; ++tz)
                        for (unsigned ty = 0; ty < block.y; ++ty)
                            for (unsigned tx = 0; tx < block.x; ++tx) {
                                blockIdx_v = uint3{bx, by, bz};
                                threadIdx_v = uint3{tx, ty, tz};
                                fn(a...);
                            }
    }
};
}  // namespace emu

#define threadIdx (::emu::threadIdx_v)
#define blockIdx (::emu::blockIdx_v)
#define blockDim (::emu::blockDim_v)
#define gridDim (::emu::gridDim_v)
// the launch syntax K<<<G, B>>>(args) is rewritten by oracle/build_ref.py into EMU_LAUNCH(K, G, B)(args); the
// generic lambda lets template kernels deduce their arguments as a launch does
#define EMU_LAUNCH(K, G, B) ::emu::Launch([](auto&... emu_a) { K(emu_a...); }, ::dim3(G), ::dim3(B))

inline cudaError_t cudaMalloc(void** p, size_t n) {
    *p = emu::alloc(n);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t n) {
    return cudaMalloc(reinterpret_cast<void**>(p), n);
}
inline cudaError_t cudaFree(void* p) {
    emu::release(p);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind) {
    if (n) std::memmove(dst, src, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemset(void* p, int v, size_t n) {
    if (n) std::memset(p, v, n);
    return cudaSuccess;
}
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaPeekAtLastError() { return cudaSuccess; }
inline const char* cudaGetErrorString(cudaError_t) { return "no error (host emulation)"; }

template <class T>
inline T atomicAdd(T* a, emu::same_t<T> v) {
    T o = *a;
    *a = o + v;
    return o;
}
template <class T>
inline T atomicMin(T* a, emu::same_t<T> v) {
    T o = *a;
    if (v < o) *a = v;
    return o;
}
template <class T>
inline T atomicMax(T* a, emu::same_t<T> v) {
    T o = *a;
    if (v > o) *a = v;
    return o;
}
template <class T>
inline T atomicExch(T* a, emu::same_t<T> v) {
    T o = *a;
    *a = v;
    return o;
}
template <class T>
inline T atomicCAS(T* a, emu::same_t<T> cmp, emu::same_t<T> v) {
    T o = *a;
    if (o == cmp) *a = v;
    return o;
}

inline int __clz(int x) { return x == 0 ? 32 : __builtin_clz(static_cast<unsigned>(x)); }
inline int __clzll(long long x) { return x == 0 ? 64 : __builtin_clzll(static_cast<unsigned long long>(x)); }

// device overloads the reference's code relies on: min/max of floats are fminf/fmaxf, and pow(float, int)
// stays in float (only squares occur: cusimp_free.cu:533,573, cusimp.cu:423,463). The device's pow(x, 2) is not
// restated here: the square is taken by multiplication, which on the GPU differs from the device function by one
// ulp for a few floats in a million (tests/test_gpu_device_pins.py measures it, and finds the CUDA path's rounds the
// same with the device function as with the multiplication)
inline float min(float a, float b) { return fminf(a, b); }
inline float max(float a, float b) { return fmaxf(a, b); }
inline double min(double a, double b) { return fmin(a, b); }
inline double max(double a, double b) { return fmax(a, b); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
inline long long min(long long a, long long b) { return a < b ? a : b; }
inline long long max(long long a, long long b) { return a > b ? a : b; }
inline unsigned long long min(unsigned long long a, unsigned long long b) { return a < b ? a : b; }
inline unsigned long long max(unsigned long long a, unsigned long long b) { return a > b ? a : b; }
inline float pow(float x, int n) {
    if (n != 2) {
        std::fprintf(stderr, "host emulation: pow(float, %d) is not emulated\n", n);
        std::abort();
    }
    return x * x;
}
