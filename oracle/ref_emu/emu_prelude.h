// Prelude of the host-emulated reference round: the CUDA runtime stand-ins, Thrust on its CPP device system
// (the reference's own Thrust calls then run on the host with the same algorithms: shuffle, stable sort, scans,
// reductions), and cub::DeviceScan::ExclusiveSum as a sequential scan. __CUDACC__ is defined only after Thrust
// is in, because the reference's LBVH headers are guarded by it (bvh/bvh.cuh:4, bvh/aabb.cuh:3) while Thrust must
// configure itself for a host compiler. Test infrastructure only.
#pragma once
#include "cuda_runtime.h"

#include <bitset>
#include <fstream>
#include <iostream>
#include <math.h>
#include <string>
#include <vector>

#include <thrust/copy.h>
#include <thrust/device_ptr.h>
#include <thrust/device_vector.h>
#include <thrust/execution_policy.h>
#include <thrust/fill.h>
#include <thrust/for_each.h>
#include <thrust/functional.h>
#include <thrust/host_vector.h>
#include <thrust/iterator/constant_iterator.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/pair.h>
#include <thrust/random.h>
#include <thrust/reduce.h>
#include <thrust/scan.h>
#include <thrust/shuffle.h>
#include <thrust/sort.h>
#include <thrust/swap.h>
#include <thrust/transform.h>
#include <thrust/tuple.h>

namespace cub {
struct DeviceScan {
    // exclusive prefix sum of n items, in place allowed (cusimp_free.cu:954-956, 970-972, 1043-1045)
    template <class In, class Out>
    static cudaError_t ExclusiveSum(void* temp, size_t& temp_bytes, In in, Out out, int n, cudaStream_t = nullptr) {
        if (temp == nullptr) {
            temp_bytes = 16;
            return cudaSuccess;
        }
        using T = typename std::decay<decltype(in[0])>::type;
        T run = T(0);
        for (int i = 0; i < n; ++i) {
            T x = in[i];
            out[i] = run;
            run = run + x;
        }
        return cudaSuccess;
    }
};
}  // namespace cub

#define __CUDACC__ 1
