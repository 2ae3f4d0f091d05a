// Compares on the GPU the device's pow(float, int) with exponent 2 (the call in the reference's skinny term,
// simp_cuda/src/cusimp_free.cu:533,573) with x * x, which the oracle uses in its place. Built with the reference's
// flags (--fmad=false). Tests 2^22 floats from a fixed LCG (half of them in the range of normalised edge lengths,
// half any finite float); prints the first few mismatches, then "<tested> <mismatches>".
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>

__global__ void k_pow2(const float* x, float* a, float* b, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float v = x[i];
        a[i] = pow(v, 2);
        b[i] = v * v;
    }
}

int main() {
    const int n = 1 << 22;
    std::vector<float> x(n);
    uint64_t s = 0x9E3779B97F4A7C15ull;
    for (int i = 0; i < n; ++i) {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        uint32_t bits = (uint32_t)(s >> 32);
        if (i % 2 == 0) {  // half in the range of edge lengths of normalised meshes, half any finite float
            float f = std::ldexp((float)(bits & 0xFFFFFF) / 16777216.0f + 0.5f, (int)((bits >> 24) % 48) - 40);
            x[i] = f;
        } else {
            bits &= 0xFF7FFFFFu;  // exponent never all ones: finite
            std::memcpy(&x[i], &bits, 4);
        }
    }
    float *dx, *da, *db;
    if (cudaMalloc(&dx, n * 4) || cudaMalloc(&da, n * 4) || cudaMalloc(&db, n * 4)) return 2;
    cudaMemcpy(dx, x.data(), n * 4, cudaMemcpyHostToDevice);
    k_pow2<<<1024, 256>>>(dx, da, db, n);
    if (cudaDeviceSynchronize() != cudaSuccess) return 3;
    std::vector<float> a(n), b(n);
    cudaMemcpy(a.data(), da, n * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(b.data(), db, n * 4, cudaMemcpyDeviceToHost);
    long bad = 0;
    for (int i = 0; i < n; ++i)
        if (std::memcmp(&a[i], &b[i], 4) != 0) {
            if (bad < 5) std::printf("# x=%a pow=%a mul=%a\n", x[i], a[i], b[i]);
            ++bad;
        }
    std::printf("%d %ld\n", n, bad);
    cudaFree(dx);
    cudaFree(da);
    cudaFree(db);
    return 0;
}
