// bench_peak.cu — integer-pipe peak for the roofline of bench.py (built into
// libftbench.so, separate from the product library).
//
// Measures 32x32->64-bit multiply-accumulate throughput (IMAD.WIDE: the
// operation the roofline's algorithmic unit counts, 64 per field
// multiplication): 8 independent accumulators per thread, each
// acc = lo32(acc) * m + acc, so no product can be strength-reduced away.
#include <cuda_runtime.h>
#include <stdint.h>

__global__ void __launch_bounds__(256) k_imad_wide(uint64_t *out, uint32_t seed, int iters)
{
    uint32_t m[8];
    uint64_t acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        m[k] = (seed + 2654435761u * (threadIdx.x + 8 * k)) | 1u;
        acc[k] = (uint64_t)(blockIdx.x + k) * 0x9e3779b97f4a7c15ull;
    }
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
#pragma unroll
            for (int k = 0; k < 8; ++k) acc[k] = (uint64_t)(uint32_t)acc[k] * m[k] + acc[k];
        }
    }
    uint64_t x = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) x ^= acc[k];
    if (x == 0x123456789abcdefull) out[blockIdx.x] = x; // keeps the work alive
}

extern "C" int ftb_imad_wide_peak(double *products_per_s, int sm_count)
{
    const int threads = 256, blocks = sm_count * 8, iters = 2048;
    uint64_t *out = nullptr;
    if (cudaMalloc(&out, sizeof(uint64_t) * blocks) != cudaSuccess) return 1;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_imad_wide<<<blocks, threads>>>(out, 7u, iters);
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(a);
        k_imad_wide<<<blocks, threads>>>(out, 11u + rep, iters);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return 2;
    *products_per_s = (double)blocks * threads * iters * 64.0 / (best * 1e-3);
    return 0;
}
