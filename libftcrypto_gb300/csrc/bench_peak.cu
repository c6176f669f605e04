// bench_peak.cu — integer-pipe peaks for the roofline of bench.py (built into
// libftbench.so, separate from the product library).
//
// Three probes, each with independent dependency chains in every thread and
// enough warps per SM that no chain latency shows:
//   k_imad_wide   one PTX mad.wide.u32 per 32x32->64 product (a 64-bit
//                 accumulator): the single-instruction product rate;
//   k_imad_lo     one PTX mad.lo.u32 per 32-bit multiply-add: the integer
//                 multiply-add issue rate (a 64-bit product takes two of
//                 these, lo and hi);
//   k_fe_mul      field multiplications of the library's own fe_mul (8 x 8
//                 limbs, carry chains, fold by 38) on registers: the rate the
//                 arithmetic of every kernel here could reach if it did
//                 nothing but multiply.
// ftb_int_peaks reports each as 32x32->64 products per second (64 per field
// multiplication; mad.lo counted as half a product), best of `reps` launches.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fe.cuh"

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
            for (int k = 0; k < 8; ++k)
                asm("mad.wide.u32 %0, %1, %2, %0;" : "+l"(acc[k]) : "r"((uint32_t)acc[k]), "r"(m[k]));
        }
    }
    uint64_t x = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) x ^= acc[k];
    if (x == 0x123456789abcdefull) out[blockIdx.x] = x; // keeps the work alive
}

__global__ void __launch_bounds__(256) k_imad_lo(uint64_t *out, uint32_t seed, int iters)
{
    uint32_t m[8], acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        m[k] = (seed + 2654435761u * (threadIdx.x + 8 * k)) | 1u;
        acc[k] = (blockIdx.x + k) * 0x9e3779b9u;
    }
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
#pragma unroll
            for (int k = 0; k < 8; ++k) asm("mad.lo.u32 %0, %0, %1, %0;" : "+r"(acc[k]) : "r"(m[k]));
        }
    }
    uint32_t x = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) x ^= acc[k];
    if (x == 0x12345678u) out[blockIdx.x] = x;
}

// two independent chains of field multiplications per thread; 128 threads x
// 4 blocks per SM (the occupancy of the library's 128-register kernels)
__global__ void __launch_bounds__(128, 4) k_fe_mul(uint64_t *out, uint32_t seed, int iters)
{
    fe x, y, c, d;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        x.v[k] = seed * (threadIdx.x + 1) + 0x9e3779b9u * k;
        y.v[k] = seed ^ (blockIdx.x * 0x85ebca6bu + k);
        c.v[k] = 0x6a09e667u + 0x3c6ef372u * k;
        d.v[k] = 0xbb67ae85u ^ (0xa54ff53au * k);
    }
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
        fe_mul(x, x, c);
        fe_mul(y, y, d);
    }
    uint32_t z = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) z ^= x.v[k] ^ y.v[k];
    if (z == 0x12345678u) out[blockIdx.x] = z;
}

namespace {

template <class F>
float best_ms(F launch, int reps, cudaEvent_t a, cudaEvent_t b)
{
    launch(1u); // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < reps; ++rep) {
        cudaEventRecord(a);
        launch(11u + rep);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) best = ms;
    }
    return best;
}

} // namespace

// out[0]: mad.wide.u32 products/s; out[1]: mad.lo.u32 multiply-adds/s / 2
// (products/s at two instructions per product); out[2]: fe_mul products/s
// (64 per multiplication).
extern "C" int ftb_int_peaks(double *out, int sm_count, int reps)
{
    const int wide_blocks = sm_count * 8, wide_iters = 2048;
    const int mul_blocks = sm_count * 4, mul_iters = 2048;
    uint64_t *buf = nullptr;
    if (cudaMalloc(&buf, sizeof(uint64_t) * wide_blocks) != cudaSuccess) return 1;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float ms_wide = best_ms([&](uint32_t s) { k_imad_wide<<<wide_blocks, 256>>>(buf, s, wide_iters); }, reps, a, b);
    float ms_lo = best_ms([&](uint32_t s) { k_imad_lo<<<wide_blocks, 256>>>(buf, s, wide_iters); }, reps, a, b);
    float ms_mul = best_ms([&](uint32_t s) { k_fe_mul<<<mul_blocks, 128>>>(buf, s, mul_iters); }, reps, a, b);
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    if (e != cudaSuccess) return 2;
    const double ops_wide = (double)wide_blocks * 256 * wide_iters * 64;
    out[0] = ops_wide / (ms_wide * 1e-3);
    out[1] = ops_wide / (ms_lo * 1e-3) / 2.0;
    out[2] = (double)mul_blocks * 128 * mul_iters * 2 * 64 / (ms_mul * 1e-3);
    return 0;
}
