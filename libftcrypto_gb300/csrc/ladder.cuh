// ladder.cuh — the constant-time variable-base ladder kernels (ft_mul /
// ft_scale; k_ft_mul and k_ft_scale, ftcrypto.cu:966-994), templated on the
// block size NT.  Each thread builds its 8-entry cached table (1 KB) and
// scans it in full under masks for each digit.  Where the table lives sets
// how many threads an SM holds:
//   NT <= 256  k_smul_var: the whole table in shared memory laid out
//              [entry][16-byte word][thread], so every table access of a warp
//              is 512 contiguous bytes (conflict-free).  NT KB per block: one
//              block of 224 threads (7 warps) is the most an SM holds.
//   NT  > 256  k_smul_var_tm: entries 1P-4P in shared memory as above
//              (512 B per thread), entries 5P-8P in tensor memory (128
//              columns of the thread's TMEM lane), so 384 or 448 threads
//              (12 or 14 warps) fit an SM; the register file then bounds the
//              registers per thread (tm_max_regs: 168 or 128).
#pragma once
#include "points.cuh"
#include "ladder_tab.cuh"

namespace ft {

FT_DEV void load_scalar(uint32_t a[8], const uint4 *sc, size_t i)
{
    uint4 s0 = sc[2 * i], s1 = sc[2 * i + 1];
    a[0] = s0.x; a[1] = s0.y; a[2] = s0.z; a[3] = s0.w;
    a[4] = s1.x; a[5] = s1.y; a[6] = s1.z; a[7] = s1.w;
}



template <int NT>
constexpr size_t ladder_smem_bytes() { return (size_t)NT * (NT > 256 ? 4 : 8) * 8 * sizeof(uint4); }

template <int NT>
__global__ void __launch_bounds__(NT, 1) k_smul_var(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step)
{
    extern __shared__ uint4 smem[];
    size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
    if (i >= n) return;
    SmemTab<NT> tab{smem + threadIdx.x};
    ge_p3 P, h;
    ld_p3(P, p, s, i);
    uint32_t a[8];
    load_scalar(a, sc, i * (size_t)sc_step);
    smul_build_table(tab, P);
    smul_ladder(h, a, tab);
    st_p3(p, s, i, h);
}

// The TMEM kernel: its shared memory (NT x 512 B > 114 KB) admits one block
// per SM, so the 512-column allocation below never waits for another
// block's.  Threads past n run the ladder on the identity with a zero scalar
// and store nothing, so every warp executes the warp-wide TMEM instructions
// converged and every thread reaches the ladder's per-window barriers; no
// thread leaves before the final barrier and the free.
// Registers per thread the launch allows: the register file is four
// 16,384-register partitions, one per warp scheduler, and the block's warps
// are spread over them, so the busiest partition holds ceil(warps / 4) warps
// (NT = 384: 168 registers; NT = 448: 128).
template <int NT>
constexpr int tm_max_regs() { return 16384 / ((NT / 32 + 3) / 4) / 32 / 8 * 8; }

template <int NT>
__global__ void __maxnreg__(tm_max_regs<NT>()) k_smul_var_tm(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step)
{
    static_assert(NT % 32 == 0 && NT <= 512, "whole warps, at most 4 per lane quarter");
    static_assert(NT <= 512 && (size_t)NT * 512 > 116 * 1024, "one block per SM, 128 columns per warp");
    extern __shared__ uint4 smem[];
    __shared__ uint32_t s_taddr;
    const int warp = threadIdx.x >> 5;
    if (warp == 0) tmem_alloc(&s_taddr, 512u);
    tmem_sync_threads();
    const size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
    const bool live = i < n;
    HybridTab<NT> tab{smem + threadIdx.x, tmem_warp_addr(s_taddr, warp, 128u * (uint32_t)(warp >> 2))};
    ge_p3 P, h;
    uint32_t a[8];
    if (live) {
        ld_p3(P, p, s, i);
        load_scalar(a, sc, i * (size_t)sc_step);
    } else {
        ge_p3_0(P);
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = 0u;
    }
    __syncwarp();
    smul_build_table(tab, P);
    tmem_wait_st();
    smul_ladder(h, a, tab, true); // every thread runs the whole ladder
    if (live) st_p3(p, s, i, h);
    tmem_sync_threads();
    if (warp == 0) tmem_free(s_taddr, 512u);
}

template <int NT>
const void *ladder_fn()
{
    if constexpr (NT > 256) return (const void *)k_smul_var_tm<NT>;
    else return (const void *)k_smul_var<NT>;
}

template <int NT>
inline SmemAttr ladder_attr;

template <int NT>
cudaError_t launch_ladder(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step, cudaStream_t st)
{
    cudaError_t e = ensure_smem_attr(ladder_attr<NT>, ladder_fn<NT>(), ladder_smem_bytes<NT>());
    if (e != cudaSuccess) return e;
    unsigned grid = (unsigned)((n + NT - 1) / NT);
    if constexpr (NT > 256) k_smul_var_tm<NT><<<grid, NT, ladder_smem_bytes<NT>(), st>>>(p, s, n, sc, sc_step);
    else k_smul_var<NT><<<grid, NT, ladder_smem_bytes<NT>(), st>>>(p, s, n, sc, sc_step);
    return cudaGetLastError();
}

// points one wave of the launch holds: resident blocks per SM (from the
// occupancy calculator) x SMs x NT; 0 if the calculator fails
template <int NT>
size_t ladder_wave()
{
    static std::atomic<size_t> known{0};
    if (const size_t w = known.load(std::memory_order_relaxed)) return w;
    if (ensure_smem_attr(ladder_attr<NT>, ladder_fn<NT>(), ladder_smem_bytes<NT>()) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ladder_fn<NT>(), NT, ladder_smem_bytes<NT>()) !=
            cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return 0;
    }
    const size_t w = (size_t)per_sm * (size_t)sm_count() * NT;
    known.store(w, std::memory_order_relaxed);
    return w;
}

} // namespace ft
