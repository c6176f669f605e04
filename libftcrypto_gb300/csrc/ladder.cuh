// ladder.cuh — the constant-time variable-base ladder kernel (ft_mul /
// ft_scale; k_ft_mul and k_ft_scale, ftcrypto.cu:966-994), templated on the
// block size NT.  Each thread keeps its 8-entry cached table (1 KB) in
// shared memory laid out [entry][16-byte word][thread], so every table access
// of a warp is 512 contiguous bytes (conflict-free); the table is scanned in
// full under masks for each digit.  Shared memory bounds the residency: NT
// threads need NT KB, so one block of 224 threads (7 warps) is the most an
// SM holds.
#pragma once
#include "points.cuh"
#include "smul.cuh"

namespace ft {

FT_DEV void load_scalar(uint32_t a[8], const uint4 *sc, size_t i)
{
    uint4 s0 = sc[2 * i], s1 = sc[2 * i + 1];
    a[0] = s0.x; a[1] = s0.y; a[2] = s0.z; a[3] = s0.w;
    a[4] = s1.x; a[5] = s1.y; a[6] = s1.z; a[7] = s1.w;
}

template <int NT>
struct SmemTab {
    uint4 *b; // &smem[threadIdx.x]
    FT_DEV void put(int k, const ge_cached &c) const
    {
        uint4 *q = b + (size_t)k * 8 * NT;
        q[0 * NT] = u4_lo(c.YplusX);
        q[1 * NT] = u4_hi(c.YplusX);
        q[2 * NT] = u4_lo(c.YminusX);
        q[3 * NT] = u4_hi(c.YminusX);
        q[4 * NT] = u4_lo(c.Z);
        q[5 * NT] = u4_hi(c.Z);
        q[6 * NT] = u4_lo(c.T2d);
        q[7 * NT] = u4_hi(c.T2d);
    }
    FT_DEV void get(int k, ge_cached &c) const
    {
        const uint4 *q = b + (size_t)k * 8 * NT;
        fe_from_u4(c.YplusX, q[0 * NT], q[1 * NT]);
        fe_from_u4(c.YminusX, q[2 * NT], q[3 * NT]);
        fe_from_u4(c.Z, q[4 * NT], q[5 * NT]);
        fe_from_u4(c.T2d, q[6 * NT], q[7 * NT]);
    }
};

template <int NT>
constexpr size_t ladder_smem_bytes() { return (size_t)NT * 8 * 8 * sizeof(uint4); }

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

template <int NT>
cudaError_t launch_ladder(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step, cudaStream_t st)
{
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_smul_var<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)ladder_smem_bytes<NT>());
        if (e != cudaSuccess) return e;
        attr = true;
    }
    unsigned grid = (unsigned)((n + NT - 1) / NT);
    k_smul_var<NT><<<grid, NT, ladder_smem_bytes<NT>(), st>>>(p, s, n, sc, sc_step);
    return cudaGetLastError();
}

} // namespace ft
