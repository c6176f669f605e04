// k_smul.cu — scalar multiplication kernels.
//
//   k_smul_var   constant-time variable-base a_i * P_i (ft_mul / ft_scale;
//                k_ft_mul and k_ft_scale, ftcrypto.cu:966-994).  Each thread
//                keeps its 8-entry cached table (1 KB) in shared memory laid
//                out [entry][16-byte word][thread] so every table access of a
//                warp is 512 contiguous bytes (conflict-free); the table is
//                scanned in full under masks for each digit.
//   k_comb_base  a_i * B by the fixed-base comb over the 24 KB table of
//                (j+1)*256^i*B staged in shared memory (ft_array_from_scalars,
//                ft_array_from_small_scalars, ft_array_init_scalar).  The
//                reference uses the variable-base ladder here
//                (ftcrypto.cu:895-913); the points are the same.
//   k_encrypt    ElGamal c1 = r*B, c2 = m*B + r*PK with both combs in shared
//                memory and m*B folded into the PK comb's accumulator.
//   k_comb_table the 32 x 8 affine comb table of a public point (PK).
#include "internal.h"
#include "points.cuh"
#include "smul.cuh"

#define FT_TABLE_QUAL static __device__ __align__(16) const
#define FT_WANT_BASE_COMB
#include "base_table.inc"

namespace ft {

#define COMB_U4 (32 * 8 * 6) // uint4 words in one comb table (24 KB)

// per-thread cached table in shared memory
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

FT_DEV void load_scalar(uint32_t a[8], const uint4 *sc, size_t i)
{
    uint4 s0 = sc[2 * i], s1 = sc[2 * i + 1];
    a[0] = s0.x; a[1] = s0.y; a[2] = s0.z; a[3] = s0.w;
    a[4] = s1.x; a[5] = s1.y; a[6] = s1.z; a[7] = s1.w;
}

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

// comb table entry (row, k) of a table of COMB_U4 uint4 in shared memory
FT_DEV void comb_get(const uint4 *t, int row, int k, ge_precomp &e)
{
    const uint4 *q = t + (row * 8 + k) * 6;
    fe_from_u4(e.yplusx, q[0], q[1]);
    fe_from_u4(e.yminusx, q[2], q[3]);
    fe_from_u4(e.xy2d, q[4], q[5]);
}

FT_DEV void stage_table(uint4 *dst, const uint4 *src)
{
    for (int j = threadIdx.x; j < COMB_U4; j += blockDim.x) dst[j] = src[j];
    __syncthreads();
}

// mode 0: 32-byte scalars (sc_step 0 = one scalar for all); mode 1: uint64
__global__ void __launch_bounds__(128) k_comb_base(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step,
                                                   const uint64_t *small)
{
    __shared__ uint4 tb[COMB_U4];
    stage_table(tb, (const uint4 *)FT_BASE_COMB_INIT);
    auto get = [&](int row, int k, ge_precomp &e) { comb_get(tb, row, k, e); };
    FT_GRID_LOOP(i, n)
    {
        uint32_t a[8];
        int nd = 64;
        if (small) {
            uint64_t m = small[i];
            a[0] = (uint32_t)m;
            a[1] = (uint32_t)(m >> 32);
#pragma unroll
            for (int k = 2; k < 8; ++k) a[k] = 0;
            nd = 17; // 16 nibbles and the recoding carry
        } else {
            load_scalar(a, sc, i * (size_t)sc_step);
        }
        ge_p3 h;
        comb_mul(h, a, nd, get);
        st_p3(p, s, i, h);
    }
}

__global__ void __launch_bounds__(128) k_encrypt(uint4 *c1, size_t s1, uint4 *c2, size_t s2, size_t n, const uint4 *r,
                                                 const uint64_t *m, int mdig, const uint4 *pktab)
{
    extern __shared__ uint4 smem[];
    uint4 *tb = smem, *tp = smem + COMB_U4;
    for (int j = threadIdx.x; j < COMB_U4; j += blockDim.x) {
        tb[j] = ((const uint4 *)FT_BASE_COMB_INIT)[j];
        tp[j] = pktab[j];
    }
    __syncthreads();
    auto getb = [&](int row, int k, ge_precomp &e) { comb_get(tb, row, k, e); };
    auto getp = [&](int row, int k, ge_precomp &e) { comb_get(tp, row, k, e); };
    FT_GRID_LOOP(i, n)
    {
        uint32_t a[8], br[8], bm[8], mw[8];
        load_scalar(a, r, i);
        recode_bias(br, a);
        uint64_t mv = m[i];
        mw[0] = (uint32_t)mv;
        mw[1] = (uint32_t)(mv >> 32);
#pragma unroll
        for (int k = 2; k < 8; ++k) mw[k] = 0;
        recode_bias(bm, mw);
        ge_p3 h;
        // c1 = r * B
        ge_p3_0(h);
        comb_accumulate(h, br, 1, 32, getb);
        ge_mul16(h);
        comb_accumulate(h, br, 0, 32, getb);
        st_p3(c1, s1, i, h);
        // c2 = r * PK + m * B in one accumulator
        ge_p3_0(h);
        comb_accumulate(h, br, 1, 32, getp);
        comb_accumulate(h, bm, 1, mdig / 2, getb);
        ge_mul16(h);
        comb_accumulate(h, br, 0, 32, getp);
        comb_accumulate(h, bm, 0, (mdig + 1) / 2, getb);
        st_p3(c2, s2, i, h);
    }
}

// thread t < 256 writes entry (t / 8, t % 8) = (t%8 + 1) * 256^(t/8) * Q
__global__ void __launch_bounds__(256) k_comb_table(uint4 *out, const uint4 *q, size_t qs)
{
    int t = threadIdx.x;
    int row = t / 8, j = t % 8;
    ge_p3 R;
    ld_p3(R, q, qs, 0);
#pragma unroll 1
    for (int k = 0; k < 8 * row; ++k) {
        ge_p1p1 r;
        ge_p3_dbl(r, R);
        ge_p1p1_to_p3(R, r);
    }
    ge_p3 acc = R;
    ge_cached c;
    ge_p3_to_cached(c, R);
#pragma unroll 1
    for (int k = 0; k < j; ++k) {
        ge_p1p1 r;
        ge_add(r, acc, c);
        ge_p1p1_to_p3(acc, r);
    }
    fe zi, x, y, xy, yp, ym, t2;
    fe_invert(zi, acc.Z);
    fe_mul(x, acc.X, zi);
    fe_mul(y, acc.Y, zi);
    fe_add(yp, y, x);
    fe_sub(ym, y, x);
    fe_mul(xy, x, y);
    fe_mul(t2, xy, fe_d2());
    fe_canon(yp, yp);
    fe_canon(ym, ym);
    fe_canon(t2, t2);
    uint4 *o = out + t * 6;
    o[0] = u4_lo(yp);
    o[1] = u4_hi(yp);
    o[2] = u4_lo(ym);
    o[3] = u4_hi(ym);
    o[4] = u4_lo(t2);
    o[5] = u4_hi(t2);
}

// ------------------------------------------------------------ launchers

static const int SMUL_NT = 128;
static const size_t SMUL_SMEM = (size_t)SMUL_NT * 8 * 8 * sizeof(uint4);

int smul_var_block() { return SMUL_NT; }

cudaError_t smul_var(View v, size_t n, const uint8_t *sc, int sc_step, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_smul_var<SMUL_NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMUL_SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    unsigned grid = (unsigned)((n + SMUL_NT - 1) / SMUL_NT);
    k_smul_var<SMUL_NT><<<grid, SMUL_NT, SMUL_SMEM, st>>>(v.p, v.s, n, (const uint4 *)sc, sc_step);
    return cudaGetLastError();
}

static unsigned comb_grid(size_t n)
{
    size_t need = (n + 127) / 128;
    size_t cap = (size_t)sm_count() * 16;
    return (unsigned)(need < cap ? (need ? need : 1) : cap);
}

cudaError_t smul_base(View v, size_t n, const uint8_t *sc, int sc_step, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    k_comb_base<<<comb_grid(n), 128, 0, st>>>(v.p, v.s, n, (const uint4 *)sc, sc_step, nullptr);
    return cudaGetLastError();
}

cudaError_t smul_base_small(View v, size_t n, const uint64_t *small, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    k_comb_base<<<comb_grid(n), 128, 0, st>>>(v.p, v.s, n, nullptr, 0, small);
    return cudaGetLastError();
}

cudaError_t build_comb_table(uint32_t *d_table, View q, cudaStream_t st)
{
    k_comb_table<<<1, 256, 0, st>>>((uint4 *)d_table, q.p, q.s);
    return cudaGetLastError();
}

cudaError_t encrypt(View c1, View c2, size_t n, const uint8_t *r, const uint64_t *m, int mdig,
                    const uint32_t *pktab, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    size_t smem = 2 * COMB_U4 * sizeof(uint4);
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_encrypt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    k_encrypt<<<comb_grid(n), 128, smem, st>>>(c1.p, c1.s, c2.p, c2.s, n, (const uint4 *)r, m, mdig,
                                               (const uint4 *)pktab);
    return cudaGetLastError();
}

} // namespace ft
