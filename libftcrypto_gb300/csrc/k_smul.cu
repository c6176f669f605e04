// k_smul.cu — scalar multiplication kernels.
//
//   smul_var     dispatch of the constant-time variable-base ladder
//                (ladder.cuh, one instantiation per block size in k_ladder.cu)
//   k_comb_base  a_i * B by the fixed-base comb over the 24 KB table of
//                (j+1)*256^i*B staged in shared memory (ft_array_from_scalars,
//                ft_array_from_small_scalars, ft_array_init_scalar).  The
//                reference uses the variable-base ladder here
//                (ftcrypto.cu:895-913); the points are the same.
#include "internal.h"
#include "points.cuh"
#include "smul.cuh"
#include "ladder.cuh"

#define FT_TABLE_QUAL static __device__ __align__(16) const
#define FT_WANT_BASE_COMB
#include "base_table.inc"

namespace ft {

#define COMB_U4 (32 * 8 * 6) // uint4 words in one comb table (24 KB)

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

// One comb row: h += digit * table[row] with the digit taken from the low
// byte of c (nibble `parity`) and c shifted down by one byte.  The kernels
// below run all of their rows through one loop so this body, the hot code,
// exists once in the instruction stream (separate inlined passes made the
// encrypt kernel stall on instruction fetch).
FT_DEV void comb_row(ge_p3 &h, uint32_t c[8], int parity, int row, bool top, const uint4 *tab)
{
    int d = (int)((c[0] >> (4 * parity)) & 15u) - (top ? 0 : 8);
    shr8_256(c);
    ge_precomp t;
    select_precomp(t, d, [&](int k, ge_precomp &e) { comb_get(tab, row, k, e); });
    ge_p1p1 r;
    ge_madd(r, h, t);
    ge_p1p1_to_p3(h, r);
}

// mode 0: 32-byte scalars (sc_step 0 = one scalar for all); mode 1: uint64
__global__ void __launch_bounds__(128) k_comb_base(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step,
                                                   const uint64_t *small)
{
    __shared__ uint4 tb[COMB_U4];
    stage_table(tb, (const uint4 *)FT_BASE_COMB_INIT);
    FT_GRID_LOOP(i, n)
    {
        uint32_t a[8], b[8];
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
        recode_bias(b, a);
        ge_p3 h;
        ge_p3_0(h);
        // pass 0: odd digits, then 16*h; pass 1: even digits (sodium_ge.cu:772-791)
#pragma unroll 1
        for (int pass = 0; pass < 2; ++pass) {
            const int parity = 1 - pass;
            const int nrows = parity ? nd / 2 : (nd + 1) / 2;
            uint32_t c[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) c[k] = b[k];
#pragma unroll 1
            for (int row = 0; row < nrows; ++row) comb_row(h, c, parity, row, 2 * row + parity == 63, tb);
            if (pass == 0) ge_mul16(h);
        }
        st_p3(p, s, i, h);
    }
}

// ------------------------------------------------------------ launchers

static int g_ladder_nt = 384; // tables half in TMEM: the fastest on GB300

int ladder_block() { return g_ladder_nt; }

int set_ladder_block(int nt)
{
    if (nt != 128 && nt != 192 && nt != 224 && nt != 384 && nt != 448) return -1;
    g_ladder_nt = nt;
    return 0;
}

cudaError_t smul_var(View v, size_t n, const uint8_t *sc, int sc_step, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    const uint4 *s4 = (const uint4 *)sc;
    switch (g_ladder_nt) {
    case 128: return ladder_launch_128(v.p, v.s, n, s4, sc_step, st);
    case 192: return ladder_launch_192(v.p, v.s, n, s4, sc_step, st);
    case 384: return ladder_launch_384(v.p, v.s, n, s4, sc_step, st);
    case 448: return ladder_launch_448(v.p, v.s, n, s4, sc_step, st);
    case 224: return ladder_launch_224(v.p, v.s, n, s4, sc_step, st);
    default: return ladder_launch_384(v.p, v.s, n, s4, sc_step, st);
    }
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

} // namespace ft
