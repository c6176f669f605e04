// k_smul.cu — scalar multiplication kernels.
//
//   smul_var     dispatch of the constant-time variable-base ladder
//                (ladder.cuh, one instantiation per block size in k_ladder.cu)
//   k_comb_base  a_i * B by the fixed-base comb over the 24 KB table of
//                (j+1)*256^i*B staged in shared memory (ft_array_from_scalars,
//                ft_array_from_small_scalars, ft_array_init_scalar).  The
//                reference uses the variable-base ladder here
//                (ftcrypto.cu:895-913); the points are the same.
//   k_encrypt    ElGamal c1 = r*B, c2 = m*B + r*PK with both combs in shared
//                memory and m*B folded into the PK comb's accumulator; with
//                ACC the products are added to c1, c2 in place
//                (re-randomisation: c + Enc(0; r)).
//   k_comb_table the 32 x 8 affine comb table of a public point (PK).
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

// dst[i] = h, or dst[i] += h with ACC
template <bool ACC>
FT_DEV void put_p3(uint4 *dst, size_t s, size_t i, const ge_p3 &h)
{
    if (ACC) {
        ge_p3 x;
        ld_p3(x, dst, s, i);
        ge_addto(x, h);
        st_p3(dst, s, i, x);
    } else {
        st_p3(dst, s, i, h);
    }
}

// four blocks per SM (128 registers, a few spills to L1) rather than three
// at 166 registers: 15.39 against 15.73 ms for 1,048,576 plaintexts
template <bool ACC>
__global__ void __launch_bounds__(128, 4) k_encrypt(uint4 *c1, size_t s1, uint4 *c2, size_t s2, size_t n, const uint4 *r,
                                                 const uint64_t *m, int mdig, const uint4 *pktab)
{
    extern __shared__ uint4 smem[];
    uint4 *tb = smem, *tp = smem + COMB_U4;
    for (int j = threadIdx.x; j < COMB_U4; j += blockDim.x) {
        tb[j] = ((const uint4 *)FT_BASE_COMB_INIT)[j];
        tp[j] = pktab[j];
    }
    __syncthreads();
    FT_GRID_LOOP(i, n)
    {
        uint32_t a[8], br[8], bm[8], mw[8];
        load_scalar(a, r, i);
        recode_bias(br, a);
        uint64_t mv = ACC ? 0 : m[i];
        mw[0] = (uint32_t)mv;
        mw[1] = (uint32_t)(mv >> 32);
#pragma unroll
        for (int k = 2; k < 8; ++k) mw[k] = 0;
        recode_bias(bm, mw);
        ge_p3 h;
        ge_p3_0(h);
        // c1 = r*B: pass 0 odd digits of r, 16*h, pass 1 even digits.
        // c2 = r*PK + m*B in one accumulator: pass 2 odd digits of r (PK
        // table), pass 3 odd digits of m (B table), 16*h, pass 4 even
        // digits of r (PK), pass 5 even digits of m (B).
#pragma unroll 1
        for (int pass = 0; pass < 6; ++pass) {
            const bool use_m = pass == 3 || pass == 5;
            const int parity = (pass == 0 || pass == 2 || pass == 3) ? 1 : 0;
            const uint4 *tab = (pass == 2 || pass == 4) ? tp : tb;
            const int nrows = use_m ? (parity ? mdig / 2 : (mdig + 1) / 2) : 32;
            uint32_t c[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) c[k] = use_m ? bm[k] : br[k];
#pragma unroll 1
            for (int row = 0; row < nrows; ++row)
                comb_row(h, c, parity, row, !use_m && 2 * row + parity == 63, tab);
            if (pass == 0 || pass == 3) ge_mul16(h);
            if (pass == 1) {
                put_p3<ACC>(c1, s1, i, h);
                ge_p3_0(h);
            }
        }
        put_p3<ACC>(c2, s2, i, h);
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

cudaError_t build_comb_table(uint32_t *d_table, View q, cudaStream_t st)
{
    k_comb_table<<<1, 256, 0, st>>>((uint4 *)d_table, q.p, q.s);
    return cudaGetLastError();
}

template <bool ACC>
static cudaError_t encrypt_launch(View c1, View c2, size_t n, const uint8_t *r, const uint64_t *m, int mdig,
                                  const uint32_t *pktab, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    size_t smem = 2 * COMB_U4 * sizeof(uint4);
    static SmemAttr attr;
    cudaError_t e = ensure_smem_attr(attr, (const void *)k_encrypt<ACC>, smem);
    if (e != cudaSuccess) return e;
    k_encrypt<ACC><<<comb_grid(n), 128, smem, st>>>(c1.p, c1.s, c2.p, c2.s, n, (const uint4 *)r, m, mdig,
                                                    (const uint4 *)pktab);
    return cudaGetLastError();
}

cudaError_t encrypt(View c1, View c2, size_t n, const uint8_t *r, const uint64_t *m, int mdig,
                    const uint32_t *pktab, cudaStream_t st)
{
    return encrypt_launch<false>(c1, c2, n, r, m, mdig, pktab, st);
}

// (c1, c2) += (r*B, r*PK)
cudaError_t rerandomise(View c1, View c2, size_t n, const uint8_t *r, const uint32_t *pktab, cudaStream_t st)
{
    return encrypt_launch<true>(c1, c2, n, r, nullptr, 0, pktab, st);
}

} // namespace ft
