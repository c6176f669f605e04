// k_encrypt.cu — the fixed-base kernels, all by the radix-32 comb of
// enc_comb.cuh over tables staged in shared memory:
//
//   k_encrypt    ElGamal encryption (ftx_encrypt; the reference composes it
//                from ft_array_from_scalars, ft_array_init_point + ft_mul and
//                ft_array_from_small_scalars + ft_add) and re-randomisation:
//                c1 = r*B, c2 = m*B + r*PK (ACC: c1 += r*B, c2 += r*PK)
//   k_comb_base  a_i * B for 32-byte scalars or uint64 values
//                (ft_array_from_scalars, ft_array_from_small_scalars,
//                ft_array_init_scalar; the reference uses its variable-base
//                ladder here, ftcrypto.cu:895-913)
//   k_enc_table  the 52 x 16 table of a point (B at init, the public key
//                per key)
//
// One 512-thread block per SM (16 warps at 128 registers) stages the tables
// (78 KB each) in shared memory; all threads of a warp read the same row
// (broadcast).  Every row of r*B, r*PK and m*B runs through one loop body
// (one copy of the hot code in the instruction stream).  Against the
// reference's 4-bit two-pass comb (64 rows and 4 doublings per product) the
// radix-32 comb has 12% fewer instructions: encryption of 1,048,576
// plaintexts 15.4 -> 14.0 ms, and with the select reading four entries per
// loop iteration instead of one 12.0 ms.  Selecting the next row's entry
// ahead of this row's addition (independent work for the scheduler) needs
// 164 registers: 9.55 ms at 384 threads per block, 9.61 ms at 512 (spills),
// against 9.19 ms; 384 threads without it 9.47 ms.
#include "internal.h"
#include "points.cuh"
#include "enc_comb.cuh"

namespace ft {

static constexpr int ENC_NT = 512;
static constexpr size_t ENC_TABLE_U4 = ENC_TABLE_WORDS / 4; // uint4 words of one table
static constexpr int ENC_SMALL_ROWS = enc_digits(64);        // rows of a uint64 scalar

// dst[i] = h, or dst[i] += h with ACC
template <bool ACC>
FT_DEV void enc_put(uint4 *dst, size_t s, size_t i, const ge_p3 &h)
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

// the radix-32 digits (biased) of the 32-byte scalar r[i], as the reference
// effectively uses it (enc_ref_scalar)
FT_DEV void enc_r_digits(uint32_t c[9], const uint4 *r, size_t i)
{
    const uint4 s0 = r[2 * i], s1v = r[2 * i + 1];
    const uint32_t a[8] = {s0.x, s0.y, s0.z, s0.w, s1v.x, s1v.y, s1v.z, s1v.w};
    uint32_t ar[8];
    enc_ref_scalar(ar, a);
    enc_recode(c, ar, ENC_ROWS);
}

// the first mdig biased digits of a 64-bit value (m + its bias < 2^70)
FT_DEV void enc_m_digits(uint32_t c[9], uint64_t mv, int mdig)
{
    const uint32_t a[8] = {(uint32_t)mv, (uint32_t)(mv >> 32), 0u, 0u, 0u, 0u, 0u, 0u};
    enc_recode(c, a, mdig);
}

#ifndef FT_ENC_SPLIT
#define FT_ENC_SPLIT 1
#endif

// Work units: half 0 of ciphertext i is c1 = r*B (52 rows of B's table),
// half 1 is c2 = r*PK + m*B (52 rows of the key's table, then mdig rows of
// B's).  With `split` the 2n halves are spread over the grid as separate
// units (a thread takes units u, u + threads, ...): 2n units make the
// last wave of the grid-stride loop fuller than n whole ciphertexts, whose
// last wave kept about half the threads idle (1,048,576 ciphertexts over
// 152 x 512 threads: 13.47 per thread).  Without it (c1 and c2 the same
// array, so its two halves must run in order in one thread) a thread takes
// both halves of each of its ciphertexts.
template <bool ACC>
__global__ void __launch_bounds__(ENC_NT, 1) k_encrypt(uint4 *c1, size_t s1, uint4 *c2, size_t s2, size_t n,
                                                      const uint4 *r, const uint64_t *m, int mdig,
                                                      const uint4 *tables, int split)
{
    extern __shared__ uint4 smem[];
    for (size_t j = threadIdx.x; j < 2 * ENC_TABLE_U4; j += ENC_NT) smem[j] = tables[j];
    __syncthreads();
    const uint4 *tb = smem, *tp = smem + ENC_TABLE_U4;
    const size_t units = split ? 2 * n : n;
    FT_GRID_LOOP(u, units)
    {
        const size_t i = split && u >= n ? u - n : u;
        const int h0 = split && u >= n ? 1 : 0, h1 = split ? h0 : 1;
#pragma unroll 1
        for (int half = h0; half <= h1; ++half) {
            // the digits of r and m are recoded from global memory where
            // their rows start, rather than kept in 12 registers throughout
            // (128 registers with 32 bytes of spills before; 9.79 -> 9.77 ms)
            uint32_t c[9];
            enc_r_digits(c, r, i);
            ge_p3 h;
            ge_p3_0(h);
            const int nrows = half ? ENC_ROWS + mdig : ENC_ROWS;
#pragma unroll 1
            for (int t = 0; t < nrows; ++t) {
                if (t == ENC_ROWS) enc_m_digits(c, ACC ? 0 : m[i], mdig);
                const int row = t < ENC_ROWS ? t : t - ENC_ROWS;
                const uint4 *tab = (half && t < ENC_ROWS) ? tp : tb;
                enc_comb_row(h, c, tab + (size_t)row * ENC_ENTRIES * 6);
            }
            if (half) enc_put<ACC>(c2, s2, i, h);
            else enc_put<ACC>(c1, s1, i, h);
        }
    }
}

// p[i] = a_i * B: 32-byte scalars (sc_step 0: one scalar for all) in
// ENC_ROWS rows, or uint64 values (small) in enc_digits(64) rows
__global__ void __launch_bounds__(ENC_NT, 1) k_comb_base(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step,
                                                        const uint64_t *small, const uint4 *btab)
{
    extern __shared__ uint4 smem[];
    for (size_t j = threadIdx.x; j < ENC_TABLE_U4; j += ENC_NT) smem[j] = btab[j];
    __syncthreads();
    const int nrows = small ? ENC_SMALL_ROWS : ENC_ROWS;
    FT_GRID_LOOP(i, n)
    {
        uint32_t a[8], c[9];
        if (small) {
            const uint64_t v = small[i];
            a[0] = (uint32_t)v;
            a[1] = (uint32_t)(v >> 32);
#pragma unroll
            for (int k = 2; k < 8; ++k) a[k] = 0u;
        } else {
            const size_t j = i * (size_t)sc_step;
            const uint4 s0 = sc[2 * j], s1v = sc[2 * j + 1];
            a[0] = s0.x; a[1] = s0.y; a[2] = s0.z; a[3] = s0.w;
            a[4] = s1v.x; a[5] = s1v.y; a[6] = s1v.z; a[7] = s1v.w;
            uint32_t ar[8];
            enc_ref_scalar(ar, a);
#pragma unroll
            for (int k = 0; k < 8; ++k) a[k] = ar[k];
        }
        enc_recode(c, a, nrows);
        ge_p3 h;
        ge_p3_0(h);
#pragma unroll 1
        for (int row = 0; row < nrows; ++row) enc_comb_row(h, c, smem + (size_t)row * ENC_ENTRIES * 6);
        st_p3(p, s, i, h);
    }
}

// thread t < rows * 16 writes entry (t / 16, t % 16) = (t%16 + 1) * 32^(t/16) * Q
__global__ void __launch_bounds__(128) k_enc_table(uint4 *out, const uint4 *q, size_t qs)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ENC_ROWS * ENC_ENTRIES) return;
    ge_p3 Q;
    ld_p3(Q, q, qs, 0);
    enc_table_entry(out + (size_t)t * 6, Q, t / ENC_ENTRIES, t % ENC_ENTRIES);
}

cudaError_t build_enc_table(uint32_t *d_table, View q, cudaStream_t st)
{
    const unsigned grid = (ENC_ROWS * ENC_ENTRIES + 127) / 128;
    k_enc_table<<<grid, 128, 0, st>>>((uint4 *)d_table, q.p, q.s);
    return cudaGetLastError();
}

static SmemAttr g_enc_attr[2], g_comb_attr;

template <bool ACC>
static cudaError_t encrypt_launch(View c1, View c2, size_t n, const uint8_t *r, const uint64_t *m, int mdig,
                                  const uint32_t *tables, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    const size_t smem = 2 * ENC_TABLE_U4 * sizeof(uint4);
    cudaError_t e = ensure_smem_attr(g_enc_attr[ACC], (const void *)k_encrypt<ACC>, smem);
    if (e != cudaSuccess) return e;
    const int split = FT_ENC_SPLIT && c1.p != c2.p;
    const size_t units = split ? 2 * n : n;
    const size_t need = (units + ENC_NT - 1) / ENC_NT, cap = (size_t)sm_count();
    const unsigned grid = (unsigned)(need < cap ? need : cap);
    k_encrypt<ACC><<<grid, ENC_NT, smem, st>>>(c1.p, c1.s, c2.p, c2.s, n, (const uint4 *)r, m, mdig,
                                               (const uint4 *)tables, split);
    return cudaGetLastError();
}

size_t encrypt_pass() { return (size_t)sm_count() * ENC_NT / (FT_ENC_SPLIT ? 2 : 1); }

cudaError_t encrypt(View c1, View c2, size_t n, const uint8_t *r, const uint64_t *m, int mdig,
                    const uint32_t *tables, cudaStream_t st)
{
    return encrypt_launch<false>(c1, c2, n, r, m, mdig, tables, st);
}

cudaError_t rerandomise(View c1, View c2, size_t n, const uint8_t *r, const uint32_t *tables, cudaStream_t st)
{
    return encrypt_launch<true>(c1, c2, n, r, nullptr, 0, tables, st);
}

static cudaError_t comb_launch(View v, size_t n, const uint4 *sc, int sc_step, const uint64_t *small,
                               const uint32_t *btab, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    const size_t smem = ENC_TABLE_U4 * sizeof(uint4);
    cudaError_t e = ensure_smem_attr(g_comb_attr, (const void *)k_comb_base, smem);
    if (e != cudaSuccess) return e;
    const size_t need = (n + ENC_NT - 1) / ENC_NT, cap = (size_t)sm_count();
    const unsigned grid = (unsigned)(need < cap ? need : cap);
    k_comb_base<<<grid, ENC_NT, smem, st>>>(v.p, v.s, n, sc, sc_step, small, (const uint4 *)btab);
    return cudaGetLastError();
}

cudaError_t smul_base(View v, size_t n, const uint8_t *sc, int sc_step, const uint32_t *btab, cudaStream_t st)
{
    return comb_launch(v, n, (const uint4 *)sc, sc_step, nullptr, btab, st);
}

cudaError_t smul_base_small(View v, size_t n, const uint64_t *small, const uint32_t *btab, cudaStream_t st)
{
    return comb_launch(v, n, nullptr, 0, small, btab, st);
}

} // namespace ft
