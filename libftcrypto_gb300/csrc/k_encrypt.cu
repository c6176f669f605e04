// k_encrypt.cu — ElGamal encryption (ftx_encrypt; the reference composes it
// from ft_array_from_scalars, ft_array_init_point + ft_mul and
// ft_array_from_small_scalars + ft_add) and re-randomisation.
//
//   c1 = r*B,  c2 = m*B + r*PK   (ACC: c1 += r*B, c2 += r*PK)
//
// Fixed-base products by a single-pass comb in signed radix 32: r is written
// as 52 digits d_i in [-16, 16) (r + sum_{i<52} 16 * 32^i, read five bits at
// a time, minus 16; exact for every 256-bit r), and
//   r*Q = sum_i d_i * (32^i * Q)
// is 52 mixed additions of a constant-time selected entry of row i of a
// table of (j+1) * 32^i * Q, j < 16 — no doublings.  The reference's comb
// (sodium_ge.cu:743-792; the 4-bit form kept in k_smul.cu for the other
// fixed-base calls) needs 64 additions and 4 doublings per product: 12% more
// instructions counted per ciphertext.  The points are the same; only the
// projective representation of the result differs, and encryption results
// are compared by their canonical encodings.
//
// The tables of B and of the public key (52 x 16 affine entries of 96 bytes:
// 78 KB each) are built on the device per key (k_enc_table) and staged in
// shared memory: one 512-thread block per SM (16 warps at 128 registers),
// all threads of a warp reading the same row (broadcast).  Every row of both
// products and of m*B runs through one loop body (one copy of the hot code
// in the instruction stream).
#include "internal.h"
#include "points.cuh"
#include "smul.cuh"

namespace ft {

static constexpr int ENC_NT = 512;
static constexpr size_t ENC_TABLE_U4 = ENC_TABLE_WORDS / 4; // uint4 words of one table

// word w of sum_{i<52} 16 * 32^i: bit 5i + 4 set for i < 52
__host__ __device__ constexpr uint32_t enc_bias_word(int w)
{
    uint32_t x = 0;
    for (int b = 0; b < 32; ++b) {
        const int bit = 32 * w + b;
        if (bit % 5 == 4 && bit <= 5 * 51 + 4) x |= 1u << b;
    }
    return x;
}

FT_DEV void shr5_288(uint32_t c[9])
{
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k] = (c[k] >> 5) | (c[k + 1] << 27);
    c[8] >>= 5;
}

// t = the entry |d| of a table row (16 entries), negated for d < 0; the
// identity for d = 0; every entry is read.  The select is spread over both
// integer pipes: with the logic pipe alone it saturated it (ALU 73% busy,
// FMA 32%) and the kernel ran 13.96 ms; split, 12.14 ms for 1,048,576
// plaintexts (measured).
FT_DEV void enc_select(ge_precomp &t, int d, const uint4 *row)
{
    const uint32_t bneg = (uint32_t)d >> 31;
    const uint32_t babs = (uint32_t)((d ^ -(int)bneg) + (int)bneg);
    // even entries masked and OR-ed (logic pipe), odd entries multiplied by
    // their 0/1 indicator and summed (multiply-add pipe): one entry at most
    // is selected, so the two partial results add up exactly
    ge_precomp a, b;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        a.yplusx.v[w] = a.yminusx.v[w] = a.xy2d.v[w] = 0u;
        b.yplusx.v[w] = b.yminusx.v[w] = b.xy2d.v[w] = 0u;
    }
    const uint32_t id = babs == 0u ? 1u : 0u; // the identity (1, 1, 0)
    a.yplusx.v[0] = id;
    a.yminusx.v[0] = id;
#pragma unroll 1
    for (int k = 0; k < ENC_ENTRIES; k += 2) {
        {
            const uint4 *q = row + 6 * k;
            const uint32_t m = ct_eq_mask(babs, (uint32_t)(k + 1));
            fe e0, e1, e2;
            fe_from_u4(e0, q[0], q[1]);
            fe_from_u4(e1, q[2], q[3]);
            fe_from_u4(e2, q[4], q[5]);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                a.yplusx.v[i] |= e0.v[i] & m;
                a.yminusx.v[i] |= e1.v[i] & m;
                a.xy2d.v[i] |= e2.v[i] & m;
            }
        }
        {
            const uint4 *q = row + 6 * (k + 1);
            const uint32_t ind = ct_eq_mask(babs, (uint32_t)(k + 2)) & 1u;
            fe e0, e1, e2;
            fe_from_u4(e0, q[0], q[1]);
            fe_from_u4(e1, q[2], q[3]);
            fe_from_u4(e2, q[4], q[5]);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                b.yplusx.v[i] = imad_u32(e0.v[i], ind, b.yplusx.v[i]);
                b.yminusx.v[i] = imad_u32(e1.v[i], ind, b.yminusx.v[i]);
                b.xy2d.v[i] = imad_u32(e2.v[i], ind, b.xy2d.v[i]);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        t.yplusx.v[i] = imad_u32(b.yplusx.v[i], 1u, a.yplusx.v[i]);
        t.yminusx.v[i] = imad_u32(b.yminusx.v[i], 1u, a.yminusx.v[i]);
        t.xy2d.v[i] = imad_u32(b.xy2d.v[i], 1u, a.xy2d.v[i]);
    }
    const uint32_t nm = 0u - bneg;
    fe nt;
    fe_neg(nt, t.xy2d);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t sw = (t.yplusx.v[k] ^ t.yminusx.v[k]) & nm;
        t.yplusx.v[k] ^= sw;
        t.yminusx.v[k] ^= sw;
    }
    fe_cmov(t.xy2d, nt, nm);
}

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

template <bool ACC>
__global__ void __launch_bounds__(ENC_NT, 1) k_encrypt(uint4 *c1, size_t s1, uint4 *c2, size_t s2, size_t n,
                                                      const uint4 *r, const uint64_t *m, int mdig,
                                                      const uint4 *tables)
{
    extern __shared__ uint4 smem[];
    for (size_t j = threadIdx.x; j < 2 * ENC_TABLE_U4; j += ENC_NT) smem[j] = tables[j];
    __syncthreads();
    const uint4 *tb = smem, *tp = smem + ENC_TABLE_U4;
    FT_GRID_LOOP(i, n)
    {
        // r + bias as 9 words (260 bits), m + bias over its mdig digits
        uint32_t br[9], bm[3], c[9];
        {
            const uint4 s0 = r[2 * i], s1v = r[2 * i + 1];
            const uint32_t a[8] = {s0.x, s0.y, s0.z, s0.w, s1v.x, s1v.y, s1v.z, s1v.w};
            br[0] = add_cc(a[0], enc_bias_word(0));
#pragma unroll
            for (int k = 1; k < 8; ++k) br[k] = addc_cc(a[k], enc_bias_word(k));
            br[8] = addc(0u, enc_bias_word(8));
        }
        {
            const uint64_t mv = ACC ? 0 : m[i];
            const int mbits = 5 * mdig; // the bias of the first mdig digits
            uint32_t bias[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int lo = 32 * k;
                const uint32_t keep = mbits >= lo + 32 ? ~0u : (mbits <= lo ? 0u : (1u << (mbits - lo)) - 1u);
                bias[k] = enc_bias_word(k) & keep;
            }
            bm[0] = add_cc((uint32_t)mv, bias[0]);
            bm[1] = addc_cc((uint32_t)(mv >> 32), bias[1]);
            bm[2] = addc(0u, bias[2]);
        }
        ge_p3 h;
        ge_p3_0(h);
        // rows 0..51: r*B; 52..103: r*PK; 104..: m*B, all through one body
        const int nrows = 2 * ENC_ROWS + mdig;
#pragma unroll
        for (int k = 0; k < 9; ++k) c[k] = br[k];
#pragma unroll 1
        for (int t = 0; t < nrows; ++t) {
            if (t == ENC_ROWS) {
                enc_put<ACC>(c1, s1, i, h);
                ge_p3_0(h);
#pragma unroll
                for (int k = 0; k < 9; ++k) c[k] = br[k];
            } else if (t == 2 * ENC_ROWS) {
                c[0] = bm[0];
                c[1] = bm[1];
                c[2] = bm[2];
#pragma unroll
                for (int k = 3; k < 9; ++k) c[k] = 0u;
            }
            const int row = t < ENC_ROWS ? t : (t < 2 * ENC_ROWS ? t - ENC_ROWS : t - 2 * ENC_ROWS);
            const uint4 *tab = (t >= ENC_ROWS && t < 2 * ENC_ROWS) ? tp : tb;
            const int d = (int)(c[0] & 31u) - 16;
            shr5_288(c);
            ge_precomp sel;
            enc_select(sel, d, tab + (size_t)row * ENC_ENTRIES * 6);
            ge_p1p1 q;
            ge_madd(q, h, sel);
            ge_p1p1_to_p3(h, q);
        }
        enc_put<ACC>(c2, s2, i, h);
    }
}

// thread t < rows * 16 writes entry (t / 16, t % 16) = (t%16 + 1) * 32^(t/16) * Q
// as (y + x, y - x, 2d x y), canonical
__global__ void __launch_bounds__(128) k_enc_table(uint4 *out, const uint4 *q, size_t qs)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ENC_ROWS * ENC_ENTRIES) return;
    const int row = t / ENC_ENTRIES, j = t % ENC_ENTRIES;
    ge_p3 R;
    ld_p3(R, q, qs, 0);
#pragma unroll 1
    for (int k = 0; k < 5 * row; ++k) {
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
    uint4 *o = out + (size_t)t * 6;
    o[0] = u4_lo(yp);
    o[1] = u4_hi(yp);
    o[2] = u4_lo(ym);
    o[3] = u4_hi(ym);
    o[4] = u4_lo(t2);
    o[5] = u4_hi(t2);
}

cudaError_t build_enc_tables(uint32_t *d_tables, View b, View pk, cudaStream_t st)
{
    const unsigned grid = (ENC_ROWS * ENC_ENTRIES + 127) / 128;
    k_enc_table<<<grid, 128, 0, st>>>((uint4 *)d_tables, b.p, b.s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_enc_table<<<grid, 128, 0, st>>>((uint4 *)d_tables + ENC_TABLE_U4, pk.p, pk.s);
    return cudaGetLastError();
}

int enc_m_digits(unsigned bits)
{
    // smallest d with 32^d - sum_{i<d} 16 * 32^i >= 2^bits (bits <= 64)
    for (int d = 1; d <= 14; ++d) {
        unsigned __int128 top = (unsigned __int128)1 << (5 * d), bias = 0;
        for (int i = 0; i < d; ++i) bias += (unsigned __int128)16 << (5 * i);
        if (top - bias >= ((unsigned __int128)1 << bits)) return d;
    }
    return 14;
}

static SmemAttr g_enc_attr[2];

template <bool ACC>
static cudaError_t encrypt_launch(View c1, View c2, size_t n, const uint8_t *r, const uint64_t *m, int mdig,
                                  const uint32_t *tables, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    const size_t smem = 2 * ENC_TABLE_U4 * sizeof(uint4);
    cudaError_t e = ensure_smem_attr(g_enc_attr[ACC], (const void *)k_encrypt<ACC>, smem);
    if (e != cudaSuccess) return e;
    const size_t need = (n + ENC_NT - 1) / ENC_NT, cap = (size_t)sm_count();
    const unsigned grid = (unsigned)(need < cap ? need : cap);
    k_encrypt<ACC><<<grid, ENC_NT, smem, st>>>(c1.p, c1.s, c2.p, c2.s, n, (const uint4 *)r, m, mdig,
                                               (const uint4 *)tables);
    return cudaGetLastError();
}

cudaError_t encrypt(View c1, View c2, size_t n, const uint8_t *r, const uint64_t *m, int mdig,
                    const uint32_t *tables, cudaStream_t st)
{
    return encrypt_launch<false>(c1, c2, n, r, m, mdig, tables, st);
}

cudaError_t rerandomise(View c1, View c2, size_t n, const uint8_t *r, const uint32_t *tables, cudaStream_t st)
{
    return encrypt_launch<true>(c1, c2, n, r, nullptr, 0, tables, st);
}

} // namespace ft
