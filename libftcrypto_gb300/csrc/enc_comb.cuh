// enc_comb.cuh — the fixed-base comb in signed radix 32 (every fixed-base
// product of the library: encryption, ft_array_from_scalars,
// ft_array_from_small_scalars, ft_array_init_scalar).
//
// A scalar a < 2^256 is written as ENC_ROWS = 52 digits d_i in [-16, 16):
// b = a + sum_{i<52} 16 * 32^i (below 2^260), d_i = bits [5i, 5i+5) of b
// minus 16.  Then
//   a*Q = sum_i d_i * (32^i * Q),
// 52 mixed additions of a constant-time selected entry of row i of a table
// of (j+1) * 32^i * Q, j < 16, with no doublings; a public bound a < 2^bits
// takes fewer rows (enc_digits in windows.h).  The reference's comb
// (ge25519_scalarmult_base, sodium_ge.cu:743-792) is 64 additions and 4
// doublings in signed radix 16; both give the same group element (for
// scalars the reference's recoding truncates, enc_ref_scalar supplies the
// scalar it effectively uses), only the projective representation differs.
//
// Table layout: entry (row, j) is 6 uint4 (yplusx, yminusx, xy2d: affine,
// canonical), row-major, ENC_ENTRIES entries a row.  This header holds no
// kernel, so the host test harness compiles it over emulated primitives.
#pragma once
#include "ge.cuh"
#include "u4.cuh"
#include "windows.h"

// word w of sum_{i<52} 16 * 32^i: bit 5i + 4 set for i < 52
FT_DEV uint32_t enc_bias_word(int w)
{
    uint32_t x = 0;
    for (int b = 0; b < 32; ++b) {
        const int bit = 32 * w + b;
        if (bit % 5 == 4 && bit <= 5 * (ENC_ROWS - 1) + 4) x |= 1u << b;
    }
    return x;
}

// b = a + the bias of the first `digits` digits (9 words; digits <= 52)
FT_DEV void enc_recode(uint32_t b[9], const uint32_t a[8], int digits)
{
    uint32_t bias[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const int lo = 32 * k, nbits = 5 * digits;
        const uint32_t keep = nbits >= lo + 32 ? ~0u : (nbits <= lo ? 0u : (1u << (nbits - lo)) - 1u);
        bias[k] = enc_bias_word(k) & keep;
    }
    b[0] = add_cc(a[0], bias[0]);
#pragma unroll
    for (int k = 1; k < 8; ++k) b[k] = addc_cc(a[k], bias[k]);
    b[8] = addc(0u, bias[8]);
}

FT_DEV void shr5_288(uint32_t c[9])
{
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k] = (c[k] >> 5) | (c[k + 1] << 27);
    c[8] >>= 5;
}

// t = the entry |d| of a table row (ENC_ENTRIES entries), negated for d < 0;
// the identity for d = 0; every entry is read and merged under its mask.
// Eight entries per iteration of a rolled loop.  With the field arithmetic
// of the time: 12.03 ms for the encryption of 1,048,576 plaintexts with
// four, 12.06 with two, 12.33 with eight, 12.71 fully unrolled and 13.96
// with one (instruction fetch and load latency); after the encryption
// stopped keeping the digits of r and m in registers: 9.78 ms with four,
// 9.90 with two, 9.72 with eight or sixteen.  Moving some entries to the multiply-add
// pipe (products by 0/1 indicators) measured 1-3% slower at every grouping.
#ifndef FT_ENC_SEL_GROUP
#define FT_ENC_SEL_GROUP 8
#endif
static constexpr int ENC_SEL_GROUP = FT_ENC_SEL_GROUP;
static_assert(ENC_ENTRIES % ENC_SEL_GROUP == 0, "select grouping");

FT_DEV void enc_select(ge_precomp &t, int d, const uint4 *row)
{
    const uint32_t bneg = (uint32_t)d >> 31;
    const uint32_t babs = (uint32_t)((d ^ -(int)bneg) + (int)bneg);
    fe_0(t.yplusx);
    fe_0(t.yminusx);
    fe_0(t.xy2d);
    const uint32_t id = babs == 0u ? 1u : 0u; // the identity (1, 1, 0)
    t.yplusx.v[0] = id;
    t.yminusx.v[0] = id;
#pragma unroll 1
    for (int k = 0; k < ENC_ENTRIES; k += ENC_SEL_GROUP) {
#pragma unroll
        for (int q = 0; q < ENC_SEL_GROUP; ++q) {
            const uint4 *e = row + 6 * (k + q);
            fe e0, e1, e2;
            fe_from_u4(e0, e[0], e[1]);
            fe_from_u4(e1, e[2], e[3]);
            fe_from_u4(e2, e[4], e[5]);
            const uint32_t m = ct_eq_mask(babs, (uint32_t)(k + q + 1));
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                t.yplusx.v[i] |= e0.v[i] & m;
                t.yminusx.v[i] |= e1.v[i] & m;
                t.xy2d.v[i] |= e2.v[i] & m;
            }
        }
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

// The scalar the reference's fixed-base product actually multiplies by.  Its
// signed radix-16 recoding (e_i = nibble_i(a + sum_{i<63} 8 * 16^i) - 8 for
// i < 63, e_63 the top nibble of that sum, up to 16) feeds an 8-entry
// select, which yields the identity for a top digit above 8: for scalars
// from about 9 * 2^252 (outside the reference's a < 2^255 contract) the
// reference computes (sum_{i<63} e_i 16^i) * B.  For those a, out =
// (a + bias) mod 2^252 + (L - bias), that value made non-negative by adding
// the group order L; otherwise out = a.  Constant time in a.
FT_DEV void enc_ref_scalar(uint32_t out[8], const uint32_t a[8])
{
    // L - sum_{i<63} 8 * 16^i
    constexpr uint32_t C[8] = {0xd46d4b65u, 0xcf89da91u, 0x1a6f144du, 0x8c567156u,
                               0x77777777u, 0x77777777u, 0x77777777u, 0x07777777u};
    uint32_t b[8];
    b[0] = add_cc(a[0], 0x88888888u);
#pragma unroll
    for (int k = 1; k < 7; ++k) b[k] = addc_cc(a[k], 0x88888888u);
    b[7] = addc_cc(a[7], 0x08888888u);
    const uint32_t top = addc(0u, 0u);                // bit 256 of the biased sum
    const uint32_t e63 = (b[7] >> 28) | (top << 4);   // the reference's top digit, 0..16
    const uint32_t m = 0u - ((8u - e63) >> 31);       // all ones iff e63 > 8
    b[7] &= 0x0fffffffu;
    uint32_t t[8];
    t[0] = add_cc(b[0], C[0]);
#pragma unroll
    for (int k = 1; k < 7; ++k) t[k] = addc_cc(b[k], C[k]);
    t[7] = addc(b[7], C[7]);
#pragma unroll
    for (int k = 0; k < 8; ++k) out[k] = (t[k] & m) | (a[k] & ~m);
}

// one comb row: h += d * table row, d from the low five bits of c, c >>= 5
FT_DEV void enc_comb_row(ge_p3 &h, uint32_t c[9], const uint4 *row)
{
    const int d = (int)(c[0] & 31u) - 16;
    shr5_288(c);
    ge_precomp sel;
    enc_select(sel, d, row);
    ge_p1p1 q;
    ge_madd(q, h, sel);
    ge_p1p1_to_p3(h, q);
}

// entry (row, j) = (j+1) * 32^row * Q as 6 uint4 (affine, canonical)
FT_DEV void enc_table_entry(uint4 out[6], const ge_p3 &Q, int row, int j)
{
    ge_p3 R = Q;
    for (int k = 0; k < 5 * row; ++k) {
        ge_p1p1 r;
        ge_p3_dbl(r, R);
        ge_p1p1_to_p3(R, r);
    }
    ge_p3 acc = R;
    ge_cached c;
    ge_p3_to_cached(c, R);
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
    out[0] = u4_lo(yp);
    out[1] = u4_hi(yp);
    out[2] = u4_lo(ym);
    out[3] = u4_hi(ym);
    out[4] = u4_lo(t2);
    out[5] = u4_hi(t2);
}
