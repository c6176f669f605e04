// ge.cuh — twisted-Edwards group arithmetic on Ed25519 (-x^2 + y^2 = 1 + d x^2 y^2).
//
// Point forms and formulas are those of the reference (sodium_ge.cu:38-69):
//   p2 (X:Y:Z), p3 (X:Y:Z:T) with XY = ZT, p1p1 ((X:Z),(Y:T)),
//   precomp (y+x, y-x, 2dxy) for affine table entries,
//   cached (Y+X, Y-X, Z, 2dT) for projective table entries.
// Every formula below performs the same field operations in the same order as
// the reference function it cites, so results agree with the reference mod p
// for every input, including inputs that are not on the curve.
#pragma once
#include "fe.cuh"

// FT_MUL_PAIRS: independent multiplications (and squarings) of a formula
// are computed two at a time with their rows interleaved (fe_mul_x2,
// fe_sq_x2): four carry chains in flight instead of two.  The same
// products, so the same values.  Measured against one at a time: CT ladder
// of 1,048,576 points 20.34 -> 20.28 ms, encryption 9.85 -> 9.80 ms, sum of
// 16,777,216 points 1.565 -> 1.538 ms, scan of 2 x 4,194,304 points 2.031 ->
// 1.997 ms (with the squarings of the doubling left unpaired the ladder
// measured 0.2% slower).
#ifndef FT_MUL_PAIRS
#define FT_MUL_PAIRS 1
#endif

struct ge_p2 { fe X, Y, Z; };
struct ge_p3 { fe X, Y, Z, T; };
struct ge_p1p1 { fe X, Y, Z, T; };
struct ge_precomp { fe yplusx, yminusx, xy2d; };
struct ge_cached { fe YplusX, YminusX, Z, T2d; };

FT_DEV void ge_p3_0(ge_p3 &h) { fe_0(h.X); fe_1(h.Y); fe_1(h.Z); fe_0(h.T); }        // sodium_ge.cu:322
FT_DEV void ge_cached_0(ge_cached &h) { fe_1(h.YplusX); fe_1(h.YminusX); fe_1(h.Z); fe_0(h.T2d); } // :331
FT_DEV void ge_precomp_0(ge_precomp &h) { fe_1(h.yplusx); fe_1(h.yminusx); fe_0(h.xy2d); }       // :408

// r = p + q  (ge25519_add, sodium_ge.cu:76-92)
FT_DEV void ge_add(ge_p1p1 &r, const ge_p3 &p, const ge_cached &q)
{
    fe t0;
    fe_add(r.X, p.Y, p.X);
    fe_sub(r.Y, p.Y, p.X);
#if FT_MUL_PAIRS
    fe_mul_x2(r.Z, r.X, q.YplusX, r.Y, r.Y, q.YminusX);
    fe_mul_x2(r.T, q.T2d, p.T, r.X, p.Z, q.Z);
#else
    fe_mul(r.Z, r.X, q.YplusX);
    fe_mul(r.Y, r.Y, q.YminusX);
    fe_mul(r.T, q.T2d, p.T);
    fe_mul(r.X, p.Z, q.Z);
#endif
    fe_add(t0, r.X, r.X);
    fe_sub(r.X, r.Z, r.Y);
    fe_add(r.Y, r.Z, r.Y);
    fe_add(r.Z, t0, r.T);
    fe_sub(r.T, t0, r.T);
}

// r = p - q  (ge25519_sub, sodium_ge.cu:517-533)
FT_DEV void ge_sub(ge_p1p1 &r, const ge_p3 &p, const ge_cached &q)
{
    fe t0;
    fe_add(r.X, p.Y, p.X);
    fe_sub(r.Y, p.Y, p.X);
    fe_mul(r.Z, r.X, q.YminusX);
    fe_mul(r.Y, r.Y, q.YplusX);
    fe_mul(r.T, q.T2d, p.T);
    fe_mul(r.X, p.Z, q.Z);
    fe_add(t0, r.X, r.X);
    fe_sub(r.X, r.Z, r.Y);
    fe_add(r.Y, r.Z, r.Y);
    fe_sub(r.Z, t0, r.T);
    fe_add(r.T, t0, r.T);
}

// r = p + q, q affine  (ge25519_madd, sodium_ge.cu:231-246)
FT_DEV void ge_madd(ge_p1p1 &r, const ge_p3 &p, const ge_precomp &q)
{
    fe t0;
    fe_add(r.X, p.Y, p.X);
    fe_sub(r.Y, p.Y, p.X);
#if FT_MUL_PAIRS
    fe_mul_x2(r.Z, r.X, q.yplusx, r.Y, r.Y, q.yminusx);
#else
    fe_mul(r.Z, r.X, q.yplusx);
    fe_mul(r.Y, r.Y, q.yminusx);
#endif
    fe_mul(r.T, q.xy2d, p.T);
    fe_add(t0, p.Z, p.Z);
    fe_sub(r.X, r.Z, r.Y);
    fe_add(r.Y, r.Z, r.Y);
    fe_add(r.Z, t0, r.T);
    fe_sub(r.T, t0, r.T);
}

FT_DEV void ge_p1p1_to_p2(ge_p2 &r, const ge_p1p1 &p) // sodium_ge.cu:273
{
#if FT_MUL_PAIRS
    fe_mul_x2(r.X, p.X, p.T, r.Y, p.Y, p.Z);
#else
    fe_mul(r.X, p.X, p.T);
    fe_mul(r.Y, p.Y, p.Z);
#endif
    fe_mul(r.Z, p.Z, p.T);
}

FT_DEV void ge_p1p1_to_p3(ge_p3 &r, const ge_p1p1 &p) // sodium_ge.cu:285
{
#if FT_MUL_PAIRS
    fe_mul_x2(r.X, p.X, p.T, r.Y, p.Y, p.Z);
    fe_mul_x2(r.Z, p.Z, p.T, r.T, p.X, p.Y);
#else
    fe_mul(r.X, p.X, p.T);
    fe_mul(r.Y, p.Y, p.Z);
    fe_mul(r.Z, p.Z, p.T);
    fe_mul(r.T, p.X, p.Y);
#endif
}

// r = 2p  (ge25519_p2_dbl, sodium_ge.cu:306-320)
FT_DEV void ge_p2_dbl(ge_p1p1 &r, const ge_p2 &p)
{
    fe t0;
#if FT_MUL_PAIRS
    fe_sq_x2(r.X, p.X, r.Z, p.Y);
    fe_add(r.Y, p.X, p.Y);
    fe_sq_x2(r.T, p.Z, t0, r.Y);
    fe_add(r.T, r.T, r.T); // fe_sq2
#else
    fe_sq(r.X, p.X);
    fe_sq(r.Z, p.Y);
    fe_sq2(r.T, p.Z);
    fe_add(r.Y, p.X, p.Y);
    fe_sq(t0, r.Y);
#endif
    fe_add(r.Y, r.Z, r.X);
    fe_sub(r.Z, r.Z, r.X);
    fe_sub(r.X, t0, r.Y);
    fe_sub(r.T, r.T, r.Z);
}

FT_DEV void ge_p3_to_p2(ge_p2 &r, const ge_p3 &p) // sodium_ge.cu:374
{
    fe_copy(r.X, p.X);
    fe_copy(r.Y, p.Y);
    fe_copy(r.Z, p.Z);
}

FT_DEV void ge_p3_dbl(ge_p1p1 &r, const ge_p3 &p) // sodium_ge.cu:400
{
    ge_p2 q;
    ge_p3_to_p2(q, p);
    ge_p2_dbl(r, q);
}

FT_DEV void ge_p3_to_cached(ge_cached &r, const ge_p3 &p) // sodium_ge.cu:344
{
    fe_add(r.YplusX, p.Y, p.X);
    fe_sub(r.YminusX, p.Y, p.X);
    fe_copy(r.Z, p.Z);
    fe_mul(r.T2d, p.T, fe_d2());
}

// dest += src  (ge25519_addto, ftcrypto.cu:143-150: 9 field multiplications)
FT_DEV void ge_addto(ge_p3 &dest, const ge_p3 &src)
{
    ge_cached c;
    ge_p1p1 s;
    ge_p3_to_cached(c, src);
    ge_add(s, dest, c);
    ge_p1p1_to_p3(dest, s);
}

// dest -= src  (ge25519_subfrom, ftcrypto.cu:153-160)
FT_DEV void ge_subfrom(ge_p3 &dest, const ge_p3 &src)
{
    ge_cached c;
    ge_p1p1 s;
    ge_p3_to_cached(c, src);
    ge_sub(s, dest, c);
    ge_p1p1_to_p3(dest, s);
}

// identity: the decoding of the folded encoding 0x01 00..00 (ftcrypto.cu:128)
// is (0 : 1 : 1 : 0)
FT_DEV void ge_zero(ge_p3 &z) { ge_p3_0(z); }

// X == 0 and Y == Z (ge25519_iszero, ftcrypto.cu:170-181)
FT_DEV int ge_iszero(const ge_p3 &e)
{
    fe ymz;
    fe_sub(ymz, e.Y, e.Z);
    return fe_iszero(e.X) & fe_iszero(ymz);
}

// equality by subtraction (ge25519_equal, ftcrypto.cu:184-190)
FT_DEV int ge_equal(const ge_p3 &a, const ge_p3 &b)
{
    ge_p3 d = a;
    ge_subfrom(d, b);
    return ge_iszero(d);
}

// canonical 32-byte encoding given 1/Z (ge25519_p3_tobytes, sodium_ge.cu:382-394)
FT_DEV void ge_encode_with_zinv(uint32_t out[8], const ge_p3 &h, const fe &zinv)
{
    fe x, y;
    fe_mul(x, h.X, zinv);
    fe_mul(y, h.Y, zinv);
    fe yc;
    fe_canon(yc, y);
    uint32_t neg = fe_isnegative(x);
#pragma unroll
    for (int k = 0; k < 8; ++k) out[k] = yc.v[k];
    out[7] ^= neg << 31;
}

// decode (ge25519_frombytes, sodium_ge.cu:137-180); returns 0 or -1.  The
// arithmetic on rejected encodings is the reference's too, so the point
// stored for a rejected input is the reference's.
FT_DEV int ge_frombytes(ge_p3 &h, const uint32_t s[8])
{
    fe u, v, v3, vxx, mchk, pchk, negx, xi;
    fe_from_words(h.Y, s);
    fe_1(h.Z);
    fe_sq(u, h.Y);
    fe_mul(v, u, fe_d());
    fe_sub(u, u, h.Z);
    fe_add(v, v, h.Z);
    fe_sq(v3, v);
    fe_mul(v3, v3, v);
    fe_sq(h.X, v3);
    fe_mul(h.X, h.X, v);
    fe_mul(h.X, h.X, u);
    fe_pow22523(h.X, h.X);
    fe_mul(h.X, h.X, v3);
    fe_mul(h.X, h.X, u);
    fe_sq(vxx, h.X);
    fe_mul(vxx, vxx, v);
    fe_sub(mchk, vxx, u);
    fe_add(pchk, vxx, u);
    int has_m = fe_iszero(mchk);
    int has_p = fe_iszero(pchk);
    fe_mul(xi, h.X, fe_sqrtm1());
    fe_cmov(h.X, xi, 0u - (uint32_t)(1 - has_m));
    fe_neg(negx, h.X);
    fe_cmov(h.X, negx, 0u - (fe_isnegative(h.X) ^ (s[7] >> 31)));
    fe_mul(h.T, h.X, h.Y);
    return (has_m | has_p) - 1;
}

// on-curve test (ge25519_is_on_curve, sodium_ge.cu:849-872)
FT_DEV int ge_is_on_curve(const ge_p3 &p)
{
    fe x2, y2, z2, z4, t0, t1;
    fe_sq(x2, p.X);
    fe_sq(y2, p.Y);
    fe_sq(z2, p.Z);
    fe_sub(t0, y2, x2);
    fe_mul(t0, t0, z2);
    fe_mul(t1, x2, y2);
    fe_mul(t1, t1, fe_d());
    fe_sq(z4, z2);
    fe_add(t1, t1, z4);
    fe_sub(t0, t0, t1);
    return fe_iszero(t0);
}

// ---- constant-time selection (ge25519_cmov8_cached / cmov8, sodium_ge.cu:458-511)

FT_DEV uint32_t ct_eq_mask(uint32_t a, uint32_t b)
{
    uint32_t x = a ^ b;
    return 0u - ((x - 1u) >> 31); // all ones iff a == b (a, b < 2^31)
}

// (the selections that use it: ge_add_select in smul.cuh, enc_select in
// enc_comb.cuh, each reading every entry and merging under masks, with no
// address or branch depending on the digit)

// ---- signed radix-16 digits (the recoding of sodium_ge.cu:693-708)
//
// For a 256-bit scalar a, b = a + sum_{i<63} 8 * 16^i (mod 2^256).  Digit i
// (i < 63) is nibble_i(b) - 8 in [-8, 7]; digit 63 is nibble_63(b).  This is
// the reference's carry recoding in closed form; for scalars at or above
// 2^255 (outside the reference's contract) nibble_63 differs from the
// reference's top digit only where both select the identity.
FT_DEV void recode_bias(uint32_t b[8], const uint32_t a[8])
{
    b[0] = add_cc(a[0], 0x88888888u);
#pragma unroll
    for (int k = 1; k < 7; ++k) b[k] = addc_cc(a[k], 0x88888888u);
    b[7] = addc(a[7], 0x08888888u);
}

FT_DEV int nibble(const uint32_t b[8], int i) // i is a compile-time constant when unrolled
{
    return (int)((b[i >> 3] >> (4 * (i & 7))) & 15u);
}

// top nibble of the 256-bit value, then shift it out (windows top-down)
FT_DEV int pop_top_nibble(uint32_t b[8])
{
    int d = (int)(b[7] >> 28);
#pragma unroll
    for (int k = 7; k > 0; --k) b[k] = (b[k] << 4) | (b[k - 1] >> 28);
    b[0] <<= 4;
    return d;
}
