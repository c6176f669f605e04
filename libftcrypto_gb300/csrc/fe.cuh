// fe.cuh — arithmetic in GF(2^255 - 19) for sm_103a.
//
// Representation: 8 x 32-bit little-endian limbs holding an integer below
// 2^256 that is congruent to the field element ("loosely reduced"; values in
// [p, 2^256) are allowed).  This is the radix that maps onto the 32-bit
// IMAD / carry-chain datapath: a product is an 8 x 8 operand-scanning
// schoolbook in mad.lo/madc.hi chains, folded with 2^256 = 38 (mod p).
// The reference's 10 x 25.5-bit signed limbs (sodium_fe.cu:30) need 100
// 32x32->64 products per multiplication against 64 here.
//
// Canonical reduction and the inversion / square-root addition chains follow
// fe25519_reduce (sodium_fe.cu:168-241), fe25519_invert (:1352-1408) and
// fe25519_pow22523 (:1410-1463) of the reference.
#pragma once
#ifdef FT_HOST_EMULATION
#include FT_HOST_EMULATION
#else
#include "ptx.cuh"
#endif

struct fe {
    uint32_t v[8];
};

FT_DEV void fe_0(fe &h)
{
#pragma unroll
    for (int k = 0; k < 8; ++k) h.v[k] = 0;
}

FT_DEV void fe_1(fe &h)
{
    fe_0(h);
    h.v[0] = 1;
}

FT_DEV fe fe_const(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                   uint32_t a4, uint32_t a5, uint32_t a6, uint32_t a7)
{
    fe r;
    r.v[0] = a0; r.v[1] = a1; r.v[2] = a2; r.v[3] = a3;
    r.v[4] = a4; r.v[5] = a5; r.v[6] = a6; r.v[7] = a7;
    return r;
}

// d = -121665/121666, 2d and sqrt(-1) (the constants of fe_constants.h)
FT_DEV fe fe_d() { return fe_const(0x135978a3u, 0x75eb4dcau, 0x4141d8abu, 0x00700a4du, 0x7779e898u, 0x8cc74079u, 0x2b6ffe73u, 0x52036ceeu); }
FT_DEV fe fe_d2() { return fe_const(0x26b2f159u, 0xebd69b94u, 0x8283b156u, 0x00e0149au, 0xeef3d130u, 0x198e80f2u, 0x56dffce7u, 0x2406d9dcu); }
FT_DEV fe fe_sqrtm1() { return fe_const(0x4a0ea0b0u, 0xc4ee1b27u, 0xad2fe478u, 0x2f431806u, 0x3dfbd7a7u, 0x2b4d0099u, 0x4fc1df0bu, 0x2b832480u); }

// h = a + b  (h < 2^256; a carry out of bit 256 is repaid as +38)
FT_DEV void fe_add(fe &h, const fe &a, const fe &b)
{
    uint32_t r[8];
    r[0] = add_cc(a.v[0], b.v[0]);
#pragma unroll
    for (int k = 1; k < 8; ++k) r[k] = addc_cc(a.v[k], b.v[k]);
    uint32_t c = addc(0u, 0u);
    r[0] = mad_lo_cc(c, 38u, r[0]);
#pragma unroll
    for (int k = 1; k < 8; ++k) r[k] = addc_cc(r[k], 0u);
    c = addc(0u, 0u);
    // r < 38 whenever c == 1, so this cannot carry
    r[0] += 38u * c;
#pragma unroll
    for (int k = 0; k < 8; ++k) h.v[k] = r[k];
}

// h = a - b  (a borrow of 2^256 is repaid as -38)
FT_DEV void fe_sub(fe &h, const fe &a, const fe &b)
{
    uint32_t r[8];
    r[0] = sub_cc(a.v[0], b.v[0]);
#pragma unroll
    for (int k = 1; k < 8; ++k) r[k] = subc_cc(a.v[k], b.v[k]);
    uint32_t bw = subc(0u, 0u); // 0 or 0xffffffff
    r[0] = sub_cc(r[0], bw & 38u);
#pragma unroll
    for (int k = 1; k < 8; ++k) r[k] = subc_cc(r[k], 0u);
    bw = subc(0u, 0u);
    // r >= 2^256 - 38 whenever bw != 0, so this cannot borrow
    r[0] -= bw & 38u;
#pragma unroll
    for (int k = 0; k < 8; ++k) h.v[k] = r[k];
}

FT_DEV void fe_neg(fe &h, const fe &f)
{
    fe z;
    fe_0(z);
    fe_sub(h, z, f);
}

// 512-bit t -> h < 2^256 with 2^256 = 38 (mod p).  r = t_lo + 38 t_hi as
// 64-bit windows of 38 * t[8 + k] at position k, in even-aligned register
// pairs as in mul_wide: the even k in one carry chain over t_lo, the odd k
// in a second array one word lower (the windows there do not overlap: no
// carries), then added; the top word (at most 38) is folded once more.
// Measured against a fold of row-by-row (lo, then hi) chains: 21.4 -> 20.4
// ms for the constant-time ladder of 1,048,576 points, same words.
// (Forming 38 t_hi as (t_hi << 5) + (t_hi << 2) + (t_hi << 1) with funnel
// shifts and carry chains instead measured slower: 23.7 ms.)
FT_DEV void fe_fold512(fe &h, const uint32_t t[16])
{
    uint32_t r[8], r8, o[8];
    r[0] = mad_lo_cc(t[8], 38u, t[0]);
    r[1] = madc_hi_cc(t[8], 38u, t[1]);
#pragma unroll
    for (int k = 2; k < 8; k += 2) {
        r[k] = madc_lo_cc(t[8 + k], 38u, t[k]);
        r[k + 1] = madc_hi_cc(t[8 + k], 38u, t[k + 1]);
    }
    r8 = addc(0u, 0u);
#pragma unroll
    for (int k = 1; k < 8; k += 2) {
        o[k - 1] = mul_lo(t[8 + k], 38u);
        o[k] = mul_hi(t[8 + k], 38u);
    }
    r[1] = add_cc(r[1], o[0]);
#pragma unroll
    for (int k = 2; k < 8; ++k) r[k] = addc_cc(r[k], o[k - 1]);
    r8 = addc(r8, o[7]);
    // value = r + r8 * 2^256 with r8 <= 38
    r[0] = mad_lo_cc(r8, 38u, r[0]);
#pragma unroll
    for (int k = 1; k < 8; ++k) r[k] = addc_cc(r[k], 0u);
    uint32_t c = addc(0u, 0u);
    r[0] += 38u * c; // r < 1482 whenever c == 1
#pragma unroll
    for (int k = 0; k < 8; ++k) h.v[k] = r[k];
}

// t = a * b (full 512-bit product).  Each product a_j * b_i is one 64-bit
// window (lo at position p = i + j, hi at p + 1) that ptxas computes with
// one IMAD.WIDE into an even-aligned register pair.  Windows at even p
// accumulate in E (E[p], E[p + 1]); windows at odd p accumulate in O one
// word lower (O[p - 1], O[p]), so that every window of both starts at an
// even index.  Row i adds its four products of each parity as one carry
// chain over consecutive windows, then its carry into the next word of that
// accumulator; t = E + O * 2^32.  (The earlier form chained row i's even-j
// products at positions i + j, odd for odd rows, and measured 60 MOV and 39
// IMAD.MOV instructions per multiplication moving words between pairs.)
// Field-multiplication throughput of other schedules, measured: one level of
// Karatsuba (48 products and ~55 more additions) 7.08 T products/s, four
// independent 4 x 4 blocks 6.83, this one 7.89.
FT_DEV void mul_row(uint32_t E[16], uint32_t O[16], const fe &a, uint32_t bi, int i)
{
    // even p = i + j: j of the parity of i
    const int je = i & 1;
    E[i + je] = mad_lo_cc(a.v[je], bi, E[i + je]);
    E[i + je + 1] = madc_hi_cc(a.v[je], bi, E[i + je + 1]);
#pragma unroll
    for (int j = je + 2; j < 8; j += 2) {
        E[i + j] = madc_lo_cc(a.v[j], bi, E[i + j]);
        E[i + j + 1] = madc_hi_cc(a.v[j], bi, E[i + j + 1]);
    }
    // the row's last window ends at E[i + je + 7]; the carry goes one
    // word up (a word only carries have reached so far; E < 2^512, so
    // past E[15] it is zero)
    if (i + je + 8 < 16) E[i + je + 8] = addc(E[i + je + 8], 0u);
    // odd p = i + j: j of the other parity, window at O[p - 1]
    const int jo = je ^ 1;
    O[i + jo - 1] = mad_lo_cc(a.v[jo], bi, O[i + jo - 1]);
    O[i + jo] = madc_hi_cc(a.v[jo], bi, O[i + jo]);
#pragma unroll
    for (int j = jo + 2; j < 8; j += 2) {
        O[i + j - 1] = madc_lo_cc(a.v[j], bi, O[i + j - 1]);
        O[i + j] = madc_hi_cc(a.v[j], bi, O[i + j]);
    }
    if (i + jo + 7 < 16) O[i + jo + 7] = addc(O[i + jo + 7], 0u);
}

// t = E + O * 2^32 (O[15] is zero: its weight is 2^512)
FT_DEV void mul_merge(uint32_t t[16], const uint32_t E[16], const uint32_t O[16])
{
    t[0] = E[0];
    t[1] = add_cc(E[1], O[0]);
#pragma unroll
    for (int k = 2; k < 15; ++k) t[k] = addc_cc(E[k], O[k - 1]);
    t[15] = addc(E[15], O[14]);
}

FT_DEV void mul_wide(uint32_t t[16], const fe &a, const fe &b)
{
    uint32_t E[16], O[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) E[k] = O[k] = 0u;
#pragma unroll
    for (int i = 0; i < 8; ++i) mul_row(E, O, a, b.v[i], i);
    mul_merge(t, E, O);
}

// two independent products with their rows interleaved (four carry chains
// in flight instead of two)
FT_DEV void mul_wide2(uint32_t t1[16], const fe &a1, const fe &b1, uint32_t t2[16], const fe &a2, const fe &b2)
{
    uint32_t E1[16], O1[16], E2[16], O2[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) E1[k] = O1[k] = E2[k] = O2[k] = 0u;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        mul_row(E1, O1, a1, b1.v[i], i);
        mul_row(E2, O2, a2, b2.v[i], i);
    }
    mul_merge(t1, E1, O1);
    mul_merge(t2, E2, O2);
}

// t = a^2: the 28 cross products a_i a_j (i < j) as 64-bit windows in even
// aligned register pairs, as in mul_wide: even p = i + j in T (T[p],
// T[p + 1]), odd p in O one word lower (O[p - 1], O[p]); row i chains its
// products of each parity.  t = 2 (T + O * 2^32) + the 8 squares a_i^2,
// whose windows (2i, 2i + 1) form one chain.
FT_DEV void sqr_row(uint32_t T[16], uint32_t O[16], const fe &a, int i)
{
    // j = i+1, i+3, ...: odd p, window at O[p - 1]
    O[2 * i] = mad_lo_cc(a.v[i], a.v[i + 1], O[2 * i]);
    O[2 * i + 1] = madc_hi_cc(a.v[i], a.v[i + 1], O[2 * i + 1]);
#pragma unroll
    for (int j = i + 3; j < 8; j += 2) {
        O[i + j - 1] = madc_lo_cc(a.v[i], a.v[j], O[i + j - 1]);
        O[i + j] = madc_hi_cc(a.v[i], a.v[j], O[i + j]);
    }
    {
        const int last = i + 1 + 2 * ((6 - i) / 2);
        if (i + last + 2 < 16) O[i + last + 1] = addc(O[i + last + 1], 0u);
    }
    // j = i+2, i+4, ...: even p
    if (i < 6) {
        T[2 * i + 2] = mad_lo_cc(a.v[i], a.v[i + 2], T[2 * i + 2]);
        T[2 * i + 3] = madc_hi_cc(a.v[i], a.v[i + 2], T[2 * i + 3]);
#pragma unroll
        for (int j = i + 4; j < 8; j += 2) {
            T[i + j] = madc_lo_cc(a.v[i], a.v[j], T[i + j]);
            T[i + j + 1] = madc_hi_cc(a.v[i], a.v[j], T[i + j + 1]);
        }
        const int last = i + 2 + 2 * ((5 - i) / 2);
        if (i + last + 2 < 16) T[i + last + 2] = addc(T[i + last + 2], 0u);
    }
}

// t = 2 (T + O * 2^32) + the squares a_i^2
FT_DEV void sqr_finish(uint32_t t[16], const uint32_t T[16], const uint32_t O[16], const fe &a)
{
    // the cross products sum to less than a^2 / 2 < 2^511: no carry out
    uint32_t c[16];
    c[0] = T[0];
    c[1] = add_cc(T[1], O[0]);
#pragma unroll
    for (int k = 2; k < 16; ++k) c[k] = addc_cc(T[k], O[k - 1]);
    t[0] = add_cc(c[0], c[0]);
#pragma unroll
    for (int k = 1; k < 16; ++k) t[k] = addc_cc(c[k], c[k]);
    t[0] = mad_lo_cc(a.v[0], a.v[0], t[0]);
    t[1] = madc_hi_cc(a.v[0], a.v[0], t[1]);
#pragma unroll
    for (int i = 1; i < 8; ++i) {
        t[2 * i] = madc_lo_cc(a.v[i], a.v[i], t[2 * i]);
        t[2 * i + 1] = madc_hi_cc(a.v[i], a.v[i], t[2 * i + 1]);
    }
}

FT_DEV void sqr_wide(uint32_t t[16], const fe &a)
{
    uint32_t T[16], O[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) T[k] = O[k] = 0u;
#pragma unroll
    for (int i = 0; i < 7; ++i) sqr_row(T, O, a, i);
    sqr_finish(t, T, O, a);
}

// two independent squarings with their rows interleaved
FT_DEV void sqr_wide2(uint32_t t1[16], const fe &a1, uint32_t t2[16], const fe &a2)
{
    uint32_t T1[16], O1[16], T2[16], O2[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) T1[k] = O1[k] = T2[k] = O2[k] = 0u;
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        sqr_row(T1, O1, a1, i);
        sqr_row(T2, O2, a2, i);
    }
    sqr_finish(t1, T1, O1, a1);
    sqr_finish(t2, T2, O2, a2);
}

FT_DEV void fe_mul(fe &h, const fe &a, const fe &b)
{
    uint32_t t[16];
    mul_wide(t, a, b);
    fe_fold512(h, t);
}

FT_DEV void fe_sq(fe &h, const fe &a)
{
    uint32_t t[16];
    sqr_wide(t, a);
    fe_fold512(h, t);
}

// h1 = a1 b1 and h2 = a2 b2, interleaved (the outputs may alias the inputs)
FT_DEV void fe_mul_x2(fe &h1, const fe &a1, const fe &b1, fe &h2, const fe &a2, const fe &b2)
{
    uint32_t t1[16], t2[16];
    mul_wide2(t1, a1, b1, t2, a2, b2);
    fe_fold512(h1, t1);
    fe_fold512(h2, t2);
}

// h1 = a1^2 and h2 = a2^2, interleaved (the outputs may alias the inputs)
FT_DEV void fe_sq_x2(fe &h1, const fe &a1, fe &h2, const fe &a2)
{
    uint32_t t1[16], t2[16];
    sqr_wide2(t1, a1, t2, a2);
    fe_fold512(h1, t1);
    fe_fold512(h2, t2);
}

// 2 * a^2 (fe25519_sq2, sodium_fe.cu:1109)
FT_DEV void fe_sq2(fe &h, const fe &a)
{
    fe s;
    fe_sq(s, a);
    fe_add(h, s, s);
}

// canonical representative in [0, p): fold bit 255 twice, then subtract p
// once if needed (the reduction of fe25519_reduce, sodium_fe.cu:168-241)
FT_DEV void fe_canon(fe &h, const fe &a)
{
    uint32_t v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = a.v[k];
#pragma unroll
    for (int round = 0; round < 2; ++round) {
        uint32_t top = v[7] >> 31;
        v[7] &= 0x7fffffffu;
        v[0] = mad_lo_cc(top, 19u, v[0]);
#pragma unroll
        for (int k = 1; k < 7; ++k) v[k] = addc_cc(v[k], 0u);
        v[7] = addc(v[7], 0u);
    }
    uint32_t u[8];
    u[0] = add_cc(v[0], 19u);
#pragma unroll
    for (int k = 1; k < 7; ++k) u[k] = addc_cc(v[k], 0u);
    u[7] = addc(v[7], 0u);
    uint32_t m = 0u - (u[7] >> 31); // all ones iff v >= p
    u[7] &= 0x7fffffffu;
#pragma unroll
    for (int k = 0; k < 8; ++k) h.v[k] = (v[k] & ~m) | (u[k] & m);
}

FT_DEV int fe_iszero(const fe &f)
{
    fe c;
    fe_canon(c, f);
    uint32_t o = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) o |= c.v[k];
    return o == 0;
}

FT_DEV uint32_t fe_isnegative(const fe &f)
{
    fe c;
    fe_canon(c, f);
    return c.v[0] & 1u;
}

// f = b ? g : f, for a mask b of all ones or all zeros
FT_DEV void fe_cmov(fe &f, const fe &g, uint32_t mask)
{
#pragma unroll
    for (int k = 0; k < 8; ++k) f.v[k] = (f.v[k] & ~mask) | (g.v[k] & mask);
}

FT_DEV void fe_copy(fe &h, const fe &f)
{
#pragma unroll
    for (int k = 0; k < 8; ++k) h.v[k] = f.v[k];
}

FT_DEV void fe_sqn(fe &h, const fe &f, int n)
{
    fe_sq(h, f);
#pragma unroll 1
    for (int i = 1; i < n; ++i) fe_sq(h, h);
}

// z^(p-2), the addition chain of fe25519_invert (sodium_fe.cu:1352-1408)
FT_DEV void fe_invert(fe &out, const fe &z)
{
    fe t0, t1, t2, t3;
    fe_sq(t0, z);
    fe_sqn(t1, t0, 2);
    fe_mul(t1, z, t1);
    fe_mul(t0, t0, t1);
    fe_sq(t2, t0);
    fe_mul(t1, t1, t2);
    fe_sqn(t2, t1, 5);
    fe_mul(t1, t2, t1);
    fe_sqn(t2, t1, 10);
    fe_mul(t2, t2, t1);
    fe_sqn(t3, t2, 20);
    fe_mul(t2, t3, t2);
    fe_sqn(t2, t2, 10);
    fe_mul(t1, t2, t1);
    fe_sqn(t2, t1, 50);
    fe_mul(t2, t2, t1);
    fe_sqn(t3, t2, 100);
    fe_mul(t2, t3, t2);
    fe_sqn(t2, t2, 50);
    fe_mul(t1, t2, t1);
    fe_sqn(t1, t1, 5);
    fe_mul(out, t1, t0);
}

// z^((p-5)/8), the chain of fe25519_pow22523 (sodium_fe.cu:1410-1463)
FT_DEV void fe_pow22523(fe &out, const fe &z)
{
    fe t0, t1, t2;
    fe_sq(t0, z);
    fe_sqn(t1, t0, 2);
    fe_mul(t1, z, t1);
    fe_mul(t0, t0, t1);
    fe_sq(t0, t0);
    fe_mul(t0, t1, t0);
    fe_sqn(t1, t0, 5);
    fe_mul(t0, t1, t0);
    fe_sqn(t1, t0, 10);
    fe_mul(t1, t1, t0);
    fe_sqn(t2, t1, 20);
    fe_mul(t1, t2, t1);
    fe_sqn(t1, t1, 10);
    fe_mul(t0, t1, t0);
    fe_sqn(t1, t0, 50);
    fe_mul(t1, t1, t0);
    fe_sqn(t2, t1, 100);
    fe_mul(t1, t2, t1);
    fe_sqn(t1, t1, 50);
    fe_mul(t0, t1, t0);
    fe_sqn(t0, t0, 2);
    fe_mul(out, t0, z);
}

// 32 little-endian bytes as 8 words, top bit ignored (fe25519_frombytes)
FT_DEV void fe_from_words(fe &h, const uint32_t w[8])
{
#pragma unroll
    for (int k = 0; k < 8; ++k) h.v[k] = w[k];
    h.v[7] &= 0x7fffffffu;
}
