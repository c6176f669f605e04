// smul.cuh — per-thread scalar multiplication cores.
//
//   smul_build_table / smul_ladder : constant-time variable-base a*P in the
//       reference's signed radix-16 window (ge25519_scalarmult,
//       sodium_ge.cu:650-731): table (k+1)*P for k < 8 built in the same
//       order, 63 x {select, add, 4 doublings} + final add.  The table lives
//       wherever the caller's accessor puts it (shared memory in the kernels).
//   smul_ladder_u32 : the same ladder for scalars under a public bound, in
//       fewer (and optionally narrower) windows.
// The fixed-base comb is in enc_comb.cuh.
#pragma once
#include "ge.cuh"
#include "windows.h"

// Tab: put(k, const ge_cached&), get(k, ge_cached&) for k in [0, 8) and
// select_fe<NE>(f, j, babs, one): coordinate j (0 YplusX, 1 YminusX, 2 Z,
// 3 T2d) of entry babs - 1 among the first NE, in constant time, the
// identity's for babs = 0.
//
// smul_build_table<NE> fills (k+1)*P for k < NE (NE = 2, 4 or 8).  Every
// entry is the reference's value: 2P, 4P, 6P, 8P are doublings of P, 2P,
// 3P, 4P and 3P, 5P, 7P are P + 2P, P + 4P, P + 6P, as in the reference.
// Only the evaluation order differs: the odd multiples read the cached even
// multiple back from the table, so at most two projective points are live
// at once (the register peak of the kernel).
template <int NE = 8, class Tab>
FT_DEV void smul_build_table(Tab &tab, const ge_p3 &p)
{
    static_assert(NE == 2 || NE == 4 || NE == 8, "tables of 2, 4 or 8 entries");
    ge_cached c;
    ge_p1p1 t;
    ge_p3 q, u;
    ge_p3_to_cached(c, p);
    tab.put(0, c); // 1P
    ge_p3_dbl(t, p);
    ge_p1p1_to_p3(q, t); // 2P
    ge_p3_to_cached(c, q);
    tab.put(1, c);
    if (NE == 2) return;
    ge_p3_dbl(t, q);
    ge_p1p1_to_p3(q, t); // 4P = 2*2P
    ge_p3_to_cached(c, q);
    tab.put(3, c);
    if (NE == 8) {
        ge_p3_dbl(t, q);
        ge_p1p1_to_p3(u, t); // 8P = 2*4P
        ge_p3_to_cached(c, u);
        tab.put(7, c);
        tab.get(3, c);
        ge_add(t, p, c);
        ge_p1p1_to_p3(u, t); // 5P = P + 4P
        ge_p3_to_cached(c, u);
        tab.put(4, c);
    }
    tab.get(1, c);
    ge_add(t, p, c);
    ge_p1p1_to_p3(q, t); // 3P = P + 2P
    ge_p3_to_cached(c, q);
    tab.put(2, c);
    if (NE == 4) return;
    ge_p3_dbl(t, q);
    ge_p1p1_to_p3(u, t); // 6P = 2*3P
    ge_p3_to_cached(c, u);
    tab.put(5, c);
    ge_add(t, p, c);
    ge_p1p1_to_p3(u, t); // 7P = P + 6P
    ge_p3_to_cached(c, u);
    tab.put(6, c);
}

// f = coordinate j of entry babs - 1 (the identity's coordinate, fe_1 or
// fe_0 as `one` says, for babs = 0); all NE entries are read.  Used by
// tables that hold every entry in one memory (Tab::get_fe).
template <int NE, class Tab>
FT_DEV void tab_select_fe(fe &f, const Tab &tab, int j, uint32_t babs, bool one)
{
    if (one) fe_1(f);
    else fe_0(f);
#pragma unroll
    for (int k = 0; k < NE; ++k) {
        fe e;
        tab.get_fe(k, j, e);
        fe_cmov(f, e, ct_eq_mask(babs, (uint32_t)(k + 1)));
    }
}

// r = p + d * P for a signed digit d in [-NE, NE], where tab holds (k+1)*P:
// the reference's cmov8_cached select (sodium_ge.cu:490-511) followed by
// ge_add (the same field operations on the same
// values), with each coordinate of the entry selected just before the
// multiplication that uses it, so that only two selected coordinates are
// live at a time.
template <int NE = 8, class Tab>
FT_DEV void ge_add_select(ge_p1p1 &r, const ge_p3 &p, const Tab &tab, int d)
{
    const uint32_t bneg = (uint32_t)d >> 31;
    const uint32_t babs = (uint32_t)((d ^ -(int)bneg) + (int)bneg);
    const uint32_t nm = 0u - bneg;
    fe a, b, t0;
    tab.template select_fe<NE>(a, 0, babs, true);
    tab.template select_fe<NE>(b, 1, babs, true);
#pragma unroll
    for (int k = 0; k < 8; ++k) { // -P swaps YplusX and YminusX
        uint32_t sw = (a.v[k] ^ b.v[k]) & nm;
        a.v[k] ^= sw;
        b.v[k] ^= sw;
    }
    fe_add(r.X, p.Y, p.X);
    fe_sub(r.Y, p.Y, p.X);
#if FT_MUL_PAIRS
    fe_mul_x2(r.Z, r.X, a, r.Y, r.Y, b);
    tab.template select_fe<NE>(a, 3, babs, false);
    fe_neg(b, a); // -P negates T2d
    fe_cmov(a, b, nm);
    tab.template select_fe<NE>(b, 2, babs, true);
    fe_mul_x2(r.T, a, p.T, r.X, p.Z, b);
#else
    fe_mul(r.Z, r.X, a);
    fe_mul(r.Y, r.Y, b);
    tab.template select_fe<NE>(a, 3, babs, false);
    fe_neg(b, a); // -P negates T2d
    fe_cmov(a, b, nm);
    fe_mul(r.T, a, p.T);
    tab.template select_fe<NE>(a, 2, babs, true);
    fe_mul(r.X, p.Z, a);
#endif
    fe_add(t0, r.X, r.X);
    fe_sub(r.X, r.Z, r.Y);
    fe_add(r.Y, r.Z, r.Y);
    fe_add(r.Z, t0, r.T);
    fe_sub(r.T, t0, r.T);
}

// h = a * P where tab holds (k+1)*P.  a is 8 little-endian words.  (The
// biased scalar stays in 8 registers: keeping it in shared memory and
// reading each window's nibble there measured 0.5% slower.)
template <class Tab>
FT_DEV void smul_ladder(ge_p3 &h, const uint32_t a[8], const Tab &tab, bool block_in_step = false)
{
    uint32_t b[8];
    recode_bias(b, a);
    ge_p3_0(h);
    ge_p1p1 r;
    ge_p2 s;
    int d = pop_top_nibble(b); // digit 63 carries no bias
#pragma unroll 1
    for (int i = 63; i > 0; --i) {
        // block_in_step (only where every thread of the block runs the whole
        // ladder): a barrier per window keeps the warps on the same stretch
        // of the loop body (~60 KB of instructions), so they share the
        // instruction caches: 25.27 -> 24.85 ms for 1,048,576 points
        if (block_in_step) __syncthreads();
        ge_add_select(r, h, tab, d);
#pragma unroll 1
        for (int k = 0; k < 4; ++k) {
            ge_p1p1_to_p2(s, r);
            ge_p2_dbl(r, s);
        }
        ge_p1p1_to_p3(h, r);
        d = pop_top_nibble(b) - 8;
    }
    ge_add_select(r, h, tab, d);
    ge_p1p1_to_p3(h, r);
}

// h = k * P for k < 2^32, constant time in k, in nwin signed radix-2^W
// windows (W = 4: the reference's radix; W = 3 or 2: smaller tables of
// 2^(W-1) entries, built by smul_build_table<2^(W-1)>), each a table
// select, an add and W doublings but the last.  The digits are exact when
// nwin = u32_ladder_windows(bits, W) for k < 2^bits (windows.h).  The point
// equals smul_ladder's for the 32-byte scalar k.
template <int W = 4, class Tab>
FT_DEV void smul_ladder_u32(ge_p3 &h, uint32_t k, const Tab &tab, int nwin = 9)
{
    constexpr int NE = 1 << (W - 1);
    constexpr uint32_t MASK = (1u << W) - 1u;
    uint64_t b = k;
#pragma unroll 1
    for (int i = 0; i < nwin; ++i) b += (uint64_t)NE << (W * i);
    ge_p3_0(h);
    ge_p1p1 r;
    ge_p2 s;
    int d = (int)((b >> (W * (nwin - 1))) & MASK) - NE;
#pragma unroll 1
    for (int i = nwin - 1; i > 0; --i) {
        ge_add_select<NE>(r, h, tab, d);
#pragma unroll 1
        for (int j = 0; j < W; ++j) {
            ge_p1p1_to_p2(s, r);
            ge_p2_dbl(r, s);
        }
        ge_p1p1_to_p3(h, r);
        d = (int)((b >> (W * (i - 1))) & MASK) - NE;
    }
    ge_add_select<NE>(r, h, tab, d);
    ge_p1p1_to_p3(h, r);
}

