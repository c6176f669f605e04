// devcode_host.cpp — host build of the library's per-thread device arithmetic
// (fe.cuh, ge.cuh, smul.cuh) over the C stand-ins of ptx_emul.h, exported for
// tests/test_devcode_host.py to compare with the oracle.  TEST HARNESS ONLY.
#include <string.h>
#include "../../libftcrypto_gb300/csrc/ladder_tab.cuh"
#include "../../libftcrypto_gb300/csrc/enc_comb.cuh"

static void ld(ge_p3 &p, const uint8_t *s) { memcpy(p.X.v, s, 32); memcpy(p.Y.v, s + 32, 32); memcpy(p.Z.v, s + 64, 32); memcpy(p.T.v, s + 96, 32); }
static void st(uint8_t *s, const ge_p3 &p) { memcpy(s, p.X.v, 32); memcpy(s + 32, p.Y.v, 32); memcpy(s + 64, p.Z.v, 32); memcpy(s + 96, p.T.v, 32); }

struct ArrTab {
    ge_cached e[8];
    void put(int k, const ge_cached &c) { e[k] = c; }
    void get(int k, ge_cached &c) const { c = e[k]; }
    void get_fe(int k, int j, fe &f) const
    {
        f = j == 0 ? e[k].YplusX : j == 1 ? e[k].YminusX : j == 2 ? e[k].Z : e[k].T2d;
    }
    template <int NE>
    void select_fe(fe &f, int j, uint32_t babs, bool one) const { tab_select_fe<NE>(f, *this, j, babs, one); }
};


// the ladder over the tables of the tensor-memory kernel (block size nt,
// 384 or 448): point i is run as thread i % nt of a block, with that
// thread's shared-memory column and warp's tensor-memory slice
template <int NT>
static void mul_hybrid(uint8_t *pts, const uint8_t *scalars, size_t n)
{
    static uint4 smem[NT * 4 * 8];
    for (size_t i = 0; i < n; ++i) {
        const int t = (int)(i % NT), warp = t / 32;
        ft::HybridTab<NT> tab{smem + t, tmem_warp_addr(0u, warp, 128u * (uint32_t)(warp >> 2)) + (uint32_t)(t % 32 << 16)};
        ge_p3 p, h; uint32_t a[8];
        ld(p, pts + 128 * i); memcpy(a, scalars + 32 * i, 32);
        smul_build_table(tab, p);
        smul_ladder(h, a, tab);
        st(pts + 128 * i, h);
    }
}
template <int W>
static void mul_u32_w(uint8_t *pts, const uint32_t *k, size_t n, unsigned bits)
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p, h; ArrTab tab;
        ld(p, pts + 128 * i);
        smul_build_table<1 << (W - 1)>(tab, p);
        smul_ladder_u32<W>(h, k[i], tab, u32_ladder_windows(bits, W));
        st(pts + 128 * i, h);
    }
}
extern "C" {

void hc_fe_mul(uint32_t *h, const uint32_t *a, const uint32_t *b)
{
    fe x, y, z;
    memcpy(x.v, a, 32); memcpy(y.v, b, 32);
    fe_mul(z, x, y);
    memcpy(h, z.v, 32);
}
void hc_mul_wide(uint32_t *t, const uint32_t *a, const uint32_t *b)
{
    fe x, y;
    memcpy(x.v, a, 32); memcpy(y.v, b, 32);
    mul_wide(t, x, y);
}
void hc_sqr_wide(uint32_t *t, const uint32_t *a) { fe x; memcpy(x.v, a, 32); sqr_wide(t, x); }
void hc_fe_sq(uint32_t *h, const uint32_t *a) { fe x, z; memcpy(x.v, a, 32); fe_sq(z, x); memcpy(h, z.v, 32); }
void hc_fe_add(uint32_t *h, const uint32_t *a, const uint32_t *b) { fe x, y, z; memcpy(x.v, a, 32); memcpy(y.v, b, 32); fe_add(z, x, y); memcpy(h, z.v, 32); }
void hc_fe_sub(uint32_t *h, const uint32_t *a, const uint32_t *b) { fe x, y, z; memcpy(x.v, a, 32); memcpy(y.v, b, 32); fe_sub(z, x, y); memcpy(h, z.v, 32); }
void hc_fe_canon(uint32_t *h, const uint32_t *a) { fe x, z; memcpy(x.v, a, 32); fe_canon(z, x); memcpy(h, z.v, 32); }
void hc_fe_invert(uint32_t *h, const uint32_t *a) { fe x, z; memcpy(x.v, a, 32); fe_invert(z, x); memcpy(h, z.v, 32); }

void hc_add(uint8_t *res, const uint8_t *b, size_t n)
{
    for (size_t i = 0; i < n; ++i) { ge_p3 p, q; ld(p, res + 128 * i); ld(q, b + 128 * i); ge_addto(p, q); st(res + 128 * i, p); }
}
void hc_sub(uint8_t *res, const uint8_t *b, size_t n)
{
    for (size_t i = 0; i < n; ++i) { ge_p3 p, q; ld(p, res + 128 * i); ld(q, b + 128 * i); ge_subfrom(p, q); st(res + 128 * i, p); }
}
void hc_mul(uint8_t *pts, const uint8_t *scalars, size_t n)
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p, h; ArrTab tab; uint32_t a[8];
        ld(p, pts + 128 * i); memcpy(a, scalars + 32 * i, 32);
        smul_build_table(tab, p);
        smul_ladder(h, a, tab);
        st(pts + 128 * i, h);
    }
}
int hc_mul_hybrid(uint8_t *pts, const uint8_t *scalars, size_t n, int nt)
{
    if (nt == 384) mul_hybrid<384>(pts, scalars, n);
    else if (nt == 448) mul_hybrid<448>(pts, scalars, n);
    else return -1;
    return 0;
}
// the small-scalar ladder of window width w (2, 3, 4) in the window count
// for k < 2^bits
int hc_mul_u32_bits(uint8_t *pts, const uint32_t *k, size_t n, unsigned bits, int w)
{
    if (w == 2) mul_u32_w<2>(pts, k, n, bits);
    else if (w == 3) mul_u32_w<3>(pts, k, n, bits);
    else if (w == 4) mul_u32_w<4>(pts, k, n, bits);
    else return -1;
    return 0;
}
void hc_mul_u32(uint8_t *pts, const uint32_t *k, size_t n)
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p, h; ArrTab tab;
        ld(p, pts + 128 * i);
        smul_build_table(tab, p);
        smul_ladder_u32(h, k[i], tab);
        st(pts + 128 * i, h);
    }
}
// a_i * Q by the radix-32 comb in nrows rows over the 52 x 16 table of Q
// (built here by enc_table_entry, kept for the next call with the same Q)
void hc_enc_comb(uint8_t *pts, const uint8_t *scalars, size_t n, int nrows, const uint8_t *q128)
{
    static uint4 tab[ENC_ROWS * ENC_ENTRIES * 6];
    static uint8_t tq[128];
    static bool have = false;
    if (!have || memcmp(tq, q128, 128) != 0) {
        ge_p3 Q;
        ld(Q, q128);
        for (int t = 0; t < ENC_ROWS * ENC_ENTRIES; ++t) enc_table_entry(tab + 6 * t, Q, t / ENC_ENTRIES, t % ENC_ENTRIES);
        memcpy(tq, q128, 128);
        have = true;
    }
    for (size_t i = 0; i < n; ++i) {
        ge_p3 h; uint32_t a[8], c[9];
        memcpy(a, scalars + 32 * i, 32);
        if (nrows == ENC_ROWS) {
            uint32_t ar[8];
            enc_ref_scalar(ar, a);
            memcpy(a, ar, 32);
        }
        enc_recode(c, a, nrows);
        ge_p3_0(h);
        for (int row = 0; row < nrows; ++row) enc_comb_row(h, c, tab + (size_t)row * ENC_ENTRIES * 6);
        st(pts + 128 * i, h);
    }
}
int hc_enc_digits(unsigned bits) { return enc_digits(bits); }
void hc_encode(uint8_t *out, const uint8_t *pts, size_t n)
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p; fe zi; uint32_t w[8];
        ld(p, pts + 128 * i);
        fe_invert(zi, p.Z);
        ge_encode_with_zinv(w, p, zi);
        memcpy(out + 32 * i, w, 32);
    }
}
long long hc_decode(uint8_t *pts, const uint8_t *in, size_t n)
{
    long long bad = -1;
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p; uint32_t w[8];
        memcpy(w, in + 32 * i, 32);
        if (ge_frombytes(p, w)) bad = (long long)i;
        st(pts + 128 * i, p);
    }
    return bad;
}

} // extern "C"
