/*
 * ftoracle.c — CPU restatement of libftcrypto's arithmetic (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py.  Never part of the product.
 *
 * Field elements are 4 x 64-bit limbs holding an integer below 2^256 that is
 * congruent mod p = 2^255 - 19 (a different representation from both the
 * reference's 10 x 25.5-bit limbs and the GPU library's 8 x 32-bit limbs).
 * Every group formula follows the reference's sequence of field operations,
 * so projective outputs agree with the reference mod p; canonical encodings
 * are therefore byte-identical.  Each function cites the reference function
 * (file:line, paths inside the reference's src/) it restates.
 */
#include "ftoracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

typedef struct { uint64_t v[4]; } fe;
typedef struct { fe X, Y, Z; } ge_p2;
typedef struct { fe X, Y, Z, T; } ge_p3;
typedef struct { fe X, Y, Z, T; } ge_p1p1;
typedef struct { fe yplusx, yminusx, xy2d; } ge_precomp;
typedef struct { fe YplusX, YminusX, Z, T2d; } ge_cached;

/* ---------------------------------------------------------------- field -- */

static const fe FE_D = {{0x75eb4dca135978a3ULL, 0x00700a4d4141d8abULL,
                         0x8cc740797779e898ULL, 0x52036cee2b6ffe73ULL}};
static const fe FE_D2 = {{0xebd69b9426b2f159ULL, 0x00e0149a8283b156ULL,
                          0x198e80f2eef3d130ULL, 0x2406d9dc56dffce7ULL}};
static const fe FE_SQRTM1 = {{0xc4ee1b274a0ea0b0ULL, 0x2f431806ad2fe478ULL,
                              0x2b4d00993dfbd7a7ULL, 0x2b8324804fc1df0bULL}};

static void fe_0(fe *h) { memset(h, 0, sizeof *h); }
static void fe_1(fe *h) { fe_0(h); h->v[0] = 1; }

/* a + b, folded with 2^256 = 38 (mod p) */
static void fe_add(fe *h, const fe *a, const fe *b)
{
    u128 c = 0;
    uint64_t r[4];
    for (int i = 0; i < 4; ++i) {
        c += (u128)a->v[i] + b->v[i];
        r[i] = (uint64_t)c;
        c >>= 64;
    }
    c *= 38;
    for (int i = 0; i < 4; ++i) {
        c += r[i];
        r[i] = (uint64_t)c;
        c >>= 64;
    }
    r[0] += (uint64_t)c * 38; /* cannot carry: r < 38 here when c == 1 */
    memcpy(h->v, r, sizeof r);
}

/* a - b, with a borrow of 2^256 repaid as 38 (mod p) */
static void fe_sub(fe *h, const fe *a, const fe *b)
{
    uint64_t r[4], borrow = 0;
    for (int i = 0; i < 4; ++i) {
        u128 t = (u128)a->v[i] - b->v[i] - borrow;
        r[i] = (uint64_t)t;
        borrow = (uint64_t)(t >> 64) & 1;
    }
    uint64_t sub = borrow * 38;
    borrow = 0;
    for (int i = 0; i < 4; ++i) {
        u128 t = (u128)r[i] - (i == 0 ? sub : 0) - borrow;
        r[i] = (uint64_t)t;
        borrow = (uint64_t)(t >> 64) & 1;
    }
    r[0] -= borrow * 38; /* cannot borrow: r >= 2^256 - 38 here */
    memcpy(h->v, r, sizeof r);
}

static void fe_neg(fe *h, const fe *f)
{
    fe z;
    fe_0(&z);
    fe_sub(h, &z, f);
}

static void fe_mul(fe *h, const fe *f, const fe *g)
{
    uint64_t r[8] = {0};
    for (int i = 0; i < 4; ++i) {
        u128 c = 0;
        for (int j = 0; j < 4; ++j) {
            c += (u128)f->v[i] * g->v[j] + r[i + j];
            r[i + j] = (uint64_t)c;
            c >>= 64;
        }
        r[i + 4] = (uint64_t)c;
    }
    u128 c = 0;
    uint64_t o[4];
    for (int k = 0; k < 4; ++k) {
        c += (u128)r[k] + (u128)r[k + 4] * 38;
        o[k] = (uint64_t)c;
        c >>= 64;
    }
    c *= 38;
    for (int k = 0; k < 4; ++k) {
        c += o[k];
        o[k] = (uint64_t)c;
        c >>= 64;
    }
    o[0] += (uint64_t)c * 38;
    memcpy(h->v, o, sizeof o);
}

static void fe_sq(fe *h, const fe *f) { fe_mul(h, f, f); }

/* 2 * f^2 (fe25519_sq2, sodium_fe.cu:1109) */
static void fe_sq2(fe *h, const fe *f)
{
    fe t;
    fe_mul(&t, f, f);
    fe_add(h, &t, &t);
}

/* Canonical value in [0, p): fold bit 255 twice, then subtract p if needed
 * (the reduction of fe25519_reduce, sodium_fe.cu:168-241). */
static void fe_canon(uint64_t o[4], const fe *a)
{
    const uint64_t M = 0x7fffffffffffffffULL;
    uint64_t t[4];
    memcpy(t, a->v, sizeof t);
    for (int round = 0; round < 2; ++round) {
        uint64_t top = t[3] >> 63;
        t[3] &= M;
        u128 c = (u128)top * 19;
        for (int i = 0; i < 4; ++i) {
            c += t[i];
            t[i] = (uint64_t)c;
            c >>= 64;
        }
    }
    uint64_t u[4];
    u128 c = 19;
    for (int i = 0; i < 4; ++i) {
        c += t[i];
        u[i] = (uint64_t)c;
        c >>= 64;
    }
    if (u[3] >> 63) {
        u[3] &= M;
        memcpy(o, u, sizeof u);
    } else {
        memcpy(o, t, sizeof t);
    }
}

/* fe25519_tobytes, sodium_fe.cu:251 */
static void fe_tobytes(uint8_t s[32], const fe *h)
{
    uint64_t c[4];
    fe_canon(c, h);
    for (int i = 0; i < 32; ++i) s[i] = (uint8_t)(c[i / 8] >> (8 * (i % 8)));
}

/* fe25519_frombytes, sodium_fe.cu:74 (top bit ignored) */
static void fe_frombytes(fe *h, const uint8_t s[32])
{
    for (int i = 0; i < 4; ++i) {
        uint64_t w = 0;
        for (int k = 0; k < 8; ++k) w |= (uint64_t)s[8 * i + k] << (8 * k);
        h->v[i] = w;
    }
    h->v[3] &= 0x7fffffffffffffffULL;
}

/* raw 32-byte load of a stored coordinate (no masking) */
static void fe_load(fe *h, const uint8_t *s)
{
    memcpy(h->v, s, 32); /* little-endian hosts only (x86-64, aarch64) */
}
static void fe_store(uint8_t *s, const fe *h) { memcpy(s, h->v, 32); }

static int fe_iszero(const fe *f) /* sodium_fe.cu:625 */
{
    uint64_t c[4];
    fe_canon(c, f);
    return (c[0] | c[1] | c[2] | c[3]) == 0;
}

static int fe_isnegative(const fe *f) /* sodium_fe.cu:607 */
{
    uint64_t c[4];
    fe_canon(c, f);
    return (int)(c[0] & 1);
}

static void fe_cmov(fe *f, const fe *g, unsigned b) /* sodium_fe.cu:446 */
{
    uint64_t m = (uint64_t)0 - (uint64_t)b;
    for (int i = 0; i < 4; ++i) f->v[i] ^= (f->v[i] ^ g->v[i]) & m;
}

static void fe_sqn(fe *h, const fe *f, int n)
{
    fe_sq(h, f);
    for (int i = 1; i < n; ++i) fe_sq(h, h);
}

/* z^(p-2): the addition chain of fe25519_invert, sodium_fe.cu:1352-1408 */
static void fe_invert(fe *out, const fe *z)
{
    fe t0, t1, t2, t3;
    fe_sq(&t0, z);
    fe_sqn(&t1, &t0, 2);
    fe_mul(&t1, z, &t1);
    fe_mul(&t0, &t0, &t1);
    fe_sq(&t2, &t0);
    fe_mul(&t1, &t1, &t2);
    fe_sqn(&t2, &t1, 5);
    fe_mul(&t1, &t2, &t1);
    fe_sqn(&t2, &t1, 10);
    fe_mul(&t2, &t2, &t1);
    fe_sqn(&t3, &t2, 20);
    fe_mul(&t2, &t3, &t2);
    fe_sqn(&t2, &t2, 10);
    fe_mul(&t1, &t2, &t1);
    fe_sqn(&t2, &t1, 50);
    fe_mul(&t2, &t2, &t1);
    fe_sqn(&t3, &t2, 100);
    fe_mul(&t2, &t3, &t2);
    fe_sqn(&t2, &t2, 50);
    fe_mul(&t1, &t2, &t1);
    fe_sqn(&t1, &t1, 5);
    fe_mul(out, &t1, &t0);
}

/* z^((p-5)/8): the chain of fe25519_pow22523, sodium_fe.cu:1410-1463 */
static void fe_pow22523(fe *out, const fe *z)
{
    fe t0, t1, t2;
    fe_sq(&t0, z);
    fe_sqn(&t1, &t0, 2);
    fe_mul(&t1, z, &t1);
    fe_mul(&t0, &t0, &t1);
    fe_sq(&t0, &t0);
    fe_mul(&t0, &t1, &t0);
    fe_sqn(&t1, &t0, 5);
    fe_mul(&t0, &t1, &t0);
    fe_sqn(&t1, &t0, 10);
    fe_mul(&t1, &t1, &t0);
    fe_sqn(&t2, &t1, 20);
    fe_mul(&t1, &t2, &t1);
    fe_sqn(&t1, &t1, 10);
    fe_mul(&t0, &t1, &t0);
    fe_sqn(&t1, &t0, 50);
    fe_mul(&t1, &t1, &t0);
    fe_sqn(&t2, &t1, 100);
    fe_mul(&t1, &t2, &t1);
    fe_sqn(&t1, &t1, 50);
    fe_mul(&t0, &t1, &t0);
    fe_sqn(&t0, &t0, 2);
    fe_mul(out, &t0, z);
}

/* ---------------------------------------------------------------- group -- */

static void ge_p3_0(ge_p3 *h) /* sodium_ge.cu:322 */
{
    fe_0(&h->X); fe_1(&h->Y); fe_1(&h->Z); fe_0(&h->T);
}

static void ge_cached_0(ge_cached *h) /* sodium_ge.cu:331 */
{
    fe_1(&h->YplusX); fe_1(&h->YminusX); fe_1(&h->Z); fe_0(&h->T2d);
}

static void ge_precomp_0(ge_precomp *h) /* sodium_ge.cu:408 */
{
    fe_1(&h->yplusx); fe_1(&h->yminusx); fe_0(&h->xy2d);
}

/* p + q, sodium_ge.cu:76-92 */
static void ge_add(ge_p1p1 *r, const ge_p3 *p, const ge_cached *q)
{
    fe t0;
    fe_add(&r->X, &p->Y, &p->X);
    fe_sub(&r->Y, &p->Y, &p->X);
    fe_mul(&r->Z, &r->X, &q->YplusX);
    fe_mul(&r->Y, &r->Y, &q->YminusX);
    fe_mul(&r->T, &q->T2d, &p->T);
    fe_mul(&r->X, &p->Z, &q->Z);
    fe_add(&t0, &r->X, &r->X);
    fe_sub(&r->X, &r->Z, &r->Y);
    fe_add(&r->Y, &r->Z, &r->Y);
    fe_add(&r->Z, &t0, &r->T);
    fe_sub(&r->T, &t0, &r->T);
}

/* p - q, sodium_ge.cu:517-533 */
static void ge_sub(ge_p1p1 *r, const ge_p3 *p, const ge_cached *q)
{
    fe t0;
    fe_add(&r->X, &p->Y, &p->X);
    fe_sub(&r->Y, &p->Y, &p->X);
    fe_mul(&r->Z, &r->X, &q->YminusX);
    fe_mul(&r->Y, &r->Y, &q->YplusX);
    fe_mul(&r->T, &q->T2d, &p->T);
    fe_mul(&r->X, &p->Z, &q->Z);
    fe_add(&t0, &r->X, &r->X);
    fe_sub(&r->X, &r->Z, &r->Y);
    fe_add(&r->Y, &r->Z, &r->Y);
    fe_sub(&r->Z, &t0, &r->T);
    fe_add(&r->T, &t0, &r->T);
}

/* p + q (q affine precomp), sodium_ge.cu:231-246 */
static void ge_madd(ge_p1p1 *r, const ge_p3 *p, const ge_precomp *q)
{
    fe t0;
    fe_add(&r->X, &p->Y, &p->X);
    fe_sub(&r->Y, &p->Y, &p->X);
    fe_mul(&r->Z, &r->X, &q->yplusx);
    fe_mul(&r->Y, &r->Y, &q->yminusx);
    fe_mul(&r->T, &q->xy2d, &p->T);
    fe_add(&t0, &p->Z, &p->Z);
    fe_sub(&r->X, &r->Z, &r->Y);
    fe_add(&r->Y, &r->Z, &r->Y);
    fe_add(&r->Z, &t0, &r->T);
    fe_sub(&r->T, &t0, &r->T);
}

static void ge_p1p1_to_p2(ge_p2 *r, const ge_p1p1 *p) /* sodium_ge.cu:273 */
{
    fe_mul(&r->X, &p->X, &p->T);
    fe_mul(&r->Y, &p->Y, &p->Z);
    fe_mul(&r->Z, &p->Z, &p->T);
}

static void ge_p1p1_to_p3(ge_p3 *r, const ge_p1p1 *p) /* sodium_ge.cu:285 */
{
    fe_mul(&r->X, &p->X, &p->T);
    fe_mul(&r->Y, &p->Y, &p->Z);
    fe_mul(&r->Z, &p->Z, &p->T);
    fe_mul(&r->T, &p->X, &p->Y);
}

static void ge_p2_dbl(ge_p1p1 *r, const ge_p2 *p) /* sodium_ge.cu:306-320 */
{
    fe t0;
    fe_sq(&r->X, &p->X);
    fe_sq(&r->Z, &p->Y);
    fe_sq2(&r->T, &p->Z);
    fe_add(&r->Y, &p->X, &p->Y);
    fe_sq(&t0, &r->Y);
    fe_add(&r->Y, &r->Z, &r->X);
    fe_sub(&r->Z, &r->Z, &r->X);
    fe_sub(&r->X, &t0, &r->Y);
    fe_sub(&r->T, &r->T, &r->Z);
}

static void ge_p3_to_p2(ge_p2 *r, const ge_p3 *p) /* sodium_ge.cu:374 */
{
    r->X = p->X; r->Y = p->Y; r->Z = p->Z;
}

static void ge_p3_dbl(ge_p1p1 *r, const ge_p3 *p) /* sodium_ge.cu:400 */
{
    ge_p2 q;
    ge_p3_to_p2(&q, p);
    ge_p2_dbl(r, &q);
}

static void ge_p3_to_cached(ge_cached *r, const ge_p3 *p) /* sodium_ge.cu:344 */
{
    fe_add(&r->YplusX, &p->Y, &p->X);
    fe_sub(&r->YminusX, &p->Y, &p->X);
    r->Z = p->Z;
    fe_mul(&r->T2d, &p->T, &FE_D2);
}

static void ge_p3_to_precomp(ge_precomp *pi, const ge_p3 *p) /* sodium_ge.cu:353 */
{
    fe recip, x, y, xy;
    fe_invert(&recip, &p->Z);
    fe_mul(&x, &p->X, &recip);
    fe_mul(&y, &p->Y, &recip);
    fe_add(&pi->yplusx, &y, &x);
    fe_sub(&pi->yminusx, &y, &x);
    fe_mul(&xy, &x, &y);
    fe_mul(&pi->xy2d, &xy, &FE_D2);
}

static void ge_p3_tobytes(uint8_t s[32], const ge_p3 *h) /* sodium_ge.cu:382 */
{
    fe recip, x, y;
    fe_invert(&recip, &h->Z);
    fe_mul(&x, &h->X, &recip);
    fe_mul(&y, &h->Y, &recip);
    fe_tobytes(s, &y);
    s[31] ^= (uint8_t)(fe_isnegative(&x) << 7);
}

/* ge25519_frombytes, sodium_ge.cu:137-180 (same arithmetic for failures) */
static int ge_frombytes(ge_p3 *h, const uint8_t s[32])
{
    fe u, v, v3, vxx, mchk, pchk, negx, xi;
    fe_frombytes(&h->Y, s);
    fe_1(&h->Z);
    fe_sq(&u, &h->Y);
    fe_mul(&v, &u, &FE_D);
    fe_sub(&u, &u, &h->Z);
    fe_add(&v, &v, &h->Z);
    fe_sq(&v3, &v);
    fe_mul(&v3, &v3, &v);
    fe_sq(&h->X, &v3);
    fe_mul(&h->X, &h->X, &v);
    fe_mul(&h->X, &h->X, &u);
    fe_pow22523(&h->X, &h->X);
    fe_mul(&h->X, &h->X, &v3);
    fe_mul(&h->X, &h->X, &u);
    fe_sq(&vxx, &h->X);
    fe_mul(&vxx, &vxx, &v);
    fe_sub(&mchk, &vxx, &u);
    fe_add(&pchk, &vxx, &u);
    int has_m = fe_iszero(&mchk);
    int has_p = fe_iszero(&pchk);
    fe_mul(&xi, &h->X, &FE_SQRTM1);
    fe_cmov(&h->X, &xi, 1 - has_m);
    fe_neg(&negx, &h->X);
    fe_cmov(&h->X, &negx, (unsigned)(fe_isnegative(&h->X) ^ (s[31] >> 7)));
    fe_mul(&h->T, &h->X, &h->Y);
    return (has_m | has_p) - 1;
}

/* --- constant-time table selection, sodium_ge.cu:416-511 --- */

static unsigned char ct_equal(signed char b, signed char c)
{
    unsigned char x = (unsigned char)b ^ (unsigned char)c;
    uint32_t y = x;
    y -= 1;
    y >>= 31;
    return (unsigned char)y;
}

static unsigned char ct_negative(signed char b)
{
    uint64_t x = (uint64_t)(int64_t)b;
    return (unsigned char)(x >> 63);
}

static void ge_cmov_cached(ge_cached *t, const ge_cached *u, unsigned char b)
{
    fe_cmov(&t->YplusX, &u->YplusX, b);
    fe_cmov(&t->YminusX, &u->YminusX, b);
    fe_cmov(&t->Z, &u->Z, b);
    fe_cmov(&t->T2d, &u->T2d, b);
}

static void ge_cmov8_cached(ge_cached *t, const ge_cached c[8], signed char b)
{
    ge_cached minust;
    unsigned char bneg = ct_negative(b);
    unsigned char babs = (unsigned char)(b - (((-bneg) & b) * 2));
    ge_cached_0(t);
    for (int k = 0; k < 8; ++k) ge_cmov_cached(t, &c[k], ct_equal((signed char)babs, (signed char)(k + 1)));
    minust.YplusX = t->YminusX;
    minust.YminusX = t->YplusX;
    minust.Z = t->Z;
    fe_neg(&minust.T2d, &t->T2d);
    ge_cmov_cached(t, &minust, bneg);
}

static void ge_cmov_precomp(ge_precomp *t, const ge_precomp *u, unsigned char b)
{
    fe_cmov(&t->yplusx, &u->yplusx, b);
    fe_cmov(&t->yminusx, &u->yminusx, b);
    fe_cmov(&t->xy2d, &u->xy2d, b);
}

static void ge_cmov8_precomp(ge_precomp *t, const ge_precomp p[8], signed char b)
{
    ge_precomp minust;
    unsigned char bneg = ct_negative(b);
    unsigned char babs = (unsigned char)(b - (((-bneg) & b) * 2));
    ge_precomp_0(t);
    for (int k = 0; k < 8; ++k) ge_cmov_precomp(t, &p[k], ct_equal((signed char)babs, (signed char)(k + 1)));
    minust.yplusx = t->yminusx;
    minust.yminusx = t->yplusx;
    fe_neg(&minust.xy2d, &t->xy2d);
    ge_cmov_precomp(t, &minust, bneg);
}

/* signed radix-16 recoding, sodium_ge.cu:693-708 */
static void recode16(signed char e[64], const uint8_t a[32])
{
    for (int i = 0; i < 32; ++i) {
        e[2 * i + 0] = (signed char)((a[i] >> 0) & 15);
        e[2 * i + 1] = (signed char)((a[i] >> 4) & 15);
    }
    signed char carry = 0;
    for (int i = 0; i < 63; ++i) {
        e[i] = (signed char)(e[i] + carry);
        carry = (signed char)((e[i] + 8) >> 4);
        e[i] = (signed char)(e[i] - carry * 16);
    }
    e[63] = (signed char)(e[63] + carry);
}

/* constant-time variable-base a*p, sodium_ge.cu:650-731 */
static void ge_scalarmult(ge_p3 *h, const uint8_t a[32], const ge_p3 *p)
{
    signed char e[64];
    ge_p1p1 r;
    ge_p2 s;
    ge_p1p1 t2, t3, t4, t5, t6, t7, t8;
    ge_p3 p2, p3, p4, p5, p6, p7, p8;
    ge_cached pi[8], t;

    ge_p3_to_cached(&pi[0], p);
    ge_p3_dbl(&t2, p);
    ge_p1p1_to_p3(&p2, &t2);
    ge_p3_to_cached(&pi[1], &p2);
    ge_add(&t3, p, &pi[1]);
    ge_p1p1_to_p3(&p3, &t3);
    ge_p3_to_cached(&pi[2], &p3);
    ge_p3_dbl(&t4, &p2);
    ge_p1p1_to_p3(&p4, &t4);
    ge_p3_to_cached(&pi[3], &p4);
    ge_add(&t5, p, &pi[3]);
    ge_p1p1_to_p3(&p5, &t5);
    ge_p3_to_cached(&pi[4], &p5);
    ge_p3_dbl(&t6, &p3);
    ge_p1p1_to_p3(&p6, &t6);
    ge_p3_to_cached(&pi[5], &p6);
    ge_add(&t7, p, &pi[5]);
    ge_p1p1_to_p3(&p7, &t7);
    ge_p3_to_cached(&pi[6], &p7);
    ge_p3_dbl(&t8, &p4);
    ge_p1p1_to_p3(&p8, &t8);
    ge_p3_to_cached(&pi[7], &p8);

    recode16(e, a);
    ge_p3_0(h);
    int i;
    for (i = 63; i != 0; i--) {
        ge_cmov8_cached(&t, pi, e[i]);
        ge_add(&r, h, &t);
        for (int k = 0; k < 4; ++k) {
            ge_p1p1_to_p2(&s, &r);
            ge_p2_dbl(&r, &s);
        }
        ge_p1p1_to_p3(h, &r);
    }
    ge_cmov8_cached(&t, pi, e[i]);
    ge_add(&r, h, &t);
    ge_p1p1_to_p3(h, &r);
}

/* base[i][j] = (j+1) * 256^i * B, the table of sodium_ge.cu:480-482,
 * regenerated here from the group law. */
static ge_precomp BASE_TABLE[32][8];
static ge_p3 GE_BASE;
static signed char L_SLIDE[256];

static const uint8_t ENC_BASE[32] = {
    0x58, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66,
    0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66,
    0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66};
static const uint8_t ENC_ZERO[32] = {1};

/* a*B by the signed-radix-16 comb, sodium_ge.cu:743-792 */
static void ge_scalarmult_base(ge_p3 *h, const uint8_t a[32])
{
    signed char e[64];
    ge_p1p1 r;
    ge_p2 s;
    ge_precomp t;
    recode16(e, a);
    ge_p3_0(h);
    for (int i = 1; i < 64; i += 2) {
        ge_cmov8_precomp(&t, BASE_TABLE[i / 2], e[i]);
        ge_madd(&r, h, &t);
        ge_p1p1_to_p3(h, &r);
    }
    ge_p3_dbl(&r, h);
    ge_p1p1_to_p2(&s, &r);
    ge_p2_dbl(&r, &s);
    ge_p1p1_to_p2(&s, &r);
    ge_p2_dbl(&r, &s);
    ge_p1p1_to_p2(&s, &r);
    ge_p2_dbl(&r, &s);
    ge_p1p1_to_p3(h, &r);
    for (int i = 0; i < 64; i += 2) {
        ge_cmov8_precomp(&t, BASE_TABLE[i / 2], e[i]);
        ge_madd(&r, h, &t);
        ge_p1p1_to_p3(h, &r);
    }
}

/* sliding-window signed digits, the recoding of slide_vartime,
 * sodium_ge.cu:95-135 (used only on the public group order) */
static void slide(signed char *r, const uint8_t *a)
{
    for (int i = 0; i < 256; ++i) r[i] = (signed char)(1 & (a[i >> 3] >> (i & 7)));
    for (int i = 0; i < 256; ++i) {
        if (!r[i]) continue;
        for (int b = 1; b <= 6 && i + b < 256; ++b) {
            if (!r[i + b]) continue;
            int ribs = r[i + b] << b;
            int cmp = r[i] + ribs;
            if (cmp <= 15) {
                r[i] = (signed char)cmp;
                r[i + b] = 0;
            } else {
                cmp = r[i] - ribs;
                if (cmp < -15) break;
                r[i] = (signed char)cmp;
                for (int k = i + b; k < 256; ++k) {
                    if (!r[k]) {
                        r[k] = 1;
                        break;
                    }
                    r[k] = 0;
                }
            }
        }
    }
}

/* L * A, the sequence of ge25519_mul_l, sodium_ge.cu:795-847 */
static void ge_mul_l(ge_p3 *r, const ge_p3 *A)
{
    ge_cached Ai[8];
    ge_p1p1 t;
    ge_p3 u, A2;
    ge_p3_to_cached(&Ai[0], A);
    ge_p3_dbl(&t, A);
    ge_p1p1_to_p3(&A2, &t);
    for (int k = 1; k < 8; ++k) {
        ge_add(&t, &A2, &Ai[k - 1]);
        ge_p1p1_to_p3(&u, &t);
        ge_p3_to_cached(&Ai[k], &u);
    }
    ge_p3_0(r);
    for (int i = 252; i >= 0; --i) {
        ge_p3_dbl(&t, r);
        if (L_SLIDE[i] > 0) {
            ge_p1p1_to_p3(&u, &t);
            ge_add(&t, &u, &Ai[L_SLIDE[i] / 2]);
        } else if (L_SLIDE[i] < 0) {
            ge_p1p1_to_p3(&u, &t);
            ge_sub(&t, &u, &Ai[(-L_SLIDE[i]) / 2]);
        }
        ge_p1p1_to_p3(r, &t);
    }
}

static int ge_is_on_curve(const ge_p3 *p) /* sodium_ge.cu:849-872 */
{
    fe x2, y2, z2, z4, t0, t1;
    fe_sq(&x2, &p->X);
    fe_sq(&y2, &p->Y);
    fe_sq(&z2, &p->Z);
    fe_sub(&t0, &y2, &x2);
    fe_mul(&t0, &t0, &z2);
    fe_mul(&t1, &x2, &y2);
    fe_mul(&t1, &t1, &FE_D);
    fe_sq(&z4, &z2);
    fe_add(&t1, &t1, &z4);
    fe_sub(&t0, &t0, &t1);
    return fe_iszero(&t0);
}

static int ge_is_on_main_subgroup(const ge_p3 *p) /* sodium_ge.cu:874-882 */
{
    ge_p3 pl;
    ge_mul_l(&pl, p);
    return fe_iszero(&pl.X);
}

/* --- helpers of the array layer, ftcrypto.cu:128-190 --- */

static void ge_zero(ge_p3 *z) { ge_frombytes(z, ENC_ZERO); } /* ftcrypto.cu:128 */

static void ge_addto(ge_p3 *dest, const ge_p3 *src) /* ftcrypto.cu:143 */
{
    ge_p1p1 s;
    ge_cached c;
    ge_p3_to_cached(&c, src);
    ge_add(&s, dest, &c);
    ge_p1p1_to_p3(dest, &s);
}

static void ge_subfrom(ge_p3 *dest, const ge_p3 *src) /* ftcrypto.cu:153 */
{
    ge_p1p1 s;
    ge_cached c;
    ge_p3_to_cached(&c, src);
    ge_sub(&s, dest, &c);
    ge_p1p1_to_p3(dest, &s);
}

static void ge_neg_quirk(ge_p3 *pt) /* ftcrypto.cu:163: negates Y and T */
{
    fe_neg(&pt->Y, &pt->Y);
    fe_neg(&pt->T, &pt->T);
}

static int ge_iszero(const ge_p3 *e) /* ftcrypto.cu:170 */
{
    fe ymz;
    fe_sub(&ymz, &e->Y, &e->Z);
    return fe_iszero(&e->X) && fe_iszero(&ymz);
}

static int ge_equal(const ge_p3 *a, const ge_p3 *b) /* ftcrypto.cu:184 */
{
    ge_p3 diff = *a;
    ge_subfrom(&diff, b);
    return ge_iszero(&diff);
}

/* --- packed128 <-> ge_p3 --- */

static void pt_load(ge_p3 *p, const uint8_t *s)
{
    fe_load(&p->X, s);
    fe_load(&p->Y, s + 32);
    fe_load(&p->Z, s + 64);
    fe_load(&p->T, s + 96);
}

static void pt_store(uint8_t *s, const ge_p3 *p)
{
    fe_store(s, &p->X);
    fe_store(s + 32, &p->Y);
    fe_store(s + 64, &p->Z);
    fe_store(s + 96, &p->T);
}

/* ------------------------------------------------------------- threads -- */

typedef void (*range_fn)(void *ctx, size_t lo, size_t hi);
struct job { range_fn fn; void *ctx; size_t lo, hi; };

static void *job_run(void *arg)
{
    struct job *j = (struct job *)arg;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}

static void parallel_for(size_t n, int threads, range_fn fn, void *ctx)
{
    if (threads <= 1 || n < 2) {
        fn(ctx, 0, n);
        return;
    }
    if ((size_t)threads > n) threads = (int)n;
    pthread_t tid[256];
    struct job jobs[256];
    if (threads > 256) threads = 256;
    for (int t = 0; t < threads; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].lo = n * (size_t)t / (size_t)threads;
        jobs[t].hi = n * (size_t)(t + 1) / (size_t)threads;
        pthread_create(&tid[t], NULL, job_run, &jobs[t]);
    }
    for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
}

/* ----------------------------------------------------------------- init -- */

static int g_inited = 0;

int fto_init(void)
{
    if (g_inited) return 0;
    ge_frombytes(&GE_BASE, ENC_BASE);
    ge_p3 row = GE_BASE;
    for (int i = 0; i < 32; ++i) {
        ge_p3 acc = row;
        ge_cached rc;
        ge_p3_to_cached(&rc, &row);
        for (int j = 0; j < 8; ++j) {
            ge_p3_to_precomp(&BASE_TABLE[i][j], &acc);
            ge_p1p1 t;
            ge_add(&t, &acc, &rc);
            ge_p1p1_to_p3(&acc, &t);
        }
        for (int k = 0; k < 8; ++k) { /* row <- 256 * row */
            ge_p1p1 t;
            ge_p3_dbl(&t, &row);
            ge_p1p1_to_p3(&row, &t);
        }
    }
    static const uint8_t L_BYTES[32] = {
        0xed, 0xd3, 0xf5, 0x5c, 0x1a, 0x63, 0x12, 0x58, 0xd6, 0x9c, 0xf7,
        0xa2, 0xde, 0xf9, 0xde, 0x14, 0x00, 0x00, 0x00, 0x00, 0x00, 0x00,
        0x00, 0x00, 0x00, 0x00, 0x00, 0x00, 0x00, 0x00, 0x00, 0x10};
    slide(L_SLIDE, L_BYTES);
    g_inited = 1;
    return 0;
}

/* ------------------------------------------------------------ array API -- */

void fto_encode(uint8_t *out32, const uint8_t *pts, size_t n)
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p;
        pt_load(&p, pts + 128 * i);
        ge_p3_tobytes(out32 + 32 * i, &p);
    }
}

/* The same canonical encodings as fto_encode, for large checks: each thread
 * encodes a contiguous range, inverting the Z coordinates of 64 points at a
 * time with one field inversion (Montgomery's simultaneous inversion:
 * prefix products, one inversion, then the inverses peeled off backwards).
 * A Z congruent to 0 is left out of the batch and gets the inverse 0, which
 * is what fe_invert returns for it (0^(p-2) = 0), so every encoding equals
 * ge_p3_tobytes's (sodium_ge.cu:382-394). */
#define ENC_BATCH 64
struct enc32_ctx { uint8_t *out; const uint8_t *pts; };

static void encode_range(void *vctx, size_t lo, size_t hi)
{
    struct enc32_ctx *c = (struct enc32_ctx *)vctx;
    ge_p3 p[ENC_BATCH];
    fe pre[ENC_BATCH], inv[ENC_BATCH];
    int zero[ENC_BATCH];
    for (size_t b0 = lo; b0 < hi; b0 += ENC_BATCH) {
        const size_t m = hi - b0 < ENC_BATCH ? hi - b0 : ENC_BATCH;
        fe acc;
        fe_1(&acc);
        for (size_t j = 0; j < m; ++j) {
            pt_load(&p[j], c->pts + 128 * (b0 + j));
            zero[j] = fe_iszero(&p[j].Z);
            pre[j] = acc; /* product of the non-zero Z before j */
            if (!zero[j]) fe_mul(&acc, &acc, &p[j].Z);
        }
        fe r;
        fe_invert(&r, &acc); /* 1 / (product of all non-zero Z) */
        for (size_t j = m; j-- > 0;) {
            if (zero[j]) {
                fe_0(&inv[j]);
                continue;
            }
            fe_mul(&inv[j], &r, &pre[j]); /* 1 / Z_j */
            fe_mul(&r, &r, &p[j].Z);     /* 1 / (product of the non-zero Z before j) */
        }
        for (size_t j = 0; j < m; ++j) {
            fe x, y;
            uint8_t *s = c->out + 32 * (b0 + j);
            fe_mul(&x, &p[j].X, &inv[j]);
            fe_mul(&y, &p[j].Y, &inv[j]);
            fe_tobytes(s, &y);
            s[31] ^= (uint8_t)(fe_isnegative(&x) << 7);
        }
    }
}

void fto_encode_mt(uint8_t *out32, const uint8_t *pts, size_t n, int threads)
{
    struct enc32_ctx c = {out32, pts};
    parallel_for(n, threads, encode_range, &c);
}

/* ftcrypto.cu:735-790: returns the last failing index, or -1 */
int64_t fto_decode(uint8_t *pts, const uint8_t *in32, size_t n)
{
    int64_t bad = -1;
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p;
        if (ge_frombytes(&p, in32 + 32 * i)) bad = (int64_t)i;
        pt_store(pts + 128 * i, &p);
    }
    return bad;
}

void fto_to_affine(uint8_t *out64, const uint8_t *pts, size_t n) /* ftcrypto.cu:659 */
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p;
        fe zi, x, y;
        pt_load(&p, pts + 128 * i);
        fe_invert(&zi, &p.Z);
        fe_mul(&x, &p.X, &zi);
        fe_mul(&y, &p.Y, &zi);
        fe_tobytes(out64 + 64 * i, &x);
        fe_tobytes(out64 + 64 * i + 32, &y);
    }
}

void fto_from_affine(uint8_t *pts, const uint8_t *in64, size_t n) /* ftcrypto.cu:793 */
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p;
        fe_frombytes(&p.X, in64 + 64 * i);
        fe_frombytes(&p.Y, in64 + 64 * i + 32);
        fe_1(&p.Z);
        fe_mul(&p.T, &p.X, &p.Y);
        pt_store(pts + 128 * i, &p);
    }
}

/* limb offsets of the reference's radix-2^25.5 fe25519 (sodium_fe.cu:30) */
static const int LIMB_OFF[10] = {0, 26, 51, 77, 102, 128, 153, 179, 204, 230};

static int64_t ld_le(const uint8_t *s, int nbytes)
{
    int64_t r = 0;
    for (int k = 0; k < nbytes; ++k) r |= (int64_t)s[k] << (8 * k);
    return r;
}

/* canonical value -> signed limbs: the load pattern and carry order of
 * fe25519_frombytes (sodium_fe.cu:74-141) applied to the canonical bytes */
static void fe_to_ref10(int32_t out[10], const fe *f)
{
    uint8_t s[32];
    fe_tobytes(s, f);
    int64_t h[10];
    h[0] = ld_le(s, 4);
    h[1] = ld_le(s + 4, 3) << 6;
    h[2] = ld_le(s + 7, 3) << 5;
    h[3] = ld_le(s + 10, 3) << 3;
    h[4] = ld_le(s + 13, 3) << 2;
    h[5] = ld_le(s + 16, 4);
    h[6] = ld_le(s + 20, 3) << 7;
    h[7] = ld_le(s + 23, 3) << 5;
    h[8] = ld_le(s + 26, 3) << 4;
    h[9] = (ld_le(s + 29, 3) & 8388607) << 2;
    int64_t carry;
    carry = (h[9] + (1LL << 24)) >> 25;
    h[0] += carry * 19;
    h[9] -= carry * (1LL << 25);
    for (int i = 1; i < 9; i += 2) {
        carry = (h[i] + (1LL << 24)) >> 25;
        h[i + 1] += carry;
        h[i] -= carry * (1LL << 25);
    }
    for (int i = 0; i < 10; i += 2) {
        carry = (h[i] + (1LL << 25)) >> 26;
        h[i + 1] += carry;
        h[i] -= carry * (1LL << 26);
    }
    for (int i = 0; i < 10; ++i) out[i] = (int32_t)h[i];
}

static void fe_from_ref10(fe *f, const int32_t in[10])
{
    /* sum limb_i * 2^off_i as a signed 320-bit integer, then reduce */
    int64_t acc[6] = {0}; /* 6 x 64-bit words, two's complement */
    for (int i = 0; i < 10; ++i) {
        int64_t l = in[i];
        int off = LIMB_OFF[i], w = off / 64, b = off % 64;
        __int128 v = (__int128)l * ((__int128)1 << b);
        /* add v (signed, < 2^(64+26)) at word w with sign extension */
        unsigned __int128 carry = 0;
        uint64_t add[6];
        uint64_t ext = v < 0 ? ~0ULL : 0ULL;
        for (int k = 0; k < 6; ++k) {
            if (k < w) add[k] = 0;
            else if (k == w) add[k] = (uint64_t)v;
            else if (k == w + 1) add[k] = (uint64_t)((unsigned __int128)v >> 64);
            else add[k] = ext;
        }
        for (int k = 0; k < 6; ++k) {
            carry += (unsigned __int128)(uint64_t)acc[k] + add[k];
            acc[k] = (int64_t)(uint64_t)carry;
            carry >>= 64;
        }
    }
    /* if negative, add 2^260 * p ... simpler: add 32p repeatedly is
     * unnecessary; use modular reduction of the two's-complement value:
     * value mod p = (acc mod 2^384) - 2^384 * sign, and 2^384 = 2^384 mod p. */
    int neg = acc[5] < 0;
    /* fold words 4,5 (value = lo256 + 2^256 * hi128): 2^256 = 38 mod p */
    fe lo = {{(uint64_t)acc[0], (uint64_t)acc[1], (uint64_t)acc[2], (uint64_t)acc[3]}};
    fe hi = {{(uint64_t)acc[4], (uint64_t)acc[5], 0, 0}};
    fe k38 = {{38, 0, 0, 0}}, t;
    fe_mul(&t, &hi, &k38);
    fe_add(f, &lo, &t);
    if (neg) {
        /* two's complement: we added 2^384 too much; 2^384 mod p = 2^129*19^... compute */
        fe two384 = {{0, 0, 0, 0}};
        /* 2^384 = 2^256 * 2^128 = 38 * 2^128 (mod p) */
        two384.v[2] = 38;
        fe_sub(f, f, &two384);
    }
}

void fto_to_ref160(uint8_t *out160, const uint8_t *pts, size_t n)
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p;
        pt_load(&p, pts + 128 * i);
        const fe *c[4] = {&p.X, &p.Y, &p.Z, &p.T};
        for (int k = 0; k < 4; ++k) {
            int32_t l[10];
            fe_to_ref10(l, c[k]);
            memcpy(out160 + 160 * i + 40 * k, l, 40);
        }
    }
}

void fto_from_ref160(uint8_t *pts, const uint8_t *in160, size_t n)
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p;
        fe *c[4] = {&p.X, &p.Y, &p.Z, &p.T};
        for (int k = 0; k < 4; ++k) {
            int32_t l[10];
            memcpy(l, in160 + 160 * i + 40 * k, 40);
            fe_from_ref10(c[k], l);
        }
        pt_store(pts + 128 * i, &p);
    }
}

void fto_set_zero(uint8_t *pts, size_t n)
{
    ge_p3 z;
    ge_zero(&z);
    for (size_t i = 0; i < n; ++i) pt_store(pts + 128 * i, &z);
}

struct smul_ctx { uint8_t *pts; const uint8_t *scalars; size_t sstride; const ge_p3 *base; int comb; };

static void smul_range(void *vctx, size_t lo, size_t hi)
{
    struct smul_ctx *c = (struct smul_ctx *)vctx;
    for (size_t i = lo; i < hi; ++i) {
        ge_p3 p, r;
        const uint8_t *s = c->scalars + c->sstride * i;
        if (c->comb) {
            ge_scalarmult_base(&r, s);
        } else {
            if (c->base) p = *c->base;
            else pt_load(&p, c->pts + 128 * i);
            ge_scalarmult(&r, s, &p);
        }
        pt_store(c->pts + 128 * i, &r);
    }
}

/* k_ft_array_from_scalars, ftcrypto.cu:895-913: s_i * B by the ladder */
void fto_from_scalars(uint8_t *pts, const uint8_t *scalars, size_t n, int threads)
{
    struct smul_ctx c = {pts, scalars, 32, &GE_BASE, 0};
    parallel_for(n, threads, smul_range, &c);
}

void fto_from_scalars_comb(uint8_t *pts, const uint8_t *scalars, size_t n, int threads)
{
    struct smul_ctx c = {pts, scalars, 32, NULL, 1};
    parallel_for(n, threads, smul_range, &c);
}

void fto_mul(uint8_t *pts, const uint8_t *scalars, size_t n, int threads) /* ftcrypto.cu:986 */
{
    struct smul_ctx c = {pts, scalars, 32, NULL, 0};
    parallel_for(n, threads, smul_range, &c);
}

void fto_scale(uint8_t *pts, const uint8_t *scalar, size_t n, int threads) /* ftcrypto.cu:966 */
{
    struct smul_ctx c = {pts, scalar, 0, NULL, 0};
    parallel_for(n, threads, smul_range, &c);
}

/* k * P for a public k < 2^64 by left-to-right double-and-add (p3
 * doubling, ge_addto for a set bit).  A faster stand-in for fto_scale with a
 * small scalar when checking large arrays: on the curve it gives the same
 * group element as the reference's ladder (ft_scale, ftcrypto.cu:966-983),
 * in other projective coordinates; compare canonical encodings only. */
struct scale64_ctx { uint8_t *pts; uint64_t k; };

static void scale64_range(void *vctx, size_t lo, size_t hi)
{
    struct scale64_ctx *c = (struct scale64_ctx *)vctx;
    int top = 63;
    while (top >= 0 && !((c->k >> top) & 1)) --top;
    for (size_t i = lo; i < hi; ++i) {
        ge_p3 p, acc;
        pt_load(&p, c->pts + 128 * i);
        ge_zero(&acc);
        for (int b = top; b >= 0; --b) {
            ge_p1p1 t;
            ge_p3_dbl(&t, &acc);
            ge_p1p1_to_p3(&acc, &t);
            if ((c->k >> b) & 1) ge_addto(&acc, &p);
        }
        pt_store(c->pts + 128 * i, &acc);
    }
}

void fto_scale_u64(uint8_t *pts, uint64_t k, size_t n, int threads)
{
    struct scale64_ctx c = {pts, k};
    parallel_for(n, threads, scale64_range, &c);
}

/* the same with a public k_i per point */
struct scale64e_ctx { uint8_t *pts; const uint64_t *k; };

static void scale64e_range(void *vctx, size_t lo, size_t hi)
{
    struct scale64e_ctx *c = (struct scale64e_ctx *)vctx;
    for (size_t i = lo; i < hi; ++i) {
        struct scale64_ctx one = {c->pts, c->k[i]};
        scale64_range(&one, i, i + 1);
    }
}

void fto_scale_u64_each(uint8_t *pts, const uint64_t *k, size_t n, int threads)
{
    struct scale64e_ctx c = {pts, k};
    parallel_for(n, threads, scale64e_range, &c);
}

struct add_ctx { uint8_t *res; const uint8_t *other; int sub; };

static void add_range(void *vctx, size_t lo, size_t hi)
{
    struct add_ctx *c = (struct add_ctx *)vctx;
    for (size_t i = lo; i < hi; ++i) {
        ge_p3 a, b;
        pt_load(&a, c->res + 128 * i);
        pt_load(&b, c->other + 128 * i);
        if (c->sub) ge_subfrom(&a, &b);
        else ge_addto(&a, &b);
        pt_store(c->res + 128 * i, &a);
    }
}

void fto_add(uint8_t *res, const uint8_t *summand, size_t n, int threads) /* ftcrypto.cu:1089 */
{
    struct add_ctx c = {res, summand, 0};
    parallel_for(n, threads, add_range, &c);
}

void fto_sub(uint8_t *res, const uint8_t *subtrahend, size_t n, int threads) /* ftcrypto.cu:1220 */
{
    struct add_ctx c = {res, subtrahend, 1};
    parallel_for(n, threads, add_range, &c);
}

void fto_neg(uint8_t *pts, size_t n) /* ftcrypto.cu:1244 */
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p;
        pt_load(&p, pts + 128 * i);
        ge_neg_quirk(&p);
        pt_store(pts + 128 * i, &p);
    }
}

void fto_index(int64_t *res, const uint8_t *pts, size_t n) /* ftcrypto.cu:1262 */
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p;
        pt_load(&p, pts + 128 * i);
        res[i] = !ge_iszero(&p);
    }
}

void fto_equal(int64_t *res, const uint8_t *a, const uint8_t *b, size_t n) /* ftcrypto.cu:1281 */
{
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p, q;
        pt_load(&p, a + 128 * i);
        pt_load(&q, b + 128 * i);
        res[i] = ge_equal(&p, &q);
    }
}

int64_t fto_validate(const uint8_t *pts, size_t n) /* ftcrypto.cu:859-892 */
{
    int64_t bad = -1;
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p;
        pt_load(&p, pts + 128 * i);
        if (!(ge_is_on_curve(&p) && ge_is_on_main_subgroup(&p))) bad = (int64_t)i;
    }
    return bad;
}

/* --- reductions (loop semantics of ftcrypto.c's array functions) --- */

struct red_ctx { const uint8_t *pts; ge_p3 *partial; size_t n; int threads; };

static void red_range(void *vctx, size_t lo, size_t hi)
{
    struct red_ctx *c = (struct red_ctx *)vctx;
    for (size_t t = lo; t < hi; ++t) {
        size_t a = c->n * t / (size_t)c->threads, b = c->n * (t + 1) / (size_t)c->threads;
        ge_p3 acc;
        ge_zero(&acc);
        for (size_t i = a; i < b; ++i) {
            ge_p3 p;
            pt_load(&p, c->pts + 128 * i);
            ge_addto(&acc, &p);
        }
        c->partial[t] = acc;
    }
}

/* sum of all points (ft_array_reduce, ftcrypto.cu:1447) */
void fto_reduce(uint8_t *out, const uint8_t *pts, size_t n, int threads)
{
    if (threads < 1) threads = 1;
    ge_p3 *partial = (ge_p3 *)calloc((size_t)threads, sizeof(ge_p3));
    struct red_ctx c = {pts, partial, n, threads};
    parallel_for((size_t)threads, threads, red_range, &c);
    ge_p3 acc;
    ge_zero(&acc);
    for (int t = 0; t < threads; ++t) ge_addto(&acc, &partial[t]);
    pt_store(out, &acc);
    free(partial);
}

/* inclusive (ft_array_scan) or exclusive (ft_array_prescan) prefix sums,
 * ftcrypto.h:416-429, restated serially */
void fto_scan(uint8_t *pts, size_t n, int exclusive)
{
    ge_p3 acc;
    ge_zero(&acc);
    for (size_t i = 0; i < n; ++i) {
        ge_p3 p;
        pt_load(&p, pts + 128 * i);
        if (exclusive) {
            pt_store(pts + 128 * i, &acc);
            ge_addto(&acc, &p);
        } else {
            ge_addto(&acc, &p);
            pt_store(pts + 128 * i, &acc);
        }
    }
}

/* fto_scan on `threads` threads, for large checks: each thread sums its
 * contiguous chunk, the chunk totals are prefixed serially, then each thread
 * rescans its chunk from its prefix.  The same group elements as the serial
 * scan (other projective coordinates): compare canonical encodings. */
struct scan_ctx { uint8_t *pts; size_t n; int threads; int exclusive; ge_p3 *part; int phase; };

static void scan_range(void *vctx, size_t lo, size_t hi)
{
    struct scan_ctx *c = (struct scan_ctx *)vctx;
    for (size_t t = lo; t < hi; ++t) {
        size_t a = c->n * t / (size_t)c->threads, b = c->n * (t + 1) / (size_t)c->threads;
        ge_p3 acc;
        if (c->phase == 0) {
            ge_zero(&acc);
            for (size_t i = a; i < b; ++i) {
                ge_p3 p;
                pt_load(&p, c->pts + 128 * i);
                ge_addto(&acc, &p);
            }
            c->part[t] = acc;
            continue;
        }
        acc = c->part[t];
        for (size_t i = a; i < b; ++i) {
            ge_p3 p;
            pt_load(&p, c->pts + 128 * i);
            if (c->exclusive) {
                pt_store(c->pts + 128 * i, &acc);
                ge_addto(&acc, &p);
            } else {
                ge_addto(&acc, &p);
                pt_store(c->pts + 128 * i, &acc);
            }
        }
    }
}

void fto_scan_mt(uint8_t *pts, size_t n, int exclusive, int threads)
{
    if (threads < 1) threads = 1;
    ge_p3 *part = (ge_p3 *)calloc((size_t)threads, sizeof(ge_p3));
    struct scan_ctx c = {pts, n, threads, exclusive, part, 0};
    parallel_for((size_t)threads, threads, scan_range, &c);
    ge_p3 run;
    ge_zero(&run);
    for (int t = 0; t < threads; ++t) { /* exclusive prefix of the chunk totals */
        ge_p3 tot = part[t];
        part[t] = run;
        ge_addto(&run, &tot);
    }
    c.phase = 1;
    parallel_for((size_t)threads, threads, scan_range, &c);
    free(part);
}

struct seg_ctx { uint8_t *out; const int32_t *off; const uint8_t *src; };

static void seg_range(void *vctx, size_t lo, size_t hi)
{
    struct seg_ctx *c = (struct seg_ctx *)vctx;
    for (size_t s = lo; s < hi; ++s) {
        ge_p3 acc;
        ge_zero(&acc);
        for (int64_t i = c->off[s]; i < c->off[s + 1]; ++i) {
            ge_p3 p;
            pt_load(&p, c->src + 128 * (size_t)i);
            ge_addto(&acc, &p);
        }
        pt_store(c->out + 128 * s, &acc);
    }
}

/* out[s] = sum of src[offsets[s] .. offsets[s+1]) — the row sums of
 * ft_sparse_matmul (ftcrypto.c:435-474) with contiguous rows */
void fto_segsum_csr(uint8_t *out, const int32_t *offsets, size_t nseg,
                    const uint8_t *src, int threads)
{
    struct seg_ctx c = {out, offsets, src};
    parallel_for(nseg, threads, seg_range, &c);
}

/* res[idxs[i]] += src[i] (ft_reduce_isum, ftcrypto.cu:1150-1217);
 * returns 4 (FT_ERR_OUT_OF_BOUNDS) if an index is out of range */
int fto_isum(uint8_t *res, size_t nres, const uint64_t *idxs, size_t n, const uint8_t *src)
{
    for (size_t i = 0; i < n; ++i)
        if (idxs[i] >= nres) return 4;
    for (size_t i = 0; i < n; ++i) {
        ge_p3 a, b;
        pt_load(&a, res + 128 * idxs[i]);
        pt_load(&b, src + 128 * i);
        ge_addto(&a, &b);
        pt_store(res + 128 * idxs[i], &a);
    }
    return 0;
}

struct enc_ctx { uint8_t *c1, *c2; const ge_p3 *pk; const uint64_t *m; const uint8_t *r; };

static void enc_range(void *vctx, size_t lo, size_t hi)
{
    struct enc_ctx *c = (struct enc_ctx *)vctx;
    for (size_t i = lo; i < hi; ++i) {
        uint8_t ms[32] = {0};
        for (int j = 0; j < 8; ++j) ms[j] = (uint8_t)(c->m[i] >> (8 * j));
        ge_p3 rb, rpk, mb;
        ge_scalarmult(&rb, c->r + 32 * i, &GE_BASE);
        ge_scalarmult(&rpk, c->r + 32 * i, c->pk);
        ge_scalarmult(&mb, ms, &GE_BASE);
        ge_addto(&mb, &rpk);
        pt_store(c->c1 + 128 * i, &rb);
        pt_store(c->c2 + 128 * i, &mb);
    }
}

int fto_encrypt(uint8_t *c1, uint8_t *c2, const uint8_t *pk32, const uint64_t *m,
                const uint8_t *r, size_t n, int threads)
{
    ge_p3 pk;
    if (ge_frombytes(&pk, pk32)) return 5; /* FT_ERR_INVALID_POINT */
    struct enc_ctx c = {c1, c2, &pk, m, r};
    parallel_for(n, threads, enc_range, &c);
    return 0;
}
