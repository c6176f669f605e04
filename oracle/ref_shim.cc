/*
 * ref_shim.cc — host build of the reference's own field/group arithmetic,
 * used only to pin the oracle (tests/golden/make_golden.py and
 * tests/test_oracle.py).  TEST INFRASTRUCTURE ONLY.
 *
 * It includes sodium_fe.cu and sodium_ge.cu from the reference source tree
 * (path given by FT_REF_SRC at compile time; see oracle/build_ref.sh) with the
 * CUDA qualifiers defined away, and exposes a small C ABI over 160-byte
 * ge25519_p3 structs (the reference's FT_EXTENDED_POINT_BYTES layout).
 * The four array-layer helpers of ftcrypto.cu:128-190 are re-expressed here
 * because ftcrypto.cu itself needs the CUDA runtime.
 */
#include <stdint.h>
#include <string.h>
#include <stddef.h>

#include "sodium_fe.cu"
#include "sodium_ge.cu"

static_assert(sizeof(ge25519_p3) == 160, "reference p3 layout");

static const unsigned char ZERO_ENC[32] = {1};
static const unsigned char GEN_ENC[32] = {
    0x58, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66,
    0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66,
    0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66, 0x66};

extern "C" {

int ref_decode(ge25519_p3 *h, const unsigned char *s) { return ge25519_frombytes(h, s); }
void ref_encode(unsigned char *s, const ge25519_p3 *h) { ge25519_p3_tobytes(s, h); }

void ref_zero(ge25519_p3 *h) { ge25519_frombytes(h, ZERO_ENC); }
void ref_base(ge25519_p3 *h) { ge25519_frombytes(h, GEN_ENC); }

void ref_scalarmult(ge25519_p3 *h, const unsigned char *a, const ge25519_p3 *p)
{
    ge25519_p3 q = *p;
    ge25519_scalarmult(h, a, &q);
}

void ref_scalarmult_base(ge25519_p3 *h, const unsigned char *a) { ge25519_scalarmult_base(h, a); }

void ref_addto(ge25519_p3 *dest, const ge25519_p3 *src)
{
    ge25519_p1p1 s;
    ge25519_cached c;
    ge25519_p3_to_cached(&c, src);
    ge25519_add(&s, dest, &c);
    ge25519_p1p1_to_p3(dest, &s);
}

void ref_subfrom(ge25519_p3 *dest, const ge25519_p3 *src)
{
    ge25519_p1p1 s;
    ge25519_cached c;
    ge25519_p3_to_cached(&c, src);
    ge25519_sub(&s, dest, &c);
    ge25519_p1p1_to_p3(dest, &s);
}

void ref_neg(ge25519_p3 *pt)
{
    fe25519_neg(pt->Y, pt->Y);
    fe25519_neg(pt->T, pt->T);
}

int ref_iszero(const ge25519_p3 *e)
{
    ge25519_p2 p2;
    ge25519_p3_to_p2(&p2, e);
    fe25519 ymz;
    fe25519_sub(ymz, p2.Y, p2.Z);
    return fe25519_iszero(p2.X) && fe25519_iszero(ymz);
}

int ref_equal(const ge25519_p3 *a, const ge25519_p3 *b)
{
    ge25519_p3 d = *a;
    ref_subfrom(&d, b);
    return ref_iszero(&d);
}

int ref_valid(const ge25519_p3 *p)
{
    return ge25519_is_on_curve(p) && ge25519_is_on_main_subgroup(p);
}

void ref_to_affine(unsigned char *out, const ge25519_p3 *p)
{
    fe25519 zi, x, y;
    fe25519_invert(zi, p->Z);
    fe25519_mul(x, p->X, zi);
    fe25519_mul(y, p->Y, zi);
    fe25519_tobytes(out, x);
    fe25519_tobytes(out + 32, y);
}

void ref_from_affine(ge25519_p3 *p, const unsigned char *in)
{
    fe25519_frombytes(p->X, in);
    fe25519_frombytes(p->Y, in + 32);
    fe25519_1(p->Z);
    fe25519_mul(p->T, p->X, p->Y);
}

/* canonical bytes of one coordinate of the reference's comb table entry */
void ref_base_table_entry(unsigned char *out96, int i, int j)
{
    const ge25519_precomp *e = &_ge25519_cmov8_base_precomp[i][j];
    fe25519_tobytes(out96, e->yplusx);
    fe25519_tobytes(out96 + 32, e->yminusx);
    fe25519_tobytes(out96 + 64, e->xy2d);
}

void ref_fe_tobytes(unsigned char *s, const int32_t *limbs) { fe25519_tobytes(s, limbs); }
void ref_fe_frombytes(int32_t *limbs, const unsigned char *s) { fe25519_frombytes(limbs, s); }

} /* extern "C" */
