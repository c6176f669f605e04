/*
 * ftoracle — CPU restatement of libftcrypto's Ed25519 arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is compared
 * against (and the timed CPU baseline of bench.py).  Nothing in the shipped
 * library links, loads or calls it.
 *
 * Parity is pinned: tests/test_oracle.py checks this restatement against
 * golden vectors produced by the reference's own host-compiled arithmetic
 * (sodium_fe.cu / sodium_ge.cu, built by oracle/build_ref.sh into
 * oracle/_ref/) and, where present, against libsodium (PyNaCl).
 *
 * Point buffers use the "packed128" layout shared with the GPU library:
 * X, Y, Z, T of an extended (p3) point, each a 32-byte little-endian integer
 * below 2^256 that is congruent to the coordinate mod p = 2^255 - 19.
 * Scalars are 32-byte little-endian.  Folded encodings are the canonical
 * 32-byte Ed25519 encoding (y, with the sign of x in bit 255).
 */
#ifndef FTORACLE_H
#define FTORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

int fto_init(void);

/* canonical encode (ge25519_p3_tobytes) / decode (ge25519_frombytes) */
void fto_encode(uint8_t *out32, const uint8_t *pts, size_t n);
int64_t fto_decode(uint8_t *pts, const uint8_t *in32, size_t n);
/* fto_encode on `threads` threads with batched inversion (same bytes) */
void fto_encode_mt(uint8_t *out32, const uint8_t *pts, size_t n, int threads);

/* affine (64 B: x || y) and reference-limb (160 B: 4 x 10 int32) formats */
void fto_to_affine(uint8_t *out64, const uint8_t *pts, size_t n);
void fto_from_affine(uint8_t *pts, const uint8_t *in64, size_t n);
void fto_to_ref160(uint8_t *out160, const uint8_t *pts, size_t n);
void fto_from_ref160(uint8_t *pts, const uint8_t *in160, size_t n);

/* constructors */
void fto_set_zero(uint8_t *pts, size_t n);
void fto_from_scalars(uint8_t *pts, const uint8_t *scalars, size_t n, int threads);
void fto_from_scalars_comb(uint8_t *pts, const uint8_t *scalars, size_t n, int threads);

/* elementwise */
void fto_add(uint8_t *res, const uint8_t *summand, size_t n, int threads);
void fto_sub(uint8_t *res, const uint8_t *subtrahend, size_t n, int threads);
void fto_neg(uint8_t *pts, size_t n);
void fto_mul(uint8_t *pts, const uint8_t *scalars, size_t n, int threads);
void fto_scale(uint8_t *pts, const uint8_t *scalar, size_t n, int threads);
/* k * P_i for a public k < 2^64 by double-and-add (same group element as
 * fto_scale; other projective coordinates) */
void fto_scale_u64(uint8_t *pts, uint64_t k, size_t n, int threads);
/* the same with a public k_i per point */
void fto_scale_u64_each(uint8_t *pts, const uint64_t *k, size_t n, int threads);
void fto_index(int64_t *res, const uint8_t *pts, size_t n);
void fto_equal(int64_t *res, const uint8_t *a, const uint8_t *b, size_t n);
int64_t fto_validate(const uint8_t *pts, size_t n);

/* reductions */
void fto_reduce(uint8_t *out, const uint8_t *pts, size_t n, int threads);
void fto_scan(uint8_t *pts, size_t n, int exclusive);
/* fto_scan on `threads` threads (chunk totals, then a rescan per chunk) */
void fto_scan_mt(uint8_t *pts, size_t n, int exclusive, int threads);
void fto_segsum_csr(uint8_t *out, const int32_t *offsets, size_t nseg,
                    const uint8_t *src, int threads);
int fto_isum(uint8_t *res, size_t nres, const uint64_t *idxs, size_t n,
             const uint8_t *src);

/* ElGamal encrypt in the reference's composition: c1 = r*B,
 * c2 = m*B + r*PK, each product by the variable-base ladder. */
int fto_encrypt(uint8_t *c1, uint8_t *c2, const uint8_t *pk32,
                const uint64_t *m, const uint8_t *r, size_t n, int threads);

#ifdef __cplusplus
}
#endif
#endif
