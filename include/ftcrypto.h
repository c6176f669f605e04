/*
 * ftcrypto.h — drop-in C interface of libftcrypto (batched additively
 * homomorphic ElGamal over Ed25519), implemented for NVIDIA GB300 (sm_103a)
 * by libftcrypto_gb300.
 *
 * Every declaration below replaces the declaration of the same name in the
 * reference's src/ftcrypto.h (the line given), with the same C signature,
 * argument meaning and error codes, so existing callers link against
 * libftcrypto.so unchanged.  Differences in behaviour are listed beside the
 * function; they concern inputs on which the reference crashes, writes out of
 * bounds or returns undefined results.
 *
 * Threading: one library CUDA stream per process; calls are not thread-safe
 * on the same handle.  Calls that only modify device arrays return before the
 * GPU work completes (as the reference's kernel launches do); calls that
 * return host data or a host-visible status synchronise first.
 */
#ifndef FT_GE25519_ARRAY
#define FT_GE25519_ARRAY

#include <stdint.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ftcrypto.h:19 */
#define FT_ED25519_SCALARBYTES 32
/* ftcrypto.h:25 */
#define FT_FOLDED_POINT_BYTES 32
/* ftcrypto.h:31: sizeof(ge25519_p3) in the reference, 4 x 10 x int32 limbs */
#define FT_EXTENDED_POINT_BYTES 160
/* ftcrypto.h:38 */
#define FT_AFFINE_POINT_BYTES (2 * FT_ED25519_SCALARBYTES)

/* ftcrypto.h:44-46: opaque handle to a device-resident array of points */
struct ft_ge25519_array_s;
typedef struct ft_ge25519_array_s *ft_ge25519_array;
typedef struct ft_ge25519_array_s const *const_ft_ge25519_array;

/* ftcrypto.h:51-63 */
typedef int ft_error;
#define FT_ERR_NO_ERROR 0
#define FT_ERR_OUT_OF_MEMORY 1
#define FT_ERR_SIZE_MISMATCH 2
#define FT_ERR_BAD_SIZE 3
#define FT_ERR_OUT_OF_BOUNDS 4
#define FT_ERR_INVALID_POINT 5
#define FT_ERR_SODIUM_INIT 6
#define FT_ERR_INSUFFICIENT_SPACE 7
#define FT_ERR_BAD_CIPHERTEXT 8
#define FT_ERR_INTERNAL_LIBRARY_ERROR 9
#define FT_ERR_INSUFFICIENT_DEVICE_OR_DRIVER 10
#define FT_ERR_MAX_ERR 10

/* ftcrypto.h:65 — same strings; "bad error value" outside 0..10 */
const char *ft_error_str(ft_error err);

/* ftcrypto.h:71 — checks for an sm_103 device and creates the library's
 * stream and memory pool.  Other calls initialise on first use as well.
 * CUDA errors are returned as codes; the library never exits the process
 * (the reference exits on any CUDA error, cuda_wrap.h:18-28). */
ft_error ft_crypto_init(void);

/* ftcrypto.h:76 */
ft_error ft_crypto_device_memory(size_t *free_mem, size_t *total_mem);

/* ftcrypto.h:86 — n_elts copies of scalar*B, or of the identity for NULL */
ft_error ft_array_init_scalar(ft_ge25519_array *array, size_t n_elts, const uint8_t *scalar);

/* ftcrypto.h:95 — n_elts copies of src[idx]; FT_ERR_OUT_OF_BOUNDS if
 * idx >= length(src) (unchecked in the reference) */
ft_error ft_array_init_point(ft_ge25519_array *array, size_t n_elts, const_ft_ge25519_array src, size_t idx);

/* ftcrypto.h:105 — FT_ERR_OUT_OF_BOUNDS for an index >= length(src) */
ft_error ft_array_get_subset(ft_ge25519_array *array, const size_t *idxs, size_t n_idxs, const_ft_ge25519_array src);

/* ftcrypto.h:116 — floor((stop - start) / step) elements, as the
 * reference's code computes (ftcrypto.cu:523; its comment says ceiling);
 * FT_ERR_BAD_SIZE for step == 0 with stop > start */
ft_error ft_array_get_range(ft_ge25519_array *array, size_t start, size_t stop, size_t step,
                            const_ft_ge25519_array src);

/* ftcrypto.h:124 */
ft_error ft_array_assign_to_subset(ft_ge25519_array array, const size_t *idxs, size_t n_idxs,
                                   const_ft_ge25519_array src);

/* ftcrypto.h:132 */
ft_error ft_array_assign_zero_to_subset(ft_ge25519_array array, const size_t *idxs, size_t n_idxs);

/* ftcrypto.h:139 */
ft_error ft_array_assign_to_range(ft_ge25519_array array, size_t start, size_t stop, size_t step,
                                  const_ft_ge25519_array src);

/* ftcrypto.h:147 — deletes the listed elements (duplicates and indices past
 * the end are ignored) */
ft_error ft_array_delete_subset(ft_ge25519_array array, const size_t *idxs, size_t n_idxs);

/* ftcrypto.h:154 — deletes start + i*step for start + i*step < stop */
ft_error ft_array_delete_range(ft_ge25519_array array, size_t start, size_t stop, size_t step);

/* ftcrypto.h:167 — canonical 32-byte encodings; writes length(array) * 32
 * bytes */
ft_error ft_array_to_bytes_folded(uint8_t *mem, size_t n_bytes, const_ft_ge25519_array array);

/* ftcrypto.h:180 — canonical x || y, 64 bytes per point */
ft_error ft_array_to_bytes_affine(uint8_t *mem, size_t n_bytes, const_ft_ge25519_array array);

/* ftcrypto.h:189 — 160 bytes per point in the reference's ge25519_p3 limb
 * layout (X, Y, Z, T as 10 x int32, radix 2^25.5), readable by the
 * reference's ft_array_from_bytes.  Limb values are those of the canonical
 * coordinates, so bytes are comparable with the reference's only after
 * folding. */
ft_error ft_array_to_bytes(uint8_t *mem, size_t n_bytes, const_ft_ge25519_array array);

/* ftcrypto.h:209 — *res = index of the last encoding that failed to decode,
 * or -1 */
ft_error ft_array_from_bytes_folded(int64_t *res, ft_ge25519_array *array, const uint8_t *mem, size_t n_bytes);

/* ftcrypto.h:228 — no validation (see ft_array_validate) */
ft_error ft_array_from_bytes_affine(ft_ge25519_array *array, const uint8_t *mem, size_t n_bytes);

/* ftcrypto.h:246 — accepts any limb values below 2^31 in magnitude; no
 * validation */
ft_error ft_array_from_bytes(ft_ge25519_array *array, const uint8_t *mem, size_t n_bytes);

/* ftcrypto.h:260 — on-curve and X(L*P) == 0, the reference's test;
 * *res = largest failing index or -1 */
ft_error ft_array_validate(int64_t *res, const_ft_ge25519_array array);

/* ftcrypto.h:274 — scalars[i] * B (fixed-base comb; constant time) */
ft_error ft_array_from_scalars(ft_ge25519_array *array, const uint8_t *scalars, size_t n_scalars);

/* ftcrypto.h:281 */
ft_error ft_array_from_small_scalars(ft_ge25519_array *array, const uint64_t *small_scalars, size_t n_scalars);

/* ftcrypto.h:288 — NULL is ignored */
void ft_array_free(ft_ge25519_array array);

/* ftcrypto.h:293 */
size_t ft_array_get_length(const_ft_ge25519_array array);

/* ftcrypto.h:307 — truncates, zero-extends, and reallocates when the new
 * length is at most half the old one or exceeds the reserve */
ft_error ft_array_set_length(ft_ge25519_array array, size_t newlen);

/* ftcrypto.h:314 */
ft_error ft_array_mux(ft_ge25519_array iftrue, const int64_t *cond, const_ft_ge25519_array iffalse);

/* ftcrypto.h:325 — compares canonical encodings (a device hash table of
 * array2's encodings probed by array1's, instead of the reference's O(n*m)
 * kernel) */
ft_error ft_array_contains(int64_t *res, const_ft_ge25519_array array1, const_ft_ge25519_array array2);

/* ftcrypto.h:334 — res[i] += summand[i]; res and summand may be the same
 * array */
ft_error ft_add(ft_ge25519_array res, const_ft_ge25519_array summand);

/* ftcrypto.h:344 — res[idxs[i]] += summand[i] for i < n_idxs; requires
 * n_idxs == length(summand) (the code's contract, ftcrypto.cu:1158) and
 * returns FT_ERR_OUT_OF_BOUNDS for an index >= length(res) without
 * modifying res.  Keys are sorted on the device. */
ft_error ft_reduce_isum(ft_ge25519_array res, const size_t *idxs, size_t n_idxs, const_ft_ge25519_array summand);

/* ftcrypto.h:353 */
ft_error ft_sub(ft_ge25519_array res, const_ft_ge25519_array summand);

/* ftcrypto.h:364 — constant time; requires scalar[31] <= 127 like the
 * reference (larger scalars give the reference's result).  Errors are
 * reported by ftx_last_error(). */
void ft_scale(ft_ge25519_array array, const uint8_t *scalar);

/* ftcrypto.h:371 — negates the Y and T coordinates, exactly as the
 * reference does (ftcrypto.cu:163-167).  NOTE: on Edwards curves -(x, y) is
 * (-x, y); the reference's (x, -y) is -P plus the 2-torsion point (0, -1).
 * Kept bit-exact for drop-in parity; use ft_sub for a true negation. */
void ft_neg(ft_ge25519_array array);

/* ftcrypto.h:382 — constant time per-element scalar multiplication */
ft_error ft_mul(ft_ge25519_array array, const uint8_t *scalars, size_t n_scalars);

/* ftcrypto.h:390 */
void ft_index(int64_t *res, const_ft_ge25519_array array);

/* ftcrypto.h:400 */
ft_error ft_equal(int64_t *res, const_ft_ge25519_array array1, const_ft_ge25519_array array2);

/* ftcrypto.h:411 */
ft_error ft_not_equal(int64_t *res, const_ft_ge25519_array array1, const_ft_ge25519_array array2);

/* ftcrypto.h:422 — exclusive prefix sums */
ft_error ft_array_prescan(ft_ge25519_array array);

/* ftcrypto.h:429 — inclusive prefix sums (correct at every length) */
ft_error ft_array_scan(ft_ge25519_array array);

/* ftcrypto.h:435 — array becomes the single-element array of its sum
 * (the identity for an empty array) */
ft_error ft_array_reduce(ft_ge25519_array array);

#ifdef __cplusplus
}
#endif

#endif /* FT_GE25519_ARRAY */
