/*
 * ftcrypto_gb300.h — extensions of the ftcrypto.h interface provided by
 * libftcrypto_gb300.  None of these replaces a reference function; they add
 * the ciphertext-level and device-pointer entry points that the batched and
 * serving forms use, and never change the behaviour of ftcrypto.h calls.
 */
#ifndef FTCRYPTO_GB300_H
#define FTCRYPTO_GB300_H

#include "ftcrypto.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Error code of the most recent call that has no return value (ft_scale,
 * ft_neg, ft_index). */
ft_error ftx_last_error(void);

/* The CUDA runtime error (a cudaError_t value) behind the most recent
 * FT_ERR_INTERNAL_LIBRARY_ERROR or FT_ERR_OUT_OF_MEMORY, 0 if none; a
 * diagnostic only. */
int ftx_last_cuda_error(void);

/* The library's CUDA stream (a cudaStream_t) on which every call runs. */
void *ftx_stream(void);

/* Waits for all work queued on the library's stream. */
ft_error ftx_synchronize(void);

/* Device address of the array's storage: 8 planes of 16-byte words, plane
 * k at planes + k * stride * 16 bytes; point i uses word i of every plane
 * (X, Y, Z, T, each as two 16-byte words, little-endian, below 2^256 and
 * congruent to the coordinate mod 2^255-19). */
ft_error ftx_array_device_view(const_ft_ge25519_array array, void **planes, size_t *stride);

/* 128 bytes per point: X, Y, Z, T as 32-byte little-endian integers (the
 * library's exact internal values; lossless and cheap). */
ft_error ftx_array_to_packed(uint8_t *mem, size_t n_bytes, const_ft_ge25519_array array);
ft_error ftx_array_from_packed(ft_ge25519_array *array, const uint8_t *mem, size_t n_bytes);

/* ft_mul with the n 32-byte scalars already in device memory. */
ft_error ftx_mul_device(ft_ge25519_array array, const uint8_t *d_scalars, size_t n_scalars);

/* ElGamal encryption of n plaintexts under the public key pk (a folded
 * 32-byte point): c1[i] = r_i * B, c2[i] = m_i * B + r_i * PK, constant
 * time in r_i and m_i.  Every m_i must be below 2^plaintext_bits
 * (1 <= plaintext_bits <= 64; FT_ERR_BAD_SIZE otherwise); r is n 32-byte
 * scalars.  The points equal the reference's composition
 * ft_array_from_scalars(r), ft_array_init_point(pk) + ft_mul(r),
 * ft_array_from_small_scalars(m) + ft_add.  FT_ERR_INVALID_POINT if pk does
 * not decode. */
ft_error ftx_encrypt(ft_ge25519_array *c1, ft_ge25519_array *c2, const uint8_t *pk, const uint64_t *m,
                     const uint8_t *r, size_t n, unsigned plaintext_bits);

/* ftx_encrypt into existing arrays of length n, with m and r already in
 * device memory (m_i < 2^plaintext_bits is not checked). */
ft_error ftx_encrypt_device(ft_ge25519_array c1, ft_ge25519_array c2, const uint8_t *pk, const uint64_t *d_m,
                            const uint8_t *d_r, size_t n, unsigned plaintext_bits);

/* Ciphertext add / subtract: (c1, c2) += (d1, d2) (resp. -=), element-wise,
 * both halves in one launch; the points equal ft_add(c1, d1) followed by
 * ft_add(c2, d2) (or ft_sub), also when arrays alias (then it runs as those
 * two calls).  Arrays of one length. */
ft_error ftx_ct_add(ft_ge25519_array c1, ft_ge25519_array c2, const_ft_ge25519_array d1, const_ft_ge25519_array d2);

/* Ciphertext prefix scan: ft_array_scan (exclusive == 0) or
 * ft_array_prescan (exclusive != 0) of c1 and of c2, both halves through the
 * same launches, so they share the scan's latency-bound lower levels
 * (ft_array_scan / ft_array_prescan, ftcrypto.cu:1474-1586, applied to each
 * half of a ciphertext array).  Arrays of one length; the same array passed
 * twice is scanned twice. */
ft_error ftx_ct_scan(ft_ge25519_array c1, ft_ge25519_array c2, int exclusive);
ft_error ftx_ct_sub(ft_ge25519_array c1, ft_ge25519_array c2, const_ft_ge25519_array d1, const_ft_ge25519_array d2);

/* Re-randomisation: (c1_i, c2_i) += (r_i * B, r_i * pk), a fresh encryption
 * of zero added in place, so the plaintexts are unchanged and the
 * ciphertexts unlinkable to the old ones.  r: n 32-byte nonces (host). */
ft_error ftx_rerandomise(ft_ge25519_array c1, ft_ge25519_array c2, const uint8_t *pk, const uint8_t *r, size_t n);

/* ftx_rerandomise with the nonces in device memory. */
ft_error ftx_rerandomise_device(ft_ge25519_array c1, ft_ge25519_array c2, const uint8_t *pk, const uint8_t *d_r,
                                size_t n);

/* Decryption of small plaintexts: m[i] is the j < m_max with
 * c2_i - sk * c1_i = j * B, or UINT64_MAX where there is none (a plaintext
 * >= m_max, or not a ciphertext under sk).  The discrete logarithm is a
 * lookup of the point's canonical encoding in a device table of j * B,
 * j < m_max, built on first use and kept for the next call with the same
 * m_max (about 80 bytes per entry).  FT_ERR_BAD_SIZE unless
 * 1 <= m_max <= FTX_DECRYPT_MAX_M; m: length(c1) entries (host). */
#define FTX_DECRYPT_MAX_M ((uint64_t)1 << 24)
ft_error ftx_decrypt(const_ft_ge25519_array c1, const_ft_ge25519_array c2, const uint8_t *sk, uint64_t m_max,
                     uint64_t *m);

/* Segmented sum over CSR offsets: out is a new array of nseg points with
 * out[s] = sum of src[offsets[s] .. offsets[s+1]) (the identity for an empty
 * segment).  offsets has nseg + 1 int32 entries, non-decreasing, from 0 to
 * length(src); FT_ERR_BAD_SIZE otherwise. */
ft_error ftx_segmented_sum_csr(ft_ge25519_array *out, const int32_t *offsets, size_t nseg,
                               const_ft_ge25519_array src);

/* The same with offsets in device memory, into an existing array of length
 * nseg (offsets are trusted). */
ft_error ftx_segmented_sum_csr_device(ft_ge25519_array out, const int32_t *d_offsets, size_t nseg,
                                      const_ft_ge25519_array src);

/* Ciphertext segmented sum: ftx_segmented_sum_csr_device of c1 into out1 and
 * of c2 into out2 over the same device offsets, both halves through the
 * same launches (the segmented sum of ft_reduce_isum, ftcrypto.cu:1113-1217,
 * over the CSR layout, applied to each half of a ciphertext array).  c1 and
 * c2 of one length, out1 and out2 of length nseg; where an output is the
 * other half's input or output the two sums run in order, as two calls
 * would (the second then reads what the first wrote). */
ft_error ftx_ct_segmented_sum_csr_device(ft_ge25519_array out1, ft_ge25519_array out2, const int32_t *d_offsets,
                                         size_t nseg, const_ft_ge25519_array c1, const_ft_ge25519_array c2);

/* out[out_idx] = sum of src, leaving src unchanged. */
ft_error ftx_reduce_into(ft_ge25519_array out, size_t out_idx, const_ft_ge25519_array src);

/* a[i] = k * a[i] for a public bound k < 2^32, constant time in k: nine
 * radix-16 windows of the reference's ladder instead of 64 (same points as
 * ft_scale with the 32-byte scalar k). */
ft_error ftx_scale_small(ft_ge25519_array array, uint32_t k);

/* ftx_scale_small for a declared public bound k < 2^bits (1 <= bits <= 32):
 * (bits + 1) / 4 + 1 windows instead of nine, constant time in k for a given
 * bits (3 windows for k < 1024).  FT_ERR_BAD_SIZE if k >= 2^bits. */
ft_error ftx_scale_bounded(ft_ge25519_array array, uint32_t k, unsigned bits);

/* Batched form: record many independent operations on arrays of any
 * lengths, then run them all in one persistent kernel launch replayed from a
 * CUDA graph.  The first ftx_batch_run uploads the work list and captures
 * the graph; later runs replay it (re-running every operation on the arrays'
 * current contents).  Operations of one batch run concurrently: an array
 * written by one operation must not appear in any other operation of the
 * batch (FT_ERR_BAD_SIZE at record time otherwise).  Arrays must stay
 * allocated and keep their storage while the batch exists: a run after
 * ft_array_set_length, ft_array_reduce or ft_array_delete_* changed a
 * recorded array returns FT_ERR_SIZE_MISMATCH and launches nothing.
 * Recording after the first run returns FT_ERR_BAD_SIZE. */
struct ftx_batch_s;
typedef struct ftx_batch_s *ftx_batch;
ft_error ftx_batch_create(ftx_batch *batch);
/* res[i] += summand[i] */
ft_error ftx_batch_add(ftx_batch batch, ft_ge25519_array res, const_ft_ge25519_array summand);
/* array[i] = k * array[i], k < 2^32 (as ftx_scale_small) */
ft_error ftx_batch_scale_small(ftx_batch batch, ft_ge25519_array array, uint32_t k);
/* array[i] = k * array[i], k < 2^bits (as ftx_scale_bounded) */
ft_error ftx_batch_scale_bounded(ftx_batch batch, ft_ge25519_array array, uint32_t k, unsigned bits);
/* out[s] = sum of src[offsets[s] .. offsets[s+1]) for s < nseg; out has
 * length nseg; offsets (host, copied) as for ftx_segmented_sum_csr */
ft_error ftx_batch_segmented_sum(ftx_batch batch, ft_ge25519_array out, const int32_t *offsets, size_t nseg,
                                 const_ft_ge25519_array src);
ft_error ftx_batch_run(ftx_batch batch);
/* number of work items and of operations recorded */
ft_error ftx_batch_info(ftx_batch batch, size_t *n_items, size_t *n_ops);
void ftx_batch_free(ftx_batch batch);

/* Serving form: a request loop with continuous batching.  A server owns a
 * public key, a budget of device memory and `slots` CUDA streams, the later
 * half of them at the device's highest stream priority (express slots).
 * Requests are queued by ftx_server_submit from any thread and admitted as
 * soon as a slot is free and their device memory (outputs, staged inputs,
 * scratch) fits in the budget: in arrival order among large requests, and
 * among small ones (work below a few milliseconds of GPU time), which use
 * the express slots first and may overtake queued large requests.  Admitted
 * requests run concurrently, so work of requests arriving while others are
 * on the GPU overlaps with theirs.  Ciphertexts stay on the device as handles: ENCRYPT and SEGSUM
 * create new arrays, RERAND and SMUL update the given arrays in place.  The
 * budget counts a request's temporaries while it runs and the arrays it
 * creates until the caller hands them back with ftx_server_release (which
 * frees them): outputs kept resident hold their share of the budget, and
 * requests wait for it (freeing such an array with ft_array_free while the
 * server lives leaves its bytes charged).  Host buffers named in a request
 * must stay valid until its result is returned; arrays of a request must not
 * be used elsewhere until then.  Results are bit-identical to the same
 * request run alone. */
#define FTX_REQ_ENCRYPT 1 /* (c1, c2) = Enc(m; r): n plaintexts < 2^bits (checked), n nonces */
#define FTX_REQ_RERAND 2  /* (c1, c2) += Enc(0; r) */
#define FTX_REQ_SMUL 3    /* (c1, c2) = k_i * (c1, c2), n 32-byte scalars, constant time */
#define FTX_REQ_SEGSUM 4  /* new (c1, c2) of nseg segment sums of the given arrays */
typedef struct {
    int op;
    size_t n;                /* ciphertexts */
    const uint64_t *m;       /* ENCRYPT */
    unsigned plaintext_bits; /* ENCRYPT */
    const uint8_t *r;        /* ENCRYPT, RERAND: n x 32 bytes */
    const uint8_t *k;        /* SMUL: n x 32 bytes */
    const int32_t *offsets;  /* SEGSUM: nseg + 1 offsets */
    size_t nseg;             /* SEGSUM */
    ft_ge25519_array c1, c2; /* RERAND, SMUL (updated); SEGSUM (source) */
} ftx_request;
typedef struct {
    ft_error err;
    ft_ge25519_array c1, c2; /* the request's output arrays */
    double queue_ms;         /* submit -> admitted */
    double latency_ms;       /* submit -> GPU work complete */
} ftx_result;
struct ftx_server_s;
typedef struct ftx_server_s *ftx_server;
ft_error ftx_server_create(ftx_server *server, const uint8_t *pk, size_t hbm_budget_bytes, int slots);
/* FT_ERR_INSUFFICIENT_SPACE if the request alone exceeds the budget */
ft_error ftx_server_submit(ftx_server server, const ftx_request *req, uint64_t *ticket);
/* blocks until the request completes */
ft_error ftx_server_wait(ftx_server server, uint64_t ticket, ftx_result *result);
/* frees an array that a request of this server created (a result's c1 or
 * c2) and returns its bytes to the budget; FT_ERR_OUT_OF_BOUNDS for an array
 * the server does not hold (not its output, or already released) */
ft_error ftx_server_release(ftx_server server, ft_ge25519_array array);
/* bytes of the budget in use (running requests, and outputs not yet
 * released) and requests queued / running */
ft_error ftx_server_stats(ftx_server server, size_t *bytes_in_use, size_t *queued, size_t *running);
/* waits for every request; frees the new arrays of results never collected
 * (collected, unreleased outputs stay valid; the caller frees them) */
void ftx_server_free(ftx_server server);

/* Launch-shape knobs, set by the autotuner (libftcrypto_gb300/autotune.py)
 * or by hand.  ftx_tune returns FT_ERR_BAD_SIZE for an unsupported value;
 * ftx_tune_get returns the current value (-1 for an unknown knob). */
#define FTX_TUNE_LADDER_BLOCK 1  /* variable-base ladder block size: 128, 192, 224 (tables in shared
                                    memory) or 384, 448 (tables half in tensor memory) */
#define FTX_TUNE_BATCH_ADD_PTS 2 /* batched form: points per thread of an ADD item (1..64) */
#define FTX_TUNE_SCALE_WINDOW 3  /* window width of the small-scalar ladder (ftx_scale_bounded and the
                                    batched scale; 2, 3 or 4 bits; a batch takes it at its first run) */
ft_error ftx_tune(int knob, int value);
int ftx_tune_get(int knob);

/* Prefix scan (exclusive if `exclusive` is non-zero, else inclusive) of n
 * points that the caller keeps in its own device memory, in this library's
 * layout (8 planes of 16-byte words, plane stride `stride` >= n, see
 * ftx_array_device_view), queued on the caller's CUDA stream.  No
 * counterpart in the reference: it exists for callers that cannot allocate
 * device memory (their memory is held by another allocator, or they must not
 * trigger cudaMalloc's synchronisation).  It allocates nothing; the scan's
 * scratch is a fixed array of about 11 MB that the library keeps on every
 * GPU that loads it.  n <= FT_NOALLOC_SCAN_MAX_POINTS (FT_ERR_BAD_SIZE
 * otherwise).  All calls share that array: calls that overlap on the GPU
 * race and must be serialised.  The first call on a device looks up the
 * array's address and keeps it for the life of the process; make it before
 * any stream capture.  A cudaDeviceReset of that device is not supported
 * afterwards (the array may move when the module is loaded again). */
#define FT_NOALLOC_SCAN_MAX_POINTS 1048576
ft_error ftx_scan_noalloc(void *d_planes, size_t stride, size_t n, int exclusive, void *stream);

#ifdef __cplusplus
}
#endif

#endif
