// internal.h — declarations shared by the host API (ft_api.cu) and the
// kernel translation units (k_*.cu).  Not installed; the public interface is
// include/ftcrypto.h and include/ftcrypto_gb300.h.
#pragma once
#include <atomic>
#include <cuda_runtime.h>
#include "windows.h"
#include <stddef.h>
#include <stdint.h>

#ifndef FT_PLANES
#define FT_PLANES 8
#endif
#define FT_PLANES_BYTES_PER_POINT ((size_t)FT_PLANES * 16)

// An array handle: device-resident structure-of-arrays planes (points.cuh).
// Allocated with new / freed with delete (ft_api.cu, serve.cu).
struct ft_ge25519_array_s {
    uint4 *planes = nullptr; // FT_PLANES planes of `cap` uint4 each (NULL when cap == 0)
    size_t n = 0;            // number of points
    size_t cap = 0;          // plane stride = number of points allocated
    // Host-side bookkeeping for exports that overlap queued work (ft_api.cu):
    // `touch` counts every hand-over of the storage to device work
    // (ft::view_of, reallocation, a batch run); `ready` is an event recorded
    // on the library stream right after a call that wrote the array marked
    // it (mark_ready), and stays valid while `touch` equals `ready_touch`.
    // `exposed`: the device address was handed out (ftx_array_device_view),
    // so writes the library does not see may follow and exports stay in
    // stream order.  `part` (valid with `ready`, when `part_end` > 0): an
    // event recorded after the marked call had written points [0, part_end),
    // so an export can copy that part while the rest is computed.
    mutable std::atomic<uint64_t> touch{0};
    cudaEvent_t ready = nullptr;
    uint64_t ready_touch = 0;
    cudaEvent_t part = nullptr;
    size_t part_end = 0;
    mutable std::atomic<bool> exposed{false};
    ft_ge25519_array_s() = default;
    ft_ge25519_array_s(const ft_ge25519_array_s &) = delete;
    ft_ge25519_array_s &operator=(const ft_ge25519_array_s &) = delete;
    ~ft_ge25519_array_s()
    {
        if (ready) cudaEventDestroy(ready);
        if (part) cudaEventDestroy(part);
    }
};

namespace ft {

// A view of n points starting at element `off` of an array.
// the dynamic shared-memory limit of a kernel, raised on its first launch
// (concurrent first launches from the serving worker and a caller thread
// may both set it, which is harmless)
struct SmemAttr {
    std::atomic<bool> done{false};
};
inline cudaError_t ensure_smem_attr(SmemAttr &a, const void *fn, size_t bytes)
{
    if (a.done.load(std::memory_order_acquire)) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) a.done.store(true, std::memory_order_release);
    return e;
}

struct View {
    uint4 *p;
    size_t s; // plane stride
};

inline View view_of(const ft_ge25519_array_s *a, size_t off = 0)
{
    a->touch.fetch_add(1, std::memory_order_relaxed);
    return View{a->planes + off, a->cap};
}

// ---- element-wise (k_elem.cu)
cudaError_t set_zero(View v, size_t n, cudaStream_t st);
// *acc = OR of v[0 .. n)
cudaError_t or_words(uint64_t *acc, const uint64_t *v, size_t n, cudaStream_t st);
cudaError_t broadcast(View dst, size_t n, View src, cudaStream_t st);
cudaError_t add(View res, View src, size_t n, int sub, cudaStream_t st);
// (r1, r2) +/-= (a1, a2) in one launch
cudaError_t add_ct(View r1, View r2, View a1, View a2, size_t n, int sub, cudaStream_t st);
cudaError_t neg(View v, size_t n, cudaStream_t st);
cudaError_t index_nonzero(int64_t *d_out, View v, size_t n, cudaStream_t st);
cudaError_t equal(int64_t *d_out, View a, View b, size_t n, int invert, cudaStream_t st);
cudaError_t mux(View t, const int64_t *d_cond, View f, size_t n, cudaStream_t st);
cudaError_t gather(View dst, View src, const uint64_t *d_idx, size_t n, cudaStream_t st);
cudaError_t scatter(View dst, View src, const uint64_t *d_idx, size_t n, cudaStream_t st);
cudaError_t scatter_zero(View dst, const uint64_t *d_idx, size_t n, cudaStream_t st);
cudaError_t gather_range(View dst, View src, size_t start, size_t step, size_t n, cudaStream_t st);
cudaError_t scatter_range(View dst, View src, size_t start, size_t step, size_t n, cudaStream_t st);
cudaError_t copy_points(View dst, View src, size_t n, cudaStream_t st);
cudaError_t encode(uint8_t *d_out32, View v, size_t n, cudaStream_t st);
cudaError_t decode(View v, const uint8_t *d_in32, size_t n, long long *d_bad, cudaStream_t st);
cudaError_t to_affine(uint8_t *d_out64, View v, size_t n, cudaStream_t st);
cudaError_t from_affine(View v, const uint8_t *d_in64, size_t n, cudaStream_t st);
cudaError_t to_ref160(uint8_t *d_out160, View v, size_t n, cudaStream_t st);
cudaError_t from_ref160(View v, const uint8_t *d_in160, size_t n, cudaStream_t st);
cudaError_t to_packed(uint8_t *d_out128, View v, size_t n, cudaStream_t st);
cudaError_t from_packed(View v, const uint8_t *d_in128, size_t n, cudaStream_t st);
cudaError_t validate(View v, size_t n, long long *d_bad, cudaStream_t st);

// ---- scalar multiplication (k_smul.cu)
// per-element (sc_step = 1) or broadcast (sc_step = 0) 32-byte scalars
cudaError_t smul_var(View v, size_t n, const uint8_t *d_scalars, int sc_step, cudaStream_t st);
// a_i * B by the radix-32 comb over B's table (btab, ENC_TABLE_WORDS words)
cudaError_t smul_base(View v, size_t n, const uint8_t *d_scalars, int sc_step, const uint32_t *btab, cudaStream_t st);
cudaError_t smul_base_small(View v, size_t n, const uint64_t *d_small, const uint32_t *btab, cudaStream_t st);
// ---- fixed-base products (k_encrypt.cu): the radix-32 comb (enc_comb.cuh)
// over tables of (j+1) * 32^row * Q, j < ENC_ENTRIES, row < ENC_ROWS (affine,
// 24 words per entry); the encryption tables are B's followed by PK's
constexpr size_t ENC_TABLE_WORDS = (size_t)ENC_ROWS * ENC_ENTRIES * 24;
constexpr size_t ENC_TABLES_BYTES = 2 * ENC_TABLE_WORDS * 4;
// the table of the point at element 0 of q
cudaError_t build_enc_table(uint32_t *d_table, View q, cudaStream_t st);
// c1 = r*B, c2 = m*B + r*PK
// ciphertexts one pass of the encryption grid takes (separate arrays)
size_t encrypt_pass();
cudaError_t encrypt(View c1, View c2, size_t n, const uint8_t *d_r, const uint64_t *d_m,
                    int m_digits, const uint32_t *d_tables, cudaStream_t st);
// (c1, c2) += (r*B, r*PK): a fresh encryption of zero added in place
cudaError_t rerandomise(View c1, View c2, size_t n, const uint8_t *d_r, const uint32_t *d_tables, cudaStream_t st);
// discrete-log table of j*B, j < m_max (k_elgamal.cu): open addressing over
// the canonical encodings, cap slots (a power of two >= 2 m_max)
struct DlogTable {
    uint32_t *state = nullptr; // 0 empty, else j + 1
    uint32_t *enc = nullptr;   // cap x 8 words
    uint64_t m_max = 0, cap = 0;
};
size_t dlog_table_bytes(uint64_t cap);
// fills a table laid out in `mem` (dlog_table_bytes(cap) bytes) mapping the
// encodings at d_enc (m_max x 32 bytes) to their indices: j*B for
// decryption, the points of an array for ft_array_contains
cudaError_t dlog_build(DlogTable &t, void *mem, uint64_t m_max, uint64_t cap, const uint8_t *d_enc, cudaStream_t st);
// m[i] = j where enc_i (n x 32 bytes) is the encoding of j*B, j < m_max; UINT64_MAX if none
cudaError_t dlog_lookup(uint64_t *d_m, const DlogTable &t, const uint8_t *d_enc, size_t n, cudaStream_t st);
cudaError_t iota_u64(uint64_t *d, size_t n, cudaStream_t st);
// ladder instantiations (k_ladder.cu) and the run-time block-size knob
cudaError_t ladder_launch_128(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step, cudaStream_t st);
cudaError_t ladder_launch_192(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step, cudaStream_t st);
cudaError_t ladder_launch_224(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step, cudaStream_t st);
cudaError_t ladder_launch_384(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step, cudaStream_t st);
cudaError_t ladder_launch_448(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step, cudaStream_t st);
size_t ladder_wave_384();
size_t ladder_wave_448();
size_t ladder_wave_128();
size_t ladder_wave_192();
size_t ladder_wave_224();
int ladder_block();
int set_ladder_block(int nt);
// points one wave of the current ladder launch holds (resident blocks x
// threads), 0 if unknown
size_t ladder_wave_points();

// ---- reductions (k_reduce.cu)
size_t reduce_scratch_bytes(size_t n);
cudaError_t reduce(View out, View src, size_t n, void *d_scratch, cudaStream_t st);
// scan: per-thread sums of scan_level_k(n) points, recursively, down to one
// block.  16 points per thread where the level fills the GPU (32 and 64
// measured slower: 1.61, 2.04 against 1.48 ms at 4M points); 4 on the
// latency-bound lower levels, whose cost is the chain of additions in one
// thread.
constexpr size_t SCAN_SMALL_MAX = 1024;
constexpr size_t scan_level_k(size_t n) { return n > ((size_t)1 << 18) ? 16 : 4; }
constexpr size_t scan_scratch_points(size_t n)
{
    return n <= SCAN_SMALL_MAX ? 0
                               : (n + scan_level_k(n) - 1) / scan_level_k(n) +
                                     scan_scratch_points((n + scan_level_k(n) - 1) / scan_level_k(n));
}
size_t scan_scratch_bytes(size_t n, int m = 1);
cudaError_t scan(View v, size_t n, int exclusive, void *d_scratch, cudaStream_t st);
// m (1 or 2) arrays of n points each scanned by the same launches
cudaError_t scan_set(const View *v, int m, size_t n, int exclusive, void *d_scratch, cudaStream_t st);
// out[s] (+)= sum of src[perm ? perm[e] : e] for e in [off[s], off[s+1])
size_t segsum_scratch_bytes(size_t nsrc, int m = 1);
cudaError_t segsum(View out, const int32_t *d_off, size_t nseg, View src, size_t nsrc,
                   const int32_t *d_perm, int accumulate, void *d_scratch, cudaStream_t st);
// m (1 or 2) segmented sums over the same offsets (out[i] from src[i]) by the
// same launches; scratch of segsum_scratch_bytes(nsrc, m)
cudaError_t segsum_set(const View *out, const View *src, int m, const int32_t *d_off, size_t nseg, size_t nsrc,
                       const int32_t *d_perm, int accumulate, void *d_scratch, cudaStream_t st);
// the same sums as segsum through one inclusive scan of the (gathered) points
// and a difference of two prefixes per segment: for layouts with long
// segments, which the walk's join adds up one thread part after another
bool segsum_prefers_prefix(size_t nsrc, size_t max_len);
size_t segsum_prefix_scratch_bytes(size_t nsrc);
cudaError_t segsum_prefix(View out, const int32_t *d_off, size_t nseg, View src, size_t nsrc,
                          const int32_t *d_perm, int accumulate, void *d_scratch, cudaStream_t st);
// *d_max = the largest segment length of a CSR layout
cudaError_t segment_maxlen(const int32_t *d_off, size_t nseg, int32_t *d_max, cudaStream_t st);
// counting sort of keys < nkeys: d_off (nkeys + 1) and d_perm (n); *d_bad set to
// the largest out-of-range position, or left at -1
size_t isum_scratch_bytes(size_t n, size_t nkeys);
cudaError_t keys_to_csr(int32_t *d_off, int32_t *d_perm, const uint64_t *d_keys, size_t n,
                        size_t nkeys, long long *d_bad, void *d_scratch, cudaStream_t st);

// ---- batched form (k_batch.cu)
enum : uint32_t { BATCH_ADD = 0, BATCH_SCALE = 1, BATCH_SEG = 2 };
struct BatchItem {
    uint32_t op;
    uint32_t count;       // points (ADD, SCALE) or segments (SEG) in this item
    uint4 *dst;           // planes of the first destination point
    size_t dst_s;
    const uint4 *src;     // ADD: summand; SEG: points the offsets index
    size_t src_s;
    const int32_t *off;   // SEG: count + 1 offsets into src
    uint32_t k;           // SCALE: the scalar
    uint32_t bits;        // SCALE: k < 2^bits
    uint32_t nwin;        // SCALE: ladder windows, u32_ladder_windows(bits, w) at upload
};
int batch_block();
size_t batch_smem_bytes();
// w: window width 2..4 of the scale items
cudaError_t batch_prepare(int w); // once, outside any stream capture
cudaError_t batch_launch(const BatchItem *d_items, int nitems, unsigned *d_counter, int w, cudaStream_t st);
// v[i] = k * v[i] in nwin constant-time windows (k < 2^bits, nwin for bits)
cudaError_t scale_small(View v, size_t n, uint32_t k, int nwin, int w, cudaStream_t st);

int sm_count();

} // namespace ft
