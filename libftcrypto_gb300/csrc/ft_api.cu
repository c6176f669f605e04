// ft_api.cu — the C ABI of include/ftcrypto.h and include/ftcrypto_gb300.h.
//
// Host logic for every entry point: argument checks with the reference's
// error codes, stream-ordered device allocation from a private memory pool,
// host<->device staging, and kernel launches (k_elem.cu, k_smul.cu,
// k_reduce.cu).  All work is queued on one library stream; calls that return
// host data synchronise that stream.  CUDA failures become FT_ERR_* codes;
// nothing here exits the process.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <set>
#include <vector>

#include "internal.h"
#include "../../include/ftcrypto.h"
#include "../../include/ftcrypto_gb300.h"

using ft::View;

namespace {

struct Ctx {
    bool inited = false;
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;
    void *scratch = nullptr;
    size_t scratch_cap = 0;
    long long *d_status = nullptr; // one device word for "last bad index"
    ft_error last_void = FT_ERR_NO_ERROR;
    // encryption tables (B's and a public key's) of the last PK_CACHE keys
    // used, least recently used replaced: a table costs ~0.55 ms to build
    // (255 doublings in sequence for its last row), so callers alternating
    // between a few keys build each once
    struct KeyTab {
        uint8_t pk[32];
        uint32_t *table = nullptr;
        uint64_t used = 0; // 0: empty
    };
    static constexpr int PK_CACHE = 4;
    KeyTab keys[PK_CACHE];
    uint64_t key_clock = 0;
    uint32_t *b_table = nullptr;  // radix-32 comb table of B (fixed-base products)
    void *dlog_mem = nullptr;     // decryption table of j*B, j < dlog.m_max
    ft::DlogTable dlog;
    // Transfers that overlap queued kernels (see export_begin, stage_scalars):
    // a second stream at the device's highest priority, an export buffer used
    // only on it, and two staging buffers for host scalars, each with the
    // events of its copy and of the kernel that read it.
    cudaStream_t xfer = nullptr;
    void *xscratch = nullptr;
    size_t xscratch_cap = 0;
    struct Stage {
        void *p = nullptr;
        size_t cap = 0;
        cudaEvent_t copied = nullptr, consumed = nullptr;
    };
    Stage stage[2];
    int stage_next = 0;
    // ftx_encrypt's input copies: the first part's on the library stream,
    // the rest's on the transfer stream
    cudaEvent_t in_ev[2] = {nullptr, nullptr};
};

Ctx g;
std::mutex g_init_mu;

std::atomic<int> g_last_cuda{0};

ft_error map_err(cudaError_t e)
{
    g_last_cuda.store((int)e);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? FT_ERR_OUT_OF_MEMORY : FT_ERR_INTERNAL_LIBRARY_ERROR;
}

#define CK(x)                                           \
    do {                                                \
        cudaError_t _e = (x);                           \
        if (_e != cudaSuccess) return map_err(_e);      \
    } while (0)

#define ENSURE_INIT()                                   \
    do {                                                \
        if (!g.inited) {                                \
            ft_error _ie = ft_crypto_init();            \
            if (_ie) return _ie;                        \
        }                                               \
    } while (0)

cudaError_t dev_alloc(void **p, size_t bytes)
{
    *p = nullptr;
    if (bytes == 0) return cudaSuccess;
    return cudaMallocFromPoolAsync(p, bytes, g.pool, g.stream);
}

void dev_free(void *p)
{
    if (p) cudaFreeAsync(p, g.stream);
}

// scratch of at least `bytes`, valid until the next scratch() call; stream
// ordering makes reuse across calls safe
cudaError_t scratch(void **p, size_t bytes)
{
    if (bytes > g.scratch_cap) {
        dev_free(g.scratch);
        g.scratch = nullptr;
        g.scratch_cap = 0;
        size_t cap = std::max(bytes, (size_t)1 << 20);
        cudaError_t e = dev_alloc(&g.scratch, cap);
        if (e != cudaSuccess) return e;
        g.scratch_cap = cap;
    }
    *p = g.scratch;
    return cudaSuccess;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

bool host_is_pinned(const void *p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// (Kernels writing exports straight into pinned caller memory over the
// host link measured 10x slower than the conversion into device memory
// followed by one copy: 13.1 against 1.24 ms for 1,048,576 raw points.)

// copy from caller memory: the caller may reuse `src` when this returns
cudaError_t h2d(void *dst, const void *src, size_t bytes)
{
    if (bytes == 0) return cudaSuccess;
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g.stream);
    if (e != cudaSuccess) return e;
    // a pageable source is staged before cudaMemcpyAsync returns; a pinned
    // one is read by DMA later, so wait for it
    if (host_is_pinned(src)) e = cudaStreamSynchronize(g.stream);
    return e;
}

cudaError_t d2h(void *dst, const void *src, size_t bytes, cudaStream_t st = nullptr)
{
    if (!st) st = g.stream;
    if (bytes) {
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
    }
    return cudaStreamSynchronize(st);
}

static cudaError_t record_on_stream(cudaEvent_t *ev)
{
    if (!*ev) {
        cudaError_t e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            *ev = nullptr;
            return e;
        }
    }
    return cudaEventRecord(*ev, g.stream);
}

// Marks that the work queued so far on the library stream has written a's
// points [0, end), the first part of a write that mark_ready(a, end) then
// completes: an export that follows copies that part while the rest is
// computed.
cudaError_t mark_part(ft_ge25519_array a)
{
    if (a->exposed.load()) return cudaSuccess;
    return record_on_stream(&a->part);
}

// Marks that the work just queued on the library stream completes a's
// writes: an export of a that follows, with no other use of a in between,
// waits for this point only (export_begin), not for everything queued after.
// part_end > 0: the call marked its first part [0, part_end) (mark_part).
cudaError_t mark_ready(ft_ge25519_array a, size_t part_end = 0)
{
    if (a->exposed.load()) return cudaSuccess;
    const uint64_t t = a->touch.load();
    const cudaError_t e = record_on_stream(&a->ready);
    a->ready_touch = e == cudaSuccess ? t : UINT64_MAX; // a failed mark keeps exports in order
    a->part_end = e == cudaSuccess ? part_end : 0;
    return e;
}

// The stream and the device buffer (at least `bytes`) an export of a
// converts and copies on.  When the call that last wrote a marked it and
// nothing has used a since, that is the transfer stream after a wait for
// the mark: the conversion and the device-to-host copy then overlap kernels
// queued later on the library stream (an export of c1 runs during the
// scalar multiplication of c2).  Otherwise the library stream and its
// scratch, in order.  The export buffer is only ever used on the transfer
// stream, and every export ends with that stream synchronised.
// *cut > 0: the marked call recorded its first part [0, *cut) (mark_part);
// the transfer stream then waits for that part only, and the caller makes
// it wait for the mark before it touches points from *cut on.
cudaError_t export_begin(const_ft_ge25519_array a, size_t bytes, void **buf, cudaStream_t *st, size_t *cut)
{
    *cut = 0;
    const bool side = a->ready && !a->exposed.load() && a->touch.load() == a->ready_touch;
    if (!side) {
        *st = g.stream;
        return scratch(buf, bytes);
    }
    cudaError_t e;
    if (bytes > g.xscratch_cap) {
        if (g.xscratch) cudaFreeAsync(g.xscratch, g.xfer);
        g.xscratch = nullptr;
        g.xscratch_cap = 0;
        size_t cap = std::max(bytes, (size_t)1 << 20);
        if ((e = cudaMallocFromPoolAsync(&g.xscratch, cap, g.pool, g.xfer)) != cudaSuccess) return e;
        g.xscratch_cap = cap;
    }
    const bool parts = a->part && a->part_end > 0 && a->part_end < a->n;
    if ((e = cudaStreamWaitEvent(g.xfer, parts ? a->part : a->ready, 0)) != cudaSuccess) return e;
    *buf = g.xscratch;
    *st = g.xfer;
    *cut = parts ? a->part_end : 0;
    return cudaSuccess;
}

// the storage of a from point `off` as a view, without counting a use (an
// export reads it on the stream export_begin chose)
View export_view(const_ft_ge25519_array a, size_t off = 0) { return View{a->planes + off, a->cap}; }

// An export to host memory: conv(out, view, count, stream) writes bpp bytes
// per point into the export buffer, which is copied to mem.  Where the call
// that wrote a marked a first part, that part is converted and copied as
// soon as it is written, then the rest after the mark.
template <class Conv>
ft_error export_to_host(uint8_t *mem, const_ft_ge25519_array a, size_t bpp, Conv conv)
{
    const size_t n = a->n;
    void *s;
    cudaStream_t st;
    size_t cut;
    CK(export_begin(a, align256(n * bpp), &s, &st, &cut));
    size_t start = 0;
    for (const size_t end : {cut, n}) {
        if (end == start) continue;
        if (start) CK(cudaStreamWaitEvent(st, a->ready, 0));
        uint8_t *buf = (uint8_t *)s + start * bpp;
        CK(conv(buf, export_view(a, start), end - start, st));
        CK(cudaMemcpyAsync(mem + start * bpp, buf, (end - start) * bpp, cudaMemcpyDeviceToHost, st));
        start = end;
    }
    CK(cudaStreamSynchronize(st));
    return FT_ERR_NO_ERROR;
}

// Copies `bytes` of pinned host memory into one of two staging buffers on
// the transfer stream, so that the copy overlaps kernels already queued on
// the library stream.  A buffer is refilled only after the kernel that last
// read it has finished (its `consumed` event, which the caller records after
// the kernel that reads this copy), and the library stream waits for the
// copy (`copied`) before that kernel.  The caller waits for `copied` before
// returning, so its buffer may be reused at once.
cudaError_t stage_scalars(void **out, Ctx::Stage **sgp, const void *src, size_t bytes)
{
    Ctx::Stage &sg = g.stage[g.stage_next];
    g.stage_next ^= 1;
    cudaError_t e;
    if (!sg.copied) {
        cudaEvent_t c1 = nullptr, c2 = nullptr;
        if ((e = cudaEventCreateWithFlags(&c1, cudaEventDisableTiming)) != cudaSuccess) return e;
        if ((e = cudaEventCreateWithFlags(&c2, cudaEventDisableTiming)) != cudaSuccess) {
            cudaEventDestroy(c1);
            return e;
        }
        sg.copied = c1;
        sg.consumed = c2; // never recorded yet: a wait on it returns at once
    }
    if (bytes > sg.cap) {
        // a kernel queued earlier may still read the old buffer: it is freed
        // in the library stream's order, after that kernel
        if (sg.p) cudaFreeAsync(sg.p, g.stream);
        sg.p = nullptr;
        sg.cap = 0;
        size_t cap = std::max(bytes, (size_t)1 << 20);
        if ((e = cudaMallocFromPoolAsync(&sg.p, cap, g.pool, g.xfer)) != cudaSuccess) return e;
        sg.cap = cap;
    }
    if ((e = cudaStreamWaitEvent(g.xfer, sg.consumed, 0)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(sg.p, src, bytes, cudaMemcpyHostToDevice, g.xfer)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(sg.copied, g.xfer)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(g.stream, sg.copied, 0)) != cudaSuccess) return e;
    *out = sg.p;
    *sgp = &sg;
    return cudaSuccess;
}

// arrays whose byte sizes (160 per point at most, in exports) overflow size_t
// can never be allocated; refusing them keeps every size product exact
bool too_long(size_t n) { return n > SIZE_MAX / 256; }

ft_error arr_new(ft_ge25519_array *out, size_t n)
{
    if (too_long(n)) return FT_ERR_OUT_OF_MEMORY;
    auto *a = new (std::nothrow) ft_ge25519_array_s();
    if (!a) return FT_ERR_OUT_OF_MEMORY;
    a->n = n;
    a->cap = n;
    cudaError_t e = dev_alloc((void **)&a->planes, n * FT_PLANES_BYTES_PER_POINT);
    if (e != cudaSuccess) {
        delete a;
        return map_err(e);
    }
    *out = a;
    return FT_ERR_NO_ERROR;
}

// replace the storage of a with a fresh buffer of `cap` points holding the
// first `keep` points of the old one
ft_error arr_realloc(ft_ge25519_array a, size_t cap, size_t keep)
{
    if (too_long(cap)) return FT_ERR_OUT_OF_MEMORY;
    uint4 *np = nullptr;
    CK(dev_alloc((void **)&np, cap * FT_PLANES_BYTES_PER_POINT));
    cudaError_t e = ft::copy_points(View{np, cap}, ft::view_of(a), std::min(keep, cap), g.stream);
    if (e != cudaSuccess) {
        dev_free(np);
        return map_err(e);
    }
    dev_free(a->planes);
    a->planes = np;
    a->cap = cap;
    return FT_ERR_NO_ERROR;
}

template <class F>
ft_error with_new_array(ft_ge25519_array *out, size_t n, F fill)
{
    ft_ge25519_array a;
    ft_error err = arr_new(&a, n);
    if (err) return err;
    err = fill(a);
    if (err) {
        ft_array_free(a);
        return err;
    }
    *out = a;
    return FT_ERR_NO_ERROR;
}

ft_error check_idxs(const size_t *idxs, size_t n, size_t bound)
{
    for (size_t i = 0; i < n; ++i)
        if (idxs[i] >= bound) return FT_ERR_OUT_OF_BOUNDS;
    return FT_ERR_NO_ERROR;
}

// keep only the listed indices (ascending) of a
ft_error compact(ft_ge25519_array a, const std::vector<uint64_t> &keep)
{
    size_t m = keep.size();
    if (m == a->n) return FT_ERR_NO_ERROR;
    void *s;
    CK(scratch(&s, align256(m * 8)));
    CK(h2d(s, keep.data(), m * 8));
    uint4 *np = nullptr;
    CK(dev_alloc((void **)&np, m * FT_PLANES_BYTES_PER_POINT));
    cudaError_t e = ft::gather(View{np, m}, ft::view_of(a), (const uint64_t *)s, m, g.stream);
    if (e != cudaSuccess) {
        dev_free(np);
        return map_err(e);
    }
    dev_free(a->planes);
    a->planes = np;
    a->cap = m;
    a->n = m;
    return FT_ERR_NO_ERROR;
}

ft_error status_reset()
{
    CK(cudaMemsetAsync(g.d_status, 0xff, sizeof(long long), g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error status_read(int64_t *res)
{
    long long v = -1;
    CK(d2h(&v, g.d_status, sizeof v));
    *res = (int64_t)v;
    return FT_ERR_NO_ERROR;
}

// the encryption tables of B and of the public key pk (32-byte folded
// encoding) into d_tables (ENC_TABLES_BYTES), queued on the library stream
ft_error build_key_tables(uint32_t *d_tables, const uint8_t *pk)
{
    ft_ge25519_array q;
    int64_t bad = -1;
    ft_error err = ft_array_from_bytes_folded(&bad, &q, pk, 32);
    if (err) return err;
    if (bad >= 0) {
        ft_array_free(q);
        return FT_ERR_INVALID_POINT;
    }
    cudaError_t e = cudaMemcpyAsync(d_tables, g.b_table, ft::ENC_TABLE_WORDS * 4, cudaMemcpyDeviceToDevice, g.stream);
    if (e == cudaSuccess) e = ft::build_enc_table(d_tables + ft::ENC_TABLE_WORDS, ft::view_of(q), g.stream);
    ft_array_free(q);
    CK(e);
    return FT_ERR_NO_ERROR;
}

// the encryption tables of pk, from the cache or built into its least
// recently used slot (kernels still queued on the library stream that read
// the slot's old tables run before the rebuild, in stream order)
ft_error ensure_pk_table(const uint8_t *pk, const uint32_t **tables)
{
    Ctx::KeyTab *slot = &g.keys[0];
    for (Ctx::KeyTab &k : g.keys) {
        if (k.used && std::memcmp(k.pk, pk, 32) == 0) {
            k.used = ++g.key_clock;
            *tables = k.table;
            return FT_ERR_NO_ERROR;
        }
        if (k.used < slot->used) slot = &k;
    }
    slot->used = 0;
    if (!slot->table) CK(dev_alloc((void **)&slot->table, ft::ENC_TABLES_BYTES));
    ft_error err = build_key_tables(slot->table, pk);
    if (err) return err;
    std::memcpy(slot->pk, pk, 32);
    slot->used = ++g.key_clock;
    *tables = slot->table;
    return FT_ERR_NO_ERROR;
}

// the decryption table for m_max, built on the device on first use
ft_error ensure_dlog(uint64_t m_max)
{
    if (g.dlog_mem && g.dlog.m_max == m_max) return FT_ERR_NO_ERROR;
    dev_free(g.dlog_mem);
    g.dlog_mem = nullptr;
    g.dlog = ft::DlogTable{};
    uint64_t cap = 64;
    while (cap < 2 * m_max) cap <<= 1;
    void *mem;
    CK(dev_alloc(&mem, ft::dlog_table_bytes(cap)));
    // j*B for j < m_max by the comb, encoded, then inserted
    void *s;
    const size_t b_pts = align256(m_max * FT_PLANES_BYTES_PER_POINT), b_js = align256(m_max * 8);
    cudaError_t e = scratch(&s, b_pts + b_js + align256(m_max * 32));
    View pts{(uint4 *)s, (size_t)m_max};
    uint64_t *js = (uint64_t *)((uint8_t *)s + b_pts);
    uint8_t *enc = (uint8_t *)s + b_pts + b_js;
    if (e == cudaSuccess) e = ft::iota_u64(js, m_max, g.stream);
    if (e == cudaSuccess) e = ft::smul_base_small(pts, m_max, js, g.b_table, g.stream);
    if (e == cudaSuccess) e = ft::encode(enc, pts, m_max, g.stream);
    if (e == cudaSuccess) e = ft::dlog_build(g.dlog, mem, m_max, cap, enc, g.stream);
    if (e != cudaSuccess) {
        dev_free(mem);
        g.dlog = ft::DlogTable{};
        return map_err(e);
    }
    g.dlog_mem = mem;
    return FT_ERR_NO_ERROR;
}

} // namespace

extern "C" {

const char *ft_error_str(ft_error err)
{
    // the reference's strings, ftcrypto.cu:34-57
    static const char *errors[] = {"no error",
                                   "out of memory",
                                   "parameter sizes did not mmatch",
                                   "bad size parameter",
                                   "index out of bounds",
                                   "invalid ed25519 point",
                                   "failed to initialise libsodium",
                                   "insufficient space in destination",
                                   "ciphertext corrupted",
                                   "internal library error",
                                   "device or driver does not support a required feature"};
    static_assert(sizeof(errors) / sizeof(errors[0]) == FT_ERR_MAX_ERR + 1, "error strings");
    if (err < 0 || err > FT_ERR_MAX_ERR) return "bad error value";
    return errors[err];
}

} // extern "C"

namespace {

// the library's stream, memory pool, status word and B's comb table
ft_error init_device(int dev)
{
    CK(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
    int prio_lo = 0, prio_hi = 0;
    CK(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
    CK(cudaStreamCreateWithPriority(&g.xfer, cudaStreamNonBlocking, prio_hi));
    for (auto &ev : g.in_ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaMemPoolProps pp;
    std::memset(&pp, 0, sizeof pp);
    pp.allocType = cudaMemAllocationTypePinned;
    pp.handleTypes = cudaMemHandleTypeNone;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = dev;
    CK(cudaMemPoolCreate(&g.pool, &pp));
    uint64_t thr = UINT64_MAX;
    CK(cudaMemPoolSetAttribute(g.pool, cudaMemPoolAttrReleaseThreshold, &thr));
    g.device = dev;
    CK(cudaMallocFromPoolAsync((void **)&g.d_status, 256, g.pool, g.stream));
    // the comb table of B, from B's encoding (y = 4/5, x even)
    uint8_t benc[32];
    std::memset(benc, 0x66, 32);
    benc[0] = 0x58;
    void *s;
    CK(dev_alloc((void **)&g.b_table, ft::ENC_TABLE_WORDS * 4));
    CK(dev_alloc(&s, align256(FT_PLANES_BYTES_PER_POINT) + 256));
    ft::View bp{(uint4 *)s, 1};
    uint8_t *d_enc = (uint8_t *)s + align256(FT_PLANES_BYTES_PER_POINT);
    CK(cudaMemcpyAsync(d_enc, benc, 32, cudaMemcpyHostToDevice, g.stream));
    CK(ft::decode(bp, d_enc, 1, g.d_status, g.stream));
    CK(ft::build_enc_table(g.b_table, bp, g.stream));
    CK(cudaStreamSynchronize(g.stream)); // benc is on the stack
    dev_free(s);
    CK(cudaStreamSynchronize(g.stream));
    return FT_ERR_NO_ERROR;
}

// undo a failed init_device, so that a later ft_crypto_init starts afresh
void init_release()
{
    if (g.stream) cudaStreamSynchronize(g.stream);
    if (g.xfer) cudaStreamSynchronize(g.xfer);
    for (auto &sg : g.stage) {
        if (sg.copied) cudaEventDestroy(sg.copied);
        if (sg.consumed) cudaEventDestroy(sg.consumed);
    }
    for (auto &ev : g.in_ev)
        if (ev) cudaEventDestroy(ev);
    if (g.pool) cudaMemPoolDestroy(g.pool); // releases its memory once nothing is outstanding
    if (g.xfer) cudaStreamDestroy(g.xfer);
    if (g.stream) cudaStreamDestroy(g.stream);
    cudaGetLastError();
    g = Ctx{};
}

} // namespace

extern "C" {

ft_error ft_crypto_init(void)
{
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (g.inited) return FT_ERR_NO_ERROR;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return FT_ERR_INSUFFICIENT_DEVICE_OR_DRIVER;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        return FT_ERR_INSUFFICIENT_DEVICE_OR_DRIVER;
    }
    // kernels are built for sm_103a only
    if (prop.major != 10 || prop.minor != 3) return FT_ERR_INSUFFICIENT_DEVICE_OR_DRIVER;
    ft_error err = init_device(dev);
    if (err) {
        init_release();
        return err;
    }
    g.inited = true;
    return FT_ERR_NO_ERROR;
}

ft_error ft_crypto_device_memory(size_t *free_mem, size_t *total_mem)
{
    ENSURE_INIT();
    CK(cudaMemGetInfo(free_mem, total_mem));
    return FT_ERR_NO_ERROR;
}

ft_error ft_array_init_scalar(ft_ge25519_array *array, size_t n, const uint8_t *scalar)
{
    ENSURE_INIT();
    return with_new_array(array, n, [&](ft_ge25519_array a) -> ft_error {
        if (n == 0) return FT_ERR_NO_ERROR;
        if (!scalar) {
            CK(ft::set_zero(ft::view_of(a), n, g.stream));
            return FT_ERR_NO_ERROR;
        }
        void *s;
        CK(scratch(&s, 256));
        CK(h2d(s, scalar, 32));
        CK(ft::smul_base(ft::view_of(a), 1, (const uint8_t *)s, 0, g.b_table, g.stream));
        CK(ft::broadcast(ft::view_of(a, 1), n - 1, ft::view_of(a), g.stream));
        return FT_ERR_NO_ERROR;
    });
}

ft_error ft_array_init_point(ft_ge25519_array *array, size_t n, const_ft_ge25519_array src, size_t idx)
{
    ENSURE_INIT();
    if (n > 0 && idx >= src->n) return FT_ERR_OUT_OF_BOUNDS;
    return with_new_array(array, n, [&](ft_ge25519_array a) -> ft_error {
        CK(ft::broadcast(ft::view_of(a), n, ft::view_of(src, idx), g.stream));
        return FT_ERR_NO_ERROR;
    });
}

ft_error ft_array_get_subset(ft_ge25519_array *array, const size_t *idxs, size_t n, const_ft_ge25519_array src)
{
    ENSURE_INIT();
    ft_error err = check_idxs(idxs, n, src->n);
    if (err) return err;
    return with_new_array(array, n, [&](ft_ge25519_array a) -> ft_error {
        if (n == 0) return FT_ERR_NO_ERROR;
        void *s;
        CK(scratch(&s, align256(n * 8)));
        CK(h2d(s, idxs, n * 8));
        CK(ft::gather(ft::view_of(a), ft::view_of(src), (const uint64_t *)s, n, g.stream));
        return FT_ERR_NO_ERROR;
    });
}

ft_error ft_array_get_range(ft_ge25519_array *array, size_t start, size_t stop, size_t step,
                            const_ft_ge25519_array src)
{
    ENSURE_INIT();
    size_t n = 0;
    if (stop > start) {
        if (step == 0) return FT_ERR_BAD_SIZE;
        n = (stop - start) / step;
    }
    if (n > src->n) return FT_ERR_SIZE_MISMATCH;
    if (n > 0 && start + (n - 1) * step >= src->n) return FT_ERR_OUT_OF_BOUNDS;
    return with_new_array(array, n, [&](ft_ge25519_array a) -> ft_error {
        CK(ft::gather_range(ft::view_of(a), ft::view_of(src), start, step, n, g.stream));
        return FT_ERR_NO_ERROR;
    });
}

ft_error ft_array_assign_to_subset(ft_ge25519_array array, const size_t *idxs, size_t n, const_ft_ge25519_array src)
{
    ENSURE_INIT();
    if (n != src->n) return FT_ERR_SIZE_MISMATCH;
    ft_error err = check_idxs(idxs, n, array->n);
    if (err) return err;
    if (n == 0) return FT_ERR_NO_ERROR;
    void *s;
    CK(scratch(&s, align256(n * 8)));
    CK(h2d(s, idxs, n * 8));
    CK(ft::scatter(ft::view_of(array), ft::view_of(src), (const uint64_t *)s, n, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ft_array_assign_zero_to_subset(ft_ge25519_array array, const size_t *idxs, size_t n)
{
    ENSURE_INIT();
    ft_error err = check_idxs(idxs, n, array->n);
    if (err) return err;
    if (n == 0) return FT_ERR_NO_ERROR;
    void *s;
    CK(scratch(&s, align256(n * 8)));
    CK(h2d(s, idxs, n * 8));
    CK(ft::scatter_zero(ft::view_of(array), (const uint64_t *)s, n, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ft_array_assign_to_range(ft_ge25519_array array, size_t start, size_t stop, size_t step,
                                  const_ft_ge25519_array src)
{
    ENSURE_INIT();
    if (stop <= start) return FT_ERR_NO_ERROR;
    if (step == 0) return FT_ERR_BAD_SIZE;
    if ((stop - start) / step > src->n) return FT_ERR_SIZE_MISMATCH;
    // the reference writes src[i] to start + i*step for every i < length(src)
    // with start + i*step < stop (ftcrypto.cu:468-479)
    size_t count = std::min(src->n, (stop - start - 1) / step + 1);
    if (count == 0) return FT_ERR_NO_ERROR;
    if (start + (count - 1) * step >= array->n) return FT_ERR_OUT_OF_BOUNDS;
    CK(ft::scatter_range(ft::view_of(array), ft::view_of(src), start, step, count, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ft_array_delete_subset(ft_ge25519_array array, const size_t *idxs, size_t n)
{
    ENSURE_INIT();
    std::vector<size_t> del(idxs, idxs + n);
    std::sort(del.begin(), del.end());
    del.erase(std::unique(del.begin(), del.end()), del.end());
    std::vector<uint64_t> keep;
    keep.reserve(array->n);
    size_t d = 0;
    for (size_t i = 0; i < array->n; ++i) {
        while (d < del.size() && del[d] < i) ++d;
        if (d < del.size() && del[d] == i) continue;
        keep.push_back(i);
    }
    return compact(array, keep);
}

ft_error ft_array_delete_range(ft_ge25519_array array, size_t start, size_t stop, size_t step)
{
    ENSURE_INIT();
    if (stop > start && step == 0) return FT_ERR_BAD_SIZE;
    std::vector<uint64_t> keep;
    keep.reserve(array->n);
    for (size_t i = 0; i < array->n; ++i) {
        if (i >= start && i < stop && (i - start) % step == 0) continue;
        keep.push_back(i);
    }
    return compact(array, keep);
}

ft_error ft_array_to_bytes_folded(uint8_t *mem, size_t n_bytes, const_ft_ge25519_array array)
{
    ENSURE_INIT();
    size_t n = array->n;
    if (n_bytes / FT_FOLDED_POINT_BYTES < n) return FT_ERR_INSUFFICIENT_SPACE;
    if (n == 0) return FT_ERR_NO_ERROR;
    return export_to_host(mem, array, 32, ft::encode);
}

ft_error ft_array_to_bytes_affine(uint8_t *mem, size_t n_bytes, const_ft_ge25519_array array)
{
    ENSURE_INIT();
    size_t n = array->n;
    if (n_bytes / FT_AFFINE_POINT_BYTES < n) return FT_ERR_INSUFFICIENT_SPACE;
    if (n == 0) return FT_ERR_NO_ERROR;
    return export_to_host(mem, array, 64, ft::to_affine);
}

ft_error ft_array_to_bytes(uint8_t *mem, size_t n_bytes, const_ft_ge25519_array array)
{
    ENSURE_INIT();
    size_t n = array->n;
    if (n_bytes / FT_EXTENDED_POINT_BYTES < n) return FT_ERR_INSUFFICIENT_SPACE;
    if (n == 0) return FT_ERR_NO_ERROR;
    return export_to_host(mem, array, 160, ft::to_ref160);
}

ft_error ft_array_from_bytes_folded(int64_t *res, ft_ge25519_array *array, const uint8_t *mem, size_t n_bytes)
{
    ENSURE_INIT();
    if (n_bytes % FT_FOLDED_POINT_BYTES) return FT_ERR_BAD_SIZE;
    size_t n = n_bytes / FT_FOLDED_POINT_BYTES;
    int64_t bad = -1;
    ft_error err = with_new_array(array, n, [&](ft_ge25519_array a) -> ft_error {
        if (n == 0) return FT_ERR_NO_ERROR;
        void *s;
        CK(scratch(&s, align256(n_bytes)));
        CK(h2d(s, mem, n_bytes));
        ft_error e2 = status_reset();
        if (e2) return e2;
        CK(ft::decode(ft::view_of(a), (const uint8_t *)s, n, g.d_status, g.stream));
        return status_read(&bad);
    });
    if (err) return err;
    *res = bad;
    return FT_ERR_NO_ERROR;
}

ft_error ft_array_from_bytes_affine(ft_ge25519_array *array, const uint8_t *mem, size_t n_bytes)
{
    ENSURE_INIT();
    if (n_bytes % FT_AFFINE_POINT_BYTES) return FT_ERR_BAD_SIZE;
    size_t n = n_bytes / FT_AFFINE_POINT_BYTES;
    return with_new_array(array, n, [&](ft_ge25519_array a) -> ft_error {
        if (n == 0) return FT_ERR_NO_ERROR;
        void *s;
        CK(scratch(&s, align256(n_bytes)));
        CK(h2d(s, mem, n_bytes));
        CK(ft::from_affine(ft::view_of(a), (const uint8_t *)s, n, g.stream));
        return FT_ERR_NO_ERROR;
    });
}

ft_error ft_array_from_bytes(ft_ge25519_array *array, const uint8_t *mem, size_t n_bytes)
{
    ENSURE_INIT();
    if (n_bytes % FT_EXTENDED_POINT_BYTES) return FT_ERR_BAD_SIZE;
    size_t n = n_bytes / FT_EXTENDED_POINT_BYTES;
    return with_new_array(array, n, [&](ft_ge25519_array a) -> ft_error {
        if (n == 0) return FT_ERR_NO_ERROR;
        void *s;
        CK(scratch(&s, align256(n_bytes)));
        CK(h2d(s, mem, n_bytes));
        CK(ft::from_ref160(ft::view_of(a), (const uint8_t *)s, n, g.stream));
        return FT_ERR_NO_ERROR;
    });
}

ft_error ft_array_validate(int64_t *res, const_ft_ge25519_array array)
{
    ENSURE_INIT();
    ft_error err = status_reset();
    if (err) return err;
    CK(ft::validate(ft::view_of(array), array->n, g.d_status, g.stream));
    return status_read(res);
}

ft_error ft_array_from_scalars(ft_ge25519_array *array, const uint8_t *scalars, size_t n)
{
    ENSURE_INIT();
    return with_new_array(array, n, [&](ft_ge25519_array a) -> ft_error {
        if (n == 0) return FT_ERR_NO_ERROR;
        void *s;
        CK(scratch(&s, align256(n * 32)));
        CK(h2d(s, scalars, n * 32));
        CK(ft::smul_base(ft::view_of(a), n, (const uint8_t *)s, 1, g.b_table, g.stream));
        return FT_ERR_NO_ERROR;
    });
}

ft_error ft_array_from_small_scalars(ft_ge25519_array *array, const uint64_t *small, size_t n)
{
    ENSURE_INIT();
    return with_new_array(array, n, [&](ft_ge25519_array a) -> ft_error {
        if (n == 0) return FT_ERR_NO_ERROR;
        void *s;
        CK(scratch(&s, align256(n * 8)));
        CK(h2d(s, small, n * 8));
        CK(ft::smul_base_small(ft::view_of(a), n, (const uint64_t *)s, g.b_table, g.stream));
        return FT_ERR_NO_ERROR;
    });
}

void ft_array_free(ft_ge25519_array array)
{
    if (!array) return;
    if (g.inited) dev_free(array->planes);
    delete array; // destroys its events
}

size_t ft_array_get_length(const_ft_ge25519_array array) { return array->n; }

// ftcrypto.cu:291-336
ft_error ft_array_set_length(ft_ge25519_array array, size_t newlen)
{
    ENSURE_INIT();
    size_t len = array->n;
    if (newlen <= len / 2) {
        ft_error err = arr_realloc(array, newlen, newlen);
        if (err) return err;
        array->n = newlen;
    } else if (newlen <= len) {
        array->n = newlen;
    } else if (newlen <= array->cap) {
        CK(ft::set_zero(ft::view_of(array, len), newlen - len, g.stream));
        array->n = newlen;
    } else {
        ft_error err = arr_realloc(array, newlen, len);
        if (err) return err;
        CK(ft::set_zero(ft::view_of(array, len), newlen - len, g.stream));
        array->n = newlen;
    }
    return FT_ERR_NO_ERROR;
}

ft_error ft_array_mux(ft_ge25519_array iftrue, const int64_t *cond, const_ft_ge25519_array iffalse)
{
    ENSURE_INIT();
    if (iftrue->n != iffalse->n) return FT_ERR_SIZE_MISMATCH;
    size_t n = iftrue->n;
    if (n == 0) return FT_ERR_NO_ERROR;
    void *s;
    CK(scratch(&s, align256(n * 8)));
    CK(h2d(s, cond, n * 8));
    CK(ft::mux(ft::view_of(iftrue), (const int64_t *)s, ft::view_of(iffalse), n, g.stream));
    return FT_ERR_NO_ERROR;
}

// res[i] = 1 iff array1[i] equals some point of array2 (ft_array_contains,
// ftcrypto.cu:1046-1086, an O(n1 * n2) comparison there): the canonical
// encodings of array2 go into a device hash table (the open-addressing
// table decryption uses, keyed by encoding, valued by index) and those of
// array1 are looked up in it, O(n1 + n2).  Equal encodings are equal points
// on the curve.
ft_error ft_array_contains(int64_t *res, const_ft_ge25519_array array1, const_ft_ge25519_array array2)
{
    ENSURE_INIT();
    const size_t n1 = array1->n, n2 = array2->n;
    if (n1 == 0) return FT_ERR_NO_ERROR;
    if (n2 == 0) {
        std::memset(res, 0, n1 * sizeof(int64_t));
        return FT_ERR_NO_ERROR;
    }
    if (n2 >= ((size_t)1 << 31)) return FT_ERR_BAD_SIZE;
    uint64_t cap = 64;
    while (cap < 2 * (uint64_t)n2) cap <<= 1;
    const size_t b1 = align256(n1 * 32), b2 = align256(n2 * 32), bt = align256(ft::dlog_table_bytes(cap));
    void *s;
    CK(scratch(&s, b1 + b2 + bt + align256(n1 * 8)));
    uint8_t *base = (uint8_t *)s;
    uint8_t *e1 = base, *e2 = base + b1;
    uint64_t *hit = (uint64_t *)(base + b1 + b2 + bt);
    CK(ft::encode(e1, ft::view_of(array1), n1, g.stream));
    CK(ft::encode(e2, ft::view_of(array2), n2, g.stream));
    ft::DlogTable t;
    CK(ft::dlog_build(t, base + b1 + b2, n2, cap, e2, g.stream));
    CK(ft::dlog_lookup(hit, t, e1, n1, g.stream));
    CK(d2h(res, hit, n1 * 8));
    for (size_t i = 0; i < n1; ++i) res[i] = (uint64_t)res[i] != ~0ull ? 1 : 0;
    return FT_ERR_NO_ERROR;
}

ft_error ft_add(ft_ge25519_array res, const_ft_ge25519_array summand)
{
    ENSURE_INIT();
    if (summand->n != res->n) return FT_ERR_SIZE_MISMATCH;
    CK(ft::add(ft::view_of(res), ft::view_of(summand), res->n, 0, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ft_reduce_isum(ft_ge25519_array res, const size_t *idxs, size_t n, const_ft_ge25519_array src)
{
    ENSURE_INIT();
    if (n != src->n) return FT_ERR_SIZE_MISMATCH;
    if (n == 0) return FT_ERR_NO_ERROR;
    size_t nk = res->n;
    if (n >= (size_t)INT32_MAX || nk >= (size_t)INT32_MAX) return FT_ERR_BAD_SIZE;
    ft_error err = check_idxs(idxs, n, nk);
    if (err) return err;
    size_t b_keys = align256(n * 8), b_off = align256((nk + 1) * 4), b_perm = align256(n * 4);
    size_t b_sort = align256(ft::isum_scratch_bytes(n, nk));
    size_t b_seg = align256(ft::segsum_scratch_bytes(n));
    void *s;
    CK(scratch(&s, b_keys + b_off + b_perm + b_sort + b_seg + 256));
    uint8_t *base = (uint8_t *)s;
    uint64_t *keys = (uint64_t *)base;
    int32_t *off = (int32_t *)(base + b_keys);
    int32_t *perm = (int32_t *)(base + b_keys + b_off);
    void *sort_tmp = base + b_keys + b_off + b_perm;
    void *seg_tmp = base + b_keys + b_off + b_perm + b_sort;
    int32_t *d_maxlen = (int32_t *)(base + b_keys + b_off + b_perm + b_sort + b_seg);
    CK(h2d(keys, idxs, n * 8));
    if ((err = status_reset())) return err;
    CK(ft::keys_to_csr(off, perm, keys, n, nk, g.d_status, sort_tmp, g.stream));
    // a key repeated thousands of times is a long segment: sum those layouts
    // through a scan (one wait for the largest count decides)
    int32_t maxlen = 0;
    CK(ft::segment_maxlen(off, nk, d_maxlen, g.stream));
    CK(d2h(&maxlen, d_maxlen, sizeof maxlen));
    if (ft::segsum_prefers_prefix(n, (size_t)maxlen)) {
        void *t = nullptr;
        CK(dev_alloc(&t, ft::segsum_prefix_scratch_bytes(n)));
        cudaError_t e = ft::segsum_prefix(ft::view_of(res), off, nk, ft::view_of(src), n, perm, 1, t, g.stream);
        dev_free(t);
        CK(e);
        return FT_ERR_NO_ERROR;
    }
    CK(ft::segsum(ft::view_of(res), off, nk, ft::view_of(src), n, perm, 1, seg_tmp, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ft_sub(ft_ge25519_array res, const_ft_ge25519_array summand)
{
    ENSURE_INIT();
    if (summand->n != res->n) return FT_ERR_SIZE_MISMATCH;
    CK(ft::add(ft::view_of(res), ft::view_of(summand), res->n, 1, g.stream));
    return FT_ERR_NO_ERROR;
}

static ft_error scale_impl(ft_ge25519_array array, const uint8_t *scalar)
{
    ENSURE_INIT();
    if (array->n == 0) return FT_ERR_NO_ERROR;
    void *s;
    CK(scratch(&s, 256));
    CK(h2d(s, scalar, 32));
    CK(ft::smul_var(ft::view_of(array), array->n, (const uint8_t *)s, 0, g.stream));
    return FT_ERR_NO_ERROR;
}

void ft_scale(ft_ge25519_array array, const uint8_t *scalar) { g.last_void = scale_impl(array, scalar); }

static ft_error neg_impl(ft_ge25519_array array)
{
    ENSURE_INIT();
    CK(ft::neg(ft::view_of(array), array->n, g.stream));
    return FT_ERR_NO_ERROR;
}

void ft_neg(ft_ge25519_array array) { g.last_void = neg_impl(array); }

ft_error ft_mul(ft_ge25519_array array, const uint8_t *scalars, size_t n)
{
    ENSURE_INIT();
    if (n != array->n) return FT_ERR_SIZE_MISMATCH;
    if (n == 0) return FT_ERR_NO_ERROR;
    const void *s;
    Ctx::Stage *sg = nullptr;
    if (host_is_pinned(scalars)) {
        void *p;
        CK(stage_scalars(&p, &sg, scalars, n * 32));
        s = p;
    } else {
        void *p;
        CK(scratch(&p, align256(n * 32)));
        CK(h2d(p, scalars, n * 32));
        s = p;
    }
    // Four or more waves of the ladder launch: all whole waves but the last
    // in one launch, then the rest, marked as two parts, so that an export
    // of the products (as the host-fed caller's next call usually is)
    // converts and copies the first part while the last wave computes.
    // Cut at a wave boundary, the two launches take as many waves as one.
    const size_t wave = ft::ladder_wave_points();
    const size_t cut = wave && n >= 4 * wave ? (n - 1) / wave * wave : 0;
    if (cut) {
        CK(ft::smul_var(ft::view_of(array), cut, (const uint8_t *)s, 1, g.stream));
        CK(mark_part(array));
        CK(ft::smul_var(ft::view_of(array, cut), n - cut, (const uint8_t *)s + cut * 32, 1, g.stream));
    } else {
        CK(ft::smul_var(ft::view_of(array), n, (const uint8_t *)s, 1, g.stream));
    }
    if (sg) CK(cudaEventRecord(sg->consumed, g.stream));
    CK(mark_ready(array, cut));
    if (sg) CK(cudaEventSynchronize(sg->copied)); // the caller may reuse its buffer
    return FT_ERR_NO_ERROR;
}

static ft_error index_impl(int64_t *res, const_ft_ge25519_array array)
{
    ENSURE_INIT();
    size_t n = array->n;
    if (n == 0) return FT_ERR_NO_ERROR;
    void *s;
    CK(scratch(&s, align256(n * 8)));
    CK(ft::index_nonzero((int64_t *)s, ft::view_of(array), n, g.stream));
    CK(d2h(res, s, n * 8));
    return FT_ERR_NO_ERROR;
}

void ft_index(int64_t *res, const_ft_ge25519_array array) { g.last_void = index_impl(res, array); }

static ft_error equal_impl(int64_t *res, const_ft_ge25519_array a, const_ft_ge25519_array b, int invert)
{
    ENSURE_INIT();
    if (a->n != b->n) return FT_ERR_SIZE_MISMATCH;
    size_t n = a->n;
    if (n == 0) return FT_ERR_NO_ERROR;
    void *s;
    CK(scratch(&s, align256(n * 8)));
    CK(ft::equal((int64_t *)s, ft::view_of(a), ft::view_of(b), n, invert, g.stream));
    CK(d2h(res, s, n * 8));
    return FT_ERR_NO_ERROR;
}

ft_error ft_equal(int64_t *res, const_ft_ge25519_array a, const_ft_ge25519_array b) { return equal_impl(res, a, b, 0); }
ft_error ft_not_equal(int64_t *res, const_ft_ge25519_array a, const_ft_ge25519_array b) { return equal_impl(res, a, b, 1); }

static ft_error scan_impl(ft_ge25519_array array, int exclusive)
{
    ENSURE_INIT();
    size_t n = array->n;
    if (n == 0) return FT_ERR_NO_ERROR;
    void *s;
    CK(scratch(&s, ft::scan_scratch_bytes(n)));
    CK(ft::scan(ft::view_of(array), n, exclusive, s, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ft_array_prescan(ft_ge25519_array array) { return scan_impl(array, 1); }
ft_error ft_array_scan(ft_ge25519_array array) { return scan_impl(array, 0); }

ft_error ftx_ct_scan(ft_ge25519_array c1, ft_ge25519_array c2, int exclusive)
{
    ENSURE_INIT();
    if (c1->n != c2->n) return FT_ERR_SIZE_MISMATCH;
    if (c1 == c2) { // the same array twice: the two ft_array_scan calls it stands for
        ft_error err = scan_impl(c1, exclusive ? 1 : 0);
        return err ? err : scan_impl(c2, exclusive ? 1 : 0);
    }
    size_t n = c1->n;
    if (n == 0) return FT_ERR_NO_ERROR;
    void *s;
    CK(scratch(&s, ft::scan_scratch_bytes(n, 2)));
    const ft::View v[2] = {ft::view_of(c1), ft::view_of(c2)};
    CK(ft::scan_set(v, 2, n, exclusive ? 1 : 0, s, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ft_array_reduce(ft_ge25519_array array)
{
    ENSURE_INIT();
    size_t n = array->n;
    if (n == 1) return FT_ERR_NO_ERROR;
    uint4 *np = nullptr;
    CK(dev_alloc((void **)&np, FT_PLANES_BYTES_PER_POINT));
    void *s;
    cudaError_t e = scratch(&s, ft::reduce_scratch_bytes(n));
    if (e == cudaSuccess) e = ft::reduce(View{np, 1}, ft::view_of(array), n, s, g.stream);
    if (e != cudaSuccess) {
        dev_free(np);
        return map_err(e);
    }
    dev_free(array->planes);
    array->planes = np;
    array->n = 1;
    array->cap = 1;
    return FT_ERR_NO_ERROR;
}

// ---------------------------------------------------------------- extensions

ft_error ftx_last_error(void) { return g.last_void; }

int ftx_last_cuda_error(void) { return g_last_cuda.load(); }

void *ftx_stream(void)
{
    if (!g.inited && ft_crypto_init()) return nullptr;
    return (void *)g.stream;
}

ft_error ftx_synchronize(void)
{
    ENSURE_INIT();
    CK(cudaStreamSynchronize(g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ftx_array_device_view(const_ft_ge25519_array array, void **planes, size_t *stride)
{
    array->exposed.store(true); // the caller may write it where the library cannot see
    *planes = (void *)array->planes;
    *stride = array->cap;
    return FT_ERR_NO_ERROR;
}

ft_error ftx_array_to_packed(uint8_t *mem, size_t n_bytes, const_ft_ge25519_array array)
{
    ENSURE_INIT();
    size_t n = array->n;
    if (n_bytes / 128 < n) return FT_ERR_INSUFFICIENT_SPACE;
    if (n == 0) return FT_ERR_NO_ERROR;
    return export_to_host(mem, array, 128, ft::to_packed);
}

ft_error ftx_array_from_packed(ft_ge25519_array *array, const uint8_t *mem, size_t n_bytes)
{
    ENSURE_INIT();
    if (n_bytes % 128) return FT_ERR_BAD_SIZE;
    size_t n = n_bytes / 128;
    return with_new_array(array, n, [&](ft_ge25519_array a) -> ft_error {
        if (n == 0) return FT_ERR_NO_ERROR;
        void *s;
        CK(scratch(&s, align256(n_bytes)));
        CK(h2d(s, mem, n_bytes));
        CK(ft::from_packed(ft::view_of(a), (const uint8_t *)s, n, g.stream));
        return FT_ERR_NO_ERROR;
    });
}

ft_error ftx_mul_device(ft_ge25519_array array, const uint8_t *d_scalars, size_t n)
{
    ENSURE_INIT();
    if (n != array->n) return FT_ERR_SIZE_MISMATCH;
    CK(ft::smul_var(ft::view_of(array), n, d_scalars, 1, g.stream));
    CK(mark_ready(array));
    return FT_ERR_NO_ERROR;
}

static int m_digits(unsigned bits) { return enc_digits(bits); }

ft_error ftx_encrypt_device(ft_ge25519_array c1, ft_ge25519_array c2, const uint8_t *pk, const uint64_t *d_m,
                            const uint8_t *d_r, size_t n, unsigned bits)
{
    ENSURE_INIT();
    if (bits < 1 || bits > 64) return FT_ERR_BAD_SIZE;
    if (c1->n != n || c2->n != n) return FT_ERR_SIZE_MISMATCH;
    const uint32_t *tab;
    ft_error err = ensure_pk_table(pk, &tab);
    if (err) return err;
    CK(ft::encrypt(ft::view_of(c1), ft::view_of(c2), n, d_r, d_m, m_digits(bits), tab, g.stream));
    CK(mark_ready(c1));
    CK(mark_ready(c2));
    return FT_ERR_NO_ERROR;
}

// The encryption of host inputs into new arrays a, b.  The inputs go over
// in two parts: the first, one pass of the encryption grid, on the library
// stream, which encrypts it while the transfer stream copies the rest; then
// the rest is encrypted.  The plaintext bound is checked on the device (an
// OR of all m after the copies), and the call returns once the inputs are
// copied and checked, with the encryption still running.  Split at one pass,
// the two launches take as many passes as one.  FT_ERR_BAD_SIZE if some
// m_i >= 2^bits (the arrays' contents are then undefined).
static ft_error encrypt_from_host(ft_ge25519_array a, ft_ge25519_array b, const uint64_t *m, const uint8_t *r,
                                  size_t n, unsigned bits, const uint32_t *tab)
{
    if (n == 0) return FT_ERR_NO_ERROR;
    void *s;
    const size_t br = align256(n * 32), bm = align256(n * 8);
    CK(scratch(&s, br + bm + 256));
    uint8_t *dr = (uint8_t *)s;
    uint64_t *dm = (uint64_t *)(dr + br), *dacc = (uint64_t *)(dr + br + bm);
    const size_t first = std::min(n, ft::encrypt_pass());
    const int mdig = m_digits(bits);
    CK(cudaMemcpyAsync(dr, r, first * 32, cudaMemcpyHostToDevice, g.stream));
    CK(cudaMemcpyAsync(dm, m, first * 8, cudaMemcpyHostToDevice, g.stream));
    CK(cudaEventRecord(g.in_ev[0], g.stream)); // the first part is copied (and the scratch free)
    CK(cudaStreamWaitEvent(g.xfer, g.in_ev[0], 0));
    if (n > first) {
        CK(cudaMemcpyAsync(dr + first * 32, r + first * 32, (n - first) * 32, cudaMemcpyHostToDevice, g.xfer));
        CK(cudaMemcpyAsync(dm + first, m + first, (n - first) * 8, cudaMemcpyHostToDevice, g.xfer));
        CK(cudaEventRecord(g.in_ev[1], g.xfer));
    }
    CK(ft::encrypt(ft::view_of(a), ft::view_of(b), first, dr, dm, mdig, tab, g.stream));
    if (n > first) {
        CK(cudaStreamWaitEvent(g.stream, g.in_ev[1], 0));
        CK(ft::encrypt(ft::view_of(a, first), ft::view_of(b, first), n - first, dr + first * 32, dm + first, mdig,
                       tab, g.stream));
    }
    CK(mark_ready(a));
    CK(mark_ready(b));
    uint64_t acc = 0;
    if (bits < 64) {
        CK(ft::or_words(dacc, dm, n, g.xfer));
        CK(cudaMemcpyAsync(&acc, dacc, sizeof acc, cudaMemcpyDeviceToHost, g.xfer));
    }
    // the caller may reuse its buffers: both parts are copied
    CK(cudaStreamSynchronize(g.xfer));
    return bits < 64 && (acc >> bits) ? FT_ERR_BAD_SIZE : FT_ERR_NO_ERROR;
}

ft_error ftx_encrypt(ft_ge25519_array *c1, ft_ge25519_array *c2, const uint8_t *pk, const uint64_t *m,
                     const uint8_t *r, size_t n, unsigned bits)
{
    ENSURE_INIT();
    if (bits < 1 || bits > 64) return FT_ERR_BAD_SIZE;
    if (too_long(n)) return FT_ERR_OUT_OF_MEMORY;
    // the key's tables first (building them uses the scratch buffer)
    const uint32_t *tab;
    ft_error err = ensure_pk_table(pk, &tab);
    if (err) return err;
    ft_ge25519_array a, b;
    if ((err = arr_new(&a, n))) return err;
    if ((err = arr_new(&b, n))) {
        ft_array_free(a);
        return err;
    }
    const ft_error res = encrypt_from_host(a, b, m, r, n, bits, tab);
    if (res) {
        ft_array_free(a); // stream-ordered: after any launch that writes it
        ft_array_free(b);
        return res;
    }
    *c1 = a;
    *c2 = b;
    return FT_ERR_NO_ERROR;
}

// (c1, c2) +/-= (d1, d2): one launch, or two in the order of ft_add(c1, d1),
// ft_add(c2, d2) when one half is read or written by the other's update
static ft_error ct_add_sub(ft_ge25519_array c1, ft_ge25519_array c2, const_ft_ge25519_array d1, const_ft_ge25519_array d2,
                    int sub)
{
    if (c1->n != c2->n || d1->n != c1->n || d2->n != c1->n) return FT_ERR_SIZE_MISMATCH;
    const size_t n = c1->n;
    if (c1 == c2 || d2 == c1 || d1 == c2) {
        CK(ft::add(ft::view_of(c1), ft::view_of(d1), n, sub, g.stream));
        CK(ft::add(ft::view_of(c2), ft::view_of(d2), n, sub, g.stream));
        return FT_ERR_NO_ERROR;
    }
    CK(ft::add_ct(ft::view_of(c1), ft::view_of(c2), ft::view_of(d1), ft::view_of(d2), n, sub, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ftx_ct_add(ft_ge25519_array c1, ft_ge25519_array c2, const_ft_ge25519_array d1, const_ft_ge25519_array d2)
{
    ENSURE_INIT();
    return ct_add_sub(c1, c2, d1, d2, 0);
}

ft_error ftx_ct_sub(ft_ge25519_array c1, ft_ge25519_array c2, const_ft_ge25519_array d1, const_ft_ge25519_array d2)
{
    ENSURE_INIT();
    return ct_add_sub(c1, c2, d1, d2, 1);
}

ft_error ftx_rerandomise_device(ft_ge25519_array c1, ft_ge25519_array c2, const uint8_t *pk, const uint8_t *d_r, size_t n)
{
    ENSURE_INIT();
    if (c1->n != n || c2->n != n) return FT_ERR_SIZE_MISMATCH;
    const uint32_t *tab;
    ft_error err = ensure_pk_table(pk, &tab);
    if (err) return err;
    CK(ft::rerandomise(ft::view_of(c1), ft::view_of(c2), n, d_r, tab, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ftx_rerandomise(ft_ge25519_array c1, ft_ge25519_array c2, const uint8_t *pk, const uint8_t *r, size_t n)
{
    ENSURE_INIT();
    if (c1->n != n || c2->n != n) return FT_ERR_SIZE_MISMATCH;
    const uint32_t *tab;
    ft_error err = ensure_pk_table(pk, &tab);
    if (err) return err;
    if (n == 0) return FT_ERR_NO_ERROR;
    void *s;
    CK(scratch(&s, align256(n * 32)));
    CK(h2d(s, r, n * 32));
    CK(ft::rerandomise(ft::view_of(c1), ft::view_of(c2), n, (const uint8_t *)s, tab, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ftx_decrypt(const_ft_ge25519_array c1, const_ft_ge25519_array c2, const uint8_t *sk, uint64_t m_max,
                     uint64_t *m)
{
    ENSURE_INIT();
    if (m_max == 0 || m_max > FTX_DECRYPT_MAX_M) return FT_ERR_BAD_SIZE;
    if (c1->n != c2->n) return FT_ERR_SIZE_MISMATCH;
    ft_error err = ensure_dlog(m_max);
    if (err) return err;
    const size_t n = c1->n;
    if (n == 0) return FT_ERR_NO_ERROR;
    // D = c2 - sk * c1, encoded, looked up
    void *s;
    const size_t b_pts = align256(n * FT_PLANES_BYTES_PER_POINT), b_enc = align256(n * 32), b_m = align256(n * 8);
    CK(scratch(&s, 2 * b_pts + b_enc + b_m + 256));
    uint8_t *base = (uint8_t *)s;
    View t{(uint4 *)base, n}, d{(uint4 *)(base + b_pts), n};
    uint8_t *enc = base + 2 * b_pts;
    uint64_t *dm = (uint64_t *)(base + 2 * b_pts + b_enc);
    uint8_t *dsk = base + 2 * b_pts + b_enc + b_m;
    CK(h2d(dsk, sk, 32));
    CK(ft::copy_points(t, ft::view_of(c1), n, g.stream));
    CK(ft::smul_var(t, n, dsk, 0, g.stream));
    CK(ft::copy_points(d, ft::view_of(c2), n, g.stream));
    CK(ft::add(d, t, n, 1, g.stream));
    CK(ft::encode(enc, d, n, g.stream));
    CK(ft::dlog_lookup(dm, g.dlog, enc, n, g.stream));
    CK(d2h(m, dm, n * 8));
    return FT_ERR_NO_ERROR;
}

ft_error ftx_segmented_sum_csr_device(ft_ge25519_array out, const int32_t *d_off, size_t nseg,
                                      const_ft_ge25519_array src)
{
    ENSURE_INIT();
    if (out->n != nseg) return FT_ERR_SIZE_MISMATCH;
    if (src->n >= (size_t)INT32_MAX || nseg >= (size_t)INT32_MAX) return FT_ERR_BAD_SIZE;
    void *s;
    CK(scratch(&s, ft::segsum_scratch_bytes(src->n)));
    CK(ft::segsum(ft::view_of(out), d_off, nseg, ft::view_of(src), src->n, nullptr, 0, s, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ftx_ct_segmented_sum_csr_device(ft_ge25519_array out1, ft_ge25519_array out2, const int32_t *d_off,
                                         size_t nseg, const_ft_ge25519_array src1, const_ft_ge25519_array src2)
{
    ENSURE_INIT();
    if (out1->n != nseg || out2->n != nseg || src1->n != src2->n) return FT_ERR_SIZE_MISMATCH;
    if (src1->n >= (size_t)INT32_MAX || nseg >= (size_t)INT32_MAX) return FT_ERR_BAD_SIZE;
    if (out1 == out2 || out1 == src2 || out2 == src1) {
        // one half's output is the other's input or output: the two sums
        // in order, as the two calls they stand for
        ft_error err = ftx_segmented_sum_csr_device(out1, d_off, nseg, src1);
        return err ? err : ftx_segmented_sum_csr_device(out2, d_off, nseg, src2);
    }
    void *s;
    CK(scratch(&s, ft::segsum_scratch_bytes(src1->n, 2)));
    const View outs[2] = {ft::view_of(out1), ft::view_of(out2)};
    const View srcs[2] = {ft::view_of(src1), ft::view_of(src2)};
    CK(ft::segsum_set(outs, srcs, 2, d_off, nseg, src1->n, nullptr, 0, s, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ftx_segmented_sum_csr(ft_ge25519_array *out, const int32_t *off, size_t nseg, const_ft_ge25519_array src)
{
    ENSURE_INIT();
    if (src->n >= (size_t)INT32_MAX || nseg >= (size_t)INT32_MAX) return FT_ERR_BAD_SIZE;
    if (off[0] != 0 || (size_t)off[nseg] != src->n) return FT_ERR_BAD_SIZE;
    size_t maxlen = 0;
    for (size_t s = 0; s < nseg; ++s) {
        if (off[s + 1] < off[s]) return FT_ERR_BAD_SIZE;
        maxlen = std::max(maxlen, (size_t)(off[s + 1] - off[s]));
    }
    // long segments go through a scan: the walk's join would add their
    // thread parts one after another
    const bool prefix = ft::segsum_prefers_prefix(src->n, maxlen);
    return with_new_array(out, nseg, [&](ft_ge25519_array a) -> ft_error {
        if (nseg == 0) return FT_ERR_NO_ERROR;
        void *s;
        size_t b_off = align256((nseg + 1) * 4);
        CK(scratch(&s, b_off + (prefix ? ft::segsum_prefix_scratch_bytes(src->n) : ft::segsum_scratch_bytes(src->n))));
        CK(h2d(s, off, (nseg + 1) * 4));
        if (prefix)
            CK(ft::segsum_prefix(ft::view_of(a), (const int32_t *)s, nseg, ft::view_of(src), src->n, nullptr, 0,
                                 (uint8_t *)s + b_off, g.stream));
        else
            CK(ft::segsum(ft::view_of(a), (const int32_t *)s, nseg, ft::view_of(src), src->n, nullptr, 0,
                          (uint8_t *)s + b_off, g.stream));
        return FT_ERR_NO_ERROR;
    });
}

static int g_batch_add_pts = 4;
// window width of the small-scalar ladder (FTX_TUNE_SCALE_WINDOW); 3 measured
// fastest on GB300 for 10-bit bounds (batched mix 33.1 ms against 37.8 at 4)
static int g_scale_w = 3;

ft_error ftx_tune(int knob, int value)
{
    switch (knob) {
    case FTX_TUNE_LADDER_BLOCK: return ft::set_ladder_block(value) ? FT_ERR_BAD_SIZE : FT_ERR_NO_ERROR;
    case FTX_TUNE_BATCH_ADD_PTS:
        if (value < 1 || value > 64) return FT_ERR_BAD_SIZE;
        g_batch_add_pts = value;
        return FT_ERR_NO_ERROR;
    case FTX_TUNE_SCALE_WINDOW:
        if (value < 2 || value > 4) return FT_ERR_BAD_SIZE;
        g_scale_w = value;
        return FT_ERR_NO_ERROR;
    default: return FT_ERR_BAD_SIZE;
    }
}

int ftx_tune_get(int knob)
{
    switch (knob) {
    case FTX_TUNE_LADDER_BLOCK: return ft::ladder_block();
    case FTX_TUNE_BATCH_ADD_PTS: return g_batch_add_pts;
    case FTX_TUNE_SCALE_WINDOW: return g_scale_w;
    default: return -1;
    }
}

ft_error ftx_reduce_into(ft_ge25519_array out, size_t out_idx, const_ft_ge25519_array src)
{
    ENSURE_INIT();
    if (out_idx >= out->n) return FT_ERR_OUT_OF_BOUNDS;
    void *s;
    CK(scratch(&s, ft::reduce_scratch_bytes(src->n)));
    CK(ft::reduce(ft::view_of(out, out_idx), ft::view_of(src), src->n, s, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ftx_scale_bounded(ft_ge25519_array array, uint32_t k, unsigned bits)
{
    ENSURE_INIT();
    if (bits < 1 || bits > 32 || (bits < 32 && (k >> bits))) return FT_ERR_BAD_SIZE;
    CK(ft::scale_small(ft::view_of(array), array->n, k, u32_ladder_windows(bits, g_scale_w), g_scale_w, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ftx_scale_small(ft_ge25519_array array, uint32_t k) { return ftx_scale_bounded(array, k, 32); }

} // extern "C"

// ---------------------------------------------------------------- serving helpers

namespace ft {

cudaMemPool_t host_pool() { return g.pool; }

// encryption tables of a public key for a server (cudaMalloc'd; the server
// frees them)
ft_error ftx_server_pk_table(const uint8_t *pk, uint32_t **table)
{
    *table = nullptr;
    cudaError_t e = cudaMalloc((void **)table, ENC_TABLES_BYTES);
    if (e != cudaSuccess) {
        *table = nullptr;
        return map_err(e);
    }
    ft_error err = build_key_tables(*table, pk);
    if (!err) {
        e = cudaStreamSynchronize(g.stream);
        if (e != cudaSuccess) err = map_err(e);
    }
    if (err) {
        cudaFree(*table);
        *table = nullptr;
    }
    return err;
}

} // namespace ft

// ---------------------------------------------------------------- batches

struct ftx_batch_s {
    std::vector<ft::BatchItem> items; // SEG items hold an index into offs in `off` until uploaded
    std::vector<int32_t> offs;
    std::set<const void *> written, read;
    // every recorded array with the storage it had then: the work items hold
    // raw device addresses, so a run refuses arrays that were reallocated
    struct Rec {
        const ft_ge25519_array_s *a;
        const uint4 *planes;
        size_t cap, n;
    };
    std::vector<Rec> arrays;
    size_t n_ops = 0;
    ft::BatchItem *d_items = nullptr;
    int32_t *d_offs = nullptr;
    unsigned *d_counter = nullptr;
    cudaGraphExec_t exec = nullptr;
    int w = 4; // window width of the scale items, fixed at upload
    bool ready = false;
};

namespace {

// an operation writing w and reading r must not touch what other operations
// of the batch write or read
ft_error claim(ftx_batch b, const void *w, const void *r)
{
    if (b->ready) return FT_ERR_BAD_SIZE;
    if (w && (b->written.count(w) || b->read.count(w))) return FT_ERR_BAD_SIZE;
    if (r && r != w && b->written.count(r)) return FT_ERR_BAD_SIZE;
    if (w) b->written.insert(w);
    if (r && r != w) b->read.insert(r);
    b->n_ops++;
    return FT_ERR_NO_ERROR;
}

void note(ftx_batch b, const_ft_ge25519_array a) { b->arrays.push_back({a, a->planes, a->cap, a->n}); }

// scales (longest ladders first), then segmented sums, then adds
int item_rank(const ft::BatchItem &it)
{
    return it.op == ft::BATCH_SCALE ? 9 - (int)it.nwin : (it.op == ft::BATCH_SEG ? 10 : 11);
}

ft_error batch_upload(ftx_batch b)
{
    // a failed upload may be retried: start from no device state
    dev_free(b->d_items);
    dev_free(b->d_offs);
    dev_free(b->d_counter);
    b->d_items = nullptr;
    b->d_offs = nullptr;
    b->d_counter = nullptr;
    b->w = g_scale_w;
    for (auto &it : b->items)
        if (it.op == ft::BATCH_SCALE) it.nwin = (uint32_t)u32_ladder_windows(it.bits, b->w);
    // costliest kinds first: the persistent blocks finish on short items
    std::stable_sort(b->items.begin(), b->items.end(),
                     [](const ft::BatchItem &x, const ft::BatchItem &y) { return item_rank(x) < item_rank(y); });
    CK(dev_alloc((void **)&b->d_offs, std::max<size_t>(b->offs.size(), 1) * sizeof(int32_t)));
    // the device copy holds offsets pointers; the host list keeps indices
    std::vector<ft::BatchItem> dev_items = b->items;
    for (auto &it : dev_items)
        if (it.op == ft::BATCH_SEG) it.off = b->d_offs + (uintptr_t)it.off;
    CK(dev_alloc((void **)&b->d_items, std::max<size_t>(b->items.size(), 1) * sizeof(ft::BatchItem)));
    CK(dev_alloc((void **)&b->d_counter, 256));
    if (!b->offs.empty())
        CK(cudaMemcpyAsync(b->d_offs, b->offs.data(), b->offs.size() * 4, cudaMemcpyHostToDevice, g.stream));
    if (!b->items.empty())
        CK(cudaMemcpyAsync(b->d_items, dev_items.data(), dev_items.size() * sizeof(ft::BatchItem),
                           cudaMemcpyHostToDevice, g.stream));
    CK(cudaStreamSynchronize(g.stream));
    CK(ft::batch_prepare(b->w));
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = ft::batch_launch(b->d_items, (int)b->items.size(), b->d_counter, b->w, g.stream);
    cudaError_t ce = cudaStreamEndCapture(g.stream, &graph);
    if (le != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return map_err(le);
    }
    CK(ce);
    cudaError_t ie = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ie);
    b->ready = true;
    return FT_ERR_NO_ERROR;
}

} // namespace

extern "C" {

ft_error ftx_batch_create(ftx_batch *batch)
{
    ENSURE_INIT();
    *batch = new (std::nothrow) ftx_batch_s();
    return *batch ? FT_ERR_NO_ERROR : FT_ERR_OUT_OF_MEMORY;
}

ft_error ftx_batch_add(ftx_batch b, ft_ge25519_array res, const_ft_ge25519_array summand)
{
    if (res->n != summand->n) return FT_ERR_SIZE_MISMATCH;
    ft_error err = claim(b, res->planes, summand->planes);
    if (err) return err;
    note(b, res);
    note(b, summand);
    const size_t per = (size_t)ft::batch_block() * g_batch_add_pts;
    for (size_t base = 0; base < res->n; base += per) {
        ft::BatchItem it{};
        it.op = ft::BATCH_ADD;
        it.count = (uint32_t)std::min(per, res->n - base);
        it.dst = res->planes + base;
        it.dst_s = res->cap;
        it.src = summand->planes + base;
        it.src_s = summand->cap;
        b->items.push_back(it);
    }
    return FT_ERR_NO_ERROR;
}

ft_error ftx_batch_scale_bounded(ftx_batch b, ft_ge25519_array a, uint32_t k, unsigned bits)
{
    if (bits < 1 || bits > 32 || (bits < 32 && (k >> bits))) return FT_ERR_BAD_SIZE;
    ft_error err = claim(b, a->planes, nullptr);
    if (err) return err;
    note(b, a);
    const size_t per = (size_t)ft::batch_block();
    for (size_t base = 0; base < a->n; base += per) {
        ft::BatchItem it{};
        it.op = ft::BATCH_SCALE;
        it.count = (uint32_t)std::min(per, a->n - base);
        it.dst = a->planes + base;
        it.dst_s = a->cap;
        it.k = k;
        it.bits = bits; // windows fixed at upload, for the batch's width
        b->items.push_back(it);
    }
    return FT_ERR_NO_ERROR;
}

ft_error ftx_batch_scale_small(ftx_batch b, ft_ge25519_array a, uint32_t k)
{
    return ftx_batch_scale_bounded(b, a, k, 32);
}

ft_error ftx_batch_segmented_sum(ftx_batch b, ft_ge25519_array out, const int32_t *off, size_t nseg,
                                 const_ft_ge25519_array src)
{
    if (out->n != nseg) return FT_ERR_SIZE_MISMATCH;
    if (src->n >= (size_t)INT32_MAX || off[0] != 0 || (size_t)off[nseg] != src->n) return FT_ERR_BAD_SIZE;
    for (size_t s = 0; s < nseg; ++s)
        if (off[s + 1] < off[s]) return FT_ERR_BAD_SIZE;
    ft_error err = claim(b, out->planes, src->planes);
    if (err) return err;
    note(b, out);
    note(b, src);
    const size_t base_off = b->offs.size();
    b->offs.insert(b->offs.end(), off, off + nseg + 1);
    const size_t per = (size_t)ft::batch_block();
    for (size_t s0 = 0; s0 < nseg; s0 += per) {
        ft::BatchItem it{};
        it.op = ft::BATCH_SEG;
        it.count = (uint32_t)std::min(per, nseg - s0);
        it.dst = out->planes + s0;
        it.dst_s = out->cap;
        it.src = src->planes;
        it.src_s = src->cap;
        it.off = (const int32_t *)(uintptr_t)(base_off + s0); // patched at upload
        b->items.push_back(it);
    }
    return FT_ERR_NO_ERROR;
}

ft_error ftx_batch_run(ftx_batch b)
{
    ENSURE_INIT();
    for (const auto &r : b->arrays)
        if (r.a->planes != r.planes || r.a->cap != r.cap || r.a->n != r.n) return FT_ERR_SIZE_MISMATCH;
    for (const auto &r : b->arrays) r.a->touch.fetch_add(1); // the run hands their storage to the kernel
    if (!b->ready) {
        ft_error err = batch_upload(b);
        if (err) return err;
    }
    CK(cudaGraphLaunch(b->exec, g.stream));
    return FT_ERR_NO_ERROR;
}

ft_error ftx_batch_info(ftx_batch b, size_t *n_items, size_t *n_ops)
{
    *n_items = b->items.size();
    *n_ops = b->n_ops;
    return FT_ERR_NO_ERROR;
}

void ftx_batch_free(ftx_batch b)
{
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (g.inited) {
        dev_free(b->d_items);
        dev_free(b->d_offs);
        dev_free(b->d_counter);
    }
    delete b;
}

} // extern "C"
