// serve.cu — the serving form (ftx_server_*): a request loop with
// continuous batching over device-resident ciphertext arrays.
//
// One worker thread per server.  Requests are queued by submit() (any
// thread) and admitted as soon as one of the server's CUDA streams ("slots")
// is free and the request's device memory fits the HBM budget.  An admitted
// request's inputs are staged and its kernels queued on its slot's stream,
// so requests in flight overlap on the GPU; a host callback at the end of
// the stream marks completion, and the worker then returns the request's
// temporary memory and budget.  The arithmetic is the library's, launched on
// the slot stream, so a request's result does not depend on what else runs.
//
// Express lane: the request mix spans four orders of magnitude of work, and
// the block scheduler dispatches a kernel's blocks in launch order, so a
// small request queued behind a large one waits for nearly all of it.  Half
// of the slots (the later ones) are created at the device's highest stream
// priority; requests whose estimated work is at most EXPRESS_COST ladder
// points (a few milliseconds of GPU time) prefer those slots, and their
// blocks are dispatched as soon as SMs free up.  Admission is FIFO within
// each class; an express request may overtake queued bulk requests (the
// requests of a server touch disjoint arrays, so order does not matter).
//
// Budget: a request is charged its temporaries (staged inputs, scratch)
// while it runs and the arrays it creates (ENCRYPT, SEGSUM outputs) from
// admission until the caller hands them back with ftx_server_release, so
// the budget bounds what the server keeps resident, not only what is in
// flight.
#include <algorithm>
#include <new>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <list>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.h"
#include "../../include/ftcrypto.h"
#include "../../include/ftcrypto_gb300.h"

namespace ft {
cudaMemPool_t host_pool(); // ft_api.cu
}

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    ftx_request r;
    uint64_t ticket = 0;
    size_t bytes = 0;     // temporaries, charged while the request runs
    size_t out_bytes = 0; // arrays it creates, charged until released
    Clock::time_point t_submit, t_admit, t_done;
    ftx_result res{};
    int slot = -1;
    bool express = false;   // small enough for the high-priority slots
    bool seg_prefix = false; // SEGSUM with long segments: summed through a scan
    bool done = false;      // set by the stream callback
    bool finished = false;  // result published
    std::vector<void *> tmp;
};

struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t lib_done = nullptr; // orders the slot after the library stream
    Req *req = nullptr;
    bool express = false;           // created at the highest stream priority
};

// estimated work in variable-base ladder points (the ladder is the unit:
// one encryption costs ~0.65 of one, a point addition ~1/40)
constexpr double EXPRESS_COST = 131072.0;

double request_cost(const ftx_request &r)
{
    switch (r.op) {
    case FTX_REQ_ENCRYPT: return 0.65 * (double)r.n;
    case FTX_REQ_RERAND: return 0.7 * (double)r.n;
    case FTX_REQ_SMUL: return 2.0 * (double)r.n;
    case FTX_REQ_SEGSUM: return 0.06 * (double)r.n;
    default: return 0.0;
    }
}

// device bytes of the arrays a request creates (its two output arrays)
size_t request_out_bytes(const ftx_request &r)
{
    const size_t pts = FT_PLANES_BYTES_PER_POINT;
    switch (r.op) {
    case FTX_REQ_ENCRYPT: return 2 * r.n * pts;
    case FTX_REQ_SEGSUM: return 2 * r.nseg * pts;
    default: return 0;
    }
}

// device bytes a request takes only while it runs (staged inputs, scratch)
size_t request_tmp_bytes(const ftx_request &r, bool seg_prefix)
{
    switch (r.op) {
    case FTX_REQ_ENCRYPT: return r.n * 40 + 4096;
    case FTX_REQ_RERAND: return r.n * 32 + 4096;
    case FTX_REQ_SMUL: return r.n * 32 + 4096;
    case FTX_REQ_SEGSUM:
        return (r.nseg + 1) * 4 + 8192 +
               2 * (seg_prefix ? ft::segsum_prefix_scratch_bytes(r.n) : ft::segsum_scratch_bytes(r.n));
    default: return 0;
    }
}

} // namespace

struct ftx_server_s {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::list<Req *> pending; // iterators stay valid while submitters append
    std::map<uint64_t, Req *> reqs;
    std::vector<Slot> slots;
    // in_use: temporaries and outputs of running requests; resident: outputs
    // of finished requests not yet released (held maps each to its bytes)
    size_t budget = 0, in_use = 0, resident = 0, running = 0;
    std::map<ft_ge25519_array, size_t> held;
    uint64_t next_ticket = 1;
    bool stop = false;
    uint32_t *pk_table = nullptr;
    int device = 0;
    std::thread worker;

    ft_error dispatch(Req *q, Slot &sl);
    Slot *free_slot(bool express);
    void admit(std::unique_lock<std::mutex> &lk, Req *q, Slot *sl);
    void loop();
};

static void CUDART_CB on_stream_done(void *arg)
{
    auto *pair = (std::pair<ftx_server, Req *> *)arg;
    ftx_server s = pair->first;
    Req *q = pair->second;
    delete pair;
    std::lock_guard<std::mutex> lk(s->mu);
    q->t_done = Clock::now();
    q->done = true;
    s->cv_work.notify_all();
}

static cudaError_t alloc_on(Req *q, void **p, size_t bytes, cudaStream_t st)
{
    *p = nullptr;
    if (!bytes) return cudaSuccess;
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes, ft::host_pool(), st);
    if (e == cudaSuccess) q->tmp.push_back(*p);
    return e;
}

static cudaError_t new_array(ft_ge25519_array *out, size_t n, cudaStream_t st)
{
    auto *a = new (std::nothrow) ft_ge25519_array_s();
    if (!a) return cudaErrorMemoryAllocation;
    a->n = a->cap = n;
    cudaError_t e = n ? cudaMallocFromPoolAsync((void **)&a->planes, n * FT_PLANES_BYTES_PER_POINT, ft::host_pool(), st)
                      : cudaSuccess;
    if (e != cudaSuccess) {
        delete a;
        return e;
    }
    *out = a;
    return cudaSuccess;
}

// queue the request's copies and kernels on the slot's stream
ft_error ftx_server_s::dispatch(Req *q, Slot &sl)
{
    const ftx_request &r = q->r;
    cudaStream_t st = sl.st;
    // arrays handed in may still be written by work queued on the library's
    // stream (ft_* calls return before their kernels finish)
    cudaError_t e = cudaEventRecord(sl.lib_done, (cudaStream_t)ftx_stream());
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, sl.lib_done, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return FT_ERR_INTERNAL_LIBRARY_ERROR;
    }
    auto enc = [&](ft_ge25519_array a, ft_ge25519_array b, const uint64_t *hm, unsigned bits) -> cudaError_t {
        void *dr, *dm;
        cudaError_t x = alloc_on(q, &dr, r.n * 32, st);
        if (x == cudaSuccess) x = alloc_on(q, &dm, r.n * 8, st);
        if (x == cudaSuccess) x = cudaMemcpyAsync(dr, r.r, r.n * 32, cudaMemcpyHostToDevice, st);
        if (x == cudaSuccess)
            x = hm ? cudaMemcpyAsync(dm, hm, r.n * 8, cudaMemcpyHostToDevice, st) : cudaMemsetAsync(dm, 0, r.n * 8, st);
        if (x == cudaSuccess)
            x = ft::encrypt(ft::view_of(a), ft::view_of(b), r.n, (const uint8_t *)dr, (const uint64_t *)dm,
                            enc_digits(bits), pk_table, st);
        return x;
    };
    switch (r.op) {
    case FTX_REQ_ENCRYPT: {
        e = new_array(&q->res.c1, r.n, st);
        if (e == cudaSuccess) e = new_array(&q->res.c2, r.n, st);
        if (e == cudaSuccess) e = enc(q->res.c1, q->res.c2, r.m, r.plaintext_bits);
        break;
    }
    case FTX_REQ_RERAND: { // (c1, c2) += Enc(0; r), fused into the encryption kernel
        void *dr;
        e = alloc_on(q, &dr, r.n * 32, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dr, r.r, r.n * 32, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = ft::rerandomise(ft::view_of(r.c1), ft::view_of(r.c2), r.n, (const uint8_t *)dr, pk_table, st);
        q->res.c1 = r.c1;
        q->res.c2 = r.c2;
        break;
    }
    case FTX_REQ_SMUL: {
        void *dk;
        e = alloc_on(q, &dk, r.n * 32, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dk, r.k, r.n * 32, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = ft::smul_var(ft::view_of(r.c1), r.n, (const uint8_t *)dk, 1, st);
        if (e == cudaSuccess) e = ft::smul_var(ft::view_of(r.c2), r.n, (const uint8_t *)dk, 1, st);
        q->res.c1 = r.c1;
        q->res.c2 = r.c2;
        break;
    }
    case FTX_REQ_SEGSUM: {
        void *doff, *s;
        e = new_array(&q->res.c1, r.nseg, st);
        if (e == cudaSuccess) e = new_array(&q->res.c2, r.nseg, st);
        if (e == cudaSuccess) e = alloc_on(q, &doff, (r.nseg + 1) * 4, st);
        const size_t sb = q->seg_prefix ? ft::segsum_prefix_scratch_bytes(r.n) : ft::segsum_scratch_bytes(r.n);
        if (e == cudaSuccess) e = alloc_on(q, &s, 2 * sb, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(doff, r.offsets, (r.nseg + 1) * 4, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && q->seg_prefix) {
            e = ft::segsum_prefix(ft::view_of(q->res.c1), (const int32_t *)doff, r.nseg, ft::view_of(r.c1), r.n,
                                  nullptr, 0, s, st);
            if (e == cudaSuccess)
                e = ft::segsum_prefix(ft::view_of(q->res.c2), (const int32_t *)doff, r.nseg, ft::view_of(r.c2), r.n,
                                      nullptr, 0, (uint8_t *)s + sb, st);
        } else if (e == cudaSuccess) {
            // both halves through the same walk and join launches
            const ft::View outs[2] = {ft::view_of(q->res.c1), ft::view_of(q->res.c2)};
            const ft::View srcs[2] = {ft::view_of(r.c1), ft::view_of(r.c2)};
            e = ft::segsum_set(outs, srcs, 2, (const int32_t *)doff, r.nseg, r.n, nullptr, 0, s, st);
        }
        break;
    }
    default: return FT_ERR_BAD_SIZE;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? FT_ERR_OUT_OF_MEMORY : FT_ERR_INTERNAL_LIBRARY_ERROR;
    }
    auto *arg = new std::pair<ftx_server, Req *>(this, q);
    if (cudaLaunchHostFunc(st, on_stream_done, arg) != cudaSuccess) {
        delete arg;
        cudaGetLastError();
        return FT_ERR_INTERNAL_LIBRARY_ERROR;
    }
    return FT_ERR_NO_ERROR;
}

// a free slot for a request of the class: express requests take an express
// slot if one is free, else any; bulk requests only bulk slots
Slot *ftx_server_s::free_slot(bool express)
{
    Slot *any = nullptr;
    for (Slot &sl : slots) {
        if (sl.req) continue;
        if (sl.express == express) return &sl;
        if (express && !any) any = &sl;
    }
    return any;
}

// start q on sl (called with the lock held; dispatch runs unlocked so that
// callbacks and submitters never wait on CUDA calls)
void ftx_server_s::admit(std::unique_lock<std::mutex> &lk, Req *q, Slot *sl)
{
    q->t_admit = Clock::now();
    q->slot = (int)(sl - slots.data());
    in_use += q->bytes + q->out_bytes;
    running++;
    sl->req = q;
    lk.unlock();
    ft_error err = dispatch(q, *sl);
    lk.lock();
    if (!err) return;
    // finish q with the error; its memory is released in stream order
    q->res.err = err;
    if (q->r.op == FTX_REQ_ENCRYPT || q->r.op == FTX_REQ_SEGSUM) {
        for (ft_ge25519_array *a : {&q->res.c1, &q->res.c2})
            if (*a) {
                if ((*a)->planes) cudaFreeAsync((*a)->planes, sl->st);
                delete *a;
                *a = nullptr;
            }
    }
    for (void *p : q->tmp) cudaFreeAsync(p, sl->st);
    q->tmp.clear();
    in_use -= q->bytes + q->out_bytes;
    running--;
    sl->req = nullptr;
    q->t_done = Clock::now();
    q->finished = true;
    cv_done.notify_all();
}

void ftx_server_s::loop()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
        // reclaim completed requests
        for (Slot &sl : slots) {
            Req *q = sl.req;
            if (!q || !q->done) continue;
            for (void *p : q->tmp) cudaFreeAsync(p, sl.st);
            q->tmp.clear();
            in_use -= q->bytes + q->out_bytes;
            running--;
            if (q->r.op == FTX_REQ_ENCRYPT || q->r.op == FTX_REQ_SEGSUM) { // charged until released
                resident += q->out_bytes;
                held[q->res.c1] = q->out_bytes / 2;
                held[q->res.c2] = q->out_bytes - q->out_bytes / 2;
            }
            q->res.queue_ms = std::chrono::duration<double, std::milli>(q->t_admit - q->t_submit).count();
            q->res.latency_ms = std::chrono::duration<double, std::milli>(q->t_done - q->t_submit).count();
            q->finished = true;
            sl.req = nullptr;
            cv_done.notify_all();
        }
        // admit in arrival order within each class while a slot is free and
        // memory fits; a bulk request that cannot start holds the later bulk
        // ones back, an express one the later express ones
        bool bulk_open = true, express_open = true;
        for (auto it = pending.begin(); it != pending.end() && (bulk_open || express_open);) {
            Req *q = *it;
            bool &open = q->express ? express_open : bulk_open;
            if (!open) {
                ++it;
                continue;
            }
            const bool fits = in_use + resident + q->bytes + q->out_bytes <= budget;
            Slot *sl = fits ? free_slot(q->express) : nullptr;
            if (!sl) {
                open = false;
                ++it;
                continue;
            }
            it = pending.erase(it);
            admit(lk, q, sl);
        }
        if (stop && pending.empty() && running == 0) break;
        // submit, stop and every completion notify cv_work; with nothing
        // queued or running the worker sleeps until one of them does
        if (pending.empty() && running == 0) cv_work.wait(lk);
        else cv_work.wait_for(lk, std::chrono::microseconds(200));
    }
}

namespace ft {
ft_error ftx_server_pk_table(const uint8_t *pk, uint32_t **table); // ft_api.cu
}

extern "C" {

ft_error ftx_server_create(ftx_server *server, const uint8_t *pk, size_t hbm_budget_bytes, int slots)
{
    if (slots < 1 || slots > 64 || hbm_budget_bytes == 0) return FT_ERR_BAD_SIZE;
    ft_error err = ft_crypto_init();
    if (err) return err;
    auto *s = new (std::nothrow) ftx_server_s();
    if (!s) return FT_ERR_OUT_OF_MEMORY;
    if ((err = ft::ftx_server_pk_table(pk, &s->pk_table))) {
        delete s;
        return err;
    }
    cudaGetDevice(&s->device);
    s->budget = hbm_budget_bytes;
    s->slots.resize(slots);
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    const int n_bulk = (slots + 1) / 2;
    for (int i = 0; i < slots; ++i) {
        Slot &sl = s->slots[i];
        sl.express = i >= n_bulk;
        if (cudaStreamCreateWithPriority(&sl.st, cudaStreamNonBlocking, sl.express ? prio_high : prio_low) !=
                cudaSuccess ||
            cudaEventCreateWithFlags(&sl.lib_done, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            ftx_server_free(s);
            return FT_ERR_INTERNAL_LIBRARY_ERROR;
        }
    }
    s->worker = std::thread([s] { s->loop(); });
    *server = s;
    return FT_ERR_NO_ERROR;
}

ft_error ftx_server_submit(ftx_server s, const ftx_request *req, uint64_t *ticket)
{
    const ftx_request &r = *req;
    if (r.op < FTX_REQ_ENCRYPT || r.op > FTX_REQ_SEGSUM) return FT_ERR_BAD_SIZE;
    if (r.op == FTX_REQ_ENCRYPT) {
        if (r.plaintext_bits < 1 || r.plaintext_bits > 64) return FT_ERR_BAD_SIZE;
        if (r.m && r.plaintext_bits < 64) { // the comb reads only the digits of the bound
            uint64_t acc = 0;
            for (size_t i = 0; i < r.n; ++i) acc |= r.m[i];
            if (acc >> r.plaintext_bits) return FT_ERR_BAD_SIZE;
        }
    }
    if (r.op != FTX_REQ_ENCRYPT && (!r.c1 || !r.c2 || r.c1->n != r.n || r.c2->n != r.n)) return FT_ERR_SIZE_MISMATCH;
    size_t maxlen = 0;
    if (r.op == FTX_REQ_SEGSUM) {
        if (r.n >= (size_t)INT32_MAX || r.offsets[0] != 0 || (size_t)r.offsets[r.nseg] != r.n) return FT_ERR_BAD_SIZE;
        for (size_t i = 0; i < r.nseg; ++i) {
            if (r.offsets[i + 1] < r.offsets[i]) return FT_ERR_BAD_SIZE;
            maxlen = std::max(maxlen, (size_t)(r.offsets[i + 1] - r.offsets[i]));
        }
    }
    auto *q = new (std::nothrow) Req();
    if (!q) return FT_ERR_OUT_OF_MEMORY;
    q->r = r;
    q->seg_prefix = r.op == FTX_REQ_SEGSUM && ft::segsum_prefers_prefix(r.n, maxlen);
    q->bytes = request_tmp_bytes(r, q->seg_prefix);
    q->out_bytes = request_out_bytes(r);
    q->express = request_cost(r) <= EXPRESS_COST;
    if (q->bytes + q->out_bytes > s->budget) {
        delete q;
        return FT_ERR_INSUFFICIENT_SPACE;
    }
    q->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    q->ticket = s->next_ticket++;
    s->reqs[q->ticket] = q;
    s->pending.push_back(q);
    *ticket = q->ticket;
    s->cv_work.notify_all();
    return FT_ERR_NO_ERROR;
}

ft_error ftx_server_wait(ftx_server s, uint64_t ticket, ftx_result *result)
{
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return FT_ERR_OUT_OF_BOUNDS;
    Req *q = it->second;
    s->cv_done.wait(lk, [q] { return q->finished; });
    *result = q->res;
    s->reqs.erase(it);
    delete q;
    return FT_ERR_NO_ERROR;
}

ft_error ftx_server_release(ftx_server s, ft_ge25519_array array)
{
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->held.find(array);
        if (it == s->held.end()) return FT_ERR_OUT_OF_BOUNDS;
        s->resident -= it->second;
        s->held.erase(it);
        s->cv_work.notify_all(); // queued requests may fit now
    }
    ft_array_free(array); // its request has completed: nothing on the GPU uses it
    return FT_ERR_NO_ERROR;
}

ft_error ftx_server_stats(ftx_server s, size_t *bytes_in_use, size_t *queued, size_t *running)
{
    std::lock_guard<std::mutex> lk(s->mu);
    *bytes_in_use = s->in_use + s->resident;
    *queued = s->pending.size();
    *running = s->running;
    return FT_ERR_NO_ERROR;
}

void ftx_server_free(ftx_server s)
{
    if (!s) return;
    if (s->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
            s->cv_work.notify_all();
        }
        s->worker.join();
    }
    for (Slot &sl : s->slots) {
        if (sl.st) {
            cudaStreamSynchronize(sl.st);
            cudaStreamDestroy(sl.st);
        }
        if (sl.lib_done) cudaEventDestroy(sl.lib_done);
    }
    // requests whose results were never collected: their new arrays are
    // nobody's, so they go with the server (the worker has drained them all)
    for (auto &kv : s->reqs) {
        Req *q = kv.second;
        if (q->finished && !q->res.err && (q->r.op == FTX_REQ_ENCRYPT || q->r.op == FTX_REQ_SEGSUM)) {
            s->held.erase(q->res.c1);
            s->held.erase(q->res.c2);
            ft_array_free(q->res.c1);
            ft_array_free(q->res.c2);
        }
        delete q;
    }
    if (s->pk_table) cudaFree(s->pk_table);
    delete s;
}

} // extern "C"
