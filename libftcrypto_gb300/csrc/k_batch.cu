// k_batch.cu — the batched form: one persistent kernel for thousands of
// independent, uneven array operations, and the small-scalar ladder.
//
// k_batch: one block per SM (384 threads: the ladder tables of the scale
//   path fill the SM's shared memory and half of its tensor memory, as in
//   k_smul_var_tm).  Each warp loops pulling a 32-thread slice of a work item
//   (item i, slice j: the item's logical threads 32j..32j+31) from an atomic
//   counter until the list is exhausted, so a warp that finishes its slice
//   early takes the next one instead of waiting at a block barrier for the
//   item's slowest warp.  Items are pre-sorted costliest first, so the tail
//   of the run is short ones (longest-processing-time order).  Item kinds:
//     ADD    dst[i] += src[i] for count points (count <= 384 x points/thread)
//     SCALE  dst[i] = k * dst[i], count <= 384 points, one per thread,
//            constant time in k < 2^bits (smul_ladder_u32 in nwin windows
//            of the batch's width W, a template parameter of the kernel)
//     SEG    dst[s] = sum of src[off[s] .. off[s+1]), count <= 384 segments,
//            one per thread (segments of the batched workload are short)
//   The host side (ft_api.cu, ftx_batch_*) captures {counter reset, k_batch}
//   in a CUDA graph and replays it.
// k_scale_small: ftx_scale_small, the same small-scalar ladder over one array.
//
// Both kernels allocate all 512 TMEM columns from warp 0 at entry and free
// them after a final barrier (tmem.cuh); their shared memory admits one
// block per SM.  In a SCALE item the warps past the item's count skip it
// (a warp-uniform test) and the lanes past it in the last warp run the
// ladder on the identity and store nothing, so every warp executes the
// warp-wide tcgen05 instructions converged.
#include "internal.h"
#include "ladder.cuh"

namespace ft {

static constexpr int BATCH_NT = 384;

// k * (point i of p) for the lanes with live set, the identity for the
// rest, in nwin windows of width W (a table of 2^(W-1) entries)
template <int W>
FT_DEV void scale_small_lane(uint4 *p, size_t s, size_t i, bool live, uint32_t k, int nwin,
                             const HybridTab<BATCH_NT> &tab)
{
    ge_p3 P, h;
    if (live) ld_p3(P, p, s, i);
    else ge_p3_0(P);
    __syncwarp();
    smul_build_table<1 << (W - 1)>(tab, P);
    tmem_wait_st();
    smul_ladder_u32<W>(h, k, tab, nwin);
    if (live) st_p3(p, s, i, h);
}

static constexpr int BATCH_WARPS = BATCH_NT / 32; // slices of an item

template <int W>
__global__ void __maxnreg__(tm_max_regs<BATCH_NT>())
    k_batch(const BatchItem *items, int nitems, unsigned *counter)
{
    extern __shared__ uint4 smem[];
    __shared__ uint32_t s_taddr;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tmem_alloc(&s_taddr, 512u);
    tmem_sync_threads();
    const HybridTab<BATCH_NT> tab{smem + tid, tmem_warp_addr(s_taddr, warp, 128u * (uint32_t)(warp >> 2))};
    const unsigned nslices = (unsigned)nitems * BATCH_WARPS; // < 2^31 (checked at launch)
    for (;;) {
        unsigned sl = 0;
        if (lane == 0) sl = atomicAdd(counter, 1u);
        sl = __shfl_sync(0xffffffffu, sl, 0);
        if (sl >= nslices) break;
        const int it = (int)(sl / BATCH_WARPS);
        const uint32_t tt = (sl % BATCH_WARPS) * 32u + (uint32_t)lane; // logical thread of the item
        const BatchItem w = items[it];
        if (w.op == BATCH_ADD) {
#pragma unroll 1
            for (uint32_t e = tt; e < w.count; e += BATCH_NT) {
                ge_p3 x, y;
                ld_p3(x, w.dst, w.dst_s, e);
                ld_p3(y, w.src, w.src_s, e);
                ge_addto(x, y);
                st_p3(w.dst, w.dst_s, e, x);
            }
        } else if (w.op == BATCH_SCALE) {
            if (tt - (uint32_t)lane < w.count) // warp-uniform
                scale_small_lane<W>(w.dst, w.dst_s, tt, tt < w.count, w.k, (int)w.nwin, tab);
        } else { // BATCH_SEG
#pragma unroll 1
            for (uint32_t sg = tt; sg < w.count; sg += BATCH_NT) {
                const int32_t a = w.off[sg], b = w.off[sg + 1];
                ge_p3 acc;
                ge_p3_0(acc);
                if (a < b) ld_p3(acc, w.src, w.src_s, a);
#pragma unroll 1
                for (int32_t e = a + 1; e < b; ++e) {
                    ge_p3 x;
                    ld_p3(x, w.src, w.src_s, e);
                    ge_addto(acc, x);
                }
                st_p3(w.dst, w.dst_s, sg, acc);
            }
        }
    }
    tmem_sync_threads();
    if (warp == 0) tmem_free(s_taddr, 512u);
}

template <int W>
__global__ void __maxnreg__(tm_max_regs<BATCH_NT>())
    k_scale_small(uint4 *p, size_t s, size_t n, uint32_t k, int nwin)
{
    extern __shared__ uint4 smem[];
    __shared__ uint32_t s_taddr;
    const int warp = threadIdx.x >> 5;
    if (warp == 0) tmem_alloc(&s_taddr, 512u);
    tmem_sync_threads();
    const size_t i = (size_t)blockIdx.x * BATCH_NT + threadIdx.x;
    const HybridTab<BATCH_NT> tab{smem + threadIdx.x, tmem_warp_addr(s_taddr, warp, 128u * (uint32_t)(warp >> 2))};
    if ((size_t)blockIdx.x * BATCH_NT + (size_t)warp * 32 < n) // warp-uniform
        scale_small_lane<W>(p, s, i, i < n, k, nwin, tab);
    tmem_sync_threads();
    if (warp == 0) tmem_free(s_taddr, 512u);
}

int batch_block() { return BATCH_NT; }

size_t batch_smem_bytes() { return ladder_smem_bytes<BATCH_NT>(); }

// the instantiations of a window width w in {2, 3, 4} (index w - 2)
static const void *const k_batch_fn[3] = {(const void *)k_batch<2>, (const void *)k_batch<3>,
                                          (const void *)k_batch<4>};
static const void *const k_scale_fn[3] = {(const void *)k_scale_small<2>, (const void *)k_scale_small<3>,
                                          (const void *)k_scale_small<4>};
static SmemAttr g_batch_attr[3], g_scale_attr[3];

static bool width_ok(int w) { return w >= 2 && w <= 4; }

cudaError_t batch_prepare(int w)
{
    if (!width_ok(w)) return cudaErrorInvalidValue;
    return ensure_smem_attr(g_batch_attr[w - 2], k_batch_fn[w - 2], batch_smem_bytes());
}

cudaError_t batch_launch(const BatchItem *d_items, int nitems, unsigned *d_counter, int w, cudaStream_t st)
{
    if (nitems < 0 || (long long)nitems * BATCH_WARPS >= (1ll << 31)) return cudaErrorInvalidValue;
    cudaError_t e = batch_prepare(w);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned), st)) != cudaSuccess) return e;
    const unsigned g = (unsigned)sm_count();
    const size_t sm = batch_smem_bytes();
    if (w == 2) k_batch<2><<<g, BATCH_NT, sm, st>>>(d_items, nitems, d_counter);
    else if (w == 3) k_batch<3><<<g, BATCH_NT, sm, st>>>(d_items, nitems, d_counter);
    else k_batch<4><<<g, BATCH_NT, sm, st>>>(d_items, nitems, d_counter);
    return cudaGetLastError();
}

cudaError_t scale_small(View v, size_t n, uint32_t k, int nwin, int w, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (!width_ok(w)) return cudaErrorInvalidValue;
    cudaError_t e = ensure_smem_attr(g_scale_attr[w - 2], k_scale_fn[w - 2], batch_smem_bytes());
    if (e != cudaSuccess) return e;
    const unsigned g = (unsigned)((n + BATCH_NT - 1) / BATCH_NT);
    const size_t sm = batch_smem_bytes();
    if (w == 2) k_scale_small<2><<<g, BATCH_NT, sm, st>>>(v.p, v.s, n, k, nwin);
    else if (w == 3) k_scale_small<3><<<g, BATCH_NT, sm, st>>>(v.p, v.s, n, k, nwin);
    else k_scale_small<4><<<g, BATCH_NT, sm, st>>>(v.p, v.s, n, k, nwin);
    return cudaGetLastError();
}

} // namespace ft
