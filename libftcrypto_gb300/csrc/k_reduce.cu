// k_reduce.cu — reductions whose combine operator is point addition.
//
//   reduce   sum of n points (ft_array_reduce; k_ft_array_reduce,
//            ftcrypto.cu:1414-1471).  Pass 1: every thread accumulates a
//            grid-strided subset with one ge_addto (9 multiplications) per
//            point, then warp-shuffle and block trees leave one partial per
//            block; pass 2 reduces the partials in one block.  ~1 addition per
//            input point (the reference's tree does the same count but with
//            most threads idle at the upper levels and 160-byte AoS loads).
//   scan     inclusive / exclusive prefix (ft_array_scan / ft_array_prescan;
//            ftcrypto.cu:1474-1586) as reduce-then-scan over chunks of
//            NT*K points: (A) per-thread sums of K consecutive points and per-
//            chunk sums, (B) exclusive scan of the chunk sums (recursively),
//            (C) block scan of the thread sums and a sequential rescan of each
//            thread's K points.  ~2 + 8/K additions per point and no waits
//            between blocks.  Correct for every length (the reference's
//            kernel indexes its tile sums wrongly above 256 x grid points,
//            ftcrypto.cu:1512).
//   segsum   out[s] = sum of src[e] (or src[perm[e]]) for e in
//            [off[s], off[s+1]): each block owns a contiguous range of whole
//            segments; within it, chunks of NT*K points in which every thread
//            sums its K consecutive points segment by segment, writes the
//            segments that begin and end inside it, and gets the partial sum
//            of the segment it starts inside from a block-wide segmented scan
//            of (has-segment-start, running sum) pairs.  ~1 + 8/K additions
//            per point.  It serves ft_reduce_isum (ftcrypto.cu:1113-1217,
//            accumulating into res) and the CSR segmented-sum extension.
//   keys_to_csr  counting sort of ft_reduce_isum's keys on the device
//            (replaces the reference's host std::sort, ftcrypto.cu:1170).
#include "internal.h"
#include "points.cuh"

namespace ft {

// ------------------------------------------------------------ block trees

// sum over the block; the result is valid in thread 0
template <int NT>
FT_DEV void block_sum(ge_p3 &acc, uint4 *sm /* (NT/32) * 8 uint4 */)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll 1
    for (int o = 16; o > 0; o >>= 1) {
        ge_p3 other;
        shfl_down_p3(other, acc, o);
        ge_addto(acc, other);
    }
    if (NT > 32) {
        if (lane == 0) sm_st_p3(sm, warp, acc);
        __syncthreads();
        if (warp == 0) {
            if (lane < NT / 32) sm_ld_p3(acc, sm, lane);
            else ge_p3_0(acc);
#pragma unroll 1
            for (int o = (NT / 64 > 0 ? NT / 64 : 1); o > 0; o >>= 1) {
                ge_p3 other;
                shfl_down_p3(other, acc, o);
                ge_addto(acc, other);
            }
        }
    }
}

template <int NT>
__global__ void __launch_bounds__(NT) k_reduce(const uint4 *p, size_t s, size_t n, uint4 *out, size_t os)
{
    __shared__ uint4 sm[(NT / 32) * 8];
    ge_p3 acc;
    size_t i = (size_t)blockIdx.x * NT + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * NT;
    if (i < n) {
        ld_p3(acc, p, s, i);
        i += stride;
    } else {
        ge_p3_0(acc);
    }
#pragma unroll 1
    for (; i < n; i += stride) {
        ge_p3 x;
        ld_p3(x, p, s, i);
        ge_addto(acc, x);
    }
    block_sum<NT>(acc, sm);
    if (threadIdx.x == 0) st_p3(out, os, blockIdx.x, acc);
}

// ------------------------------------------------------------ scan

// inclusive scan over the warp; returns the lane's inclusive sum in acc
FT_DEV void warp_scan_incl(ge_p3 &acc)
{
    const int lane = threadIdx.x & 31;
#pragma unroll 1
    for (int o = 1; o < 32; o <<= 1) {
        ge_p3 up, sum;
        shfl_up_p3(up, acc, o);
        sum = up;
        ge_addto(sum, acc);
        if (lane >= o) acc = sum;
    }
}

// exclusive block scan of x; returns the thread's exclusive prefix.  NT <= 1024.
template <int NT>
FT_DEV void block_scan_excl(ge_p3 &ex, const ge_p3 &x, uint4 *sm /* (NT/32) * 8 */)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ge_p3 incl = x;
    warp_scan_incl(incl);
    if (lane == 31) sm_st_p3(sm, warp, incl);
    __syncthreads();
    if (warp == 0) {
        ge_p3 w;
        if (lane < NT / 32) sm_ld_p3(w, sm, lane);
        else ge_p3_0(w);
        warp_scan_incl(w);
        ge_p3 wex;
        shfl_up_p3(wex, w, 1);
        if (lane == 0) ge_p3_0(wex);
        __syncwarp();
        if (lane < NT / 32) sm_st_p3(sm, lane, wex);
    }
    __syncthreads();
    ge_p3 lex;
    shfl_up_p3(lex, incl, 1);
    if (lane == 0) ge_p3_0(lex);
    sm_ld_p3(ex, sm, warp);
    ge_addto(ex, lex);
}

// (A) thread sums tt[c*NT + t] of K consecutive points; chunk sums ct[c]
template <int NT, int K>
__global__ void __launch_bounds__(NT) k_scan_sums(const uint4 *p, size_t s, size_t n, uint4 *tt, size_t ts,
                                                  uint4 *ct, size_t cs)
{
    __shared__ uint4 sm[(NT / 32) * 8];
    const size_t c = blockIdx.x;
    const size_t e0 = c * (size_t)(NT * K) + (size_t)threadIdx.x * K;
    ge_p3 acc;
    ge_p3_0(acc);
    if (e0 < n) ld_p3(acc, p, s, e0);
#pragma unroll 1
    for (int k = 1; k < K; ++k) {
        size_t e = e0 + k;
        if (e >= n) break;
        ge_p3 x;
        ld_p3(x, p, s, e);
        ge_addto(acc, x);
    }
    st_p3(tt, ts, c * NT + threadIdx.x, acc);
    block_sum<NT>(acc, sm);
    if (threadIdx.x == 0) st_p3(ct, cs, c, acc);
}

// (C) rescan each thread's K points from its exclusive prefix
template <int NT, int K>
__global__ void __launch_bounds__(NT) k_scan_apply(uint4 *p, size_t s, size_t n, const uint4 *tt, size_t ts,
                                                   const uint4 *ct, size_t cs, int exclusive)
{
    __shared__ uint4 sm[(NT / 32) * 8];
    const size_t c = blockIdx.x;
    const size_t e0 = c * (size_t)(NT * K) + (size_t)threadIdx.x * K;
    ge_p3 x, pre;
    ld_p3(x, tt, ts, c * NT + threadIdx.x);
    block_scan_excl<NT>(pre, x, sm);
    ge_p3 cp;
    ld_p3(cp, ct, cs, c);
    ge_addto(pre, cp);
#pragma unroll 1
    for (int k = 0; k < K; ++k) {
        size_t e = e0 + k;
        if (e >= n) break;
        ld_p3(x, p, s, e);
        if (exclusive) {
            st_p3(p, s, e, pre);
            ge_addto(pre, x);
        } else {
            ge_addto(pre, x);
            st_p3(p, s, e, pre);
        }
    }
}

static const int SCAN_NT = 128, SCAN_K = 8;
static const size_t SCAN_CHUNK = (size_t)SCAN_NT * SCAN_K;

size_t scan_scratch_bytes(size_t n)
{
    size_t pts = 0;
    while (n > 1) {
        size_t nch = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
        pts += nch * SCAN_NT + nch;
        n = nch;
    }
    return pts * 128 + 256;
}

cudaError_t scan(View v, size_t n, int exclusive, void *scratch, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    size_t nch = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    View tt{(uint4 *)scratch, nch * SCAN_NT};
    View ct{tt.p + FT_PLANES * tt.s, nch};
    void *rest = ct.p + FT_PLANES * ct.s;
    k_scan_sums<SCAN_NT, SCAN_K><<<(unsigned)nch, SCAN_NT, 0, st>>>(v.p, v.s, n, tt.p, tt.s, ct.p, ct.s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (nch > 1) {
        e = scan(ct, nch, 1, rest, st);
        if (e != cudaSuccess) return e;
    } else {
        e = set_zero(ct, 1, st);
        if (e != cudaSuccess) return e;
    }
    k_scan_apply<SCAN_NT, SCAN_K><<<(unsigned)nch, SCAN_NT, 0, st>>>(v.p, v.s, n, tt.p, tt.s, ct.p, ct.s, exclusive);
    return cudaGetLastError();
}

// ------------------------------------------------------------ reduce launcher

static const int RED_NT = 128;

static unsigned reduce_grid(size_t n)
{
    size_t need = (n + RED_NT - 1) / RED_NT;
    size_t cap = (size_t)sm_count() * 4;
    return (unsigned)(need < cap ? (need ? need : 1) : cap);
}

size_t reduce_scratch_bytes(size_t n) { return (size_t)reduce_grid(n) * 128 + 256; }

cudaError_t reduce(View out, View src, size_t n, void *scratch, cudaStream_t st)
{
    unsigned g = reduce_grid(n);
    if (n == 0) return set_zero(out, 1, st);
    if (g == 1) {
        k_reduce<RED_NT><<<1, RED_NT, 0, st>>>(src.p, src.s, n, out.p, out.s);
        return cudaGetLastError();
    }
    View part{(uint4 *)scratch, g};
    k_reduce<RED_NT><<<g, RED_NT, 0, st>>>(src.p, src.s, n, part.p, part.s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_reduce<RED_NT><<<1, RED_NT, 0, st>>>(part.p, part.s, g, out.p, out.s);
    return cudaGetLastError();
}

// ------------------------------------------------------------ segmented sum

// segmented combine: (f1, v1) then (f2, v2) -> (f1 | f2, f2 ? v2 : v1 + v2)
FT_DEV void seg_combine(int &f, ge_p3 &v, int f_prev, const ge_p3 &v_prev)
{
    ge_p3 sum = v_prev;
    ge_addto(sum, v);
    if (!f) v = sum;
    f |= f_prev;
}

FT_DEV int lower_bound_i32(const int32_t *a, int lo, int hi, long long x) // first i in [lo,hi) with a[i] >= x
{
    while (lo < hi) {
        int mid = lo + ((hi - lo) >> 1);
        if ((long long)a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

FT_DEV int upper_bound_i32(const int32_t *a, int lo, int hi, long long x) // first i in [lo,hi) with a[i] > x
{
    while (lo < hi) {
        int mid = lo + ((hi - lo) >> 1);
        if ((long long)a[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

template <int NT, int K>
__global__ void __launch_bounds__(NT) k_segsum(uint4 *op, size_t os, const int32_t *off, int nseg, const uint4 *sp,
                                               size_t ss, long long nsrc, const int32_t *perm, int accumulate)
{
    constexpr int NW = NT / 32;
    __shared__ uint4 s_wv[NW * 8];
    __shared__ int s_wf[NW];
    __shared__ uint4 s_carry[8];
    __shared__ int s_cf;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long G = gridDim.x, b = blockIdx.x;

    // this block's whole segments [s0, s1) and their points [E0, E1)
    const int s0 = b == 0 ? 0 : lower_bound_i32(off, 0, nseg + 1, nsrc * b / G);
    const int s1 = b == G - 1 ? nseg : lower_bound_i32(off, 0, nseg + 1, nsrc * (b + 1) / G);
    if (s0 >= s1) return;
    const long long E0 = off[s0], E1 = off[s1];

    // empty segments produce the identity (or leave res untouched)
    if (!accumulate) {
        for (int sg = s0 + threadIdx.x; sg < s1; sg += NT) {
            if (off[sg] == off[sg + 1]) {
                ge_p3 z;
                ge_p3_0(z);
                st_p3(op, os, sg, z);
            }
        }
    }
    if (threadIdx.x == 0) {
        ge_p3 z;
        ge_p3_0(z);
        sm_st_p3(s_carry, 0, z);
        s_cf = 0;
    }
    __syncthreads();

#pragma unroll 1
    for (long long c0 = E0; c0 < E1; c0 += (long long)NT * K) {
        const long long cend = min(E1, c0 + (long long)NT * K);
        const long long e0 = c0 + (long long)threadIdx.x * K;
        // pass 1: walk this thread's points
        int fstart = 0, head_pending = 0, head_seg = 0, any = 0, open_before = 1;
        ge_p3 acc, head;
        ge_p3_0(acc);
        ge_p3_0(head);
        if (e0 < cend) {
            int sg = upper_bound_i32(off, s0, s1 + 1, e0) - 1;
#pragma unroll 1
            for (int k = 0; k < K; ++k) {
                const long long e = e0 + k;
                if (e >= cend) break;
                while ((long long)off[sg + 1] <= e) ++sg;
                ge_p3 x;
                ld_p3(x, sp, ss, perm ? (size_t)perm[e] : (size_t)e);
                if ((long long)off[sg] == e) {
                    fstart = 1;
                    open_before = 0;
                    acc = x;
                } else if (!any) {
                    acc = x;
                } else {
                    ge_addto(acc, x);
                }
                any = 1;
                if ((long long)off[sg + 1] == e + 1) { // last point of segment sg
                    if (open_before) {
                        head = acc;
                        head_pending = 1;
                        head_seg = sg;
                        open_before = 0;
                    } else {
                        ge_p3 o = acc;
                        if (accumulate) {
                            ge_p3 r;
                            ld_p3(r, op, os, sg);
                            ge_addto(r, o);
                            o = r;
                        }
                        st_p3(op, os, sg, o);
                    }
                }
            }
        }
        // block-wide exclusive segmented scan of (fstart, acc), seeded by the
        // carry from the previous chunk
        int f = fstart;
        ge_p3 v = acc;
#pragma unroll 1
        for (int o = 1; o < 32; o <<= 1) {
            ge_p3 vu;
            shfl_up_p3(vu, v, o);
            int fu = __shfl_up_sync(0xffffffffu, f, o);
            int f2 = f;
            ge_p3 v2 = v;
            seg_combine(f2, v2, fu, vu);
            if (lane >= o) {
                f = f2;
                v = v2;
            }
        }
        if (lane == 31) {
            sm_st_p3(s_wv, warp, v);
            s_wf[warp] = f;
        }
        __syncthreads();
        if (warp == 0) {
            // scan of [carry, warp totals...]; lane w ends with the prefix of warp w
            int wf = 0;
            ge_p3 wv;
            ge_p3_0(wv);
            if (lane < NW) {
                sm_ld_p3(wv, s_wv, lane);
                wf = s_wf[lane];
            }
#pragma unroll 1
            for (int o = 1; o < 32; o <<= 1) {
                ge_p3 vu;
                shfl_up_p3(vu, wv, o);
                int fu = __shfl_up_sync(0xffffffffu, wf, o);
                int f2 = wf;
                ge_p3 v2 = wv;
                seg_combine(f2, v2, fu, vu);
                if (lane >= o) {
                    wf = f2;
                    wv = v2;
                }
            }
            // exclusive prefix of warp w = carry (+) inclusive of warps < w
            ge_p3 ex;
            shfl_up_p3(ex, wv, 1);
            int exf = __shfl_up_sync(0xffffffffu, wf, 1);
            ge_p3 cv;
            sm_ld_p3(cv, s_carry, 0);
            int cf = s_cf;
            if (lane == 0) {
                ex = cv;
                exf = cf;
            } else {
                seg_combine(exf, ex, cf, cv);
            }
            // new carry = carry (+) all warps
            ge_p3 tot = wv;
            int totf = wf;
            seg_combine(totf, tot, cf, cv);
            __syncwarp();
            if (lane < NW) {
                sm_st_p3(s_wv, lane, ex);
                s_wf[lane] = exf;
            }
            if (lane == NW - 1) {
                sm_st_p3(s_carry, 0, tot);
                s_cf = totf;
            }
        }
        __syncthreads();
        // carry into this thread = warp prefix (+) lanes before it
        ge_p3 lv;
        shfl_up_p3(lv, v, 1);
        int lf = __shfl_up_sync(0xffffffffu, f, 1);
        ge_p3 cin;
        sm_ld_p3(cin, s_wv, warp);
        int cinf = s_wf[warp];
        if (lane > 0) {
            seg_combine(lf, lv, cinf, cin);
            cin = lv;
        }
        if (head_pending) {
            ge_addto(cin, head);
            if (accumulate) {
                ge_p3 r;
                ld_p3(r, op, os, head_seg);
                ge_addto(r, cin);
                cin = r;
            }
            st_p3(op, os, head_seg, cin);
        }
        __syncthreads(); // s_wv and the carry are rewritten next chunk
    }
}

static const int SEG_NT = 128, SEG_K = 16;

cudaError_t segsum(View out, const int32_t *off, size_t nseg, View src, size_t nsrc, const int32_t *perm,
                   int accumulate, cudaStream_t st)
{
    if (nseg == 0) return cudaSuccess;
    size_t per_block = (size_t)SEG_NT * SEG_K * 8;
    size_t g = (nsrc + per_block - 1) / per_block;
    size_t cap = (size_t)sm_count() * 6;
    if (g > cap) g = cap;
    if (g == 0) g = 1;
    k_segsum<SEG_NT, SEG_K><<<(unsigned)g, SEG_NT, 0, st>>>(out.p, out.s, off, (int)nseg, src.p, src.s,
                                                             (long long)nsrc, perm, accumulate);
    return cudaGetLastError();
}

// ------------------------------------------------------------ counting sort

__global__ void k_key_hist(const uint64_t *keys, size_t n, size_t nkeys, int32_t *cnt, long long *bad)
{
    FT_GRID_LOOP(i, n)
    {
        uint64_t k = keys[i];
        if (k >= nkeys) atomicMax(bad, (long long)i);
        else atomicAdd(&cnt[k], 1);
    }
}

__global__ void k_key_place(const uint64_t *keys, size_t n, size_t nkeys, int32_t *cur, int32_t *perm)
{
    FT_GRID_LOOP(i, n)
    {
        uint64_t k = keys[i];
        if (k < nkeys) perm[atomicAdd(&cur[k], 1)] = (int32_t)i;
    }
}

// exclusive scan of int32 in blocks of 1024 x 4; block totals scanned recursively
__global__ void __launch_bounds__(1024) k_iscan_block(int32_t *a, size_t n, int32_t *bsum)
{
    __shared__ int32_t ws[32];
    const size_t base = (size_t)blockIdx.x * 4096 + threadIdx.x * 4;
    int32_t v[4], t = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = base + k < n ? a[base + k] : 0;
        t += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t incl = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int32_t w = ws[lane];
        int32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t u = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += u;
        }
        ws[lane] = wi - w;
        if (lane == 31 && bsum) bsum[blockIdx.x] = wi;
    }
    __syncthreads();
    int32_t run = ws[warp] + incl - t;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) a[base + k] = run;
        run += v[k];
    }
}

__global__ void k_iscan_add(int32_t *a, size_t n, const int32_t *bsum)
{
    FT_GRID_LOOP(i, n) a[i] += bsum[i / 4096];
}

static cudaError_t iscan_excl(int32_t *a, size_t n, int32_t *tmp, cudaStream_t st)
{
    size_t nb = (n + 4095) / 4096;
    k_iscan_block<<<(unsigned)nb, 1024, 0, st>>>(a, n, nb > 1 ? tmp : nullptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || nb == 1) return e;
    e = iscan_excl(tmp, nb, tmp + nb, st);
    if (e != cudaSuccess) return e;
    k_iscan_add<<<(unsigned)((n + 255) / 256 < 65535 ? (n + 255) / 256 : 65535), 256, 0, st>>>(a, n, tmp);
    return cudaGetLastError();
}

size_t isum_scratch_bytes(size_t n, size_t nkeys)
{
    (void)n;
    size_t t = 0, m = nkeys + 1;
    while (m > 1) {
        m = (m + 4095) / 4096;
        t += m;
    }
    return (nkeys + 1 + t + 64) * sizeof(int32_t);
}

cudaError_t keys_to_csr(int32_t *off, int32_t *perm, const uint64_t *keys, size_t n, size_t nkeys,
                        long long *bad, void *scratch, cudaStream_t st)
{
    int32_t *cur = (int32_t *)scratch;
    int32_t *tmp = cur + nkeys + 1;
    cudaError_t e = cudaMemsetAsync(off, 0, (nkeys + 1) * sizeof(int32_t), st);
    if (e != cudaSuccess) return e;
    unsigned g = (unsigned)((n + 255) / 256 < 65535 ? ((n + 255) / 256 ? (n + 255) / 256 : 1) : 65535);
    k_key_hist<<<g, 256, 0, st>>>(keys, n, nkeys, off, bad);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = iscan_excl(off, nkeys + 1, tmp, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(cur, off, (nkeys + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return e;
    k_key_place<<<g, 256, 0, st>>>(keys, n, nkeys, cur, perm);
    return cudaGetLastError();
}

} // namespace ft
