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
//            ftcrypto.cu:1474-1586): per-thread sums of K consecutive points
//            (16 on levels that fill the GPU, 4 below), an exclusive scan of
//            those sums by the same routine (one block once at most 1,024
//            remain), then each thread rescans its K points from its prefix.
//            ~2 + 2/16 additions per point, one
//            point-addition site per kernel, no waits between blocks.  Correct
//            for every length (the reference's kernel indexes its tile sums
//            wrongly above 256 x grid points, ftcrypto.cu:1512).
//   segsum   out[s] = sum of src[e] (or src[perm[e]]) for e in
//            [off[s], off[s+1]): each thread sums SEG_K = 32 consecutive points
//            segment by segment, writes the segments that begin and end inside
//            it and records the parts of the segments crossing its edges; a
//            second kernel joins those parts (k_seg_walk / k_seg_join).
//            ~1 + 1/32 additions per point.  It serves ft_reduce_isum
//            (ftcrypto.cu:1113-1217, accumulating into res) and the CSR
//            segmented-sum extension.
//   keys_to_csr  counting sort of ft_reduce_isum's keys on the device
//            (replaces the reference's host std::sort, ftcrypto.cu:1170).
#include <algorithm>

#include <cmath>
#include <mutex>

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

// A minimum of one block per SM in the launch bounds lets ptxas take 124
// registers instead of 106 (still four blocks of 128 threads per SM): the
// sum of 16,777,216 points 1.539 -> 1.483 ms.  Two points per step (158
// registers, three blocks per SM) measured 1.546 ms, with 128 registers
// forced (spills) 1.559 ms.
template <int NT>
__global__ void __launch_bounds__(NT, 1) k_reduce(const uint4 *p, size_t s, size_t n, uint4 *out, size_t os)
{
    __shared__ uint4 sm[(NT / 32) * 8];
    ge_p3 acc;
    const size_t stride = (size_t)gridDim.x * NT;
    size_t base = (size_t)blockIdx.x * NT;
    if (base + threadIdx.x < n) ld_p3(acc, p, s, base + threadIdx.x);
    else ge_p3_0(acc);
    // block-uniform steps with a barrier each: the warps stay on the same
    // stretch of the addition's code and share the instruction caches
    // (instruction-fetch stalls were 0.75 per issue): 2.09 -> 2.01 ms for
    // 16,777,216 points
#pragma unroll 1
    for (base += stride; base < n; base += stride) {
        __syncthreads();
        const size_t i = base + threadIdx.x;
        if (i < n) {
            ge_p3 x;
            ld_p3(x, p, s, i);
            ge_addto(acc, x);
        }
    }
    block_sum<NT>(acc, sm);
    if (threadIdx.x == 0) st_p3(out, os, blockIdx.x, acc);
}

// ------------------------------------------------------------ scan

// inclusive scan over the first `width` lanes of the warp (a power of two);
// returns the lane's inclusive sum in acc
FT_DEV void warp_scan_incl(ge_p3 &acc, int width = 32)
{
    const int lane = threadIdx.x & 31;
#pragma unroll 1
    for (int o = 1; o < width; o <<= 1) {
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
    static_assert(NT >= 64 && NT <= 1024 && (NT & (NT - 1)) == 0, "a power-of-two number of warps");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ge_p3 incl = x;
    warp_scan_incl(incl);
    if (lane == 31) sm_st_p3(sm, warp, incl);
    __syncthreads();
    if (warp == 0) {
        ge_p3 w;
        if (lane < NT / 32) sm_ld_p3(w, sm, lane);
        else ge_p3_0(w);
        warp_scan_incl(w, NT / 32); // the warps' totals: log2(NT/32) levels, not 5
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

// The scan kernels take up to two arrays of one length (the two halves of a
// ciphertext array, ftx_ct_scan): blockIdx.y selects the array, so both are
// scanned by the same launches and share the latency-bound lower levels.
struct ScanSet {
    uint4 *p[2];
    size_t s[2];
    // array blockIdx.y, chosen by selects (indexing the parameter array with
    // blockIdx.y would copy it to local memory)
    FT_DEV uint4 *ptr() const { return blockIdx.y ? p[1] : p[0]; }
    FT_DEV size_t stride() const { return blockIdx.y ? s[1] : s[0]; }
};

// blocks per SM the scan's and the segmented sum's walks are compiled for
// (__launch_bounds__ minimum; 1 leaves the register count to ptxas).
// Measured on GB300 for the 2 x 4,194,304-point ciphertext scan: 1.95 ms
// unconstrained (sums ~152 registers, apply ~184), 2.09 ms at 3 blocks,
// 2.11 ms at 4 for the sums and 3 for the rescan, 2.68 ms at 4 for both
// (128 registers, spills); the segmented-sum walk 1.73 ms at 4 blocks
// (128 registers) against 1.81 ms at 3.
#ifndef FT_SCAN_SUMS_MINB
#define FT_SCAN_SUMS_MINB 1
#endif
#ifndef FT_SCAN_APPLY_MINB
#define FT_SCAN_APPLY_MINB 1
#endif
#ifndef FT_SEG_WALK_MINB
#define FT_SEG_WALK_MINB 4
#endif


#ifndef FT_WAVE_FIT
#define FT_WAVE_FIT 1
#endif

// Blocks of `fn` (block size `nt`, no dynamic shared memory) resident on the
// whole GPU at once, from the occupancy calculator; cached by the caller.
static int resident_blocks(const void *fn, int nt)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, nt, 0) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm * sm_count();
}

// Of the points-per-thread candidates ks[0..nk) (ascending), the one whose
// launch of ceil(ceil(n / k) / 128) * m blocks of 128 threads fills its last
// wave of `resident` blocks best (waves / ceil(waves) highest; ties go to
// the smaller k).  One walk per thread, so a last wave at 74% leaves a
// quarter of the GPU idle for 1/7 of the launch (16,777,216 points at 32 per
// thread in four 128-thread blocks per SM: 6.74 waves; at 36: 5.99).
static int wave_fit_k(size_t n, int m, const int *ks, int nk, const int *resident)
{
    int best = ks[0];
    double best_eff = -1.0;
    for (int i = 0; i < nk; ++i) {
        const size_t blocks = ((n + ks[i] - 1) / ks[i] + 127) / 128 * (size_t)m;
        const double waves = (double)blocks / resident[i];
        const double eff = waves / std::ceil(waves);
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = ks[i];
        }
    }
    return best;
}

// (An L1 prefetch of the thread's next pair of points before each step
// measured slower: the two-half scan of 4,194,304 points 1.93 -> 1.96 ms,
// the segmented sum of 16,777,216 points 1.66 -> 1.77 ms.  Copying the
// rescan's next pair into shared memory with cp.async while the current
// pair is added — no registers held for it, 64 KB per block, still three
// blocks per SM — measured the same for both halves, 1.046 -> 1.062 ms for
// one array and 1.014 -> 1.064 ms for the prescan.)
#ifndef FT_WALK_PAIRS
#define FT_WALK_PAIRS 1
#endif

// per-thread sums of K consecutive points: ts[t] = sum of p[tK .. tK+K).
// With FT_WALK_PAIRS the thread loads its points two at a time: the two
// 16-byte words of a pair fill one 32-byte sector of each plane, which is
// then read from DRAM once (one point at a time, the sector's second half
// can be evicted before the next step and read again: 1.29x the
// algorithmic bytes in the sums, 1.39x in the rescan, measured), and the
// rescan waits for memory once per two points.  2 x 4,194,304-point
// ciphertext scan: 2.045 -> 2.020 ms.
template <int K>
__global__ void __launch_bounds__(128, FT_SCAN_SUMS_MINB) k_scan_sums(ScanSet in, size_t n, ScanSet ts)
{
    const uint4 *p = in.ptr();
    const size_t s = in.stride();
    uint4 *tp = ts.ptr();
    const size_t tss = ts.stride();
    const size_t nt = (n + K - 1) / K;
    FT_GRID_LOOP(t, nt)
    {
        const size_t e0 = t * K;
        ge_p3 acc;
#if FT_WALK_PAIRS
        static_assert(K % 2 == 0, "pairs of points");
        ge_p3 x;
        ld_p3(acc, p, s, e0);
        if (e0 + 1 < n) {
            ld_p3(x, p, s, e0 + 1);
            ge_addto(acc, x);
        }
#pragma unroll 1
        for (int k = 2; k < K; k += 2) {
            const size_t e = e0 + k;
            if (e >= n) break;
            ge_p3 y;
            ld_p3(x, p, s, e);
            const bool two = e + 1 < n;
            if (two) ld_p3(y, p, s, e + 1);
            ge_addto(acc, x);
            if (!two) break;
            ge_addto(acc, y);
        }
#else
        ld_p3(acc, p, s, e0);
#pragma unroll 1
        for (int k = 1; k < K; ++k) {
            const size_t e = e0 + k;
            if (e >= n) break;
            ge_p3 x;
            ld_p3(x, p, s, e);
            ge_addto(acc, x);
        }
#endif
        st_p3(tp, tss, t, acc);
    }
}

// rescan each thread's K points starting from its exclusive prefix ts[t];
// `exclusive` a template parameter: as a run-time flag the inclusive form
// needed 210 registers (two blocks per SM) instead of 168 (three)
template <int K, int exclusive>
__global__ void __launch_bounds__(128, FT_SCAN_APPLY_MINB) k_scan_apply(ScanSet io, size_t n, ScanSet ts)
{
    uint4 *p = io.ptr();
    const size_t s = io.stride();
    const uint4 *tp = ts.ptr();
    const size_t tss = ts.stride();
    const size_t nt = (n + K - 1) / K;
    FT_GRID_LOOP(t, nt)
    {
        ge_p3 pre;
        ld_p3(pre, tp, tss, t);
#if FT_WALK_PAIRS
        static_assert(K % 2 == 0, "pairs of points");
#pragma unroll 1
        for (int k = 0; k < K; k += 2) {
            const size_t e = t * K + k;
            if (e >= n) break;
            ge_p3 x, y;
            ld_p3(x, p, s, e);
            const bool two = e + 1 < n;
            if (two) ld_p3(y, p, s, e + 1);
            if (exclusive) st_p3(p, s, e, pre);
            ge_addto(pre, x);
            if (!exclusive) st_p3(p, s, e, pre);
            if (!two) break;
            if (exclusive) st_p3(p, s, e + 1, pre);
            ge_addto(pre, y);
            if (!exclusive) st_p3(p, s, e + 1, pre);
        }
#else
#pragma unroll 1
        for (int k = 0; k < K; ++k) {
            const size_t e = t * K + k;
            if (e >= n) break;
            ge_p3 x;
            ld_p3(x, p, s, e);
            if (exclusive) st_p3(p, s, e, pre);
            ge_addto(pre, x);
            if (!exclusive) st_p3(p, s, e, pre);
        }
#endif
    }
}

// one block per array scans n <= NT * kpt points in place: sums of kpt
// consecutive points per thread, a block-wide exclusive scan of them, then
// the sequential rescan.  One block is latency-bound, so the points are
// spread over all NT threads (kpt = ceil(n / NT)): the last level of a
// 4M-point scan (1,024 points) is a chain of 17 dependent additions instead
// of 41 with a fixed 16 points per thread (194 us per launch).
template <int NT>
__global__ void __launch_bounds__(NT) k_scan_small(ScanSet io, size_t n, int kpt, int exclusive)
{
    __shared__ uint4 sm[(NT / 32) * 8];
    uint4 *p = io.ptr();
    const size_t s = io.stride();
    const size_t e0 = (size_t)threadIdx.x * kpt;
    ge_p3 acc;
    ge_p3_0(acc);
    if (e0 < n) ld_p3(acc, p, s, e0);
#pragma unroll 1
    for (int k = 1; k < kpt; ++k) {
        const size_t e = e0 + k;
        if (e >= n) break;
        ge_p3 x;
        ld_p3(x, p, s, e);
        ge_addto(acc, x);
    }
    ge_p3 pre;
    block_scan_excl<NT>(pre, acc, sm);
#pragma unroll 1
    for (int k = 0; k < kpt; ++k) {
        const size_t e = e0 + k;
        if (e >= n) break;
        ge_p3 x;
        ld_p3(x, p, s, e);
        if (exclusive) st_p3(p, s, e, pre);
        ge_addto(pre, x);
        if (!exclusive) st_p3(p, s, e, pre);
    }
}

static const int SMALL_NT = 256;

size_t scan_scratch_bytes(size_t n, int m) { return (size_t)m * scan_scratch_points(n) * 128 + 256; }

// thread sums of K = scan_level_k(n) points, an exclusive scan of those sums
// (the same routine on arrays K times shorter, until one block suffices),
// then the rescan: about 2 + 2/K additions per point, no waits between blocks.
// At 4M points the lower levels (262,144 points down to 4,096) take 4 points
// per thread: 16 made each of their launches a 16-addition chain in
// under-filled waves (~60 us each).  m arrays (1 or 2) of n points each go
// through the same launches; scratch holds m x scan_scratch_points(n) points.
cudaError_t scan_set(const View *v, int m, size_t n, int exclusive, void *scratch, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (m < 1 || m > 2) return cudaErrorInvalidValue;
    ScanSet io{};
    for (int i = 0; i < m; ++i) {
        io.p[i] = v[i].p;
        io.s[i] = v[i].s;
    }
    if (n <= SCAN_SMALL_MAX) {
        const int kpt = (int)((n + SMALL_NT - 1) / SMALL_NT);
        k_scan_small<SMALL_NT><<<dim3(1, m), SMALL_NT, 0, st>>>(io, n, kpt, exclusive);
        return cudaGetLastError();
    }
    // points per thread: 16 above 2^18 points, 4 on the latency-bound lower
    // levels.  (Choosing 16, 18 or 20 by how well the last wave fills, as
    // the segmented walk does, measured 7% slower: at 18 and 20 points the
    // sums pass takes 170 registers and two blocks per SM instead of three.)
    const size_t K = scan_level_k(n);
    const size_t nt = (n + K - 1) / K;
    View ts[2];
    ScanSet tset{};
    for (int i = 0; i < m; ++i) {
        ts[i] = View{(uint4 *)scratch + (size_t)i * FT_PLANES * nt, nt};
        tset.p[i] = ts[i].p;
        tset.s[i] = nt;
    }
    void *rest = (uint4 *)scratch + (size_t)m * FT_PLANES * nt;
    const dim3 grid((unsigned)((nt + 127) / 128), m);
    if (K == 16) k_scan_sums<16><<<grid, 128, 0, st>>>(io, n, tset);
    else k_scan_sums<4><<<grid, 128, 0, st>>>(io, n, tset);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if ((e = scan_set(ts, m, nt, 1, rest, st)) != cudaSuccess) return e;
    if (K == 16 && exclusive) k_scan_apply<16, 1><<<grid, 128, 0, st>>>(io, n, tset);
    else if (K == 16) k_scan_apply<16, 0><<<grid, 128, 0, st>>>(io, n, tset);
    else if (exclusive) k_scan_apply<4, 1><<<grid, 128, 0, st>>>(io, n, tset);
    else k_scan_apply<4, 0><<<grid, 128, 0, st>>>(io, n, tset);
    return cudaGetLastError();
}

cudaError_t scan(View v, size_t n, int exclusive, void *scratch, cudaStream_t st)
{
    return scan_set(&v, 1, n, exclusive, scratch, st);
}

// ------------------------------------------------------------ reduce launcher

static const int RED_NT = 128;

static unsigned reduce_grid(size_t n)
{
    // one wave of the first pass: every block resident at once
    static std::once_flag once;
    static size_t resident;
    std::call_once(once, [] { resident = (size_t)resident_blocks((const void *)k_reduce<RED_NT>, RED_NT); });
    size_t need = (n + RED_NT - 1) / RED_NT;
    return (unsigned)(need < resident ? (need ? need : 1) : resident);
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

FT_DEV int upper_bound_i32(const int32_t *a, int lo, int hi, long long x) // first i in [lo,hi) with a[i] > x
{
    while (lo < hi) {
        int mid = lo + ((hi - lo) >> 1);
        if ((long long)a[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

FT_DEV void seg_write(uint4 *op, size_t os, int sg, const ge_p3 &v, int accumulate)
{
    if (accumulate) {
        ge_p3 r;
        ld_p3(r, op, os, sg);
        ge_addto(r, v);
        st_p3(op, os, sg, r);
    } else {
        st_p3(op, os, sg, v);
    }
}

// record flags of a thread in the segmented sum
#define SEG_HEAD 1u   // H[t] holds the part of a segment that began before the thread
#define SEG_CLOSE 2u  // ... and that segment ends inside the thread (or at its last point)
#define SEG_TAIL 4u   // L[t] holds the start of segment lseg[t], which continues past the thread

// The arrays of one or two segmented sums over the same offsets (the two
// halves of a ciphertext array): output, source and scratch of sum y in
// slot y, chosen by blockIdx.y (a select, not an index, so the struct stays
// in parameter space).
struct SegSet {
    uint4 *op[2];
    size_t os[2];
    const uint4 *sp[2];
    size_t ss[2];
    uint4 *H[2];
    uint4 *Lp[2];
    uint32_t *flags[2];
    int32_t *lseg[2];
    template <class T>
    FT_DEV static T pick(const T (&a)[2]) { return blockIdx.y ? a[1] : a[0]; }
};

// Pass 1: thread t sums its K consecutive points segment by segment.  A
// segment that begins and ends inside the thread is written at once; the
// parts of segments crossing the thread's edges go to H / L.
// four blocks per SM (128 registers, a few spills to L1) rather than two at
// 202 registers: 2.58 against 2.68 ms for 16,777,216 points (measured)
template <int K>
__global__ void __launch_bounds__(128, FT_SEG_WALK_MINB) k_seg_walk(SegSet set, const int32_t *off, int nseg,
                                                                    long long nsrc, const int32_t *perm, int accumulate,
                                                                    size_t hs)
{
    uint4 *op = SegSet::pick(set.op);
    const size_t os = SegSet::pick(set.os);
    const uint4 *sp = SegSet::pick(set.sp);
    const size_t ss = SegSet::pick(set.ss);
    uint4 *H = SegSet::pick(set.H);
    uint4 *Lp = SegSet::pick(set.Lp);
    uint32_t *flags = SegSet::pick(set.flags);
    int32_t *lseg = SegSet::pick(set.lseg);
    const long long nt = (nsrc + K - 1) / K;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; // the launch covers nt
    const bool live = t < nt;
    {
        const long long e0 = live ? t * K : 0;
        const long long e1 = live ? min(e0 + K, nsrc) : 0;
        int sg = live ? upper_bound_i32(off, 0, nseg + 1, e0) - 1 : 0; // segment holding e0 (skips empty ones)
        bool open_before = live && (long long)off[sg] < e0;
        uint32_t fl = 0;
        ge_p3 acc;
        ge_p3_0(acc);
        // every thread of the block takes the K steps, with a barrier each:
        // the warps stay on the same stretch of code and share the
        // instruction caches (instruction-fetch stalls were 1.45 per issue):
        // 2.32 -> 2.21 ms for 16,777,216 points in 1,048,576 segments
#pragma unroll 1
        for (int k = 0; k < K; ++k) {
            __syncthreads();
            const long long e = e0 + k;
            if (e >= e1) continue;
            while ((long long)off[sg + 1] <= e) ++sg;
            ge_p3 x;
            ld_p3(x, sp, ss, perm ? (size_t)perm[e] : (size_t)e);
            if ((long long)off[sg] == e || e == e0) acc = x;
            else ge_addto(acc, x);
            if ((long long)off[sg + 1] == e + 1) { // last point of segment sg
                if (open_before) {
                    st_p3(H, hs, t, acc);
                    fl |= SEG_HEAD | SEG_CLOSE;
                    open_before = false;
                } else {
                    seg_write(op, os, sg, acc, accumulate);
                }
            }
        }
        if (live && (long long)off[sg + 1] > e1) { // the last segment continues past the thread
            if (open_before) {
                st_p3(H, hs, t, acc);
                fl |= SEG_HEAD;
            } else {
                st_p3(Lp, hs, t, acc);
                fl |= SEG_TAIL;
                lseg[t] = sg;
            }
        }
        if (live) flags[t] = fl;
    }
}

// Pass 2: a segment started in thread t and continuing past it totals
// L[t] + H[t+1] + ... + H[u], u the first later thread whose head closes it.
__global__ void __launch_bounds__(128) k_seg_join(SegSet set, size_t hs, size_t nt, int accumulate)
{
    uint4 *op = SegSet::pick(set.op);
    const size_t os = SegSet::pick(set.os);
    const uint4 *H = SegSet::pick(set.H);
    const uint4 *Lp = SegSet::pick(set.Lp);
    const uint32_t *flags = SegSet::pick(set.flags);
    const int32_t *lseg = SegSet::pick(set.lseg);
    FT_GRID_LOOP(t, nt)
    {
        if (!(flags[t] & SEG_TAIL)) continue;
        ge_p3 sum;
        ld_p3(sum, Lp, hs, t);
#pragma unroll 1
        for (size_t u = t + 1; u < nt; ++u) {
            ge_p3 h;
            ld_p3(h, H, hs, u);
            ge_addto(sum, h);
            if (flags[u] & SEG_CLOSE) break;
        }
        seg_write(op, os, lseg[t], sum, accumulate);
    }
}

__global__ void __launch_bounds__(256) k_seg_empty(SegSet set, const int32_t *off, size_t nseg)
{
    uint4 *op = SegSet::pick(set.op);
    const size_t os = SegSet::pick(set.os);
    FT_GRID_LOOP(sg, nseg)
    {
        if (off[sg] == off[sg + 1]) {
            ge_p3 z;
            ge_p3_0(z);
            st_p3(op, os, sg, z);
        }
    }
}

// points per thread of the walk: 32 rather than 16 halves the threads' fixed
// costs (the binary search for the first segment, the edge partials, the
// join): 2.59 -> 2.32 ms for 16,777,216 points in 1,048,576 segments (64 and
// 128 measure the same as 32; 8 is 3.84 ms)
static const int SEG_K = 32;

size_t segsum_scratch_bytes(size_t nsrc, int m)
{
    size_t nt = (nsrc + SEG_K - 1) / SEG_K;
    const size_t one = ((2 * nt * 128 + 2 * nt * 4 + 1024) + 255) / 256 * 256; // each sum's part 256-byte aligned
    return (size_t)m * one;
}

// out[s] (+)= sum of src[perm ? perm[e] : e], e in [off[s], off[s+1]):
// ~1 + 1/SEG_K additions per point, two kernels, no waits between blocks.
// A segment spanning m threads costs m sequential additions in pass 2
// (m ~ length / 32; 1-2 for the benchmark's mean lengths 8-32).  m (1 or
// 2) sums over the same offsets and source length go through the same
// launches (grid dimension y); scratch holds m x segsum_scratch_bytes(nsrc).
cudaError_t segsum_set(const View *out, const View *src, int m, const int32_t *off, size_t nseg, size_t nsrc,
                       const int32_t *perm, int accumulate, void *scratch, cudaStream_t st)
{
    if (nseg == 0) return cudaSuccess;
    if (m < 1 || m > 2) return cudaErrorInvalidValue;
    SegSet set{};
    for (int i = 0; i < m; ++i) {
        set.op[i] = out[i].p;
        set.os[i] = out[i].s;
        set.sp[i] = src[i].p;
        set.ss[i] = src[i].s;
    }
    cudaError_t e;
    if (!accumulate) {
        const dim3 g((unsigned)std::min<size_t>((nseg + 255) / 256, 65535), m);
        k_seg_empty<<<g, 256, 0, st>>>(set, off, nseg);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (nsrc == 0) return cudaSuccess;
    // points per thread: 32, 36 or 40, whichever fills the walk's last wave
    // best (at least 32, so the scratch sized for SEG_K suffices)
    static const int ks[3] = {32, 36, 40};
    static int res[3];
    static std::once_flag once;
    std::call_once(once, [] {
        res[0] = resident_blocks((const void *)k_seg_walk<32>, 128);
        res[1] = resident_blocks((const void *)k_seg_walk<36>, 128);
        res[2] = resident_blocks((const void *)k_seg_walk<40>, 128);
    });
    const int K = FT_WAVE_FIT ? wave_fit_k(nsrc, m, ks, 3, res) : SEG_K;
    const size_t nt = (nsrc + K - 1) / K;
    for (int i = 0; i < m; ++i) {
        uint8_t *base = (uint8_t *)scratch + (size_t)i * segsum_scratch_bytes(nsrc, 1);
        set.H[i] = (uint4 *)base;
        set.Lp[i] = set.H[i] + FT_PLANES * nt;
        set.flags[i] = (uint32_t *)(set.Lp[i] + FT_PLANES * nt);
        set.lseg[i] = (int32_t *)(set.flags[i] + nt);
    }
    const dim3 grid((unsigned)((nt + 127) / 128), m);
    switch (K) {
    case 36: k_seg_walk<36><<<grid, 128, 0, st>>>(set, off, (int)nseg, (long long)nsrc, perm, accumulate, nt); break;
    case 40: k_seg_walk<40><<<grid, 128, 0, st>>>(set, off, (int)nseg, (long long)nsrc, perm, accumulate, nt); break;
    default: k_seg_walk<SEG_K><<<grid, 128, 0, st>>>(set, off, (int)nseg, (long long)nsrc, perm, accumulate, nt); break;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_seg_join<<<grid, 128, 0, st>>>(set, nt, nt, accumulate);
    return cudaGetLastError();
}

cudaError_t segsum(View out, const int32_t *off, size_t nseg, View src, size_t nsrc, const int32_t *perm,
                   int accumulate, void *scratch, cudaStream_t st)
{
    return segsum_set(&out, &src, 1, off, nseg, nsrc, perm, accumulate, scratch, st);
}

// ------------------------------------------------------------ long segments

// dst[e] = src[perm[e]]
__global__ void __launch_bounds__(256) k_gather_i32(uint4 *d, size_t ds, const uint4 *s, size_t ss,
                                                    const int32_t *perm, size_t n)
{
    FT_GRID_LOOP(e, n)
    {
        const size_t j = (size_t)perm[e];
#pragma unroll
        for (int k = 0; k < FT_PLANES; ++k) d[k * ds + e] = s[k * ss + j];
    }
}

// out[s] (+)= P[off[s+1] - 1] - P[off[s] - 1], P the inclusive prefix sums
// (P[-1] the identity): each segment as a difference of two prefixes
__global__ void __launch_bounds__(128) k_seg_diff(uint4 *op, size_t os, const int32_t *off, size_t nseg,
                                                  const uint4 *P, size_t ps, int accumulate)
{
    FT_GRID_LOOP(sg, nseg)
    {
        const int32_t a = off[sg], b = off[sg + 1];
        ge_p3 v;
        if (a == b) {
            if (accumulate) continue;
            ge_p3_0(v);
        } else {
            ld_p3(v, P, ps, (size_t)b - 1);
            if (a > 0) {
                ge_p3 q;
                ld_p3(q, P, ps, (size_t)a - 1);
                ge_subfrom(v, q);
            }
        }
        seg_write(op, os, (int)sg, v, accumulate);
    }
}

// the largest off[s+1] - off[s] into *d_max (which the caller zeroes)
__global__ void __launch_bounds__(256) k_seg_maxlen(const int32_t *off, size_t nseg, int32_t *d_max)
{
    int32_t m = 0;
    FT_GRID_LOOP(sg, nseg) m = max(m, off[sg + 1] - off[sg]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(d_max, m);
}

cudaError_t segment_maxlen(const int32_t *d_off, size_t nseg, int32_t *d_max, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(d_max, 0, sizeof(int32_t), st);
    if (e != cudaSuccess || nseg == 0) return e;
    k_seg_maxlen<<<(unsigned)std::min<size_t>((nseg + 255) / 256, 1024), 256, 0, st>>>(d_off, nseg, d_max);
    return cudaGetLastError();
}

bool segsum_prefers_prefix(size_t nsrc, size_t max_len)
{
    // the walk's join adds the parts of a segment spanning m threads one
    // after another (m = length / 32, ~7 us each); the prefix path costs
    // about one scan more than the walk, whatever the lengths
    return max_len > std::max<size_t>(2048, nsrc / 1024);
}

size_t segsum_prefix_scratch_bytes(size_t nsrc)
{
    return ((nsrc * 128 + 255) / 256) * 256 + scan_scratch_bytes(nsrc);
}

// the same sums through one inclusive scan of the (gathered) points and a
// difference of two prefixes per segment: ~2 additions per point, and no
// chain of additions longer than the scan's whatever the segment lengths
cudaError_t segsum_prefix(View out, const int32_t *off, size_t nseg, View src, size_t nsrc, const int32_t *perm,
                          int accumulate, void *scratch, cudaStream_t st)
{
    if (nseg == 0) return cudaSuccess;
    View P{(uint4 *)scratch, nsrc};
    void *scan_tmp = (uint8_t *)scratch + ((nsrc * 128 + 255) / 256) * 256;
    cudaError_t e = cudaSuccess;
    if (nsrc) {
        if (perm) {
            k_gather_i32<<<(unsigned)std::min<size_t>((nsrc + 255) / 256, (size_t)sm_count() * 16), 256, 0, st>>>(
                P.p, P.s, src.p, src.s, perm, nsrc);
            e = cudaGetLastError();
        } else {
            e = copy_points(P, src, nsrc, st);
        }
        if (e == cudaSuccess) e = scan(P, nsrc, 0, scan_tmp, st);
        if (e != cudaSuccess) return e;
    }
    k_seg_diff<<<(unsigned)std::min<size_t>((nseg + 127) / 128, (size_t)sm_count() * 32), 128, 0, st>>>(
        out.p, out.s, off, nseg, P.p, P.s, accumulate);
    return cudaGetLastError();
}

// ------------------------------------------------------------ counting sort

// Lanes of a warp holding the same key add their count with one atomic (the
// lowest of them): repeated keys, up to all keys equal, do not serialise on
// one counter.
__global__ void k_key_hist(const uint64_t *keys, size_t n, size_t nkeys, int32_t *cnt, long long *bad)
{
    FT_GRID_LOOP(i, n)
    {
        const uint64_t k = keys[i];
        const unsigned peers = __match_any_sync(__activemask(), k);
        if (k >= nkeys) atomicMax(bad, (long long)i);
        else if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&cnt[k], __popc(peers));
    }
}

// places index i of key k at cur[k] + its rank among the warp's lanes of key k
__global__ void k_key_place(const uint64_t *keys, size_t n, size_t nkeys, int32_t *cur, int32_t *perm)
{
    FT_GRID_LOOP(i, n)
    {
        const uint64_t k = keys[i];
        const unsigned peers = __match_any_sync(__activemask(), k);
        const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
        int32_t base = 0;
        if (k < nkeys && lane == leader) base = atomicAdd(&cur[k], __popc(peers));
        base = __shfl_sync(peers, base, leader);
        if (k < nkeys) perm[base + __popc(peers & ((1u << lane) - 1u))] = (int32_t)i;
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
