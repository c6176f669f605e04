// k_elem.cu — element-wise kernels: group ops, comparisons, gather/scatter and
// the wire formats (folded 32 B, affine 64 B, reference-limb 160 B, packed 128 B).
//
// Kernel <-> reference kernel (ftcrypto.cu):
//   k_set_zero        k_ft_array_set_zero (252)       k_broadcast   k_ft_array_set_point (275)
//   k_add (sub=0/1)   k_ft_add (1089) / k_ft_sub (1220) k_neg        k_ft_neg (1244)
//   k_index           k_ft_index (1262)                k_equal       k_ft_equal (1281)
//   k_mux             k_ft_array_mux (1014)
//   k_gather/k_scatter/k_scatter_zero/k_gather_range/k_scatter_range
//                     k_ft_array_{get_subset,assign_to_subset,assign_zero_to_subset,get_range,assign_to_range} (390-515)
//   k_encode          k_ft_array_to_bytes_folded (629), batched inversion
//   k_decode          k_ft_array_from_bytes_folded (735)
//   k_to_affine       k_ft_array_to_bytes_affine (659)  k_from_affine k_ft_array_from_bytes_affine (793)
//   k_validate        k_ft_array_validate (859)
#include "internal.h"
#include "points.cuh"

#define FT_TABLE_QUAL static __constant__
#define FT_WANT_L_SLIDE
#include "base_table.inc"

namespace ft {

static int g_sm_count = 0;
int sm_count()
{
    if (!g_sm_count) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (g_sm_count <= 0) g_sm_count = 1;
    }
    return g_sm_count;
}

static inline unsigned grid_for(size_t n, int block, int per_sm = 8)
{
    size_t need = (n + block - 1) / block;
    size_t cap = (size_t)sm_count() * per_sm;
    if (need > cap) need = cap;
    if (need == 0) need = 1;
    return (unsigned)need;
}

// ------------------------------------------------------------ group ops

__global__ void __launch_bounds__(256) k_set_zero(uint4 *p, size_t s, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        ge_p3 z;
        ge_zero(z);
        st_p3(p, s, i, z);
    }
}

__global__ void __launch_bounds__(256) k_broadcast(uint4 *p, size_t s, size_t n, const uint4 *q, size_t qs)
{
    FT_GRID_LOOP(i, n)
    {
#pragma unroll
        for (int k = 0; k < FT_PLANES; ++k) p[k * s + i] = q[k * qs];
    }
}

__global__ void __launch_bounds__(128, 4) k_add(uint4 *r, size_t rs, const uint4 *a, size_t as, size_t n, int sub)
{
    FT_GRID_LOOP(i, n)
    {
        ge_p3 x, y;
        ld_p3(x, r, rs, i);
        ld_p3(y, a, as, i);
        if (sub) ge_subfrom(x, y);
        else ge_addto(x, y);
        st_p3(r, rs, i, x);
    }
}

// ciphertext add: (r1, r2) += (a1, a2) over one index space of 2n points,
// so both halves of a ciphertext array share one launch
__global__ void __launch_bounds__(128, 4) k_add_ct(uint4 *r1, size_t r1s, const uint4 *a1, size_t a1s, uint4 *r2,
                                                   size_t r2s, const uint4 *a2, size_t a2s, size_t n, int sub)
{
    FT_GRID_LOOP(j, 2 * n)
    {
        const bool hi = j >= n;
        const size_t i = hi ? j - n : j;
        uint4 *r = hi ? r2 : r1;
        const uint4 *a = hi ? a2 : a1;
        const size_t rs = hi ? r2s : r1s, as = hi ? a2s : a1s;
        ge_p3 x, y;
        ld_p3(x, r, rs, i);
        ld_p3(y, a, as, i);
        if (sub) ge_subfrom(x, y);
        else ge_addto(x, y);
        st_p3(r, rs, i, x);
    }
}

// negates Y and T, as ge25519_neg of ftcrypto.cu:163-167 does
__global__ void __launch_bounds__(256) k_neg(uint4 *p, size_t s, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        ge_p3 x;
        ld_p3(x, p, s, i);
        fe_neg(x.Y, x.Y);
        fe_neg(x.T, x.T);
        st_p3(p, s, i, x);
    }
}

__global__ void __launch_bounds__(256) k_index(int64_t *out, const uint4 *p, size_t s, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        ge_p3 x;
        ld_p3(x, p, s, i);
        out[i] = !ge_iszero(x);
    }
}

__global__ void __launch_bounds__(128, 4) k_equal(int64_t *out, const uint4 *a, size_t as, const uint4 *b, size_t bs,
                                                  size_t n, int invert)
{
    FT_GRID_LOOP(i, n)
    {
        ge_p3 x, y;
        ld_p3(x, a, as, i);
        ld_p3(y, b, bs, i);
        out[i] = ge_equal(x, y) ^ invert;
    }
}

__global__ void __launch_bounds__(256) k_mux(uint4 *t, size_t ts, const int64_t *cond, const uint4 *f, size_t fs, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        if (cond[i] == 0) {
#pragma unroll
            for (int k = 0; k < FT_PLANES; ++k) t[k * ts + i] = f[k * fs + i];
        }
    }
}

__global__ void __launch_bounds__(256) k_gather(uint4 *d, size_t ds, const uint4 *s, size_t ss, const uint64_t *idx, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        size_t j = idx[i];
#pragma unroll
        for (int k = 0; k < FT_PLANES; ++k) d[k * ds + i] = s[k * ss + j];
    }
}

__global__ void __launch_bounds__(256) k_scatter(uint4 *d, size_t ds, const uint4 *s, size_t ss, const uint64_t *idx, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        size_t j = idx[i];
#pragma unroll
        for (int k = 0; k < FT_PLANES; ++k) d[k * ds + j] = s[k * ss + i];
    }
}

__global__ void __launch_bounds__(256) k_scatter_zero(uint4 *d, size_t ds, const uint64_t *idx, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        ge_p3 z;
        ge_zero(z);
        st_p3(d, ds, idx[i], z);
    }
}

__global__ void __launch_bounds__(256) k_gather_range(uint4 *d, size_t ds, const uint4 *s, size_t ss, size_t start,
                                                      size_t step, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        size_t j = start + i * step;
#pragma unroll
        for (int k = 0; k < FT_PLANES; ++k) d[k * ds + i] = s[k * ss + j];
    }
}

__global__ void __launch_bounds__(256) k_scatter_range(uint4 *d, size_t ds, const uint4 *s, size_t ss, size_t start,
                                                       size_t step, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        size_t j = start + i * step;
#pragma unroll
        for (int k = 0; k < FT_PLANES; ++k) d[k * ds + j] = s[k * ss + i];
    }
}

// ------------------------------------------------------------ wire formats

// Batched inversion (Montgomery's trick) over K consecutive points per
// thread: one fe_invert and 3(K-1) multiplications instead of K inversions.
// A zero Z is replaced by 1 inside the product and its inverse reported as 0,
// which is what fe25519_invert(0) = 0 gives the reference.
template <int K, class Emit>
FT_DEV void batch_zinv(const uint4 *p, size_t s, size_t n, size_t base, Emit emit)
{
    fe q[K];
    uint32_t zero_bits = 0;
    fe acc;
    fe_1(acc);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        size_t i = base + k;
        fe z;
        if (i < n) fe_from_u4(z, p[4 * s + i], p[5 * s + i]);
        else fe_1(z);
        uint32_t zm = 0u - (uint32_t)fe_iszero(z);
        zero_bits |= (zm & 1u) << k;
        fe one;
        fe_1(one);
        fe_cmov(z, one, zm);
        if (k == 0) fe_copy(acc, z);
        else fe_mul(acc, acc, z);
        fe_copy(q[k], acc);
    }
    fe inv;
    fe_invert(inv, acc);
#pragma unroll
    for (int k = K - 1; k >= 0; --k) {
        size_t i = base + k;
        fe zinv;
        if (k > 0) {
            fe_mul(zinv, inv, q[k - 1]);
            fe z;
            if (i < n) fe_from_u4(z, p[4 * s + i], p[5 * s + i]);
            else fe_1(z);
            fe one;
            fe_1(one);
            fe_cmov(z, one, 0u - ((zero_bits >> k) & 1u));
            fe_mul(inv, inv, z);
        } else {
            fe_copy(zinv, inv);
        }
        fe zero;
        fe_0(zero);
        fe_cmov(zinv, zero, 0u - ((zero_bits >> k) & 1u));
        if (i < n) emit(i, zinv);
    }
}

template <int K>
__global__ void __launch_bounds__(128) k_encode(uint4 *out, const uint4 *p, size_t s, size_t n)
{
    size_t groups = (n + K - 1) / K;
    FT_GRID_LOOP(g, groups)
    {
        batch_zinv<K>(p, s, n, g * K, [&](size_t i, const fe &zinv) {
            ge_p3 h;
            ld_p3(h, p, s, i);
            uint32_t w[8];
            ge_encode_with_zinv(w, h, zinv);
            out[2 * i] = make_uint4(w[0], w[1], w[2], w[3]);
            out[2 * i + 1] = make_uint4(w[4], w[5], w[6], w[7]);
        });
    }
}

template <int K>
__global__ void __launch_bounds__(128) k_to_affine(uint4 *out, const uint4 *p, size_t s, size_t n)
{
    size_t groups = (n + K - 1) / K;
    FT_GRID_LOOP(g, groups)
    {
        batch_zinv<K>(p, s, n, g * K, [&](size_t i, const fe &zinv) {
            ge_p3 h;
            ld_p3(h, p, s, i);
            fe x, y;
            fe_mul(x, h.X, zinv);
            fe_mul(y, h.Y, zinv);
            fe_canon(x, x);
            fe_canon(y, y);
            out[4 * i + 0] = u4_lo(x);
            out[4 * i + 1] = u4_hi(x);
            out[4 * i + 2] = u4_lo(y);
            out[4 * i + 3] = u4_hi(y);
        });
    }
}

__global__ void __launch_bounds__(128) k_decode(uint4 *p, size_t s, const uint4 *in, size_t n, long long *bad)
{
    FT_GRID_LOOP(i, n)
    {
        uint4 a = in[2 * i], b = in[2 * i + 1];
        uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        ge_p3 h;
        int r = ge_frombytes(h, w);
        st_p3(p, s, i, h);
        if (r) atomicMax(bad, (long long)i);
    }
}

// X, Y from bytes (top bit ignored), Z = 1, T = XY; no validation
__global__ void __launch_bounds__(256) k_from_affine(uint4 *p, size_t s, const uint4 *in, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        uint4 w[4] = {in[4 * i], in[4 * i + 1], in[4 * i + 2], in[4 * i + 3]};
        uint32_t xw[8] = {w[0].x, w[0].y, w[0].z, w[0].w, w[1].x, w[1].y, w[1].z, w[1].w};
        uint32_t yw[8] = {w[2].x, w[2].y, w[2].z, w[2].w, w[3].x, w[3].y, w[3].z, w[3].w};
        ge_p3 h;
        fe_from_words(h.X, xw);
        fe_from_words(h.Y, yw);
        fe_1(h.Z);
        fe_mul(h.T, h.X, h.Y);
        st_p3(p, s, i, h);
    }
}

// bits [lo, lo + nb) of a 256-bit little-endian value, nb <= 32, lo constant
FT_DEV int64_t bits_at(const fe &c, int lo, int nb)
{
    int w = lo >> 5, b = lo & 31;
    uint64_t x = c.v[w];
    if (w + 1 < 8) x |= (uint64_t)c.v[w + 1] << 32;
    x >>= b;
    return (int64_t)(x & ((1ull << nb) - 1));
}

// canonical value -> the 10 signed limbs fe25519_frombytes (sodium_fe.cu:74-141)
// produces from the canonical bytes: same loads, same carry order
FT_DEV void fe_to_ref10(int32_t out[10], const fe &f)
{
    fe c;
    fe_canon(c, f);
    int64_t h[10];
    h[0] = bits_at(c, 0, 32);
    h[1] = bits_at(c, 32, 24) << 6;
    h[2] = bits_at(c, 56, 24) << 5;
    h[3] = bits_at(c, 80, 24) << 3;
    h[4] = bits_at(c, 104, 24) << 2;
    h[5] = bits_at(c, 128, 32);
    h[6] = bits_at(c, 160, 24) << 7;
    h[7] = bits_at(c, 184, 24) << 5;
    h[8] = bits_at(c, 208, 24) << 4;
    h[9] = (bits_at(c, 232, 24) & 8388607) << 2;
    int64_t carry;
    carry = (h[9] + (1LL << 24)) >> 25;
    h[0] += carry * 19;
    h[9] -= carry * (1LL << 25);
#pragma unroll
    for (int i = 1; i < 9; i += 2) {
        carry = (h[i] + (1LL << 24)) >> 25;
        h[i + 1] += carry;
        h[i] -= carry * (1LL << 25);
    }
#pragma unroll
    for (int i = 0; i < 10; i += 2) {
        carry = (h[i] + (1LL << 25)) >> 26;
        h[i + 1] += carry;
        h[i] -= carry * (1LL << 26);
    }
#pragma unroll
    for (int i = 0; i < 10; ++i) out[i] = (int32_t)h[i];
}

// sum of limb_i * 2^off_i (limbs signed, any magnitude below 2^31) mod p:
// positive and negative limbs go to two 288-bit accumulators, each folded
// with 2^256 = 38, and the results are subtracted
FT_DEV void fe_from_ref10(fe &f, const int32_t l[10])
{
    const int off[10] = {0, 26, 51, 77, 102, 128, 153, 179, 204, 230};
    uint32_t pos[16], neg[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) pos[k] = neg[k] = 0;
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        int32_t v = l[i];
        uint32_t m = 0u - (uint32_t)(v < 0);
        uint32_t mag = ((uint32_t)v ^ m) - m;
        int w = off[i] >> 5, b = off[i] & 31;
        uint64_t sh = (uint64_t)mag << b;
        uint32_t lo = (uint32_t)sh, hi = (uint32_t)(sh >> 32);
        uint32_t cp = 0, cn = 0;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            uint64_t add = (k == w) ? lo : (k == w + 1 ? hi : 0u);
            uint64_t tp = (uint64_t)pos[k] + (add & ~(uint64_t)m) + cp;
            uint64_t tn = (uint64_t)neg[k] + (add & (uint64_t)m) + cn;
            pos[k] = (uint32_t)tp;
            cp = (uint32_t)(tp >> 32);
            neg[k] = (uint32_t)tn;
            cn = (uint32_t)(tn >> 32);
        }
    }
    fe a, b;
    fe_fold512(a, pos);
    fe_fold512(b, neg);
    fe_sub(f, a, b);
}

// Each warp converts 32 consecutive points into shared memory (rows of 41
// words: conflict-free) and writes their 5,120 contiguous bytes with
// coalesced stores; one thread writing its 160-byte struct directly made
// every store instruction of a warp touch 32 sectors.
__global__ void __launch_bounds__(128) k_to_ref160(int32_t *out, const uint4 *p, size_t s, size_t n)
{
    __shared__ int32_t stage[4][32 * 41];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t *row = stage[warp] + 41 * lane;
#pragma unroll 1
    for (size_t base = (size_t)blockIdx.x * 128 + 32 * warp; base < n; base += (size_t)gridDim.x * 128) {
        const size_t i = base + lane;
        if (i < n) {
            ge_p3 h;
            ld_p3(h, p, s, i);
            fe_to_ref10(row, h.X);
            fe_to_ref10(row + 10, h.Y);
            fe_to_ref10(row + 20, h.Z);
            fe_to_ref10(row + 30, h.T);
        }
        __syncwarp();
        const int words = 40 * (int)(n - base < 32 ? n - base : 32);
        int32_t *o = out + 40 * base;
#pragma unroll 1
        for (int k = lane; k < words; k += 32) o[k] = stage[warp][41 * (k / 40) + k % 40];
        __syncwarp();
    }
}

// the mirror of k_to_ref160: each warp reads its 32 structs with coalesced
// loads into shared memory, then each thread converts its own
__global__ void __launch_bounds__(128) k_from_ref160(uint4 *p, size_t s, const int32_t *in, size_t n)
{
    __shared__ int32_t stage[4][32 * 41];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int32_t *row = stage[warp] + 41 * lane;
#pragma unroll 1
    for (size_t base = (size_t)blockIdx.x * 128 + 32 * warp; base < n; base += (size_t)gridDim.x * 128) {
        const int words = 40 * (int)(n - base < 32 ? n - base : 32);
        const int32_t *q = in + 40 * base;
#pragma unroll 1
        for (int k = lane; k < words; k += 32) stage[warp][41 * (k / 40) + k % 40] = q[k];
        __syncwarp();
        const size_t i = base + lane;
        if (i < n) {
            ge_p3 h;
            int32_t l[10];
#pragma unroll
            for (int j = 0; j < 10; ++j) l[j] = row[j];
            fe_from_ref10(h.X, l);
#pragma unroll
            for (int j = 0; j < 10; ++j) l[j] = row[10 + j];
            fe_from_ref10(h.Y, l);
#pragma unroll
            for (int j = 0; j < 10; ++j) l[j] = row[20 + j];
            fe_from_ref10(h.Z, l);
#pragma unroll
            for (int j = 0; j < 10; ++j) l[j] = row[30 + j];
            fe_from_ref10(h.T, l);
            st_p3(p, s, i, h);
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(256) k_to_packed(uint4 *out, const uint4 *p, size_t s, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
#pragma unroll
        for (int k = 0; k < FT_PLANES; ++k) out[8 * i + k] = p[k * s + i];
    }
}

__global__ void __launch_bounds__(256) k_from_packed(uint4 *p, size_t s, const uint4 *in, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
#pragma unroll
        for (int k = 0; k < FT_PLANES; ++k) p[k * s + i] = in[8 * i + k];
    }
}

// ------------------------------------------------------------ validation

// L * A in the sliding-window sequence of ge25519_mul_l (sodium_ge.cu:795-847);
// variable time in the public group order only.
FT_DEV void ge_mul_l(ge_p3 &r, const ge_p3 &A)
{
    ge_cached Ai[8];
    ge_p1p1 t;
    ge_p3 u, A2;
    ge_p3_to_cached(Ai[0], A);
    ge_p3_dbl(t, A);
    ge_p1p1_to_p3(A2, t);
#pragma unroll 1
    for (int k = 1; k < 8; ++k) {
        ge_add(t, A2, Ai[k - 1]);
        ge_p1p1_to_p3(u, t);
        ge_p3_to_cached(Ai[k], u);
    }
    ge_p3_0(r);
#pragma unroll 1
    for (int i = 252; i >= 0; --i) {
        ge_p3_dbl(t, r);
        int d = FT_L_SLIDE_INIT[i];
        if (d > 0) {
            ge_p1p1_to_p3(u, t);
            ge_add(t, u, Ai[d / 2]);
        } else if (d < 0) {
            ge_p1p1_to_p3(u, t);
            ge_sub(t, u, Ai[(-d) / 2]);
        }
        ge_p1p1_to_p3(r, t);
    }
}

__global__ void __launch_bounds__(128) k_validate(const uint4 *p, size_t s, size_t n, long long *bad)
{
    FT_GRID_LOOP(i, n)
    {
        ge_p3 h;
        ld_p3(h, p, s, i);
        int ok = ge_is_on_curve(h);
        if (ok) {
            ge_p3 pl;
            ge_mul_l(pl, h);
            ok = fe_iszero(pl.X);
        }
        if (!ok) atomicMax(bad, (long long)i);
    }
}

// ------------------------------------------------------------ launchers

// *acc |= OR of v[0 .. n): one 64-bit atomic per warp
__global__ void __launch_bounds__(256) k_or_words(unsigned long long *acc, const uint64_t *v, size_t n)
{
    uint64_t x = 0;
    FT_GRID_LOOP(i, n) x |= v[i];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x |= __shfl_xor_sync(0xffffffffu, x, d);
    if ((threadIdx.x & 31) == 0 && x) atomicOr(acc, (unsigned long long)x);
}

#define FT_LAUNCH(kern, n, block, ...)                                  \
    do {                                                                 \
        if ((n) == 0) return cudaSuccess;                                \
        kern<<<grid_for((n), (block)), (block), 0, st>>>(__VA_ARGS__);   \
        return cudaGetLastError();                                       \
    } while (0)

cudaError_t set_zero(View v, size_t n, cudaStream_t st) { FT_LAUNCH(k_set_zero, n, 256, v.p, v.s, n); }

cudaError_t or_words(uint64_t *acc, const uint64_t *v, size_t n, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(uint64_t), st);
    if (e != cudaSuccess) return e;
    FT_LAUNCH(k_or_words, n, 256, (unsigned long long *)acc, v, n);
}
cudaError_t broadcast(View d, size_t n, View q, cudaStream_t st) { FT_LAUNCH(k_broadcast, n, 256, d.p, d.s, n, q.p, q.s); }
cudaError_t add(View r, View a, size_t n, int sub, cudaStream_t st) { FT_LAUNCH(k_add, n, 128, r.p, r.s, a.p, a.s, n, sub); }
cudaError_t add_ct(View r1, View r2, View a1, View a2, size_t n, int sub, cudaStream_t st)
{
    FT_LAUNCH(k_add_ct, 2 * n, 128, r1.p, r1.s, a1.p, a1.s, r2.p, r2.s, a2.p, a2.s, n, sub);
}
cudaError_t neg(View v, size_t n, cudaStream_t st) { FT_LAUNCH(k_neg, n, 256, v.p, v.s, n); }
cudaError_t index_nonzero(int64_t *o, View v, size_t n, cudaStream_t st) { FT_LAUNCH(k_index, n, 256, o, v.p, v.s, n); }
cudaError_t equal(int64_t *o, View a, View b, size_t n, int inv, cudaStream_t st) { FT_LAUNCH(k_equal, n, 128, o, a.p, a.s, b.p, b.s, n, inv); }
cudaError_t mux(View t, const int64_t *c, View f, size_t n, cudaStream_t st) { FT_LAUNCH(k_mux, n, 256, t.p, t.s, c, f.p, f.s, n); }
cudaError_t gather(View d, View s, const uint64_t *ix, size_t n, cudaStream_t st) { FT_LAUNCH(k_gather, n, 256, d.p, d.s, s.p, s.s, ix, n); }
cudaError_t scatter(View d, View s, const uint64_t *ix, size_t n, cudaStream_t st) { FT_LAUNCH(k_scatter, n, 256, d.p, d.s, s.p, s.s, ix, n); }
cudaError_t scatter_zero(View d, const uint64_t *ix, size_t n, cudaStream_t st) { FT_LAUNCH(k_scatter_zero, n, 256, d.p, d.s, ix, n); }
cudaError_t gather_range(View d, View s, size_t a, size_t b, size_t n, cudaStream_t st) { FT_LAUNCH(k_gather_range, n, 256, d.p, d.s, s.p, s.s, a, b, n); }
cudaError_t scatter_range(View d, View s, size_t a, size_t b, size_t n, cudaStream_t st) { FT_LAUNCH(k_scatter_range, n, 256, d.p, d.s, s.p, s.s, a, b, n); }
cudaError_t decode(View v, const uint8_t *in, size_t n, long long *bad, cudaStream_t st) { FT_LAUNCH(k_decode, n, 128, v.p, v.s, (const uint4 *)in, n, bad); }
cudaError_t from_affine(View v, const uint8_t *in, size_t n, cudaStream_t st) { FT_LAUNCH(k_from_affine, n, 256, v.p, v.s, (const uint4 *)in, n); }
cudaError_t to_ref160(uint8_t *o, View v, size_t n, cudaStream_t st) { FT_LAUNCH(k_to_ref160, n, 128, (int32_t *)o, v.p, v.s, n); }
cudaError_t from_ref160(View v, const uint8_t *in, size_t n, cudaStream_t st) { FT_LAUNCH(k_from_ref160, n, 128, v.p, v.s, (const int32_t *)in, n); }
cudaError_t to_packed(uint8_t *o, View v, size_t n, cudaStream_t st) { FT_LAUNCH(k_to_packed, n, 256, (uint4 *)o, v.p, v.s, n); }
cudaError_t from_packed(View v, const uint8_t *in, size_t n, cudaStream_t st) { FT_LAUNCH(k_from_packed, n, 256, v.p, v.s, (const uint4 *)in, n); }
cudaError_t validate(View v, size_t n, long long *bad, cudaStream_t st) { FT_LAUNCH(k_validate, n, 128, v.p, v.s, n, bad); }

static const int ENC_K = 8;
cudaError_t encode(uint8_t *o, View v, size_t n, cudaStream_t st)
{
    size_t groups = (n + ENC_K - 1) / ENC_K;
    FT_LAUNCH(k_encode<ENC_K>, groups, 128, (uint4 *)o, v.p, v.s, n);
}
cudaError_t to_affine(uint8_t *o, View v, size_t n, cudaStream_t st)
{
    size_t groups = (n + ENC_K - 1) / ENC_K;
    FT_LAUNCH(k_to_affine<ENC_K>, groups, 128, (uint4 *)o, v.p, v.s, n);
}

cudaError_t copy_points(View d, View s, size_t n, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    return cudaMemcpy2DAsync(d.p, d.s * sizeof(uint4), s.p, s.s * sizeof(uint4), n * sizeof(uint4), FT_PLANES,
                             cudaMemcpyDeviceToDevice, st);
}

} // namespace ft
