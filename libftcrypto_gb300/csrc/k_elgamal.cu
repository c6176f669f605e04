// k_elgamal.cu — caller-side ElGamal helpers: the discrete-log table of
// small plaintexts that decryption looks messages up in.
//
// Decryption of (c1, c2) under sk gives the point D = c2 - sk*c1 = m*B; m is
// found by looking the canonical encoding of D up in a table of the
// encodings of j*B, j < m_max.  The table is open addressing with linear
// probing over cap = a power of two >= 2 m_max slots:
//   state[slot]  0 empty, else j + 1 (claimed with atomicCAS by the thread
//                inserting j, which then writes the encoding)
//   enc[slot]    the 32-byte encoding of j*B, as 8 words
// A lookup probes from the encoding's hash until it finds the encoding
// (m = state - 1) or an empty slot (no such m).  Every probe loop is bounded
// by cap: an insert always finds a slot (the table is at most half full) and
// a lookup always meets an empty one; no thread waits on another.
#include "internal.h"
#include "points.cuh"

namespace ft {

FT_DEV uint64_t dlog_hash(const uint32_t e[8])
{
    uint64_t h = ((uint64_t)e[1] << 32 | e[0]) ^ ((uint64_t)e[3] << 32 | e[2]) * 0x9e3779b97f4a7c15ull;
    h ^= h >> 29;
    h *= 0xbf58476d1ce4e5b9ull;
    return h ^ (h >> 32);
}

FT_DEV void load_enc(uint32_t e[8], const uint8_t *p)
{
    const uint4 *q = (const uint4 *)p;
    uint4 a = q[0], b = q[1];
    e[0] = a.x; e[1] = a.y; e[2] = a.z; e[3] = a.w;
    e[4] = b.x; e[5] = b.y; e[6] = b.z; e[7] = b.w;
}

__global__ void k_dlog_insert(uint32_t *state, uint32_t *enc, uint64_t cap, const uint8_t *d_enc, uint64_t m_max)
{
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m_max; j += (uint64_t)blockDim.x * gridDim.x) {
        uint32_t e[8];
        load_enc(e, d_enc + 32 * j);
        uint64_t slot = dlog_hash(e) & (cap - 1);
        for (uint64_t probe = 0; probe < cap; ++probe) {
            if (atomicCAS(&state[slot], 0u, (uint32_t)(j + 1)) == 0u) {
                uint4 *q = (uint4 *)(enc + 8 * slot);
                q[0] = make_uint4(e[0], e[1], e[2], e[3]);
                q[1] = make_uint4(e[4], e[5], e[6], e[7]);
                break;
            }
            slot = (slot + 1) & (cap - 1);
        }
    }
}

__global__ void k_dlog_lookup(uint64_t *m, const uint32_t *state, const uint32_t *enc, uint64_t cap,
                              const uint8_t *d_enc, size_t n)
{
    FT_GRID_LOOP(i, n)
    {
        uint32_t e[8];
        load_enc(e, d_enc + 32 * i);
        uint64_t slot = dlog_hash(e) & (cap - 1), out = ~0ull;
        for (uint64_t probe = 0; probe < cap; ++probe) {
            const uint32_t st = state[slot];
            if (st == 0u) break;
            const uint4 *q = (const uint4 *)(enc + 8 * slot);
            const uint4 a = q[0], b = q[1];
            if (a.x == e[0] && a.y == e[1] && a.z == e[2] && a.w == e[3] && b.x == e[4] && b.y == e[5] &&
                b.z == e[6] && b.w == e[7]) {
                out = st - 1u;
                break;
            }
            slot = (slot + 1) & (cap - 1);
        }
        m[i] = out;
    }
}

__global__ void k_iota_u64(uint64_t *d, size_t n)
{
    FT_GRID_LOOP(i, n) d[i] = i;
}

static unsigned grid_for(size_t n)
{
    size_t need = (n + 255) / 256, cap = (size_t)sm_count() * 8;
    return (unsigned)(need < cap ? (need ? need : 1) : cap);
}

size_t dlog_table_bytes(uint64_t cap) { return ((cap * 4 + 255) & ~(uint64_t)255) + cap * 32; }

cudaError_t dlog_build(DlogTable &t, void *mem, uint64_t m_max, uint64_t cap, const uint8_t *d_enc, cudaStream_t st)
{
    t.state = (uint32_t *)mem;
    t.enc = (uint32_t *)((uint8_t *)mem + ((cap * 4 + 255) & ~(uint64_t)255));
    t.m_max = m_max;
    t.cap = cap;
    cudaError_t e = cudaMemsetAsync(t.state, 0, cap * 4, st);
    if (e != cudaSuccess) return e;
    k_dlog_insert<<<grid_for(m_max), 256, 0, st>>>(t.state, t.enc, cap, d_enc, m_max);
    return cudaGetLastError();
}

cudaError_t dlog_lookup(uint64_t *d_m, const DlogTable &t, const uint8_t *d_enc, size_t n, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    k_dlog_lookup<<<grid_for(n), 256, 0, st>>>(d_m, t.state, t.enc, t.cap, d_enc, n);
    return cudaGetLastError();
}

cudaError_t iota_u64(uint64_t *d, size_t n, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    k_iota_u64<<<grid_for(n), 256, 0, st>>>(d, n);
    return cudaGetLastError();
}

} // namespace ft
