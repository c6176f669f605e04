// ladder_tab.cuh — per-thread tables of the variable-base ladder: (k+1)*P in
// cached form for k < 8, 1 KB per thread.
//   SmemTab<NT>    all entries in shared memory, [entry][16-byte word][thread]
//                  with stride NT: a warp's access to one word of one entry
//                  is 512 contiguous bytes (conflict-free).
//   HybridTab<NT>  entries 0-3 in shared memory (same layout), 4-7 in the
//                  thread's tensor-memory lane (tmem.cuh).
// Both satisfy the Tab interface of smul.cuh.  This header holds no kernel,
// so the host test harness compiles it against emulated shared and tensor
// memory.
#pragma once
#include "smul.cuh"
#include "u4.cuh"
#ifndef FT_HOST_EMULATION
#include "tmem.cuh"
#define FT_TAB_FN __device__ __forceinline__
#else
#define FT_TAB_FN inline
#endif

#ifndef FT_TMEM_SEL_COLS
#define FT_TMEM_SEL_COLS 8
#endif
static_assert(FT_TMEM_SEL_COLS == 8 || FT_TMEM_SEL_COLS == 16 || FT_TMEM_SEL_COLS == 32, "TMEM select load width");

namespace ft {

template <int NT>
struct SmemTab {
    uint4 *b; // &smem[threadIdx.x]
    FT_TAB_FN void put(int k, const ge_cached &c) const
    {
        uint4 *q = b + (size_t)k * 8 * NT;
        q[0 * NT] = u4_lo(c.YplusX);
        q[1 * NT] = u4_hi(c.YplusX);
        q[2 * NT] = u4_lo(c.YminusX);
        q[3 * NT] = u4_hi(c.YminusX);
        q[4 * NT] = u4_lo(c.Z);
        q[5 * NT] = u4_hi(c.Z);
        q[6 * NT] = u4_lo(c.T2d);
        q[7 * NT] = u4_hi(c.T2d);
    }
    // coordinate j of entry k: 0 YplusX, 1 YminusX, 2 Z, 3 T2d
    FT_TAB_FN void get_fe(int k, int j, fe &f) const
    {
        const uint4 *q = b + (size_t)(k * 8 + 2 * j) * NT;
        fe_from_u4(f, q[0], q[NT]);
    }
    template <int NE>
    FT_TAB_FN void select_fe(fe &f, int j, uint32_t babs, bool one) const
    {
        tab_select_fe<NE>(f, *this, j, babs, one);
    }
    FT_TAB_FN void get(int k, ge_cached &c) const
    {
        const uint4 *q = b + (size_t)k * 8 * NT;
        fe_from_u4(c.YplusX, q[0 * NT], q[1 * NT]);
        fe_from_u4(c.YminusX, q[2 * NT], q[3 * NT]);
        fe_from_u4(c.Z, q[4 * NT], q[5 * NT]);
        fe_from_u4(c.T2d, q[6 * NT], q[7 * NT]);
    }
};

// Entries 0-3 in shared memory ([entry][word][thread], stride NT), entries
// 4-7 in TMEM at columns col + 32 j + 8 (k - 4) of the thread's lane: the
// four entries' coordinate j are 32 consecutive columns (read 8 at a time).
template <int NT>
struct HybridTab {
    uint4 *b;     // &smem[threadIdx.x]
    uint32_t col; // TMEM address of this warp's lane quarter and column slice
    FT_TAB_FN void put(int k, const ge_cached &c) const
    {
        if (k < 4) {
            uint4 *q = b + (size_t)k * 8 * NT;
            q[0 * NT] = u4_lo(c.YplusX);
            q[1 * NT] = u4_hi(c.YplusX);
            q[2 * NT] = u4_lo(c.YminusX);
            q[3 * NT] = u4_hi(c.YminusX);
            q[4 * NT] = u4_lo(c.Z);
            q[5 * NT] = u4_hi(c.Z);
            q[6 * NT] = u4_lo(c.T2d);
            q[7 * NT] = u4_hi(c.T2d);
        } else {
            const uint32_t a = col + 8u * (uint32_t)(k - 4);
            tmem_st8(a + 0, c.YplusX.v);
            tmem_st8(a + 32, c.YminusX.v);
            tmem_st8(a + 64, c.Z.v);
            tmem_st8(a + 96, c.T2d.v);
        }
    }
    FT_TAB_FN void get(int k, ge_cached &c) const
    {
        if (k < 4) {
            const uint4 *q = b + (size_t)k * 8 * NT;
            fe_from_u4(c.YplusX, q[0 * NT], q[1 * NT]);
            fe_from_u4(c.YminusX, q[2 * NT], q[3 * NT]);
            fe_from_u4(c.Z, q[4 * NT], q[5 * NT]);
            fe_from_u4(c.T2d, q[6 * NT], q[7 * NT]);
        } else {
            tmem_wait_st();
            const uint32_t a = col + 8u * (uint32_t)(k - 4);
            tmem_ld8(a + 0, c.YplusX.v);
            tmem_ld8(a + 32, c.YminusX.v);
            tmem_ld8(a + 64, c.Z.v);
            tmem_ld8(a + 96, c.T2d.v);
        }
    }
    // entries k < min(NE, 4) from shared memory, 4 <= k < NE from TMEM
    template <int NE>
    FT_TAB_FN void select_fe(fe &f, int j, uint32_t babs, bool one) const
    {
        if (one) fe_1(f);
        else fe_0(f);
#pragma unroll
        for (int k = 0; k < (NE < 4 ? NE : 4); ++k) {
            const uint4 *q = b + (size_t)(k * 8 + 2 * j) * NT;
            fe e;
            fe_from_u4(e, q[0], q[NT]);
            fe_cmov(f, e, ct_eq_mask(babs, (uint32_t)(k + 1)));
        }
        if (NE <= 4) return;
        // (a select with some entries multiplied by 0/1 indicators on the
        // multiply-add pipe instead of masked measured 3% slower: the field
        // multiplications keep that pipe busy)
        // FT_TMEM_SEL_COLS columns per load (8: one entry, 16: two, 32: all
        // four), each load waited for before its entries are merged.
        // Ladder of 1,048,576 points: 20.31 ms with one load of 32 columns
        // (32 registers in flight), 20.24 ms with two of 16, 20.19 ms with
        // four of 8.
        constexpr int EPL = FT_TMEM_SEL_COLS / 8; // entries per load
#pragma unroll
        for (int k0 = 0; k0 < 4; k0 += EPL) {
            uint32_t r[FT_TMEM_SEL_COLS];
            const uint32_t a = col + 32u * (uint32_t)j + 8u * (uint32_t)k0;
            if constexpr (EPL == 1) tmem_ld8(a, r);
            else if constexpr (EPL == 2) tmem_ld16(a, r);
            else tmem_ld32(a, r);
#pragma unroll
            for (int q = 0; q < EPL; ++q) {
                const uint32_t m = ct_eq_mask(babs, (uint32_t)(k0 + q + 5));
#pragma unroll
                for (int w = 0; w < 8; ++w) f.v[w] ^= (f.v[w] ^ r[8 * q + w]) & m;
            }
        }
    }
};

} // namespace ft
