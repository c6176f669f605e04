// tmem.cuh — tensor memory (TMEM) as per-thread storage.
//
// TMEM is 128 lanes x 512 columns of 32-bit cells per SM.  With the
// 32x32b access shape, thread t of warp w reads and writes lane
// 32*(w % 4) + t, N consecutive columns per instruction, so a column range
// given to a warp is private storage of 4*N bytes per thread.  Warps with the
// same w % 4 share lanes and are given disjoint column ranges.
//
// Protocol (every kernel that uses these):
//   * warp 0 allocates with tmem_alloc (whole warp), the address is published
//     through shared memory behind tmem_sync_threads(), and warp 0 frees the
//     same columns after a final tmem_sync_threads();
//   * a kernel allocates only when it is the only CTA its SM can hold (its
//     shared memory exceeds half of the SM's), so an allocation never waits
//     for another CTA's columns;
//   * the .sync.aligned forms are executed by every thread of a warp
//     together: the kernels run no divergent code around them;
//   * loads complete inside the same asm statement (tcgen05.wait::ld), so the
//     compiler never sees their destination registers before they are
//     written; stores are completed with tmem_wait_st() before any load of
//     the same cells.
#pragma once
#include <cstdint>

#define FT_DEV_TM __device__ __forceinline__

namespace ft {

FT_DEV_TM void tmem_alloc(uint32_t *smem_dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"((uint32_t)__cvta_generic_to_shared(smem_dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

FT_DEV_TM void tmem_free(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// __syncthreads with the fences that order TMEM accesses across it
FT_DEV_TM void tmem_sync_threads()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

FT_DEV_TM void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// address of column `col` in this warp's lane quarter
FT_DEV_TM uint32_t tmem_warp_addr(uint32_t base, int warp, uint32_t col)
{
    return base + ((uint32_t)(32 * (warp & 3)) << 16) + col;
}

FT_DEV_TM void tmem_st8(uint32_t ta, const uint32_t v[8])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(ta), "r"(v[0]),
                 "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}

FT_DEV_TM void tmem_ld8(uint32_t ta, uint32_t r[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n\t"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(ta)
                 : "memory");
}

FT_DEV_TM void tmem_ld16(uint32_t ta, uint32_t r[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(ta)
                 : "memory");
}

FT_DEV_TM void tmem_ld32(uint32_t ta, uint32_t r[32])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                   "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                   "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(ta)
                 : "memory");
}

} // namespace ft
