// ptx_emul.h — C stand-ins for the PTX carry-chain primitives of
// libftcrypto_gb300/csrc/ptx.cuh, so the device field/group code can be
// compiled with g++ and checked against the oracle on a machine without a
// GPU.  TEST HARNESS ONLY (tests/host/devcode_host.cpp); never part of the
// shipped library.
#pragma once
#include <stdint.h>
#include <string.h>
#include <stdlib.h>

#define FT_DEV static inline

static thread_local uint32_t g_cf; // the PTX carry flag

static inline uint32_t add_cc(uint32_t a, uint32_t b) { uint64_t t = (uint64_t)a + b; g_cf = (uint32_t)(t >> 32); return (uint32_t)t; }
static inline uint32_t addc_cc(uint32_t a, uint32_t b) { uint64_t t = (uint64_t)a + b + g_cf; g_cf = (uint32_t)(t >> 32); return (uint32_t)t; }
static inline uint32_t addc(uint32_t a, uint32_t b) { return a + b + g_cf; }
static inline uint32_t sub_cc(uint32_t a, uint32_t b) { uint64_t t = (uint64_t)a - b; g_cf = (uint32_t)(t >> 32) & 1u; return (uint32_t)t; }
static inline uint32_t subc_cc(uint32_t a, uint32_t b) { uint64_t t = (uint64_t)a - b - g_cf; g_cf = (uint32_t)(t >> 32) & 1u; return (uint32_t)t; }
static inline uint32_t subc(uint32_t a, uint32_t b) { return a - b - g_cf; }
static inline uint32_t mad_lo_cc(uint32_t a, uint32_t b, uint32_t c) { uint64_t t = (uint64_t)(uint32_t)(a * b) + c; g_cf = (uint32_t)(t >> 32); return (uint32_t)t; }
static inline uint32_t madc_lo_cc(uint32_t a, uint32_t b, uint32_t c) { uint64_t t = (uint64_t)(uint32_t)(a * b) + c + g_cf; g_cf = (uint32_t)(t >> 32); return (uint32_t)t; }
static inline uint32_t madc_lo(uint32_t a, uint32_t b, uint32_t c) { return (uint32_t)(a * b) + c + g_cf; }
static inline uint32_t mad_hi_cc(uint32_t a, uint32_t b, uint32_t c) { uint64_t t = (((uint64_t)a * b) >> 32) + c; g_cf = (uint32_t)(t >> 32); return (uint32_t)t; }
static inline uint32_t madc_hi_cc(uint32_t a, uint32_t b, uint32_t c) { uint64_t t = (((uint64_t)a * b) >> 32) + c + g_cf; g_cf = (uint32_t)(t >> 32); return (uint32_t)t; }
static inline uint32_t madc_hi(uint32_t a, uint32_t b, uint32_t c) { return (uint32_t)(((uint64_t)a * b) >> 32) + c + g_cf; }
static inline uint32_t mul_lo(uint32_t a, uint32_t b) { return a * b; }
static inline uint32_t mul_hi(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }

// 16-byte word of the device code (CUDA's uint4)
struct uint4 {
    uint32_t x, y, z, w;
};
static inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return uint4{x, y, z, w}; }

// Tensor memory of one SM (128 lanes x 512 columns) for the tcgen05 helpers
// of tmem.cuh.  An address is lane << 16 | column; an access outside the
// allocation aborts, so the tests also check the kernels' column arithmetic.
static thread_local uint32_t g_tmem[128][512];
static inline uint32_t *tmem_cell(uint32_t ta, int n)
{
    uint32_t lane = ta >> 16, col = ta & 0xffffu;
    if (lane >= 128u || col + (uint32_t)n > 512u) abort();
    return &g_tmem[lane][col];
}
static inline uint32_t tmem_warp_addr(uint32_t base, int warp, uint32_t col)
{
    return base + ((uint32_t)(32 * (warp & 3)) << 16) + col;
}
static inline void tmem_st8(uint32_t ta, const uint32_t v[8]) { memcpy(tmem_cell(ta, 8), v, 32); }
static inline void tmem_ld8(uint32_t ta, uint32_t r[8]) { memcpy(r, tmem_cell(ta, 8), 32); }
static inline void tmem_ld16(uint32_t ta, uint32_t r[16]) { memcpy(r, tmem_cell(ta, 16), 64); }
static inline void tmem_ld32(uint32_t ta, uint32_t r[32]) { memcpy(r, tmem_cell(ta, 32), 128); }
static inline void tmem_wait_st() {}
// one emulated thread at a time: a block barrier has nothing to wait for
static inline void __syncthreads() {}
