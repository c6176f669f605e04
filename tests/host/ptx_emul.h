// ptx_emul.h — C stand-ins for the PTX carry-chain primitives of
// libftcrypto_gb300/csrc/ptx.cuh, so the device field/group code can be
// compiled with g++ and checked against the oracle on a machine without a
// GPU.  TEST HARNESS ONLY (tests/host/devcode_host.cpp); never part of the
// shipped library.
#pragma once
#include <stdint.h>

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
