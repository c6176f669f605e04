// points.cuh — structure-of-arrays point storage in HBM.
//
// An array of n points is 8 planes of 16-byte words (uint4), plane stride
// `s` elements (s >= n):
//   plane 0,1: X words 0-3, 4-7     plane 4,5: Z words 0-3, 4-7
//   plane 2,3: Y words 0-3, 4-7     plane 6,7: T words 0-3, 4-7
// Thread i reads point i with eight 16-byte loads; a warp's load of one plane
// is 512 contiguous bytes.  128 bytes per point, the algorithmic minimum for
// an extended point (the reference stores 160-byte AoS ge25519_p3 structs).
#pragma once
#include "ge.cuh"
#include "u4.cuh"

#define FT_PLANES 8


FT_DEV void ld_p3(ge_p3 &r, const uint4 *__restrict__ p, size_t s, size_t i)
{
    uint4 w[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) w[k] = p[k * s + i];
    fe_from_u4(r.X, w[0], w[1]);
    fe_from_u4(r.Y, w[2], w[3]);
    fe_from_u4(r.Z, w[4], w[5]);
    fe_from_u4(r.T, w[6], w[7]);
}

FT_DEV void st_p3(uint4 *__restrict__ p, size_t s, size_t i, const ge_p3 &r)
{
    p[0 * s + i] = u4_lo(r.X);
    p[1 * s + i] = u4_hi(r.X);
    p[2 * s + i] = u4_lo(r.Y);
    p[3 * s + i] = u4_hi(r.Y);
    p[4 * s + i] = u4_lo(r.Z);
    p[5 * s + i] = u4_hi(r.Z);
    p[6 * s + i] = u4_lo(r.T);
    p[7 * s + i] = u4_hi(r.T);
}

// warp shuffle of a whole point
FT_DEV void shfl_down_p3(ge_p3 &o, const ge_p3 &v, int delta)
{
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        o.X.v[k] = __shfl_down_sync(0xffffffffu, v.X.v[k], delta);
        o.Y.v[k] = __shfl_down_sync(0xffffffffu, v.Y.v[k], delta);
        o.Z.v[k] = __shfl_down_sync(0xffffffffu, v.Z.v[k], delta);
        o.T.v[k] = __shfl_down_sync(0xffffffffu, v.T.v[k], delta);
    }
}

FT_DEV void shfl_up_p3(ge_p3 &o, const ge_p3 &v, int delta)
{
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        o.X.v[k] = __shfl_up_sync(0xffffffffu, v.X.v[k], delta);
        o.Y.v[k] = __shfl_up_sync(0xffffffffu, v.Y.v[k], delta);
        o.Z.v[k] = __shfl_up_sync(0xffffffffu, v.Z.v[k], delta);
        o.T.v[k] = __shfl_up_sync(0xffffffffu, v.T.v[k], delta);
    }
}

FT_DEV void shfl_idx_p3(ge_p3 &o, const ge_p3 &v, int lane)
{
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        o.X.v[k] = __shfl_sync(0xffffffffu, v.X.v[k], lane);
        o.Y.v[k] = __shfl_sync(0xffffffffu, v.Y.v[k], lane);
        o.Z.v[k] = __shfl_sync(0xffffffffu, v.Z.v[k], lane);
        o.T.v[k] = __shfl_sync(0xffffffffu, v.T.v[k], lane);
    }
}

// shared-memory staging of one point per slot, stored as 8 uint4
FT_DEV void sm_st_p3(uint4 *sm, int slot, const ge_p3 &r)
{
    uint4 *q = sm + 8 * slot;
    q[0] = u4_lo(r.X); q[1] = u4_hi(r.X); q[2] = u4_lo(r.Y); q[3] = u4_hi(r.Y);
    q[4] = u4_lo(r.Z); q[5] = u4_hi(r.Z); q[6] = u4_lo(r.T); q[7] = u4_hi(r.T);
}

FT_DEV void sm_ld_p3(ge_p3 &r, const uint4 *sm, int slot)
{
    const uint4 *q = sm + 8 * slot;
    fe_from_u4(r.X, q[0], q[1]);
    fe_from_u4(r.Y, q[2], q[3]);
    fe_from_u4(r.Z, q[4], q[5]);
    fe_from_u4(r.T, q[6], q[7]);
}

// grid-stride loop bounds in size_t
#define FT_GRID_LOOP(i, n) \
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (size_t)blockDim.x * gridDim.x)
