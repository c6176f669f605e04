// u4.cuh — a field element as two 16-byte words (the unit of every point and
// table access).
#pragma once
#include "fe.cuh"

FT_DEV void fe_from_u4(fe &f, const uint4 &a, const uint4 &b)
{
    f.v[0] = a.x; f.v[1] = a.y; f.v[2] = a.z; f.v[3] = a.w;
    f.v[4] = b.x; f.v[5] = b.y; f.v[6] = b.z; f.v[7] = b.w;
}

FT_DEV uint4 u4_lo(const fe &f) { return make_uint4(f.v[0], f.v[1], f.v[2], f.v[3]); }
FT_DEV uint4 u4_hi(const fe &f) { return make_uint4(f.v[4], f.v[5], f.v[6], f.v[7]); }
