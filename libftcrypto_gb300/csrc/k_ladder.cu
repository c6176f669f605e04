// k_ladder.cu — one instantiation of the variable-base ladder kernel
// (ladder.cuh) per block size.  build.py compiles this file once per
// FT_LADDER_NT value into separate objects (in parallel); k_smul.cu picks
// the instantiation at run time (ftx_tune, FTX_TUNE_LADDER_BLOCK).
#include "internal.h"
#include "ladder.cuh"

#ifndef FT_LADDER_NT
#error "compile with -DFT_LADDER_NT=<block size>"
#endif

#define FT_CAT2(a, b) a##b
#define FT_CAT(a, b) FT_CAT2(a, b)

namespace ft {

cudaError_t FT_CAT(ladder_launch_, FT_LADDER_NT)(uint4 *p, size_t s, size_t n, const uint4 *sc, int sc_step,
                                                 cudaStream_t st)
{
    return launch_ladder<FT_LADDER_NT>(p, s, n, sc, sc_step, st);
}

size_t FT_CAT(ladder_wave_, FT_LADDER_NT)() { return ladder_wave<FT_LADDER_NT>(); }

} // namespace ft
