// k_smul.cu — dispatch of the constant-time variable-base ladder (ladder.cuh,
// one instantiation per block size in k_ladder.cu) by the run-time block
// size knob.  The fixed-base kernels are in k_encrypt.cu.
#include "internal.h"
#include "ladder.cuh"

namespace ft {

// ------------------------------------------------------------ launchers

static int g_ladder_nt = 384; // tables half in TMEM: the fastest on GB300

int ladder_block() { return g_ladder_nt; }

int set_ladder_block(int nt)
{
    if (nt != 128 && nt != 192 && nt != 224 && nt != 384 && nt != 448) return -1;
    g_ladder_nt = nt;
    return 0;
}

size_t ladder_wave_points()
{
    switch (g_ladder_nt) {
    case 128: return ladder_wave_128();
    case 192: return ladder_wave_192();
    case 224: return ladder_wave_224();
    case 448: return ladder_wave_448();
    default: return ladder_wave_384();
    }
}

cudaError_t smul_var(View v, size_t n, const uint8_t *sc, int sc_step, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    const uint4 *s4 = (const uint4 *)sc;
    switch (g_ladder_nt) {
    case 128: return ladder_launch_128(v.p, v.s, n, s4, sc_step, st);
    case 192: return ladder_launch_192(v.p, v.s, n, s4, sc_step, st);
    case 384: return ladder_launch_384(v.p, v.s, n, s4, sc_step, st);
    case 448: return ladder_launch_448(v.p, v.s, n, s4, sc_step, st);
    case 224: return ladder_launch_224(v.p, v.s, n, s4, sc_step, st);
    default: return ladder_launch_384(v.p, v.s, n, s4, sc_step, st);
    }
}

} // namespace ft
