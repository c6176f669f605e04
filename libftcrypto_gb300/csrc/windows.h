// windows.h — window count of the small-scalar ladder (smul_ladder_u32),
// shared by the device code and the host side that records work items.
//
// The signed radix-16 digits of k under the bias sum_{i<nwin} 8 * 16^i are
// exact when k + bias < 16^nwin.  For k < 2^bits, nwin = (bits + 1) / 4 + 1
// gives 16^nwin >= 2^(bits+2) while the bias stays below 16^nwin / 2; any
// 32-bit k takes nine windows.
#pragma once

constexpr int u32_ladder_windows(unsigned bits) { return (int)((bits + 1) / 4) + 1; }
static_assert(u32_ladder_windows(32) == 9 && u32_ladder_windows(10) == 3 && u32_ladder_windows(7) == 3,
              "window counts");
