// windows.h — window count of the small-scalar ladder (smul_ladder_u32),
// shared by the device code and the host side that records work items.
//
// In signed radix 2^w, k is written with m digits in [-2^(w-1), 2^(w-1))
// by adding the bias sum_{i<m} 2^(w-1) * 2^(w i) and reading w-bit digits
// minus 2^(w-1); the digits are exact when k + bias < 2^(w m).  For k <
// 2^bits the ladder takes the smallest such m (nine windows of width 4 for
// any 32-bit k, three for k < 2^10).
#pragma once

constexpr unsigned long long u32_ladder_bias(int w, int m)
{
    unsigned long long b = 0;
    for (int i = 0; i < m; ++i) b += (1ull << (w - 1)) << (w * i);
    return b;
}

constexpr int u32_ladder_windows(unsigned bits, int w = 4)
{
    int m = 1;
    while (m * w < 62 && (1ull << (w * m)) - u32_ladder_bias(w, m) < (1ull << bits)) ++m;
    return m;
}

static_assert(u32_ladder_windows(32) == 9 && u32_ladder_windows(10) == 3 && u32_ladder_windows(7) == 3 &&
                  u32_ladder_windows(10, 3) == 4 && u32_ladder_windows(10, 2) == 6,
              "window counts");

// The radix-32 fixed-base comb (enc_comb.cuh): ENC_ROWS rows of ENC_ENTRIES
// entries (j+1) * 32^row * Q, and the rows a scalar below 2^bits needs
// (bits <= 256): the smallest d with a + sum_{i<d} 16 * 32^i < 32^d for every
// a < 2^bits, i.e. 15 * 32^d + 16 >= 31 * 2^bits.
constexpr int ENC_ROWS = 52, ENC_ENTRIES = 16;

constexpr int enc_digits(unsigned bits)
{
    int d = 1;
    // 5d >= bits + 2 always suffices; 5d = bits + 1 only when 2^bits <= 16
    while (5 * d < (int)bits + 2 && !(5 * d == (int)bits + 1 && bits <= 4)) ++d;
    return d;
}
static_assert(enc_digits(256) == 52 && enc_digits(253) == 51 && enc_digits(64) == 14 && enc_digits(8) == 2 &&
                  enc_digits(4) == 1 && enc_digits(3) == 1 && enc_digits(5) == 2,
              "comb rows");
