// rows.cuh -- packed candidate words.
//
// A candidate of length L over an alphabet of k values {-c, -c+2, ..., c}
// (the reference's alphabets, src/utils/golay.cpp:60-75, are all of this
// form) is stored as one 128-bit word: digit j (value (v + c) / 2) in bits
// [b(L-1-j), b(L-j)), b = bits per digit.  Position 0 is the most
// significant digit, so the numeric order of words is the lexicographic
// order of sequences, which is the order the reference enumerates them in.
#pragma once
#include <cstdint>

#include "gp_internal.h"

namespace gp {

struct u128w {
    uint64_t lo, hi;
};

__host__ __device__ __forceinline__ int word_digit(uint64_t lo, uint64_t hi, int b, int L, int j) {
    const int pos = b * (L - 1 - j);  // lowest bit of digit j
    const uint64_t m = (1ull << b) - 1ull;
    if (pos >= 64) return (int)((hi >> (pos - 64)) & m);
    uint64_t v = lo >> pos;
    if (pos + b > 64 && pos > 0) v |= hi << (64 - pos);
    return (int)(v & m);
}

// Writes the row's L values as int8.
__device__ __forceinline__ void decode_row(const RowSrc& s, int64_t row, int8_t* out) {
    if (s.seqs) {
        for (int j = 0; j < s.L; ++j) out[j] = s.seqs[row * s.L + j];
        return;
    }
    const uint4 w = s.words[row];
    const uint64_t lo = ((uint64_t)w.y << 32) | w.x;
    const uint64_t hi = ((uint64_t)w.w << 32) | w.z;
    for (int j = 0; j < s.L; ++j) out[j] = (int8_t)(2 * word_digit(lo, hi, s.pack_bits, s.L, j) - s.alpha_c);
}

}  // namespace gp
