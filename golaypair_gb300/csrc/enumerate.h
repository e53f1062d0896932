// enumerate.h -- arguments of the rank-window necklace enumerator.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "gp_internal.h"

namespace gp {

constexpr int kMaxDigitSum = 1023;

struct EnumArgs {
    int L;                     // sequence length
    int b;                     // bits per digit
    struct {
        uint64_t lo, hi;
    } maxpat;                  // digit k-1 at every position
    struct {
        uint64_t lo, hi;
    } plane[4];                // bit t of every digit
    const uint8_t* roles;      // [kMaxDigitSum+1]: bit0 = A row sum, bit1 = B row sum
    uint4* cur;                // per window: next word to visit (updated on exit)
    const uint4* end;          // per window: first word past the window
    int64_t nwin;
    uint4* words;              // out: candidate words
    uint8_t* out_roles;        // out: role bits per candidate
    unsigned long long* count; // out: candidates appended
    int64_t cap;               // hard capacity of words/out_roles
    int64_t soft_cap;          // stop when count reaches this
    unsigned long long* necklaces;  // out: necklaces visited
    int* incomplete;           // out: 1 if some window is unfinished
    int* status;
};

cudaError_t launch_enumerate(const EnumArgs& a, int num_sms, cudaStream_t st);

}  // namespace gp
