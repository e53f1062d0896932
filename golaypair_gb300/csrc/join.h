// join.h -- device-resident signature join (join.cu).
#pragma once
#include <cstdint>
#include <utility>
#include <vector>

#include "ctx.h"

namespace gp {

// One side of the join: n records in device memory (packed words and
// signatures of L-1 values each).
struct JoinSide {
    const uint4* words;
    const uint16_t* sig;
    int64_t n;
};

// Pairs (row in A, row in B) whose signature strings are equal and whose
// PAF vectors add up to `target` at every shift 1..L/2; unordered.
int device_join(gp_ctx* c, const JoinSide& A, const JoinSide& B, int L, int pack_bits, int alpha_c, int target,
                std::vector<std::pair<uint32_t, uint32_t>>& matches);

}  // namespace gp
