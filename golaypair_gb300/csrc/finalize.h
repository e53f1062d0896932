// finalize.h -- exact FP64 recheck + canonical check + signature records.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "gp_internal.h"

namespace gp {

struct FinalizeArgs {
    RowSrc src;                 // candidates (packed words)
    const uint8_t* roles;       // per candidate role bits (bit0 A, bit1 B), or nullptr
    uint8_t fixed_role;         // role bits when roles == nullptr
    const uint32_t* idx;        // candidate rows to finalize
    const unsigned long long* n_idx;
    int64_t idx_cap;
    const double* tw;           // FP64 twiddles
    double thr;                 // 2n - paf + 0.001
    int bound;                  // 2n - paf (inverted signatures)
    int invert_roles;           // bit r set: role r writes bound - rint(psd)
    int check_canonical;
    const int16_t* units;       // units mod L (affine group multipliers)
    int n_units;
    // outputs
    uint4* rec_words;
    uint8_t* rec_role;
    uint16_t* rec_sig;          // (L-1) per record
    uint32_t* rec_src;          // optional: candidate row of each record
    unsigned long long* rec_count;
    int64_t rec_cap;
    unsigned long long* psd_pass;
    int* status;
    // optional spectral pruning (nullptr = off): prune_tab[m] bit 0 = m is a
    // square, bit 1 = m is a norm a^2 - ab + b^2 of an Eisenstein integer,
    // for 0 <= m <= bound.  A candidate is dropped when bound - p(L/2) (even
    // L) is not a square, or bound - p(L/3) (L divisible by 3) not a norm:
    // no complementary partner can exist (p_A(k) + p_B(k) = bound exactly).
    const uint8_t* prune_tab = nullptr;
};

// Lists the set bits of mask[0 .. n) (n = min(n, *n_dev) when n_dev is set).
cudaError_t launch_mask_to_list(const uint32_t* mask, int64_t n, uint32_t* out, unsigned long long* count,
                                int64_t cap, int* status, int num_sms, cudaStream_t st,
                                const unsigned long long* n_dev = nullptr);
cudaError_t launch_finalize(const FinalizeArgs& a, int64_t max_rows, int num_sms, cudaStream_t st);

// The same two steps for several jobs in one launch each (grid row y = job y).
constexpr int kMaxMultiJobs = 8;
struct ListJob {
    const uint32_t* mask;
    int64_t n;                          // rows (capacity), or min(n, *n_dev)
    const unsigned long long* n_dev;
    uint32_t* out;
    unsigned long long* count;
    int64_t cap;
};
struct ListMultiArgs {
    ListJob job[kMaxMultiJobs];
    int njobs;
    int* status;
};
struct FinalizeMultiArgs {
    FinalizeArgs job[kMaxMultiJobs];
    int njobs;
};
cudaError_t launch_mask_to_list_multi(const ListMultiArgs& a, int num_sms, cudaStream_t st);
// max_rows[j]: the most rows job j can list (its index capacity)
cudaError_t launch_finalize_multi(const FinalizeMultiArgs& a, const int64_t* max_rows, int num_sms,
                                  cudaStream_t st);

}  // namespace gp
