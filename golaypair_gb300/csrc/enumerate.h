// enumerate.h -- arguments of the rank-window necklace enumerator.
//
// One launch enumerates the windows of up to kMaxEnumJobs jobs (orders /
// compressions of different lengths): every window carries its job, and each
// job has its own digit layout, row-sum table and output buffer.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "gp_internal.h"

namespace gp {

constexpr int kMaxDigitSum = 1023;
constexpr int kMaxEnumJobs = 8;
// Steps between a lane's checks of its job's candidate count against the
// soft capacity (a step is a block of up to k^2 words; see enumerate.cu).
constexpr int kCapCheck = 2;
constexpr int kEnumQueue = 264;  // candidates a warp queues in shared memory (written out from 232; static shared memory stays under 48 KB)

struct U128p {
    uint64_t lo, hi;
};

struct EnumJob {
    int L;                     // sequence length
    int b;                     // bits per digit
    U128p maxpat;              // digit k-1 at every position
    U128p plane[4];            // bit t of every digit
    uint4* words;              // out: candidate words
    uint8_t* out_roles;        // out: role bits per candidate
    unsigned long long* count; // out: candidates appended
    int64_t cap;               // hard capacity of words / out_roles
    int64_t soft_cap;          // stop when count reaches this
    unsigned long long* necklaces;  // out: necklaces visited
};

struct EnumArgs {
    const EnumJob* jobs;       // device array of njobs jobs
    int njobs;
    const uint8_t* roles;      // [njobs][kMaxDigitSum+1]: bit0 = A row sum, bit1 = B row sum
    uint4* cur;                // per window: next word to visit (updated on exit)
    const uint4* end;          // per window: first word past the window
    const uint8_t* win_job;    // per window: its job
    int64_t nwin;
    unsigned long long* next_win;  // window handout counter (zero before the launch)
    int* incomplete;           // out: 1 if some window is unfinished
    int* status;
    int narrow;                // 1: every job's word fits 63 bits (b * L <= 63): the 64-bit kernel
};

// variant 0: unrestricted registers; 1: 32 registers, full occupancy
cudaError_t launch_enumerate(const EnumArgs& a, int num_sms, cudaStream_t st, int variant = 0);

}  // namespace gp
