// gp_internal.h -- declarations shared by the kernels (.cu) and the host
// runtime behind the C ABI.  Not part of the public interface.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

// Kernel status word values (device side).  0 = ok.
#define GP_KSTATUS_TIMEOUT_BASE 1000  // + site id
#define GP_KSTATUS_OVERFLOW 2000      // an output list ran out of room

namespace gp {

constexpr int kTileM = 128;     // candidates per tensor-core tile (TMEM lanes)
constexpr int kMaxTcK = 128;    // longest sequence the tensor-core filter takes
constexpr int kMaxLen = 512;    // longest sequence any kernel takes

// ------------------------------------------------------------ PSD filter
struct PsdTcArgs {
    const int8_t* seqs;      // n x L, row-major
    int64_t n;
    int L;
    const void* bimage;      // twiddles: hi tile then lo tile, UMMA smem image
    float thr;               // T = 2n - paf + 0.001
    float guard_cfg;         // configured guard band (absolute)
    float err_coef;          // per-row |X| error bound = S_row * err_coef
    uint32_t* mask;          // ceil(n/32) words; bit = sure pass or unsure
    int64_t mask_words;
    uint32_t* unsure;        // indices of unsure candidates (chunk-local)
    unsigned long long* unsure_count;
    int64_t unsure_cap;
    float* psd_out;          // optional n x (K/2) PSD values
    int* status;
};

// Builds the B-operand image (hi tile, lo tile) for length L, K = padded L.
// Returns its size in bytes; writes it to out when out != nullptr.
size_t build_twiddle_image(int L, int K, void* out);
int tc_k_for_len(int L);               // padded K (multiple of 16), or 0 if unsupported
float tc_err_coef(int K);              // |X| error per unit of sum|x|

cudaError_t launch_psd_tc(const PsdTcArgs& a, int num_sms, cudaStream_t st);

struct PsdF64Args {
    const int8_t* seqs;
    int64_t n;
    int L;
    double thr;
    uint32_t* mask;
    int64_t mask_words;
};
cudaError_t launch_psd_fp64(const PsdF64Args& a, cudaStream_t st);

// FP64 recheck of the unsure list: clears the mask bit of every unsure
// candidate that fails the exact filter.
cudaError_t launch_psd_recheck(const int8_t* seqs, int L, double thr, const uint32_t* unsure,
                               const unsigned long long* unsure_count, int64_t cap, uint32_t* mask,
                               cudaStream_t st);

// Exact FP64 PSD values (all L bins) for a list of rows (testing/signatures)
cudaError_t launch_psd_fp64_values(const int8_t* seqs, int64_t n, int L, double* out, cudaStream_t st);

}  // namespace gp
