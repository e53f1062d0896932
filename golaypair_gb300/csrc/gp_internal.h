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
    const int8_t* seqs;      // n x L, row-major (int8 input), or nullptr
    const uint4* words;      // n packed words (packed input), or nullptr
    int pack_bits;           // packed: bits per digit (1..4)
    int alpha_c;             // packed: value = 2*digit - alpha_c (also bounds |value|)
    int64_t n;               // rows (or the capacity when n_dev is set)
    const unsigned long long* n_dev = nullptr;  // optional: row count read on the device, min(n, *n_dev)
    int grid_per_sm = 0;     // CTAs per SM (0 = as many as fit)
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
    unsigned long long* trace;  // optional per-role cycle counters (diagnostics)
};

// Diagnostics counters written when PsdTcArgs::trace is set (summed over
// CTAs, in SM clock cycles, one sample per warp and tile).
enum TcTrace {
    kTrConvWaitRaw = 0, kTrConvWaitA, kTrConvWork,
    kTrEpiWaitAcc, kTrEpiWaitStash, kTrEpiWork,
    kTrMmaWaitA, kTrMmaWaitAcc, kTrMmaIssue,
    kTrProdWait, kTrProdIssue, kTrTiles, kTrConvFence, kTrMmaCommit, kTrCount
};

// Builds the B-operand image (hi tile, lo tile) for length L, K = padded L.
// Returns its size in bytes; writes it to out when out != nullptr.
size_t build_twiddle_image(int L, int K, void* out);
int tc_k_for_len(int L);               // padded K (multiple of 16), or 0 if unsupported
bool tc_packed_supported(int L, int b);  // packed-word input with b bits per digit
float tc_err_coef(int K);              // |X| error per unit of sum|x|

cudaError_t launch_psd_tc(const PsdTcArgs& a, int num_sms, cudaStream_t st);

// Where the FP64 kernels read candidate rows: int8 rows or packed words.
struct RowSrc {
    const int8_t* seqs;
    const uint4* words;
    int L;
    int pack_bits;
    int alpha_c;
};

// FP64 twiddle table: tw[m] = (cos, sin)(2 pi m / L), m = 0..L-1
void build_twiddle64(int L, double* out /* 2L doubles */);

struct PsdF64Args {
    RowSrc src;
    const double* tw;
    int64_t n;
    double thr;
    uint32_t* mask;
    int64_t mask_words;
};
cudaError_t launch_psd_fp64(const PsdF64Args& a, cudaStream_t st);

// FP64 recheck of the unsure list (one warp per row): clears the mask bit of
// every unsure candidate that fails the exact filter.
cudaError_t launch_psd_recheck(const RowSrc& src, const double* tw, double thr, const uint32_t* unsure,
                               const unsigned long long* unsure_count, int64_t cap, uint32_t* mask,
                               int num_sms, cudaStream_t st);

// Exact FP64 PSD values (all L bins) of rows 0..n-1 (testing)
cudaError_t launch_psd_fp64_values(const RowSrc& src, const double* tw, int64_t n, double* out, cudaStream_t st);

}  // namespace gp
