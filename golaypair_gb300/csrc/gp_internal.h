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
constexpr int kMaxTcK = 128;    // largest padded K of the tensor-core filter (L <= 127)
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
    // int8 rows: 1 = each row is read from the 4-byte boundary at or below
    // its first byte and sits s = (row * L) mod 4 columns along A, the bytes
    // of neighbouring rows masked; the image then carries tc_i8_wrap_rows(L)
    // wrapped twiddle rows past L (tc_i8_shifted(L) must hold)
    int i8_shift = 0;
    int* status;
    unsigned long long* trace;  // optional per-role cycle counters (diagnostics)
};

// Diagnostics counters written when PsdTcArgs::trace is set (summed over
// CTAs, in SM clock cycles, one sample per warp and tile).  conv_work
// includes conv_st (from the converted row to the end of the TMEM stores'
// wait); epi_work includes
// epi_ld (up to the hi accumulator columns landing in registers) and
// epi_tail (after the accumulator is released).
enum TcTrace {
    kTrConvWaitRaw = 0, kTrConvWaitA, kTrConvWork,
    kTrEpiWaitAcc, kTrEpiLd, kTrEpiWork,
    kTrMmaWaitA, kTrMmaWaitAcc, kTrMmaIssue,
    kTrProdWait, kTrProdIssue, kTrTiles, kTrConvFence, kTrMmaCommit,
    kTrConvSt, kTrEpiTail, kTrCount
};

// Builds the B-operand image (hi and lo twiddles) for length L, K = padded L.
// Rows j = L .. L + wrap - 1 of the sequence axis hold the twiddles of
// j - L (the DFT's period), for int8 rows loaded with a shift; every other
// row past L is zero.  Returns its size in bytes; writes it to out when
// out != nullptr.
size_t build_twiddle_image(int L, int K, void* out, int wrap = 0);
int tc_k_for_len(int L);               // padded K (multiple of 16, > L), or 0 if unsupported

// Shifted loads of int8 rows (PsdTcArgs::i8_shift).  A row of length L that
// starts s bytes past a 4-byte boundary (s = (row * L) mod 4: 0 when L is a
// multiple of 4, 0 or 2 when L = 2 mod 4, 0..3 when L is odd) is placed s
// columns along A; shifting a sequence multiplies X_k by a unit phase, so
// the PSD is unchanged when the twiddle rows continue periodically past L.
// Applies when K <= 64 and L + max s <= K.
bool tc_i8_shifted(int L);
int tc_i8_wrap_rows(int L);  // wrapped image rows for the shifted loads (max s), 0 if they do not apply

// Where twiddle row `nrow` (0..K-1), column j (0..K-1), part (0 hi, 1 lo)
// sits in the B image, as an index of fp16 elements.  The image is a 2K x K
// fp16 matrix (hi part at row nrow, lo part at row K + nrow) in the
// canonical no-swizzle K-major layout of 8 x 8 core matrices: core matrix
// (n/8, j/8) at byte (j/8) * (2K/8) * 128 + (n/8) * 128, row n%8 at +16,
// column j%8 at +2.
__host__ __device__ inline size_t tc_image_index(int nrow, int j, int part, int K) {
    const int n = nrow + part * K;
    return ((size_t)(j / 8) * (2 * K / 8) * 128 + (size_t)(n / 8) * 128 + (size_t)(n % 8) * 16 + (j % 8) * 2) / 2;
}

// Bin of twiddle row nrow: cosine rows 0..K/2-1 are bins 1..K/2, sine rows
// K/2..K-1 bins 1..K/2.  Bins above L/2 are zero rows, except the last
// cosine row (bin K/2 > L/2 since K > L): all ones, the row sum X_0.
// Returns 0 (zero row), 1 (cosine of *bin), 2 (sine of *bin) or 3 (ones).
__host__ __device__ inline int tc_row_kind(int nrow, int L, int K, int* bin) {
    const bool is_sin = nrow >= K / 2;
    *bin = (is_sin ? nrow - K / 2 : nrow) + 1;
    if (*bin <= L / 2) return is_sin ? 2 : 1;
    return (!is_sin && nrow == K / 2 - 1) ? 3 : 0;
}
bool tc_packed_supported(int L, int b);  // packed-word input with b bits per digit
float tc_err_coef(int K);              // |X| error per unit of sum|x|

cudaError_t launch_psd_tc(const PsdTcArgs& a, int num_sms, cudaStream_t st);

// Several jobs' tensor-core filters (packed words, lengths up to 63) in one
// launch: each CTA serves one job for its whole life, with that job's
// one-job kernel body; CTAs are shared out in proportion to the jobs' tile
// counts read on the device.  Every job as for launch_psd_tc (n = its
// capacity, n_dev its count), one status word for all.
constexpr int kMaxTcJobs = 8;
constexpr int kMaxMultiK = 64;  // largest padded K of a multi-job launch
struct PsdTcMultiArgs {
    PsdTcArgs job[kMaxTcJobs];
    int njobs;
    int grid_per_sm;  // CTAs per SM (0 = as many as fit)
};
cudaError_t launch_psd_tc_multi(const PsdTcMultiArgs& a, int num_sms, cudaStream_t st);
// True when a multi-job launch takes packed rows of length L with b bits per
// digit (padded K at most kMaxMultiK).
bool tc_multi_supported(int L, int b);

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

// The same recheck for several jobs in one launch (one grid row per job).
struct RecheckJob {
    RowSrc src;
    const double* tw;
    double thr;
    const uint32_t* unsure;
    const unsigned long long* unsure_count;
    int64_t cap;
    uint32_t* mask;
};
struct RecheckMultiArgs {
    RecheckJob job[8];
    int njobs;
};
cudaError_t launch_psd_recheck_multi(const RecheckMultiArgs& a, int num_sms, cudaStream_t st);

// Exact FP64 PSD values (all L bins) of rows 0..n-1 (testing)
cudaError_t launch_psd_fp64_values(const RowSrc& src, const double* tw, int64_t n, double* out, cudaStream_t st);

}  // namespace gp
