// psd_fp64.cu -- plain FP64 CUDA-core PSD kernels.
//
// Restates src/utils/fourier.cpp:25-52 in double precision as a direct DFT
// whose twiddle for (j, k) is exp(-2 pi i ((j k) mod L) / L), kept in shared
// memory.  Three uses:
//   * psd_fp64_filter: the plain FP64 filter (the comparator of the
//     tensor-core path): one candidate per thread, bins k = 1..L/2 in order,
//     stopping at the first bin above the bound;
//   * psd_recheck: exact verdict for the tensor core's "unsure" candidates;
//   * psd_fp64_values: every bin of a batch (signatures and tests).
#include "gp_internal.h"

namespace gp {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ void load_twiddles(double* cs, double* sn, int L) {
    const double two_pi = 6.283185307179586476925286766559;
    for (int m = threadIdx.x; m < L; m += blockDim.x) {
        double s, c;
        sincospi(2.0 * (double)m / (double)L, &s, &c);
        cs[m] = c;
        sn[m] = s;
        (void)two_pi;
    }
}

// Stages a block's rows (blockDim x L bytes) into shared memory with
// coalesced loads; returns the row of this thread.
__device__ __forceinline__ const int8_t* stage_rows(const int8_t* seqs, int64_t n, int L, int8_t* srows) {
    const int64_t row0 = (int64_t)blockIdx.x * blockDim.x;
    int64_t rows = n - row0;
    if (rows > blockDim.x) rows = blockDim.x;
    const int64_t bytes = rows * L;
    const int8_t* src = seqs + row0 * L;
    for (int64_t i = threadIdx.x; i < bytes; i += blockDim.x) srows[i] = src[i];
    __syncthreads();
    return srows + (int64_t)threadIdx.x * L;
}

__device__ __forceinline__ bool fp64_pass(const int8_t* x, int L, const double* cs, const double* sn, double thr) {
    const int H = L / 2;
    for (int k = 1; k <= H; ++k) {
        double re = 0.0, im = 0.0;
        int m = 0;
        for (int j = 0; j < L; ++j) {
            const double v = (double)x[j];
            re = fma(v, cs[m], re);
            im = fma(-v, sn[m], im);
            m += k;
            if (m >= L) m -= L;
        }
        if (re * re + im * im > thr) return false;
    }
    return true;
}

__global__ void __launch_bounds__(kBlock) psd_fp64_filter_kernel(PsdF64Args a) {
    extern __shared__ double sh64[];
    double* cs = sh64;
    double* sn = sh64 + a.L;
    int8_t* srows = reinterpret_cast<int8_t*>(sn + a.L);
    load_twiddles(cs, sn, a.L);
    const int8_t* x = stage_rows(a.seqs, a.n, a.L, srows);
    const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = row < a.n;
    const bool pass = valid && fp64_pass(x, a.L, cs, sn, a.thr);
    const uint32_t bits = __ballot_sync(0xFFFFFFFFu, pass);
    const int64_t word = row >> 5;
    if ((threadIdx.x & 31) == 0 && word < a.mask_words) a.mask[word] = bits;
}

__global__ void __launch_bounds__(kBlock) psd_recheck_kernel(const int8_t* seqs, int L, double thr,
                                                             const uint32_t* unsure,
                                                             const unsigned long long* unsure_count, int64_t cap,
                                                             uint32_t* mask) {
    extern __shared__ double sh64[];
    double* cs = sh64;
    double* sn = sh64 + L;
    load_twiddles(cs, sn, L);
    __syncthreads();
    int64_t cnt = (int64_t)*unsure_count;
    if (cnt > cap) cnt = cap;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t row = unsure[i];
        if (!fp64_pass(seqs + (int64_t)row * L, L, cs, sn, thr)) atomicAnd(&mask[row >> 5], ~(1u << (row & 31)));
    }
}

__global__ void __launch_bounds__(kBlock) psd_values_kernel(const int8_t* seqs, int64_t n, int L, double* out) {
    extern __shared__ double sh64[];
    double* cs = sh64;
    double* sn = sh64 + L;
    int8_t* srows = reinterpret_cast<int8_t*>(sn + L);
    load_twiddles(cs, sn, L);
    const int8_t* x = stage_rows(seqs, n, L, srows);
    const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    for (int k = 0; k < L; ++k) {
        double re = 0.0, im = 0.0;
        int m = 0;
        for (int j = 0; j < L; ++j) {
            const double v = (double)x[j];
            re = fma(v, cs[m], re);
            im = fma(-v, sn[m], im);
            m += k;
            if (m >= L) m -= L;
        }
        out[row * L + k] = re * re + im * im;
    }
}

}  // namespace

cudaError_t launch_psd_fp64(const PsdF64Args& a, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    const int64_t blocks = (a.n + kBlock - 1) / kBlock;
    const size_t smem = 2 * sizeof(double) * a.L + (size_t)kBlock * a.L + 16;
    cudaError_t e = cudaFuncSetAttribute(psd_fp64_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    psd_fp64_filter_kernel<<<(unsigned)blocks, kBlock, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_psd_recheck(const int8_t* seqs, int L, double thr, const uint32_t* unsure,
                               const unsigned long long* unsure_count, int64_t cap, uint32_t* mask,
                               cudaStream_t st) {
    if (cap <= 0) return cudaSuccess;
    int64_t blocks = (cap + kBlock - 1) / kBlock;
    if (blocks > 4096) blocks = 4096;
    const size_t smem = 2 * sizeof(double) * L;
    psd_recheck_kernel<<<(unsigned)blocks, kBlock, smem, st>>>(seqs, L, thr, unsure, unsure_count, cap, mask);
    return cudaGetLastError();
}

cudaError_t launch_psd_fp64_values(const int8_t* seqs, int64_t n, int L, double* out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const int64_t blocks = (n + kBlock - 1) / kBlock;
    const size_t smem = 2 * sizeof(double) * L + (size_t)kBlock * L + 16;
    cudaError_t e = cudaFuncSetAttribute(psd_values_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    psd_values_kernel<<<(unsigned)blocks, kBlock, smem, st>>>(seqs, n, L, out);
    return cudaGetLastError();
}

}  // namespace gp
