// psd_fp64.cu -- plain FP64 CUDA-core PSD kernels.
//
// Restates src/utils/fourier.cpp:25-52 in double precision as a direct DFT
// whose twiddle for (j, k) is exp(-2 pi i ((j k) mod L) / L), read from a
// table kept in shared memory.  Three uses:
//   * psd_fp64_filter: the plain FP64 filter (the comparator of the
//     tensor-core path): one candidate per thread, bins k = 1..L/2 in order,
//     stopping at the first bin above the bound;
//   * psd_recheck: exact verdict for the tensor core's "unsure" candidates,
//     one warp per candidate (lanes split the bins);
//   * psd_fp64_values: every bin of a batch (tests).
#include <cmath>

#include "gp_device.cuh"
#include "rows.cuh"

namespace gp {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ void load_tw(double2* stw, const double* tw, int L) {
    for (int m = threadIdx.x; m < L; m += blockDim.x) stw[m] = make_double2(tw[2 * m], tw[2 * m + 1]);
}

__device__ __forceinline__ double bin_power(const int8_t* x, int L, int k, const double2* tw) {
    double re = 0.0, im = 0.0;
    int m = 0;
    for (int j = 0; j < L; ++j) {
        const double v = (double)x[j];
        const double2 w = tw[m];
        re = fma(v, w.x, re);
        im = fma(-v, w.y, im);
        m += k;
        if (m >= L) m -= L;
    }
    return re * re + im * im;
}

__global__ void __launch_bounds__(kBlock) psd_fp64_filter_kernel(PsdF64Args a) {
    extern __shared__ double2 sh_tw[];
    const int L = a.src.L;
    int8_t* srows = reinterpret_cast<int8_t*>(sh_tw + L);
    load_tw(sh_tw, a.tw, L);
    const int64_t row0 = (int64_t)blockIdx.x * blockDim.x;
    int64_t rows = a.n - row0;
    if (rows > blockDim.x) rows = blockDim.x;
    // stage this block's rows (coalesced)
    if (a.src.seqs) {
        const int8_t* src = a.src.seqs + row0 * L;
        for (int64_t i = threadIdx.x; i < rows * L; i += blockDim.x) srows[i] = src[i];
    } else {
        for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) decode_row(a.src, row0 + r, srows + r * L);
    }
    __syncthreads();
    const int64_t row = row0 + threadIdx.x;
    bool pass = false;
    if (row < a.n) {
        const int8_t* x = srows + (int64_t)threadIdx.x * L;
        pass = true;
        for (int k = 1; k <= L / 2; ++k)
            if (bin_power(x, L, k, sh_tw) > a.thr) {
                pass = false;
                break;
            }
    }
    const uint32_t bits = __ballot_sync(0xFFFFFFFFu, pass);
    const int64_t word = row >> 5;
    if ((threadIdx.x & 31) == 0 && word < a.mask_words) a.mask[word] = bits;
}

// one warp per unsure row; lane l computes bins l+1, l+33, ...
__device__ __forceinline__ void recheck_rows(const RowSrc& src, const double* tw, double thr, const uint32_t* unsure,
                                             const unsigned long long* unsure_count, int64_t cap, uint32_t* mask,
                                             double2* sh_tw) {
    const int L = src.L;
    int8_t* xs = reinterpret_cast<int8_t*>(sh_tw + L) + (threadIdx.x >> 5) * kMaxLen;
    load_tw(sh_tw, tw, L);
    __syncthreads();
    int64_t cnt = (int64_t)*unsure_count;
    if (cnt > cap) cnt = cap;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < cnt; i += warps) {
        const uint32_t row = unsure[i];
        if (src.seqs) {
            for (int j = lane; j < L; j += 32) xs[j] = src.seqs[(int64_t)row * L + j];
        } else if (lane == 0) {
            decode_row(src, row, xs);
        }
        __syncwarp();
        bool fail = false;
        for (int k = lane + 1; k <= L / 2; k += 32) fail |= bin_power(xs, L, k, sh_tw) > thr;
        fail = __any_sync(0xFFFFFFFFu, fail);
        if (fail && lane == 0) atomicAnd(&mask[row >> 5], ~(1u << (row & 31)));
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kBlock) psd_recheck_kernel(RowSrc src, const double* tw, double thr,
                                                             const uint32_t* unsure,
                                                             const unsigned long long* unsure_count, int64_t cap,
                                                             uint32_t* mask) {
    extern __shared__ double2 sh_tw[];
    recheck_rows(src, tw, thr, unsure, unsure_count, cap, mask, sh_tw);
}

// every job's unsure rows in one launch: grid row y serves job y
__global__ void __launch_bounds__(kBlock) psd_recheck_multi_kernel(RecheckMultiArgs a) {
    extern __shared__ double2 sh_tw[];
    const RecheckJob& j = a.job[blockIdx.y];
    recheck_rows(j.src, j.tw, j.thr, j.unsure, j.unsure_count, j.cap, j.mask, sh_tw);
}

__global__ void __launch_bounds__(kBlock) psd_values_kernel(RowSrc src, const double* tw, int64_t n, double* out) {
    extern __shared__ double2 sh_tw[];
    const int L = src.L;
    int8_t* xs = reinterpret_cast<int8_t*>(sh_tw + L) + (int64_t)threadIdx.x * L;
    load_tw(sh_tw, tw, L);
    __syncthreads();
    const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    decode_row(src, row, xs);
    for (int k = 0; k < L; ++k) out[row * L + k] = bin_power(xs, L, k, sh_tw);
}

}  // namespace

void build_twiddle64(int L, double* out) {
    for (int m = 0; m < L; ++m) {
        const long double ang = 6.283185307179586476925286766559L * (long double)m / (long double)L;
        out[2 * m] = (double)std::cos(ang);
        out[2 * m + 1] = (double)std::sin(ang);
    }
}

cudaError_t launch_psd_fp64(const PsdF64Args& a, cudaStream_t st) {
    if (a.n == 0) return cudaSuccess;
    const int64_t blocks = (a.n + kBlock - 1) / kBlock;
    const size_t smem = sizeof(double2) * a.src.L + (size_t)kBlock * a.src.L + 16;
    cudaError_t e =
        cudaFuncSetAttribute(psd_fp64_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    psd_fp64_filter_kernel<<<(unsigned)blocks, kBlock, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_psd_recheck(const RowSrc& src, const double* tw, double thr, const uint32_t* unsure,
                               const unsigned long long* unsure_count, int64_t cap, uint32_t* mask, int num_sms,
                               cudaStream_t st) {
    if (cap <= 0) return cudaSuccess;
    int64_t blocks = (cap + (kBlock / 32) - 1) / (kBlock / 32);
    if (blocks > (int64_t)num_sms * 8) blocks = (int64_t)num_sms * 8;
    const size_t smem = sizeof(double2) * src.L + (size_t)(kBlock / 32) * kMaxLen;
    cudaError_t e = cudaFuncSetAttribute(psd_recheck_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    psd_recheck_kernel<<<(unsigned)blocks, kBlock, smem, st>>>(src, tw, thr, unsure, unsure_count, cap, mask);
    return cudaGetLastError();
}

cudaError_t launch_psd_recheck_multi(const RecheckMultiArgs& a, int num_sms, cudaStream_t st) {
    if (a.njobs <= 0) return cudaSuccess;
    int maxL = 1;
    int64_t maxcap = 0;
    for (int j = 0; j < a.njobs; ++j) {
        maxL = a.job[j].src.L > maxL ? a.job[j].src.L : maxL;
        maxcap = a.job[j].cap > maxcap ? a.job[j].cap : maxcap;
    }
    if (maxcap <= 0) return cudaSuccess;
    int64_t blocks = (maxcap + (kBlock / 32) - 1) / (kBlock / 32);
    // per job as many blocks as its own launch would take: blocks of a job
    // with fewer rows end at once
    if (blocks > (int64_t)num_sms * 8) blocks = (int64_t)num_sms * 8;
    const size_t smem = sizeof(double2) * maxL + (size_t)(kBlock / 32) * kMaxLen;
    cudaError_t e =
        cudaFuncSetAttribute(psd_recheck_multi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    psd_recheck_multi_kernel<<<dim3((unsigned)blocks, (unsigned)a.njobs), kBlock, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_psd_fp64_values(const RowSrc& src, const double* tw, int64_t n, double* out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const int64_t blocks = (n + kBlock - 1) / kBlock;
    const size_t smem = sizeof(double2) * src.L + (size_t)kBlock * src.L + 16;
    cudaError_t e = cudaFuncSetAttribute(psd_values_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    psd_values_kernel<<<(unsigned)blocks, kBlock, smem, st>>>(src, tw, n, out);
    return cudaGetLastError();
}

}  // namespace gp
