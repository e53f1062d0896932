// noalloc.cu -- gp_psd_filter_noalloc: the batched tensor-core PSD filter
// for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory pool or allocator hooks, inside a real-time loop that
// forbids allocator calls, or on a device whose memory is fully reserved by
// its owner.  This entry point runs the same kernels as gp_psd_filter_device
// (psd_tc_kernel, then the FP64 recheck) but takes every working buffer it
// needs -- the unsure-row list and its counter, the kernel status word, the
// tensor-core twiddle image and the FP64 twiddle table -- from one fixed
// array in static device memory, g_noalloc_scratch, instead of allocating.
//
// Properties a caller must know:
//   * The array is a file-scope __device__ variable: every GPU that loads
//     this library holds kNoAllocScratchBytes of it until the process exits.
//   * Batches are limited to kNoAllocMaxRows rows (the unsure list must be
//     able to hold every row); larger n is rejected with GP_ERR_ARG.
//   * The first call on a device looks up the array's device address there
//     (cudaGetSymbolAddress) with that device current and keeps it for the
//     life of the process; make that first call before any stream capture.
//     A device reset (cudaDeviceReset) invalidates the kept address: do not
//     call the entry point on that device again in the same process.
//   * Every call shares the array and it keeps the last call's contents;
//     the call clears the counter and status words it relies on.  Calls that
//     overlap on the GPU (other streams, other threads) race on it.
//   * The call is synchronous: it reads the kernel status word on its own
//     stream and waits for that stream (a timed-out device wait returns
//     GP_ERR_TIMEOUT); it does not wait on the device's other streams.
#include <cmath>
#include <cstdio>
#include <mutex>

#include <cuda_fp16.h>

#include "../../include/golaypair_gb300.h"
#include "gp_internal.h"

namespace gp {
namespace {

constexpr int64_t kNoAllocMaxRows = int64_t(1) << 20;
constexpr size_t kImageBytes = 2 * (size_t)kMaxTcK * kMaxTcK * 2;  // hi + lo tiles at K = 128
constexpr size_t kTw64Bytes = 2 * (size_t)kMaxTcK * sizeof(double);
// layout of the scratch array (byte offsets, 256-aligned)
constexpr size_t kOffStatus = 0;                            // int status
constexpr size_t kOffCounter = 256;                         // unsigned long long unsure count
constexpr size_t kOffImage = 512;                           // tensor-core twiddle image
constexpr size_t kOffTw64 = kOffImage + kImageBytes;        // FP64 twiddle table
constexpr size_t kOffUnsure = kOffTw64 + kTw64Bytes;        // uint32 unsure rows
constexpr size_t kNoAllocScratchBytes = kOffUnsure + (size_t)kNoAllocMaxRows * 4;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Twiddles built on the device: the tensor-core image in the same canonical
// layout as build_twiddle_image (wrap: rows L .. L + wrap - 1 continue the
// period, for shifted int8 loads), and the FP64 (cos, sin) table.
__global__ void noalloc_twiddles_kernel(unsigned char* scratch, int L, int K, int wrap) {
    uint16_t* img = reinterpret_cast<uint16_t*>(scratch + kOffImage);
    double* tw = reinterpret_cast<double*>(scratch + kOffTw64);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < K * K; e += gridDim.x * blockDim.x) {
        const int nrow = e / K, j = e % K;
        int bin = 0;
        const int kind = tc_row_kind(nrow, L, K, &bin);
        double w = 0.0;
        if (kind != 0 && j < L + wrap) {
            const int m = (int)(((long long)(j % L) * bin) % L);
            double s, c;
            sincospi(2.0 * (double)m / (double)L, &s, &c);
            w = kind == 3 ? 1.0 : kind == 2 ? s : c;
        }
        const __half h = __double2half(w);
        const __half l = __double2half(w - (double)__half2float(h));
        img[tc_image_index(nrow, j, 0, K)] = __half_as_ushort(h);
        img[tc_image_index(nrow, j, 1, K)] = __half_as_ushort(l);
    }
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < L; m += gridDim.x * blockDim.x) {
        double s, c;
        sincospi(2.0 * (double)m / (double)L, &s, &c);
        tw[2 * m] = c;
        tw[2 * m + 1] = s;
    }
}

// per-device address of g_noalloc_scratch, looked up once per device
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};

int setup_device(int dev, unsigned char** addr, int* sms) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            fprintf(stderr, "gp_psd_filter_noalloc: cudaGetSymbolAddress failed on device %d: %s\n", dev,
                    cudaGetErrorString(e));
            return GP_ERR_CUDA;
        }
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GP_ERR_CUDA;
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
        g_num_sms[dev] = n;
    }
    *addr = g_scratch_addr[dev];
    *sms = g_num_sms[dev];
    return GP_OK;
}

}  // namespace
}  // namespace gp

extern "C" int gp_psd_filter_noalloc(const int8_t* d_seqs, int64_t n, int L, int order, int paf, uint32_t* d_pass_mask,
                                     void* stream) {
    using namespace gp;
    if (n < 0 || (n > 0 && (!d_seqs || !d_pass_mask))) return GP_ERR_ARG;
    if (n > kNoAllocMaxRows) {
        fprintf(stderr, "gp_psd_filter_noalloc: %lld rows exceed the fixed scratch limit of %lld rows\n",
                (long long)n, (long long)kNoAllocMaxRows);
        return GP_ERR_ARG;
    }
    const int K = tc_k_for_len(L);
    if (!K) return GP_ERR_UNSUPPORTED;
    if (n == 0) return GP_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GP_ERR_CUDA;
    unsigned char* s = nullptr;
    int sms = 0;
    int rc = setup_device(dev, &s, &sms);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // clear what the kernels count from zero; the rest is overwritten
    if (cudaMemsetAsync(s + kOffStatus, 0, 512, st) != cudaSuccess) return GP_ERR_CUDA;
    noalloc_twiddles_kernel<<<64, 256, 0, st>>>(s, L, K, tc_i8_wrap_rows(L));
    if (cudaGetLastError() != cudaSuccess) return GP_ERR_CUDA;
    const double thr = 2.0 * order - paf + 0.001;
    PsdTcArgs a;
    a.seqs = d_seqs;
    a.words = nullptr;
    a.pack_bits = 0;
    a.alpha_c = 0;
    a.n = n;
    a.L = L;
    a.bimage = s + kOffImage;
    a.i8_shift = tc_i8_shifted(L) ? 1 : 0;
    a.thr = (float)thr;
    a.guard_cfg = (float)(2e-3 * order);
    a.err_coef = tc_err_coef(K);
    a.mask = d_pass_mask;
    a.mask_words = (n + 31) / 32;
    a.unsure = reinterpret_cast<uint32_t*>(s + kOffUnsure);
    a.unsure_count = reinterpret_cast<unsigned long long*>(s + kOffCounter);
    a.unsure_cap = n;
    a.psd_out = nullptr;
    a.status = reinterpret_cast<int*>(s + kOffStatus);
    a.trace = nullptr;
    if (launch_psd_tc(a, sms, st) != cudaSuccess) return GP_ERR_CUDA;
    RowSrc src{d_seqs, nullptr, L, 0, 0};
    if (launch_psd_recheck(src, reinterpret_cast<const double*>(s + kOffTw64), thr, a.unsure, a.unsure_count, n,
                           d_pass_mask, sms, st) != cudaSuccess)
        return GP_ERR_CUDA;
    // the status word is read on the caller's stream: nothing here waits on
    // other streams of the device
    int status = 0;
    if (cudaMemcpyAsync(&status, s + kOffStatus, sizeof status, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return GP_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return GP_ERR_CUDA;
    if (status >= GP_KSTATUS_TIMEOUT_BASE && status < GP_KSTATUS_OVERFLOW) return GP_ERR_TIMEOUT;
    if (status) return GP_ERR_OVERFLOW;
    return GP_OK;
}
