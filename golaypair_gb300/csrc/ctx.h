// ctx.h -- the context behind gp_ctx: device, streams, grow-only device
// buffers, cached twiddle images.  Host-side runtime, not public.
#pragma once
#include <cstdarg>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/golaypair_gb300.h"
#include "gp_internal.h"

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    // Grows to at least `bytes` (contents not preserved).  false on failure.
    bool ensure(size_t bytes) {
        if (bytes <= cap) return true;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = bytes < 256 ? 256 : bytes;
        if (cudaMalloc(&p, want) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        cap = want;
        return true;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

struct HostPinned {
    void* p = nullptr;
    size_t cap = 0;
    HostPinned() = default;
    HostPinned(const HostPinned&) = delete;
    HostPinned& operator=(const HostPinned&) = delete;
    ~HostPinned() { release(); }
    bool ensure(size_t bytes) {
        if (bytes <= cap) return true;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        if (cudaMallocHost(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        cap = bytes;
        return true;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// An NVTX range over one stage call, named for the entry point: the stages
// show on a profiler's timeline (no cost without a tool attached).
struct StageRange {
    explicit StageRange(const char* name) { nvtxRangePushA(name); }
    ~StageRange() { nvtxRangePop(); }
    StageRange(const StageRange&) = delete;
    StageRange& operator=(const StageRange&) = delete;
};

// entries of the spectral pruning table (values 0 .. kPruneTab - 1; orders
// whose bound 2n - paf is larger are not pruned)
constexpr int kPruneTab = 4096;

struct gp_ctx {
    int device = 0;
    int num_sms = 0;
    int out_format = 0;  // GP_FORMAT_TEXT or GP_FORMAT_BINARY (generation files)
    int spectral_prune = 0;  // gp_set_spectral_prune
    DevBuf prune_tab;        // uint8_t[kPruneTab]: bit 0 square, bit 1 Eisenstein norm
    cudaStream_t s_comp = nullptr;
    cudaStream_t s_copy = nullptr;
    static constexpr int kCopyStreams = 4;   // host->device copies of a chunk are split over these
    cudaStream_t s_copies[kCopyStreams] = {};
    cudaEvent_t ev_part[kCopyStreams] = {};
    cudaEvent_t ev_h2d[2] = {nullptr, nullptr};
    cudaEvent_t ev_done[2] = {nullptr, nullptr};
    std::string err;
    std::mutex err_mu;
    // status word and counters (device)
    DevBuf status;          // int
    DevBuf counts;          // unsigned long long [8]
    HostPinned h_counts;    // mirror of counts, per chunk
    HostPinned h_ux;        // uncompression: record counts of the two sides
    // PSD filter staging
    DevBuf seq_buf[2];
    DevBuf mask_buf[2];
    DevBuf unsure_buf[2];
    std::map<int, DevBuf> twiddles;    // tensor-core B images, by 4 L + wrapped rows
    std::map<int, DevBuf> twiddles64;  // FP64 (cos, sin) tables, by L
    // optional CUDA-event timing of the main filter kernel (profiling)
    bool timing = false;
    bool trace_on = false;  // per-role cycle counters of the tensor-core filter
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timed;
    void time_begin(cudaStream_t st, cudaEvent_t* b) {
        *b = nullptr;
        if (!timing) return;
        cudaEventCreate(b);
        cudaEventRecord(*b, st);
    }
    void time_end(cudaStream_t st, cudaEvent_t b) {
        if (!timing || !b) return;
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, st);
        timed.emplace_back(b, e);
    }
    // generic scratch arenas used by the stage pipelines
    DevBuf scratch[16];
    // grow-only scratch of the uncompression stage (kept across pairs: a
    // cudaFree per pair would synchronise the device every pair)
    DevBuf ux[66];
    HostPinned hscratch[4];
    // batched generation: one stream per job branch, fork/join events
    static constexpr int kJobStreams = 8;
    cudaStream_t s_jobs[kJobStreams] = {};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[kJobStreams] = {};
    bool ensure_job_streams();
    // tuned settings of batched generation and of the sort, by workload key
    std::map<std::string, std::vector<int64_t>> tuned;

    int fail(int code, const char* fmt, ...) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        std::lock_guard<std::mutex> lock(err_mu);  // host threads of one call may fail together
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what) {
        return fail(GP_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }
    // device twiddle image for length L (tensor-core filter)
    // tensor-core B image of length L: with the wrapped rows of shifted int8
    // loads when int8_rows and the length takes them (*shift set to 1)
    const void* twiddle_image(int L, bool int8_rows = false, int* shift = nullptr);
    // Multi-job tensor-core filter of device batches (packed words) followed
    // by the FP64 recheck of every job's unsure rows: two launches on st for
    // up to eight jobs, each job's tiles at its own padded K.  Per job as
    // enqueue_filter_dev; unsure counts must be zero.
    int enqueue_filter_multi(const gp::RowSrc* src, const int64_t* cap, const unsigned long long* const* n_dev,
                             const int* order, const int* paf, uint32_t* const* d_mask, uint32_t* const* d_unsure,
                             unsigned long long* const* d_ucount, int njobs, int grid_per_sm, cudaStream_t st);
    // device FP64 twiddle table for length L
    const double* twiddle64(int L);
    // Enqueues the PSD filter of a device batch (int8 rows or packed words)
    // on st: mask bit = pass; TC mode rechecks its unsure rows in FP64.
    int enqueue_filter(const gp::RowSrc& src, int64_t n, int order, int paf, int mode, uint32_t* d_mask,
                       uint32_t* d_unsure, unsigned long long* d_ucount, cudaStream_t st);
    // TC-mode filter of a device batch whose row count is read on the device
    // (*n_dev, at most cap rows): nothing here depends on the count, so the
    // sequence can be captured in a CUDA graph.  *d_ucount must be zero.
    int enqueue_filter_dev(const gp::RowSrc& src, int64_t cap, const unsigned long long* n_dev, int order, int paf,
                           uint32_t* d_mask, uint32_t* d_unsure, unsigned long long* d_ucount, int grid_per_sm,
                           cudaStream_t st);
    // reads the kernel status word; resets it; returns a GP code
    int check_status(const char* what);
};

#define GP_CUDA_TRY(ctx, expr)                                  \
    do {                                                        \
        cudaError_t _e = (expr);                                \
        if (_e != cudaSuccess) return (ctx)->cuda_fail(_e, #expr); \
    } while (0)
