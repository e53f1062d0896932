// capi_psd.cu -- context management and the batched PSD filter entry points.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ctx.h"
#include "gp_device.cuh"

namespace {

constexpr int64_t kChunkRows = int64_t(1) << 25;  // rows per pipelined chunk (multiple of 128)

double threshold(int order, int paf) { return 2.0 * order - paf + 0.001; }

// configured guard band: 1e-3 * 2n (absolute PSD units)
float guard_band(int order) { return (float)(2e-3 * order); }

}  // namespace

const void* gp_ctx::twiddle_image(int L, bool int8_rows, int* shift) {
    const bool sh = int8_rows && gp::tc_i8_shifted(L);
    if (shift) *shift = sh ? 1 : 0;
    const int wrap = sh ? gp::tc_i8_wrap_rows(L) : 0;
    const int key = 4 * L + wrap;
    auto it = twiddles.find(key);
    if (it != twiddles.end()) return it->second.p;
    const int K = gp::tc_k_for_len(L);
    if (!K) return nullptr;
    const size_t bytes = gp::build_twiddle_image(L, K, nullptr, wrap);
    std::vector<uint8_t> img(bytes);
    gp::build_twiddle_image(L, K, img.data(), wrap);
    DevBuf& b = twiddles[key];
    if (!b.ensure(bytes)) return nullptr;
    if (cudaMemcpy(b.p, img.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return b.p;
}

const double* gp_ctx::twiddle64(int L) {
    auto it = twiddles64.find(L);
    if (it != twiddles64.end()) return it->second.as<double>();
    std::vector<double> t(2 * (size_t)L);
    gp::build_twiddle64(L, t.data());
    DevBuf& b = twiddles64[L];
    if (!b.ensure(t.size() * 8)) return nullptr;
    if (cudaMemcpy(b.p, t.data(), t.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return b.as<double>();
}

int gp_ctx::enqueue_filter(const gp::RowSrc& src, int64_t n, int order, int paf, int mode, uint32_t* d_mask,
                           uint32_t* d_unsure, unsigned long long* d_ucount, cudaStream_t st) {
    const int L = src.L;
    const int64_t words = (n + 31) / 32;
    const double* tw = twiddle64(L);
    if (!tw) return fail(GP_ERR_NOMEM, "twiddle table");
    if (mode == GP_PSD_FP64) {
        gp::PsdF64Args a{src, tw, n, threshold(order, paf), d_mask, words};
        cudaEvent_t tb;
        time_begin(st, &tb);
        GP_CUDA_TRY(this, gp::launch_psd_fp64(a, st));
        time_end(st, tb);
        return GP_OK;
    }
    int shift = 0;
    const void* img = twiddle_image(L, src.seqs != nullptr, &shift);
    if (!img) return fail(GP_ERR_UNSUPPORTED, "tensor-core filter: unsupported length %d", L);
    if (src.words && !gp::tc_packed_supported(L, src.pack_bits))
        return fail(GP_ERR_UNSUPPORTED, "tensor-core filter: packed length %d x %d bits", L, src.pack_bits);
    GP_CUDA_TRY(this, cudaMemsetAsync(d_ucount, 0, sizeof(unsigned long long), st));
    gp::PsdTcArgs a;
    a.i8_shift = shift;
    a.seqs = src.seqs;
    a.words = src.words;
    a.pack_bits = src.pack_bits;
    a.alpha_c = src.alpha_c;
    a.n = n;
    a.L = L;
    a.bimage = img;
    a.thr = (float)threshold(order, paf);
    a.guard_cfg = guard_band(order);
    a.err_coef = gp::tc_err_coef(gp::tc_k_for_len(L));
    a.mask = d_mask;
    a.mask_words = words;
    a.unsure = d_unsure;
    a.unsure_count = d_ucount;
    a.unsure_cap = n;
    a.psd_out = nullptr;
    a.status = status.as<int>();
    a.trace = trace_on ? counts.as<unsigned long long>() + 16 : nullptr;
    cudaEvent_t tb;
    time_begin(st, &tb);
    GP_CUDA_TRY(this, gp::launch_psd_tc(a, num_sms, st));
    time_end(st, tb);
    GP_CUDA_TRY(this, gp::launch_psd_recheck(src, tw, threshold(order, paf), d_unsure, d_ucount, n, d_mask, num_sms, st));
    return GP_OK;
}

int gp_ctx::enqueue_filter_dev(const gp::RowSrc& src, int64_t cap, const unsigned long long* n_dev, int order,
                               int paf, uint32_t* d_mask, uint32_t* d_unsure, unsigned long long* d_ucount,
                               int grid_per_sm, cudaStream_t st) {
    const int L = src.L;
    const double* tw = twiddle64(L);
    int shift = 0;
    const void* img = twiddle_image(L, src.seqs != nullptr, &shift);
    if (!tw || !img) return fail(GP_ERR_UNSUPPORTED, "tensor-core filter: unsupported length %d", L);
    if (src.words && !gp::tc_packed_supported(L, src.pack_bits))
        return fail(GP_ERR_UNSUPPORTED, "tensor-core filter: packed length %d x %d bits", L, src.pack_bits);
    gp::PsdTcArgs a;
    a.i8_shift = shift;
    a.seqs = src.seqs;
    a.words = src.words;
    a.pack_bits = src.pack_bits;
    a.alpha_c = src.alpha_c;
    a.n = cap;
    a.n_dev = n_dev;
    a.grid_per_sm = grid_per_sm;
    a.L = L;
    a.bimage = img;
    a.thr = (float)threshold(order, paf);
    a.guard_cfg = guard_band(order);
    a.err_coef = gp::tc_err_coef(gp::tc_k_for_len(L));
    a.mask = d_mask;
    a.mask_words = (cap + 31) / 32;
    a.unsure = d_unsure;
    a.unsure_count = d_ucount;
    a.unsure_cap = cap;
    a.psd_out = nullptr;
    a.status = status.as<int>();
    a.trace = nullptr;
    GP_CUDA_TRY(this, gp::launch_psd_tc(a, num_sms, st));
    GP_CUDA_TRY(this, gp::launch_psd_recheck(src, tw, threshold(order, paf), d_unsure, d_ucount, cap, d_mask, num_sms, st));
    return GP_OK;
}

int gp_ctx::enqueue_filter_multi(const gp::RowSrc* src, const int64_t* cap, const unsigned long long* const* n_dev,
                                 const int* order, const int* paf, uint32_t* const* d_mask,
                                 uint32_t* const* d_unsure, unsigned long long* const* d_ucount, int njobs,
                                 int grid_per_sm, cudaStream_t st) {
    if (njobs < 1 || njobs > gp::kMaxTcJobs) return fail(GP_ERR_ARG, "multi-job filter: %d jobs", njobs);
    gp::PsdTcMultiArgs m{};
    gp::RecheckMultiArgs r{};
    m.njobs = r.njobs = njobs;
    m.grid_per_sm = grid_per_sm;
    for (int j = 0; j < njobs; ++j) {
        const int L = src[j].L;
        if (!src[j].words || !gp::tc_multi_supported(L, src[j].pack_bits))
            return fail(GP_ERR_UNSUPPORTED, "multi-job filter: length %d x %d bits", L, src[j].pack_bits);
        const double* tw = twiddle64(L);
        const void* img = twiddle_image(L);
        if (!tw || !img) return fail(GP_ERR_NOMEM, "multi-job filter: twiddle tables for length %d", L);
        // each job's arguments as enqueue_filter_dev forms them
        gp::PsdTcArgs& a = m.job[j];
        a.seqs = nullptr;
        a.words = src[j].words;
        a.pack_bits = src[j].pack_bits;
        a.alpha_c = src[j].alpha_c;
        a.n = cap[j];
        a.n_dev = n_dev[j];
        a.grid_per_sm = grid_per_sm;
        a.L = L;
        a.bimage = img;
        a.thr = (float)threshold(order[j], paf[j]);
        a.guard_cfg = guard_band(order[j]);
        a.err_coef = gp::tc_err_coef(gp::tc_k_for_len(L));
        a.mask = d_mask[j];
        a.mask_words = (cap[j] + 31) / 32;
        a.unsure = d_unsure[j];
        a.unsure_count = d_ucount[j];
        a.unsure_cap = cap[j];
        a.psd_out = nullptr;
        a.status = status.as<int>();
        a.trace = nullptr;
        gp::RecheckJob& w = r.job[j];
        w.src = src[j];
        w.tw = tw;
        w.thr = threshold(order[j], paf[j]);
        w.unsure = d_unsure[j];
        w.unsure_count = d_ucount[j];
        w.cap = cap[j];
        w.mask = d_mask[j];
    }
    GP_CUDA_TRY(this, gp::launch_psd_tc_multi(m, num_sms, st));
    GP_CUDA_TRY(this, gp::launch_psd_recheck_multi(r, num_sms, st));
    return GP_OK;
}

bool gp_ctx::ensure_job_streams() {
    if (ev_fork) return true;
    for (int i = 0; i < kJobStreams; ++i) {
        if (cudaStreamCreateWithFlags(&s_jobs[i], cudaStreamNonBlocking) != cudaSuccess) return false;
        if (cudaEventCreateWithFlags(&ev_join[i], cudaEventDisableTiming) != cudaSuccess) return false;
    }
    return cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming) == cudaSuccess;
}

namespace {

// One thread waits on an mbarrier that nothing arrives on.  The wait is the
// bounded loop of every pipeline kernel, with the caller's limit: it gives
// up, records its site in the status word and returns.
__global__ void wait_timeout_kernel(uint64_t limit_ns, int* status) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        gp::mbar_init(&bar, 1);
        gp::mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint64_t t0 = gp::globaltimer_ns();
        while (!gp::mbar_try_wait(&bar, 0)) {
            if (gp::globaltimer_ns() - t0 > limit_ns) {
                atomicCAS(status, 0, GP_KSTATUS_TIMEOUT_BASE + 99);
                break;
            }
        }
    }
}

}  // namespace

int gp_ctx::check_status(const char* what) {
    int st = 0;
    cudaError_t e = cudaMemcpy(&st, status.p, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (st == 0) return GP_OK;
    cudaMemset(status.p, 0, sizeof(int));
    if (st >= GP_KSTATUS_TIMEOUT_BASE && st < GP_KSTATUS_OVERFLOW)
        return fail(GP_ERR_TIMEOUT, "%s: device wait timed out at site %d", what, st - GP_KSTATUS_TIMEOUT_BASE);
    if (st == GP_KSTATUS_OVERFLOW) return fail(GP_ERR_OVERFLOW, "%s: device output list overflow", what);
    return fail(GP_ERR_CUDA, "%s: kernel status %d", what, st);
}

extern "C" {

int gp_debug_wait_timeout(gp_ctx* c, int64_t limit_ns) {
    if (!c || limit_ns < 0 || limit_ns > (int64_t)gp::kWaitTimeoutNs) return GP_ERR_ARG;
    cudaSetDevice(c->device);
    wait_timeout_kernel<<<1, 32, 0, c->s_comp>>>((uint64_t)limit_ns, c->status.as<int>());
    GP_CUDA_TRY(c, cudaGetLastError());
    GP_CUDA_TRY(c, cudaStreamSynchronize(c->s_comp));
    return c->check_status("gp_debug_wait_timeout");
}

int gp_ctx_create(gp_ctx** out, int device) {
    if (!out) return GP_ERR_ARG;
    *out = nullptr;
    gp_ctx* c = new gp_ctx();
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    int major = 0, minor = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return GP_ERR_CUDA;
    }
    if (major != 10 || minor != 3) {
        // kernels are built for sm_103a only
        delete c;
        return GP_ERR_UNSUPPORTED;
    }
    if (cudaStreamCreateWithFlags(&c->s_comp, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->s_copy, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return GP_ERR_CUDA;
    }
    for (int i = 0; i < 2; ++i) {
        cudaEventCreateWithFlags(&c->ev_h2d[i], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&c->ev_done[i], cudaEventDisableTiming);
    }
    for (int i = 0; i < gp_ctx::kCopyStreams; ++i) {
        if (cudaStreamCreateWithFlags(&c->s_copies[i], cudaStreamNonBlocking) != cudaSuccess) {
            delete c;
            return GP_ERR_CUDA;
        }
        cudaEventCreateWithFlags(&c->ev_part[i], cudaEventDisableTiming);
    }
    if (!c->status.ensure(sizeof(int)) || !c->counts.ensure(64 * sizeof(unsigned long long)) ||
        !c->h_counts.ensure(64 * sizeof(unsigned long long))) {
        delete c;
        return GP_ERR_NOMEM;
    }
    cudaMemset(c->status.p, 0, sizeof(int));
    cudaMemset(c->counts.p, 0, 64 * sizeof(unsigned long long));
    cudaDeviceSynchronize();
    *out = c;
    return GP_OK;
}

int gp_ctx_destroy(gp_ctx* c) {
    if (!c) return GP_OK;
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    c->status.release();
    c->counts.release();
    c->h_counts.release();
    for (int i = 0; i < 2; ++i) {
        c->seq_buf[i].release();
        c->mask_buf[i].release();
        c->unsure_buf[i].release();
        if (c->ev_h2d[i]) cudaEventDestroy(c->ev_h2d[i]);
        if (c->ev_done[i]) cudaEventDestroy(c->ev_done[i]);
    }
    for (auto& kv : c->twiddles) kv.second.release();
    for (auto& kv : c->twiddles64) kv.second.release();
    for (auto& b : c->scratch) b.release();
    for (auto& b : c->ux) b.release();
    for (auto& b : c->hscratch) b.release();
    if (c->s_comp) cudaStreamDestroy(c->s_comp);
    if (c->s_copy) cudaStreamDestroy(c->s_copy);
    for (int i = 0; i < gp_ctx::kCopyStreams; ++i) {
        if (c->s_copies[i]) cudaStreamDestroy(c->s_copies[i]);
        if (c->ev_part[i]) cudaEventDestroy(c->ev_part[i]);
    }
    for (int i = 0; i < gp_ctx::kJobStreams; ++i) {
        if (c->s_jobs[i]) cudaStreamDestroy(c->s_jobs[i]);
        if (c->ev_join[i]) cudaEventDestroy(c->ev_join[i]);
    }
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    delete c;
    return GP_OK;
}

const char* gp_last_error(const gp_ctx* c) { return c ? c->err.c_str() : "no context"; }

int gp_kernel_timing(gp_ctx* c, int enable) {
    if (!c) return GP_ERR_ARG;
    c->timing = enable != 0;
    return GP_OK;
}

int gp_debug_tc_trace(gp_ctx* c, int enable, uint64_t* out, int nout) {
    if (!c) return GP_ERR_ARG;
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    if (out && nout > 0) {
        unsigned long long h[gp::kTrCount];
        GP_CUDA_TRY(c, cudaMemcpy(h, c->counts.as<unsigned long long>() + 16, sizeof h, cudaMemcpyDeviceToHost));
        for (int i = 0; i < nout && i < gp::kTrCount; ++i) out[i] = h[i];
    }
    GP_CUDA_TRY(c, cudaMemset(c->counts.as<unsigned long long>() + 16, 0, sizeof(unsigned long long) * gp::kTrCount));
    c->trace_on = enable != 0;
    return GP_OK;
}

int gp_kernel_time(gp_ctx* c, double* total_ms, int64_t* launches) {
    if (!c) return GP_ERR_ARG;
    double tot = 0;
    int64_t n = 0;
    for (auto& pr : c->timed) {
        float ms = 0;
        if (cudaEventSynchronize(pr.second) == cudaSuccess && cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess) {
            tot += ms;
            ++n;
        }
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    c->timed.clear();
    if (total_ms) *total_ms = tot;
    if (launches) *launches = n;
    return GP_OK;
}

int gp_device_sm_count(const gp_ctx* c) { return c ? c->num_sms : 0; }

static gp::RowSrc int8_src(const int8_t* d, int L) {
    gp::RowSrc r;
    r.seqs = d;
    r.words = nullptr;
    r.L = L;
    r.pack_bits = 0;
    r.alpha_c = 0;
    return r;
}

// *out += number of set bits in w[0 .. nwords)
__global__ void popcount_add_kernel(const uint32_t* w, int64_t nwords, unsigned long long* out) {
    unsigned long long s = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nwords; i += (int64_t)gridDim.x * blockDim.x)
        s += (unsigned long long)__popc(w[i]);
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

constexpr int kPassCountSlot = 40;  // counts[]: passes of the current gp_psd_filter call

static int check_args(gp_ctx* c, int64_t n, int L, int mode) {
    if (!c) return GP_ERR_ARG;
    if (n < 0 || L < 1 || L > gp::kMaxLen) return c->fail(GP_ERR_ARG, "bad n=%lld or L=%d", (long long)n, L);
    if (mode != GP_PSD_FP64 && mode != GP_PSD_TC_GUARDED) return c->fail(GP_ERR_ARG, "bad mode %d", mode);
    if (mode == GP_PSD_TC_GUARDED && !gp::tc_k_for_len(L))
        return c->fail(GP_ERR_UNSUPPORTED, "tensor-core filter supports 2 <= L <= %d", gp::kMaxTcK - 1);
    return GP_OK;
}

int gp_psd_filter(gp_ctx* c, const int8_t* seqs, int64_t n, int L, int order, int paf, int mode,
                  uint32_t* pass_mask, gp_psd_stats* stats) {
    StageRange nvtx_range("gp_psd_filter");
    int rc = check_args(c, n, L, mode);
    if (rc) return rc;
    if (n > 0 && (!seqs || !pass_mask)) return c->fail(GP_ERR_ARG, "null buffer");
    cudaSetDevice(c->device);
    const int64_t chunk = std::min<int64_t>(kChunkRows, std::max<int64_t>(n, 1));
    for (int b = 0; b < 2; ++b) {
        if (!c->seq_buf[b].ensure((size_t)chunk * L + 16) || !c->mask_buf[b].ensure((size_t)(chunk + 31) / 32 * 4) ||
            !c->unsure_buf[b].ensure((size_t)chunk * 4))
            return c->fail(GP_ERR_NOMEM, "psd filter: device allocation failed");
    }
    auto* d_counts = c->counts.as<unsigned long long>();
    auto* h_counts = c->h_counts.as<unsigned long long>();
    const int64_t nchunks = (n + chunk - 1) / chunk;
    if (stats) GP_CUDA_TRY(c, cudaMemsetAsync(d_counts + kPassCountSlot, 0, sizeof(unsigned long long), c->s_comp));
    int64_t unsure_total = 0;
    for (int64_t ci = 0; ci < nchunks; ++ci) {
        const int b = (int)(ci & 1);
        const int64_t r0 = ci * chunk;
        const int64_t rows = std::min(chunk, n - r0);
        // the chunk's host->device copy is split over several copy streams
        // (several copy engines in flight); compute waits for all parts
        const size_t bytes = (size_t)rows * L;
        const size_t part = (bytes / gp_ctx::kCopyStreams + 4095) & ~size_t(4095);
        for (int q = 0; q < gp_ctx::kCopyStreams; ++q) {
            const size_t o = (size_t)q * part;
            if (o >= bytes) break;
            const size_t nb = std::min(part, bytes - o);
            if (ci >= 2) GP_CUDA_TRY(c, cudaStreamWaitEvent(c->s_copies[q], c->ev_done[b], 0));
            GP_CUDA_TRY(c, cudaMemcpyAsync(static_cast<uint8_t*>(c->seq_buf[b].p) + o,
                                           reinterpret_cast<const uint8_t*>(seqs) + r0 * L + o, nb,
                                           cudaMemcpyHostToDevice, c->s_copies[q]));
            GP_CUDA_TRY(c, cudaEventRecord(c->ev_part[q], c->s_copies[q]));
            GP_CUDA_TRY(c, cudaStreamWaitEvent(c->s_comp, c->ev_part[q], 0));
        }
        rc = c->enqueue_filter(int8_src(c->seq_buf[b].as<int8_t>(), L), rows, order, paf, mode,
                               c->mask_buf[b].as<uint32_t>(), c->unsure_buf[b].as<uint32_t>(), d_counts + b, c->s_comp);
        if (rc) return rc;
        GP_CUDA_TRY(c, cudaMemcpyAsync(pass_mask + r0 / 32, c->mask_buf[b].p, (size_t)(rows + 31) / 32 * 4,
                                       cudaMemcpyDeviceToHost, c->s_comp));
        if (stats) {
            const int64_t words = (rows + 31) / 32;
            const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((words + 255) / 256, (int64_t)c->num_sms * 4));
            popcount_add_kernel<<<(unsigned)blocks, 256, 0, c->s_comp>>>(c->mask_buf[b].as<uint32_t>(), words,
                                                                         d_counts + kPassCountSlot);
            GP_CUDA_TRY(c, cudaGetLastError());
        }
        if (mode == GP_PSD_TC_GUARDED)
            GP_CUDA_TRY(c, cudaMemcpyAsync(h_counts + 2 + ci % 62, d_counts + b, sizeof(unsigned long long),
                                           cudaMemcpyDeviceToHost, c->s_comp));
        GP_CUDA_TRY(c, cudaEventRecord(c->ev_done[b], c->s_comp));
        if (mode == GP_PSD_TC_GUARDED && (ci % 62) == 61) {
            GP_CUDA_TRY(c, cudaStreamSynchronize(c->s_comp));
            for (int k = 0; k < 62; ++k) unsure_total += (int64_t)h_counts[2 + k];
        }
    }
    GP_CUDA_TRY(c, cudaStreamSynchronize(c->s_comp));
    for (int q = 0; q < gp_ctx::kCopyStreams; ++q) GP_CUDA_TRY(c, cudaStreamSynchronize(c->s_copies[q]));
    if (mode == GP_PSD_TC_GUARDED)
        for (int64_t k = 0; k < nchunks % 62; ++k) unsure_total += (int64_t)h_counts[2 + k];
    rc = c->check_status("gp_psd_filter");
    if (rc) return rc;
    if (stats) {
        unsigned long long passes = 0;
        GP_CUDA_TRY(c, cudaMemcpy(&passes, d_counts + kPassCountSlot, sizeof passes, cudaMemcpyDeviceToHost));
        stats->n = n;
        stats->n_pass = (int64_t)passes;
        stats->n_unsure = unsure_total;
        stats->guard = guard_band(order);
        stats->err_coef = mode == GP_PSD_TC_GUARDED ? gp::tc_err_coef(gp::tc_k_for_len(L)) : 0.f;
    }
    return GP_OK;
}

int gp_psd_filter_device(gp_ctx* c, const int8_t* d_seqs, int64_t n, int L, int order, int paf, int mode,
                         uint32_t* d_mask, void* stream, gp_psd_stats* stats) {
    StageRange nvtx_range("gp_psd_filter_device");
    int rc = check_args(c, n, L, mode);
    if (rc) return rc;
    if (n >= (int64_t(1) << 31)) return c->fail(GP_ERR_ARG, "device batch too large (n < 2^31)");
    cudaSetDevice(c->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->s_comp;
    if (mode == GP_PSD_TC_GUARDED && !c->unsure_buf[0].ensure((size_t)std::max<int64_t>(n, 1) * 4))
        return c->fail(GP_ERR_NOMEM, "psd filter: device allocation failed");
    rc = c->enqueue_filter(int8_src(d_seqs, L), n, order, paf, mode, d_mask, c->unsure_buf[0].as<uint32_t>(),
                           c->counts.as<unsigned long long>(), st);
    if (rc) return rc;
    if (stats) {
        GP_CUDA_TRY(c, cudaStreamSynchronize(st));
        rc = c->check_status("gp_psd_filter_device");
        if (rc) return rc;
        unsigned long long* pc = c->counts.as<unsigned long long>() + kPassCountSlot;
        GP_CUDA_TRY(c, cudaMemsetAsync(pc, 0, sizeof(unsigned long long), st));
        const int64_t words = (n + 31) / 32;
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((words + 255) / 256, (int64_t)c->num_sms * 4));
        popcount_add_kernel<<<(unsigned)blocks, 256, 0, st>>>(d_mask, words, pc);
        GP_CUDA_TRY(c, cudaGetLastError());
        unsigned long long u = 0, passes = 0;
        GP_CUDA_TRY(c, cudaMemcpyAsync(&passes, pc, sizeof passes, cudaMemcpyDeviceToHost, st));
        GP_CUDA_TRY(c, cudaStreamSynchronize(st));
        GP_CUDA_TRY(c, cudaMemcpy(&u, c->counts.p, sizeof u, cudaMemcpyDeviceToHost));
        stats->n = n;
        stats->n_pass = (int64_t)passes;
        stats->n_unsure = mode == GP_PSD_TC_GUARDED ? (int64_t)u : 0;
        stats->guard = guard_band(order);
        stats->err_coef = mode == GP_PSD_TC_GUARDED ? gp::tc_err_coef(gp::tc_k_for_len(L)) : 0.f;
    }
    return GP_OK;
}

int gp_check(gp_ctx* c, void* stream) {
    if (!c) return GP_ERR_ARG;
    cudaSetDevice(c->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->s_comp;
    GP_CUDA_TRY(c, cudaStreamSynchronize(st));
    return c->check_status("gp_check");
}

int gp_psd_tc_values(gp_ctx* c, const int8_t* seqs, int64_t n, int L, float* out) {
    int rc = check_args(c, n, L, GP_PSD_TC_GUARDED);
    if (rc) return rc;
    if (n >= (int64_t(1) << 31)) return c->fail(GP_ERR_ARG, "batch too large");
    if (n == 0) return GP_OK;
    cudaSetDevice(c->device);
    const int K = gp::tc_k_for_len(L);
    DevBuf& ds = c->scratch[0];
    DevBuf& dm = c->scratch[1];
    DevBuf& du = c->scratch[2];
    DevBuf& dp = c->scratch[3];
    if (!ds.ensure((size_t)n * L + 16) || !dm.ensure((size_t)(n + 31) / 32 * 4) || !du.ensure((size_t)n * 4) ||
        !dp.ensure((size_t)n * (K / 2) * 4))
        return c->fail(GP_ERR_NOMEM, "allocation failed");
    GP_CUDA_TRY(c, cudaMemcpy(ds.p, seqs, (size_t)n * L, cudaMemcpyHostToDevice));
    int shift = 0;
    const void* img = c->twiddle_image(L, true, &shift);
    if (!img) return c->fail(GP_ERR_UNSUPPORTED, "length %d", L);
    GP_CUDA_TRY(c, cudaMemset(c->counts.p, 0, sizeof(unsigned long long)));
    gp::PsdTcArgs a;
    a.i8_shift = shift;
    a.seqs = ds.as<int8_t>();
    a.words = nullptr;
    a.pack_bits = 0;
    a.alpha_c = 0;
    a.n = n;
    a.L = L;
    a.bimage = img;
    a.thr = 1e30f;
    a.guard_cfg = 0.f;
    a.err_coef = 0.f;
    a.mask = dm.as<uint32_t>();
    a.mask_words = (n + 31) / 32;
    a.unsure = du.as<uint32_t>();
    a.unsure_count = c->counts.as<unsigned long long>();
    a.unsure_cap = n;
    a.psd_out = dp.as<float>();
    a.status = c->status.as<int>();
    a.trace = nullptr;
    GP_CUDA_TRY(c, gp::launch_psd_tc(a, c->num_sms, c->s_comp));
    GP_CUDA_TRY(c, cudaStreamSynchronize(c->s_comp));
    rc = c->check_status("gp_psd_tc_values");
    if (rc) return rc;
    std::vector<float> full((size_t)n * (K / 2));
    GP_CUDA_TRY(c, cudaMemcpy(full.data(), dp.p, full.size() * 4, cudaMemcpyDeviceToHost));
    const int H = L / 2;
    for (int64_t i = 0; i < n; ++i) std::memcpy(out + i * H, full.data() + i * (K / 2), (size_t)H * 4);
    return GP_OK;
}

int gp_psd_fp64_values(gp_ctx* c, const int8_t* seqs, int64_t n, int L, double* out) {
    int rc = check_args(c, n, L, GP_PSD_FP64);
    if (rc) return rc;
    if (n == 0) return GP_OK;
    cudaSetDevice(c->device);
    DevBuf& ds = c->scratch[0];
    DevBuf& dv = c->scratch[4];
    if (!ds.ensure((size_t)n * L + 16) || !dv.ensure((size_t)n * L * 8))
        return c->fail(GP_ERR_NOMEM, "allocation failed");
    GP_CUDA_TRY(c, cudaMemcpy(ds.p, seqs, (size_t)n * L, cudaMemcpyHostToDevice));
    const double* tw = c->twiddle64(L);
    if (!tw) return c->fail(GP_ERR_NOMEM, "twiddle table");
    GP_CUDA_TRY(c, gp::launch_psd_fp64_values(int8_src(ds.as<int8_t>(), L), tw, n, dv.as<double>(), c->s_comp));
    GP_CUDA_TRY(c, cudaStreamSynchronize(c->s_comp));
    GP_CUDA_TRY(c, cudaMemcpy(out, dv.p, (size_t)n * L * 8, cudaMemcpyDeviceToHost));
    return GP_OK;
}

}  // extern "C"
