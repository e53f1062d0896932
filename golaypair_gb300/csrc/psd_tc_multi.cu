// psd_tc_multi.cu -- the tensor-core PSD filter over several jobs in one
// launch (the batch engine's one-launch-per-iteration mode).
//
// Each CTA serves one job for its whole life and runs that job's one-job
// body (psd_tc_body.cuh) at the job's own padded K and packing, over the
// tiles first, first + stride, ... of the job.  The CTAs are shared out at
// the start of the launch, from the jobs' row counts on the device: one CTA
// per job that has rows, the rest in proportion to the jobs' work (rounded
// down), what rounding leaves to the job with the most work.  A tile's work
// is taken as K + 32 (the one-job kernel's time per tile on GB300 fits
// c (K + 35) for packed words at K = 32 and 48).  Every CTA computes the
// same split.  Per-job constants (length, packing, bound,
// twiddles) are then fixed for the CTA, so its loop is the one-job kernel's
// loop: no per-tile dispatch.
#include "psd_tc_body.cuh"

namespace gp {

namespace {

struct MultiSlot {
    int job, first, stride;
};

// tc_k_for_len on the device: L + 1 rounded up to 16
__device__ __forceinline__ int tc_k_for_len_dev(int L) { return (L + 16) / 16 * 16; }

__device__ MultiSlot multi_slot(const PsdTcMultiArgs& m) {
    int64_t work[kMaxTcJobs];
    int64_t total = 0;
    int nonempty = 0, big = 0;
    for (int j = 0; j < m.njobs; ++j) {
        int64_t n = m.job[j].n;
        if (m.job[j].n_dev) {
            const int64_t nd = (int64_t)*reinterpret_cast<const volatile unsigned long long*>(m.job[j].n_dev);
            if (nd < n) n = nd;
        }
        work[j] = (n + kTileM - 1) / kTileM * (tc_k_for_len_dev(m.job[j].L) + 32);
        total += work[j];
        nonempty += work[j] > 0;
        if (work[j] > work[big]) big = j;
    }
    MultiSlot s{-1, 0, 1};
    const int G = (int)gridDim.x;
    if (total == 0 || G < nonempty) return s;  // the launch gives at least one CTA per job
    const int64_t spare = G - nonempty;
    int c = (int)blockIdx.x, used = 0;
    int g[kMaxTcJobs];
    for (int j = 0; j < m.njobs; ++j) {
        g[j] = work[j] ? 1 + (int)(spare * work[j] / total) : 0;
        used += g[j];
    }
    g[big] += G - used;
    for (int j = 0; j < m.njobs; ++j) {
        if (c < g[j]) {
            s.job = j;
            s.first = c;
            s.stride = g[j];
            break;
        }
        c -= g[j];
    }
    return s;
}

// Calls f(std::integral_constant<int, K>) for the job's padded K (16..KMAX).
template <int KMAX, class F>
__device__ __forceinline__ void with_k(int K, F&& f) {
    if (K == 16) {
        f(std::integral_constant<int, 16>{});
    } else if (K == 32) {
        f(std::integral_constant<int, 32>{});
    } else if (K == 48) {
        f(std::integral_constant<int, 48>{});
    } else if constexpr (KMAX >= 64) {
        if (K == 64) f(std::integral_constant<int, 64>{});
    }
}

// KMAX 48: two CTAs per SM (every job's TMEM share is 256 columns);
// KMAX 64: one CTA per SM.
template <int KMAX>
__global__ void __launch_bounds__(kThreads, KMAX <= 48 ? 2 : 1) psd_tc_multi_kernel(PsdTcMultiArgs m, SmemLayout lay) {
    const MultiSlot s = multi_slot(m);
    if (s.job < 0) return;
    const PsdTcArgs& a = m.job[s.job];
    const int bits = a.pack_bits;
    with_k<KMAX>(tc_k_for_len_dev(a.L), [&](auto kc) {
        constexpr int K = decltype(kc)::value;
        switch (bits) {
            case 1: tc_body<K, 1, false, false>(a, lay, s.first, s.stride); break;
            case 2: tc_body<K, 2, false, false>(a, lay, s.first, s.stride); break;
            case 3:
                if constexpr (K <= 48) tc_body<K, 3, false, false>(a, lay, s.first, s.stride);
                break;
            default:
                if constexpr (K <= 48) tc_body<K, 4, false, false>(a, lay, s.first, s.stride);
                break;
        }
    });
}

// The layout of the largest job's one-job kernel, with the barrier region
// sized for any K's stage counts and at most one (KMAX 64) or two CTAs per SM.
template <int KMAX>
SmemLayout multi_layout() {
    SmemLayout s;
    uint32_t off = 0;
    s.b_off = off;
    off += TcCfg<KMAX>::B_BYTES;
    off = (off + 1023) & ~1023u;
    s.lut_off = off;
    off += kLutBytes;
    s.bar_off = off;
    off += (2 * kMaxRawStages + 2 * 4 + 2 * 4 + 2) * 8;  // AS, NACC <= 4 for every K
    s.misc_off = off;
    off += 16;
    off = (off + 127) & ~127u;
    s.raw_stride = (uint32_t)((kTileM * 16 + kRawSlack + 127) & ~127);
    s.raw_off = off;
    const uint32_t budget = (KMAX <= 48 ? kSmemBudget2Cta : kSmemBudget1Cta) - 1024;
    int st = budget > off ? (int)((budget - off) / s.raw_stride) : 0;
    if (st > kMaxRawStages) st = kMaxRawStages;
    if (st < 2) st = 2;
    s.raw_stages = (uint32_t)st;
    off += st * s.raw_stride;
    s.total = off + 1024;
    // TMEM: two CTAs of 256 columns, or one of up to 512
    const uint32_t floor = KMAX <= 48 ? 96 * 1024 : 116 * 1024;
    if (s.total < floor) s.total = floor;
    return s;
}

template <int KMAX>
cudaError_t launch_multi(const PsdTcMultiArgs& a, int num_sms, cudaStream_t st) {
    const SmemLayout lay = multi_layout<KMAX>();
    auto kern = psd_tc_multi_kernel<KMAX>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.total);
    if (e != cudaSuccess) return e;
    int64_t cap_tiles = 0;
    for (int j = 0; j < a.njobs; ++j) cap_tiles += (a.job[j].n + kTileM - 1) / kTileM;
    if (cap_tiles == 0) return cudaSuccess;
    const int fit = KMAX <= 48 ? 2 : 1;
    const int per_sm = a.grid_per_sm > 0 && a.grid_per_sm < fit ? a.grid_per_sm : fit;
    int64_t grid = (int64_t)num_sms * per_sm;
    if (grid > cap_tiles) grid = cap_tiles;
    if (grid < a.njobs) grid = a.njobs;  // one CTA per job at least
    kern<<<(unsigned)grid, kThreads, lay.total, st>>>(a, lay);
    return cudaGetLastError();
}

}  // namespace

bool tc_multi_supported(int L, int b) { return tc_packed_supported(L, b) && tc_k_for_len(L) <= kMaxMultiK; }

cudaError_t launch_psd_tc_multi(const PsdTcMultiArgs& a, int num_sms, cudaStream_t st) {
    if (a.njobs < 1 || a.njobs > kMaxTcJobs) return cudaErrorInvalidValue;
    int kmax = 0;
    for (int j = 0; j < a.njobs; ++j) {
        const PsdTcArgs& q = a.job[j];
        if (!q.words || q.psd_out || q.trace || !tc_multi_supported(q.L, q.pack_bits) || q.n < 0 ||
            q.n >= (int64_t(1) << 31))
            return cudaErrorInvalidValue;
        const int K = tc_k_for_len(q.L);
        kmax = K > kmax ? K : kmax;
    }
    return kmax <= 48 ? launch_multi<48>(a, num_sms, st) : launch_multi<64>(a, num_sms, st);
}

}  // namespace gp
