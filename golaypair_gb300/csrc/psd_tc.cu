// psd_tc.cu -- guarded-FP32 tensor-core PSD filter (tcgen05 + TMEM + bulk copy).
//
// Restates src/utils/fourier.cpp:25-52 (FFTW c2c PSD, then reject if any
// psd[k] > 2n - paf + 0.001 for k = 1..L/2) as a batched dense contraction:
//
//   X[M=128 candidates x K] (fp16, exact small integers)
//     * W[K x N] (cos/sin twiddles, split hi + lo fp16, both accumulated into
//       one fp32 TMEM accumulator)   ->   re_k, im_k  ->  p_k = re^2 + im^2.
//
// Row n < N/2 of W is the cosine of bin n+1, row N/2 + n the sine of bin n+1;
// bins above L/2 are zero rows.  K = N = L rounded up to 16.
//
// Each candidate is classified against T = 2n - paf + 0.001 with a guard g
// (the configured band, widened per row to a rigorous bound on the fp32
// error): max p < T - g -> pass, max p > T + g -> reject, else "unsure",
// appended to a list that an FP64 kernel rechecks exactly.  The pass mask
// bit is set for pass and unsure; the recheck clears the failing unsure ones.
//
// Persistent kernel, one 128-candidate tile per step, warp roles:
//   warps 0-3  convert: int8 rows (staged by the bulk-copy engine) -> fp16
//              A tile in the UMMA canonical K-major layout, plus sum |x|
//   warps 4-7  epilogue: TMEM -> registers -> PSD max -> mask / unsure list
//   warp 8     producer: cp.async.bulk of each 128 x L byte tile
//   warp 9     MMA issuer (one lane) and TMEM owner
#include <cmath>
#include <cstring>
#include <vector>

#include "gp_device.cuh"

namespace gp {

namespace {

constexpr int kThreads = 320;
constexpr int kRawSlack = 64;

template <int K>
struct TcCfg {
    static constexpr int M = kTileM;
    static constexpr int N = K;
    static constexpr int KCH = K / 8;                  // core-matrix columns along K
    static constexpr int KSTEPS = K / 16;              // UMMA instructions per pass
    static constexpr int A_BYTES = M * K * 2;
    static constexpr int A_KSTRIDE = (M / 8) * 128;    // bytes between K-adjacent core matrices
    static constexpr int B_BYTES = N * K * 2;
    static constexpr int B_KSTRIDE = (N / 8) * 128;
    static constexpr int STAGES = K <= 64 ? 4 : 2;
    static constexpr int NACC = (256 / N) < 4 ? (256 / N) : 4;
    static constexpr int RING = STAGES + NACC;         // sum|x| stash slots
    static constexpr int TMEM_COLS = 256;
    static constexpr int MIN_BLOCKS = K <= 64 ? 2 : 1;
};

struct SmemLayout {
    uint32_t b_off, a_off, raw_off, raw_stride, stash_off, bar_off, misc_off, total;
};

template <int K>
SmemLayout smem_layout(int L) {
    using C = TcCfg<K>;
    SmemLayout s;
    uint32_t off = 0;
    s.b_off = off;
    off += 2 * C::B_BYTES;
    off = (off + 1023) & ~1023u;
    s.a_off = off;
    off += C::STAGES * C::A_BYTES;
    s.raw_stride = (uint32_t)((kTileM * L + kRawSlack + 127) & ~127);
    s.raw_off = off;
    off += C::STAGES * s.raw_stride;
    s.stash_off = off;
    off += C::RING * kTileM * 4;
    off = (off + 7) & ~7u;
    s.bar_off = off;
    off += (4 * C::STAGES + 2 * C::NACC + C::RING + 2) * 8;
    s.misc_off = off;
    off += 16;
    s.total = off + 1024;  // slack for the 1024-byte alignment of the base
    // At most two CTAs per SM: each holds 256 TMEM columns (512 per SM).
    if (s.total < 96 * 1024) s.total = 96 * 1024;
    return s;
}

template <int K, bool WRITE_PSD>
__global__ void __launch_bounds__(kThreads, TcCfg<K>::MIN_BLOCKS) psd_tc_kernel(PsdTcArgs a, SmemLayout lay) {
    using C = TcCfg<K>;
    extern __shared__ uint8_t smem_raw_base[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw_base) + 1023) & ~uintptr_t(1023));

    uint8_t* sB = smem + lay.b_off;
    uint8_t* sA = smem + lay.a_off;
    uint8_t* sRaw = smem + lay.raw_off;
    float* stash = reinterpret_cast<float*>(smem + lay.stash_off);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + lay.bar_off);
    uint64_t* raw_full = bars;
    uint64_t* raw_empty = bars + C::STAGES;
    uint64_t* a_full = bars + 2 * C::STAGES;
    uint64_t* a_empty = bars + 3 * C::STAGES;
    uint64_t* acc_full = bars + 4 * C::STAGES;
    uint64_t* acc_empty = acc_full + C::NACC;
    uint64_t* b_full = acc_empty + C::NACC;
    uint64_t* final_bar = b_full + 1;
    uint64_t* stash_full = final_bar + 1;  // RING barriers: sum|x| of a tile is written
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + lay.misc_off);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + lay.misc_off + 4);

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int L = a.L;
    const int64_t n = a.n;
    const int64_t ntiles = (n + kTileM - 1) / kTileM;
    const bool aligned = (reinterpret_cast<uintptr_t>(a.seqs) & 15) == 0;

    if (threadIdx.x == 0) {
        for (int i = 0; i < C::STAGES; ++i) {
            mbar_init(&raw_full[i], 1);
            mbar_init(&raw_empty[i], 4);
            mbar_init(&a_full[i], 4);
            mbar_init(&a_empty[i], 1);
        }
        for (int i = 0; i < C::NACC; ++i) {
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], 4);
        }
        mbar_init(b_full, 1);
        mbar_init(final_bar, 1);
        for (int i = 0; i < C::RING; ++i) mbar_init(&stash_full[i], 4);
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 9) {
        tmem_alloc(tmem_slot, C::TMEM_COLS);
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *reinterpret_cast<volatile uint32_t*>(tmem_slot);

    if (warp < 4) {
        // ------------------------------------------------ converters
        const int r = threadIdx.x;  // row of the tile
        uint32_t mlo[C::KCH], mhi[C::KCH];
#pragma unroll
        for (int c = 0; c < C::KCH; ++c) {
            int v = L - 8 * c;
            mlo[c] = v >= 4 ? 0xFFFFFFFFu : (v <= 0 ? 0u : ((1u << (8 * v)) - 1u));
            mhi[c] = v >= 8 ? 0xFFFFFFFFu : (v <= 4 ? 0u : ((1u << (8 * (v - 4))) - 1u));
        }
        int64_t it = 0;
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
            const int s = (int)(it % C::STAGES);
            const uint32_t ph = (uint32_t)((it / C::STAGES) & 1);
            if (!mbar_wait(&raw_full[s], ph, abort_flag, a.status, 1)) break;
            if (!mbar_wait(&a_empty[s], ph ^ 1u, abort_flag, a.status, 2)) break;
            uint8_t* A = sA + s * C::A_BYTES;
            const int64_t row = t * kTileM + r;
            const bool full_tile = aligned && (t + 1) * kTileM <= n;
            uint32_t sabs = 0;
            if (full_tile) {
                const uint8_t* raw = sRaw + s * lay.raw_stride;
                const int off = r * L;
#pragma unroll
                for (int c = 0; c < C::KCH; ++c) {
                    const int o = off + 8 * c;
                    const int base = o & ~3;
                    const uint32_t sh = (uint32_t)(o & 3) * 8u;
                    const uint32_t w0 = *reinterpret_cast<const uint32_t*>(raw + base);
                    const uint32_t w1 = *reinterpret_cast<const uint32_t*>(raw + base + 4);
                    const uint32_t w2 = *reinterpret_cast<const uint32_t*>(raw + base + 8);
                    const uint32_t lo = __funnelshift_r(w0, w1, sh) & mlo[c];
                    const uint32_t hi = __funnelshift_r(w1, w2, sh) & mhi[c];
                    sabs = __dp4a(__vabs4(lo), 0x01010101u, sabs);
                    sabs = __dp4a(__vabs4(hi), 0x01010101u, sabs);
                    uint4 h;
                    i8x4_to_h2x2(lo, h.x, h.y);
                    i8x4_to_h2x2(hi, h.z, h.w);
                    *reinterpret_cast<uint4*>(A + c * C::A_KSTRIDE + r * 16) = h;
                }
            } else {
                const bool valid = row < n;
                const int8_t* src = a.seqs + (valid ? row : 0) * (int64_t)L;
#pragma unroll
                for (int c = 0; c < C::KCH; ++c) {
                    uint32_t w[2] = {0u, 0u};
#pragma unroll
                    for (int b = 0; b < 8; ++b) {
                        const int j = 8 * c + b;
                        const uint32_t v = (valid && j < L) ? (uint32_t)(uint8_t)src[j] : 0u;
                        w[b >> 2] |= v << (8 * (b & 3));
                    }
                    sabs = __dp4a(__vabs4(w[0]), 0x01010101u, sabs);
                    sabs = __dp4a(__vabs4(w[1]), 0x01010101u, sabs);
                    uint4 h;
                    i8x4_to_h2x2(w[0], h.x, h.y);
                    i8x4_to_h2x2(w[1], h.z, h.w);
                    *reinterpret_cast<uint4*>(A + c * C::A_KSTRIDE + r * 16) = h;
                }
            }
            stash[(int)(it % C::RING) * kTileM + r] = (float)sabs;
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&stash_full[(int)(it % C::RING)]);
                mbar_arrive(&a_full[s]);
                mbar_arrive(&raw_empty[s]);
            }
        }
    } else if (warp < 8) {
        // ------------------------------------------------ epilogue
        const int q = warp - 4;  // TMEM lane quarter
        const float thr = a.thr;
        const float sq = sqrtf(thr);
        int64_t it = 0;
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
            const int b = (int)(it % C::NACC);
            const uint32_t ph = (uint32_t)((it / C::NACC) & 1);
            if (!mbar_wait(&acc_full[b], ph, abort_flag, a.status, 3)) break;
            tc_fence_after();
            float v[C::N];
            const uint32_t taddr = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * C::N);
#pragma unroll
            for (int c = 0; c < C::N / 16; ++c) tmem_ld16(taddr + 16 * c, v + 16 * c);
            tmem_wait_ld();
            const int r = q * 32 + lane;
            // The converters wrote sum|x| for this tile before the A tile was
            // released to the MMA, and cannot lap the RING slots: the MMA of
            // a later use waits for this epilogue to free its accumulator.
            const int slot = (int)(it % C::RING);
            if (!mbar_wait(&stash_full[slot], (uint32_t)((it / C::RING) & 1), abort_flag, a.status, 11)) break;
            const float sabs = stash[slot * kTileM + r];
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[b]);

            float pmax = 0.f;
#pragma unroll
            for (int k = 0; k < C::N / 2; ++k) {
                const float p = fmaf(v[k], v[k], v[C::N / 2 + k] * v[C::N / 2 + k]);
                pmax = fmaxf(pmax, p);
            }
            const int64_t row = t * kTileM + r;
            const bool valid = row < n;
            const float d = sabs * a.err_coef;
            const float g = fmaxf(a.guard_cfg, 2.f * sq * d + 3.f * d * d + 1e-4f);
            const bool sure = valid && pmax < thr - g;
            const bool unsure = valid && !sure && pmax <= thr + g;
            const uint32_t bits = __ballot_sync(0xFFFFFFFFu, sure || unsure);
            const int64_t word = t * 4 + q;
            if (lane == 0 && word < a.mask_words) a.mask[word] = bits;
            const uint32_t ub = __ballot_sync(0xFFFFFFFFu, unsure);
            if (ub) {
                unsigned long long basei = 0;
                if (lane == 0) basei = atomicAdd(a.unsure_count, (unsigned long long)__popc(ub));
                basei = __shfl_sync(0xFFFFFFFFu, basei, 0);
                if (unsure) {
                    const unsigned long long pos = basei + __popc(ub & ((1u << lane) - 1u));
                    if ((int64_t)pos < a.unsure_cap)
                        a.unsure[pos] = (uint32_t)row;
                    else
                        atomicCAS(a.status, 0, GP_KSTATUS_OVERFLOW);
                }
            }
            if constexpr (WRITE_PSD) {
                if (valid) {
#pragma unroll
                    for (int k = 0; k < C::N / 2; ++k)
                        a.psd_out[row * (C::N / 2) + k] = fmaf(v[k], v[k], v[C::N / 2 + k] * v[C::N / 2 + k]);
                }
            }
        }
    } else if (warp == 8) {
        // ------------------------------------------------ producer
        int64_t it = 0;
        if (lane == 0) {
            mbar_arrive_expect_tx(b_full, 2 * C::B_BYTES);
            bulk_g2s(sB, a.bimage, 2 * C::B_BYTES, b_full);
            for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
                const int s = (int)(it % C::STAGES);
                const uint32_t ph = (uint32_t)((it / C::STAGES) & 1);
                if (!mbar_wait(&raw_empty[s], ph ^ 1u, abort_flag, a.status, 4)) break;
                const bool full_tile = aligned && (t + 1) * kTileM <= n;
                if (full_tile) {
                    const uint32_t bytes = (uint32_t)(kTileM * L);
                    mbar_arrive_expect_tx(&raw_full[s], bytes);
                    bulk_g2s(sRaw + s * lay.raw_stride, a.seqs + t * kTileM * (int64_t)L, bytes, &raw_full[s]);
                } else {
                    mbar_arrive(&raw_full[s]);
                }
            }
            // Do not leave the CTA with copies in flight: wait (bounded, even
            // after an abort) for the last phase issued on every stage.
            int issued = (int)(it < C::STAGES ? it : C::STAGES);
            for (int k = 0; k < issued; ++k) {
                const int64_t j = it - 1 - k;
                const int s = (int)(j % C::STAGES);
                const uint32_t ph = (uint32_t)((j / C::STAGES) & 1);
                const uint64_t t0 = globaltimer_ns();
                while (!mbar_try_wait(&raw_full[s], ph)) {
                    if (globaltimer_ns() - t0 > kWaitTimeoutNs) {
                        atomicCAS(a.status, 0, GP_KSTATUS_TIMEOUT_BASE + 7);
                        break;
                    }
                }
            }
            const uint64_t t0 = globaltimer_ns();
            while (!mbar_try_wait(b_full, 0)) {
                if (globaltimer_ns() - t0 > kWaitTimeoutNs) {
                    atomicCAS(a.status, 0, GP_KSTATUS_TIMEOUT_BASE + 8);
                    break;
                }
            }
        }
    } else {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_f16_f32(C::M, C::N);
            const uint32_t aBase = smem_u32(sA);
            const uint32_t bBase = smem_u32(sB);
            bool ok = mbar_wait(b_full, 0, abort_flag, a.status, 5);
            int64_t it = 0;
            for (int64_t t = blockIdx.x; ok && t < ntiles; t += gridDim.x, ++it) {
                const int s = (int)(it % C::STAGES);
                const uint32_t ph = (uint32_t)((it / C::STAGES) & 1);
                const int b = (int)(it % C::NACC);
                const uint32_t aph = (uint32_t)((it / C::NACC) & 1);
                if (!mbar_wait(&a_full[s], ph, abort_flag, a.status, 6)) break;
                if (!mbar_wait(&acc_empty[b], aph ^ 1u, abort_flag, a.status, 9)) break;
                tc_fence_after();
                const uint32_t d = tmem_base + (uint32_t)(b * C::N);
                const uint32_t aS = aBase + (uint32_t)(s * C::A_BYTES);
#pragma unroll
                for (int pass = 0; pass < 2; ++pass) {
#pragma unroll
                    for (int ks = 0; ks < C::KSTEPS; ++ks) {
                        const uint64_t ad = sdesc_noswizzle(aS + (uint32_t)(ks * 2 * C::A_KSTRIDE), C::A_KSTRIDE, 128);
                        const uint64_t bd = sdesc_noswizzle(
                            bBase + (uint32_t)(pass * C::B_BYTES + ks * 2 * C::B_KSTRIDE), C::B_KSTRIDE, 128);
                        umma_f16(d, ad, bd, idesc, (pass | ks) != 0 ? 1u : 0u);
                    }
                }
                umma_commit(&a_empty[s]);
                umma_commit(&acc_full[b]);
            }
            // every MMA this thread issued is complete before TMEM is freed
            umma_commit(final_bar);
            const uint64_t t0 = globaltimer_ns();
            while (!mbar_try_wait(final_bar, 0)) {
                if (globaltimer_ns() - t0 > kWaitTimeoutNs) {
                    atomicCAS(a.status, 0, GP_KSTATUS_TIMEOUT_BASE + 10);
                    break;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 9) {
        tc_fence_after();
        tmem_dealloc(tmem_base, C::TMEM_COLS);
    }
}

template <int K>
cudaError_t launch_k(const PsdTcArgs& a, int num_sms, cudaStream_t st) {
    const SmemLayout lay = smem_layout<K>(a.L);
    const int64_t ntiles = (a.n + kTileM - 1) / kTileM;
    if (ntiles == 0) return cudaSuccess;
    const bool wpsd = a.psd_out != nullptr;
    auto kern = wpsd ? psd_tc_kernel<K, true> : psd_tc_kernel<K, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.total);
    if (e != cudaSuccess) return e;
    int64_t grid = (int64_t)num_sms * TcCfg<K>::MIN_BLOCKS;
    if (grid > ntiles) grid = ntiles;
    kern<<<(unsigned)grid, kThreads, lay.total, st>>>(a, lay);
    return cudaGetLastError();
}

// IEEE binary16 round-to-nearest-even from double (host side).
uint16_t half_bits(double x) {
    uint16_t sign = 0;
    if (x < 0) {
        sign = 0x8000;
        x = -x;
    }
    if (x == 0) return sign;
    int e;
    double m = std::frexp(x, &e);  // x = m * 2^e, m in [0.5, 1)
    int exp = e - 1;               // x = (2m) * 2^exp
    if (exp < -14) {
        // subnormal: units of 2^-24
        double q = std::nearbyint(x * 16777216.0);
        return (uint16_t)(sign | (uint16_t)q);
    }
    double frac = (2 * m - 1) * 1024.0;
    double q = std::nearbyint(frac);
    if (q >= 1024.0) {
        q = 0;
        exp += 1;
    }
    if (exp > 15) return (uint16_t)(sign | 0x7C00);
    return (uint16_t)(sign | (uint16_t)((exp + 15) << 10) | (uint16_t)q);
}

double half_value(uint16_t h) {
    int s = h >> 15, e = (h >> 10) & 31, m = h & 1023;
    double v = e == 0 ? std::ldexp((double)m, -24) : std::ldexp(1.0 + m / 1024.0, e - 15);
    return s ? -v : v;
}

}  // namespace

int tc_k_for_len(int L) {
    if (L < 2 || L > kMaxTcK) return 0;
    return (L + 15) / 16 * 16;
}

// |X_k - X^_k| <= sum|x| * err_coef:  twiddle residual after the hi + lo
// split (<= 2^-24) plus fp32 accumulation in the tensor core, bounded
// generously as 17 roundings of relative size 2^-22 per UMMA step (2K/16
// steps + the final) applied to partial sums no larger than sum|x|.
float tc_err_coef(int K) {
    const double steps = 2.0 * K / 16.0 + 1.0;
    return (float)(std::ldexp(1.0, -24) + steps * 17.0 * std::ldexp(1.0, -22));
}

size_t build_twiddle_image(int L, int K, void* out) {
    const int N = K;
    const size_t tile = (size_t)N * K * 2;
    if (!out) return 2 * tile;
    std::vector<uint16_t> hi((size_t)N * K, 0), lo((size_t)N * K, 0);
    const int H = L / 2;
    const double two_pi = 6.283185307179586476925286766559;
    for (int nrow = 0; nrow < N; ++nrow) {
        const bool is_sin = nrow >= N / 2;
        const int bin = (is_sin ? nrow - N / 2 : nrow) + 1;
        if (bin > H) continue;
        for (int j = 0; j < L; ++j) {
            const int m = (int)(((long long)j * bin) % L);
            const double w = is_sin ? std::sin(two_pi * m / L) : std::cos(two_pi * m / L);
            const uint16_t h = half_bits(w);
            const uint16_t l = half_bits(w - half_value(h));
            // canonical no-swizzle K-major layout: core matrix (n/8, j/8) at
            // (j/8) * (N/8) * 128 + (n/8) * 128, row n%8 at +16, col j%8 at +2
            const size_t byte = (size_t)(j / 8) * (N / 8) * 128 + (size_t)(nrow / 8) * 128 + (nrow % 8) * 16 + (j % 8) * 2;
            hi[byte / 2] = h;
            lo[byte / 2] = l;
        }
    }
    std::memcpy(out, hi.data(), tile);
    std::memcpy(static_cast<uint8_t*>(out) + tile, lo.data(), tile);
    return 2 * tile;
}

cudaError_t launch_psd_tc(const PsdTcArgs& a, int num_sms, cudaStream_t st) {
    switch (tc_k_for_len(a.L)) {
        case 16: return launch_k<16>(a, num_sms, st);
        case 32: return launch_k<32>(a, num_sms, st);
        case 48: return launch_k<48>(a, num_sms, st);
        case 64: return launch_k<64>(a, num_sms, st);
        case 80: return launch_k<80>(a, num_sms, st);
        case 96: return launch_k<96>(a, num_sms, st);
        case 112: return launch_k<112>(a, num_sms, st);
        case 128: return launch_k<128>(a, num_sms, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace gp
