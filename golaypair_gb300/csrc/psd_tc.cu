// psd_tc.cu -- guarded-FP32 tensor-core PSD filter (tcgen05 + TMEM + bulk copy).
//
// Restates src/utils/fourier.cpp:25-52 (FFTW c2c PSD, then reject if any
// psd[k] > 2n - paf + 0.001 for k = 1..L/2) as a batched dense contraction:
//
//   X[M=128 candidates x K] (fp16, exact small integers)
//     * W[K x N] (cos/sin twiddles, each split into hi + lo fp16)
//     -> D[128 x N] fp32 in TMEM, p_k = re_k^2 + im_k^2.
//
// Row n < K/2 of W is the cosine of bin n+1, row K/2 + n the sine of bin
// n+1; bins above L/2 and columns j >= L are zero, so the padding columns of
// X never contribute.  K = L + 1 rounded up to 16, so the last cosine row
// (bin K/2) is always beyond L/2: it holds ones instead, and that column of
// D is the row sum X_0 (exact).  By Parseval, L sum x^2 = X_0^2 + 2 sum_k p_k
// (bin L/2 of an even L counted twice: an upper bound) <= X_0^2 + 2 (L/2)
// max_k p_k, which gives the per-row error bound from the values the
// epilogue computes anyway.
//
// The hi and lo twiddles sit side by side along N: the B image is 2K x K,
// one UMMA of N = 2K per 16-wide K step.  A tcgen05.mma of M = 128, K = 16
// takes ~46 cycles for any N up to 96 (measured on GB300), so one N = 2K
// instruction per step costs half of two N = K instructions.  The epilogue
// decides from the hi columns alone, with a guard widened by the hi-only
// twiddle error; only a warp with a row inside that wider band reads the lo
// columns too and decides again (about 1e-5 of the warps on int8 input).
//
// Each candidate is classified against T = 2n - paf + 0.001 with a guard g
// (the configured band, widened per row to a rigorous bound on the fp32
// error): max p < T - g -> pass, max p > T + g -> reject, else "unsure",
// appended to a list that an FP64 kernel rechecks exactly.  The pass mask
// bit is set for pass and unsure; the recheck clears the failing unsure ones.
//
// Two input forms:
//   int8 rows    n x L bytes (the batched filter's input);
//   packed words one 16-byte word per candidate, digit j in bits
//                [b(L-1-j), b(L-j)), value = 2*digit - c (the enumerator's
//                and the uncompression expander's output).
//
// The A operand (the candidates) lives in tensor memory: each converter
// thread owns one row = one TMEM lane and writes its fp16 pairs with
// tcgen05.st, so shared memory only carries the raw input (written once by
// the bulk-copy engine, read once by the converters) and the constant B.
//
// Persistent kernel, one 128-candidate tile per step, warp roles:
//   warps 0-3  convert: staged tile -> fp16 row in TMEM
//   warps 4-7  epilogue: TMEM -> registers -> PSD max -> mask / unsure list
//   warp 8     producer: cp.async.bulk of each tile into a deep ring
//   warp 9     MMA issuer (one lane) and TMEM owner
// Rings of mbarriers hand tiles between the roles; every wait is bounded
// (a timeout records a site code and the CTA unwinds).  With as many A
// stages as accumulators, the MMAs of a tile free its A stage when they
// complete, so one commit (accumulator full) serves the epilogue and the
// converters.
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "gp_device.cuh"

namespace gp {

namespace {

constexpr int kThreads = 320;
constexpr int kConvWarps = 4;
constexpr int kRawSlack = 64;
constexpr int kMaxRawStages = 12;
constexpr uint32_t kSmemBudget2Cta = 112 * 1024;  // two CTAs per SM
constexpr uint32_t kSmemBudget1Cta = 220 * 1024;
constexpr int kLutBytes = 4096;

// accumulator buffers and TMEM A stages per K (columns: NACC*N + AS*K/2)
constexpr int tc_nacc(int K) { return K == 16 ? 4 : K == 32 ? 3 : K == 48 ? 2 : K == 64 ? 3 : K <= 96 ? 2 : K == 112 ? 2 : 1; }
constexpr int tc_as(int K) { return K == 16 ? 4 : K == 32 ? 3 : K == 48 ? 2 : K <= 80 ? 4 : K == 96 ? 2 : K == 112 ? 1 : 4; }

template <int K>
struct TcCfg {
    static constexpr int M = kTileM;
    static constexpr int N = 2 * K;                    // UMMA N: K/2 cosine + K/2 sine bins, hi then lo
    static constexpr int KCH = K / 8;                  // 8-element chunks along K
    static constexpr int KW = K / 4 + 1;               // 32-bit words covering a row's K bytes + misalignment
    static constexpr int KSTEPS = K / 16;              // UMMA K steps (instructions) per tile
    static constexpr int B_BYTES = 2 * K * K * 2;      // whole B image (hi and lo)
    static constexpr int B_KSTRIDE = (N / 8) * 128;    // bytes between core matrices adjacent in K
    static constexpr int MIN_BLOCKS = K <= 48 ? 2 : 1;
    static constexpr int TMEM_COLS = MIN_BLOCKS == 2 ? 256 : 512;
    static constexpr int NACC = tc_nacc(K);
    static constexpr int AS = tc_as(K);                // A stages in TMEM
    static constexpr int A_COL0 = NACC * N;            // first TMEM column of the A stages
    static_assert(NACC * N + AS * K / 2 <= TMEM_COLS, "TMEM budget");
};

struct SmemLayout {
    uint32_t b_off, lut_off, raw_off, raw_stride, raw_stages, bar_off, misc_off, total;
};

template <int K>
SmemLayout smem_layout(int row_bytes) {
    using C = TcCfg<K>;
    SmemLayout s;
    uint32_t off = 0;
    s.b_off = off;
    off += C::B_BYTES;
    off = (off + 1023) & ~1023u;
    s.lut_off = off;
    off += kLutBytes;
    s.bar_off = off;
    off += (2 * kMaxRawStages + 2 * C::AS + 2 * C::NACC + 2) * 8;
    s.misc_off = off;
    off += 16;
    off = (off + 127) & ~127u;
    s.raw_stride = (uint32_t)((kTileM * row_bytes + kRawSlack + 127) & ~127);
    s.raw_off = off;
    const uint32_t budget = (C::MIN_BLOCKS == 2 ? kSmemBudget2Cta : kSmemBudget1Cta) - 1024;
    int st = budget > off ? (int)((budget - off) / s.raw_stride) : 0;
    if (st > kMaxRawStages) st = kMaxRawStages;
    if (st < 2) st = 2;
    s.raw_stages = (uint32_t)st;
    off += st * s.raw_stride;
    s.total = off + 1024;  // slack for the 1024-byte alignment of the base
    // At most two CTAs per SM: each holds 256 TMEM columns (512 per SM).
    if (s.total < 96 * 1024) s.total = 96 * 1024;
    return s;
}

// Builds the packed-digit lookup table: for b in {1,2,4} a byte of 8/b
// digits maps to 8/b halves; for b = 3 six bits (two digits) map to a half2.
// Value of a digit: 2*digit - c.
__device__ void build_lut(uint8_t* lut, int b, int c) {
    const int entries = b == 3 ? 64 : 256;
    const int per = b == 3 ? 2 : 8 / b;  // digits per entry
    const int bits = b == 3 ? 6 : 8;
    for (int e = threadIdx.x; e < entries; e += blockDim.x) {
        for (int d = 0; d < per; ++d) {
            const int digit = (e >> (bits - b * (d + 1))) & ((1 << b) - 1);
            reinterpret_cast<__half*>(lut)[e * per + d] = __int2half_rn(2 * digit - c);
        }
    }
}

// Normalises a packed word: the 128-bit left shift by norm (0..127) that
// puts digit 0 at bit 127.  sw[0] holds bits 0-31 ... sw[3] bits 96-127.
// norm is the same for every row of a tile, so the word shift is a uniform
// branch and the bit shift four funnel shifts.
__device__ __forceinline__ void shl128(uint4 v, int norm, uint32_t (&sw)[4]) {
    uint32_t a0 = v.x, a1 = v.y, a2 = v.z, a3 = v.w;
    switch (norm >> 5) {
        case 1: a3 = a2; a2 = a1; a1 = a0; a0 = 0u; break;
        case 2: a3 = a1; a2 = a0; a1 = 0u; a0 = 0u; break;
        case 3: a3 = a0; a2 = 0u; a1 = 0u; a0 = 0u; break;
        default: break;
    }
    const uint32_t bs = (uint32_t)norm & 31u;
    sw[3] = __funnelshift_l(a2, a3, bs);
    sw[2] = __funnelshift_l(a1, a2, bs);
    sw[1] = __funnelshift_l(a0, a1, bs);
    sw[0] = a0 << bs;
}

// 8 halves of digits 8*ch .. 8*ch+7 from the normalised word (digit 0 at bit
// 127).  w[0] holds bits 0-31 ... w[3] bits 96-127.
template <int B, int CH>
__device__ __forceinline__ uint4 packed_chunk(const uint32_t (&w)[4], const uint8_t* lut) {
    constexpr int WIDTH = 8 * B;
    constexpr int HI = 128 - WIDTH * CH;  // exclusive top bit of the field
    constexpr int LO = HI - WIDTH;
    uint32_t field;
    if constexpr (HI <= 0) {
        field = 0;
    } else if constexpr (LO >= 0) {
        constexpr int wi = LO >> 5, sh = LO & 31;
        const uint32_t lo = w[wi];
        const uint32_t hi = (wi + 1 < 4) ? w[(wi + 1 < 4) ? wi + 1 : 3] : 0u;
        const uint64_t v = ((uint64_t)hi << 32) | lo;
        field = (uint32_t)(v >> sh);
        if constexpr (WIDTH < 32) field &= (1u << WIDTH) - 1u;
    } else {
        // field straddles bit 0: the digits below it are padding
        const uint32_t top = w[0] & ((HI >= 32) ? 0xFFFFFFFFu : ((1u << (HI & 31)) - 1u));
        field = top << ((-LO) & 31);
    }
    uint4 out;
    if constexpr (B == 1) {
        out = reinterpret_cast<const uint4*>(lut)[field & 0xFF];
    } else if constexpr (B == 2) {
        const uint2 x = reinterpret_cast<const uint2*>(lut)[(field >> 8) & 0xFF];
        const uint2 y = reinterpret_cast<const uint2*>(lut)[field & 0xFF];
        out = make_uint4(x.x, x.y, y.x, y.y);
    } else if constexpr (B == 3) {
        const uint32_t* l = reinterpret_cast<const uint32_t*>(lut);
        out = make_uint4(l[(field >> 18) & 63], l[(field >> 12) & 63], l[(field >> 6) & 63], l[field & 63]);
    } else {
        const uint32_t* l = reinterpret_cast<const uint32_t*>(lut);
        out = make_uint4(l[(field >> 24) & 255], l[(field >> 16) & 255], l[(field >> 8) & 255], l[field & 255]);
    }
    return out;
}

template <int B, int CH, int CHEND>
__device__ __forceinline__ void packed_row(const uint32_t (&w)[4], const uint8_t* lut, uint32_t* h) {
    if constexpr (CH < CHEND) {
        const uint4 v = packed_chunk<B, CH>(w, lut);
        h[4 * CH] = v.x;
        h[4 * CH + 1] = v.y;
        h[4 * CH + 2] = v.z;
        h[4 * CH + 3] = v.w;
        packed_row<B, CH + 1, CHEND>(w, lut, h);
    }
}

// B = 0: int8 rows; B = 1..4: packed words with B bits per digit.
// Cycle counter for the per-role diagnostics; compiled out when TR is false.
template <bool TR>
__device__ __forceinline__ long long tclock() {
    if constexpr (TR) return clock64();
    return 0;
}

// Stage index and phase parity of a ring of S stages, advanced once per tile.
struct Ring {
    int slot = 0;
    uint32_t phase = 0;
    __device__ __forceinline__ void next(int S) {
        if (++slot == S) {
            slot = 0;
            phase ^= 1u;
        }
    }
};

__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Eight bins from column c0 of one accumulator row: re = cos hi + cos lo,
// im = sin hi + sin lo, p = re^2 + im^2; folds max p into pmax, except for
// column HB - 1, which is the row sum X_0 (stored in x0).  (Measured: x8
// loads per chunk beat x16 loads of 16 bins by 9 %.)
template <int HB, bool WRITE_PSD>
__device__ __forceinline__ void psd_chunk(uint32_t taddr, int c0, float& pmax, float& x0, float* psd_row) {
    constexpr int K = 2 * HB, W = 8;
    float chi[W], shi[W], clo[W], slo[W];
    tmem_ld8(taddr + c0, chi);
    tmem_ld8(taddr + HB + c0, shi);
    tmem_ld8(taddr + K + c0, clo);
    tmem_ld8(taddr + K + HB + c0, slo);
    tmem_wait_ld();
#pragma unroll
    for (int k = 0; k < W; k += 2) {
        const float2 re = __fadd2_rn(make_float2(chi[k], chi[k + 1]), make_float2(clo[k], clo[k + 1]));
        const float2 im = __fadd2_rn(make_float2(shi[k], shi[k + 1]), make_float2(slo[k], slo[k + 1]));
        const float2 p = __ffma2_rn(re, re, __fmul2_rn(im, im));
        if (c0 + k + 1 == HB - 1) {
            pmax = fmaxf(pmax, p.x);
            x0 = re.y;
        } else {
            pmax = fmax3(pmax, p.x, p.y);
        }
        if constexpr (WRITE_PSD) {
            if (psd_row) {
                psd_row[c0 + k] = p.x;
                psd_row[c0 + k + 1] = p.y;
            }
        }
    }
}

// The hi twiddles alone: eight bins from column c0, p = c_hi^2 + s_hi^2.
template <int HB>
__device__ __forceinline__ void psd_chunk_hi(uint32_t taddr, int c0, float& pmax, float& x0) {
    float chi[8], shi[8];
    tmem_ld8(taddr + c0, chi);
    tmem_ld8(taddr + HB + c0, shi);
    tmem_wait_ld();
#pragma unroll
    for (int k = 0; k < 8; k += 2) {
        const float2 re = make_float2(chi[k], chi[k + 1]);
        const float2 im = make_float2(shi[k], shi[k + 1]);
        const float2 p = __ffma2_rn(re, re, __fmul2_rn(im, im));
        if (c0 + k + 1 == HB - 1) {
            pmax = fmaxf(pmax, p.x);
            x0 = re.y;  // the ones row has no lo part: X_0 is exact here
        } else {
            pmax = fmax3(pmax, p.x, p.y);
        }
    }
}

// The hi twiddles alone over all HB bins: every load issued before one wait.
// t_ld: the cycle counter when the loads have landed (TR builds).
template <int HB, bool TR>
__device__ __forceinline__ void psd_hi_all(uint32_t taddr, float& pmax, float& x0, long long& t_ld) {
    // the cosine and sine columns are contiguous: [0, HB) and [HB, 2 HB)
    float v[2 * HB];
    tmem_ld_cols<2 * HB>(taddr, v);
    const float* chi = v;
    const float* shi = v + HB;
    tmem_wait_ld();
    t_ld = tclock<TR>();
    float pm[2] = {pmax, 0.f};  // two independent max chains
#pragma unroll
    for (int k = 0; k < HB; k += 2) {
        const float2 re = make_float2(chi[k], chi[k + 1]);
        const float2 im = make_float2(shi[k], shi[k + 1]);
        const float2 p = __ffma2_rn(re, re, __fmul2_rn(im, im));
        float& m = pm[(k >> 1) & 1];
        if (k + 1 == HB - 1) {
            m = fmaxf(m, p.x);
            x0 = re.y;  // the ones row has no lo part: X_0 is exact here
        } else {
            m = fmax3(m, p.x, p.y);
        }
    }
    pmax = fmaxf(pm[0], pm[1]);
}

// A row of a tile that is not whole or not bulk-copied (the last tile, or
// an input not 16-byte aligned): byte loads from global memory, zeros past
// row n or column L, stored as the A row at TMEM address aaddr.  Out of line: it runs at most once per CTA on aligned
// input, and keeps its unrolled loads out of the hot loop's code.
template <int K>
__device__ __noinline__ void partial_row_store(const int8_t* seqs, int row, int n, int L, uint32_t aaddr) {
    uint32_t h[K / 2];
    const bool valid = row < n;
    const int8_t* src = seqs + (int64_t)(valid ? row : 0) * L;
#pragma unroll
    for (int c = 0; c < K / 8; ++c) {
        uint32_t w[2] = {0u, 0u};
#pragma unroll
        for (int bb = 0; bb < 8; ++bb) {
            const int j = 8 * c + bb;
            const uint32_t v = (valid && j < L) ? (uint32_t)(uint8_t)src[j] : 0u;
            w[bb >> 2] |= v << (8 * (bb & 3));
        }
        i8x4_to_h2x2(w[0], h[4 * c], h[4 * c + 1]);
        i8x4_to_h2x2(w[1], h[4 * c + 2], h[4 * c + 3]);
    }
#pragma unroll
    for (int g = 0; g < K / 16; ++g) tmem_st8(aaddr + 8 * g, h + 8 * g);
}

// Both twiddle halves over all HB bins (the exact pass): max p and X_0.
// Out of line: it runs for about 1e-5 of the warps of the int8 workload.
template <int HB, bool WRITE_PSD>
__device__ __noinline__ float2 exact_pass(uint32_t taddr, float* psd_row) {
    float pmax = 0.f, x0 = 0.f;
#pragma unroll
    for (int c0 = 0; c0 < HB; c0 += 8) psd_chunk<HB, WRITE_PSD>(taddr, c0, pmax, x0, psd_row);
    return make_float2(pmax, x0);
}

// TR: per-role cycle counters (diagnostics build of the kernel).
template <int K, int B, bool WRITE_PSD, bool TR>
__global__ void __launch_bounds__(kThreads, TcCfg<K>::MIN_BLOCKS) psd_tc_kernel(PsdTcArgs a, SmemLayout lay) {
    using C = TcCfg<K>;
    extern __shared__ uint8_t smem_raw_base[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw_base) + 1023) & ~uintptr_t(1023));

    uint8_t* sB = smem + lay.b_off;
    uint8_t* sLut = smem + lay.lut_off;
    uint8_t* sRaw = smem + lay.raw_off;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + lay.bar_off);
    uint64_t* raw_full = bars;
    uint64_t* raw_empty = bars + kMaxRawStages;
    uint64_t* a_full = bars + 2 * kMaxRawStages;
    uint64_t* a_empty = a_full + C::AS;
    uint64_t* acc_full = a_empty + C::AS;
    uint64_t* acc_empty = acc_full + C::NACC;
    uint64_t* b_full = acc_empty + C::NACC;
    uint64_t* final_bar = b_full + 1;
    // 32-bit shared-window addresses of the barrier rings (8 bytes apart)
    const uint32_t u_raw_full = smem_u32(raw_full), u_raw_empty = smem_u32(raw_empty);
    const uint32_t u_a_full = smem_u32(a_full), u_a_empty = smem_u32(a_empty);
    const uint32_t u_acc_full = smem_u32(acc_full), u_acc_empty = smem_u32(acc_empty);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + lay.misc_off);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + lay.misc_off + 4);

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int L = a.L;
    int64_t n = a.n;
    if (a.n_dev) {
        const int64_t nd = (int64_t)*reinterpret_cast<const volatile unsigned long long*>(a.n_dev);
        if (nd < n) n = nd;
    }
    // tile and row indices fit 32 bits (the launch refuses n >= 2^31)
    const int ntiles = (int)((n + kTileM - 1) / kTileM);
    const int n32 = (int)n;
    const int RS = (int)lay.raw_stages;
    const int row_bytes = B == 0 ? L : 16;
    const bool aligned =
        (reinterpret_cast<uintptr_t>(B == 0 ? (const void*)a.seqs : (const void*)a.words) & 15) == 0;
    // tiles below nfull are whole and bulk-copied into shared memory
    const int nfull = aligned ? (int)(n / kTileM) : 0;

    if (threadIdx.x == 0) {
        for (int i = 0; i < RS; ++i) {
            mbar_init(&raw_full[i], 1);
            mbar_init(&raw_empty[i], kConvWarps);
        }
        for (int i = 0; i < C::AS; ++i) {
            mbar_init(&a_full[i], kConvWarps);
            mbar_init(&a_empty[i], 1);
        }
        for (int i = 0; i < C::NACC; ++i) {
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], 4);
        }
        mbar_init(b_full, 1);
        mbar_init(final_bar, 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    if constexpr (B != 0) build_lut(sLut, B, a.alpha_c);
    if (warp == 9) {
        tmem_alloc(tmem_slot, C::TMEM_COLS);
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *reinterpret_cast<volatile uint32_t*>(tmem_slot);

    if (warp < kConvWarps) {
        // ------------------------------------------------ converters
        // Row r's bytes L..K-1 in a full tile are the next row's first
        // bytes: they land in A columns whose B rows are all zero, so they
        // add nothing and are not masked.
        const int r = threadIdx.x;  // row of the tile = TMEM lane
        const int norm = 128 - B * L;  // packed: left shift that puts digit 0 at bit 127
        const uint32_t lane_base = tmem_base + ((uint32_t)(warp * 32) << 16) + (uint32_t)C::A_COL0;
        int it = 0;
        Ring raw, ast;
        unsigned long long tr0 = 0, tr1 = 0, tr2 = 0, tr3 = 0, tr4 = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it, raw.next(RS), ast.next(C::AS)) {
            const int rs = raw.slot;
            const uint32_t rph = raw.phase;
            const int as = ast.slot;
            const uint32_t aph = ast.phase;
            const long long c0t = tclock<TR>();
            if (!mbar_wait(u_raw_full + 8u * rs, rph, abort_flag, a.status, 1)) break;
            const long long c1t = tclock<TR>();
            // with as many A stages as accumulators, the MMAs of the tile that
            // last used this A stage completed when its accumulator was
            // committed full: acc_full of the same slot stands for a_empty
            if (!mbar_wait((C::AS == C::NACC ? u_acc_full : u_a_empty) + 8u * as, aph ^ 1u, abort_flag, a.status, 2))
                break;
            const long long c2t = tclock<TR>();
            tr0 += c1t - c0t;
            tr1 += c2t - c1t;
            tc_fence_after();
            const int row = t * kTileM + r;
            const bool full_tile = t < nfull;
            uint32_t h[K / 2];  // the row as fp16 pairs
            const uint32_t aaddr = lane_base + (uint32_t)(as * (K / 2));
            if constexpr (B == 0) {
                if (full_tile) {
                    const uint8_t* raw = sRaw + rs * lay.raw_stride;
                    const int off = r * L;
                    const uint32_t* wp = reinterpret_cast<const uint32_t*>(raw + (off & ~3));
                    const uint32_t sh = (uint32_t)(off & 3) * 8u;
                    uint32_t wv[C::KW];
#pragma unroll
                    for (int i = 0; i < C::KW; ++i) wv[i] = wp[i];
#pragma unroll
                    for (int c = 0; c < C::KCH; ++c) {
                        const uint32_t lo = __funnelshift_r(wv[2 * c], wv[2 * c + 1], sh);
                        const uint32_t hi = __funnelshift_r(wv[2 * c + 1], wv[2 * c + 2], sh);
                        i8x4_to_h2x2(lo, h[4 * c], h[4 * c + 1]);
                        i8x4_to_h2x2(hi, h[4 * c + 2], h[4 * c + 3]);
                    }
                } else {
                    partial_row_store<K>(a.seqs, row, n32, L, aaddr);
                }
            } else {
                uint4 wv;
                if (full_tile) {
                    wv = *reinterpret_cast<const uint4*>(sRaw + rs * lay.raw_stride + r * 16);
                } else {
                    wv = row < n ? a.words[row] : make_uint4(0, 0, 0, 0);
                }
                uint32_t sw[4];
                shl128(wv, norm, sw);
                packed_row<B, 0, C::KCH>(sw, sLut, h);
            }
            const long long c25t = tclock<TR>();
            if (B != 0 || full_tile) {
#pragma unroll
                for (int g = 0; g < K / 16; ++g) tmem_st8(aaddr + 8 * g, h + 8 * g);
            }
            tmem_wait_st();
            const long long c3t = tclock<TR>();
            tr3 += c3t - c2t;
            tr4 += c3t - c25t;
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(u_a_full + 8u * as);
                mbar_arrive(u_raw_empty + 8u * rs);
            }
            tr2 += tclock<TR>() - c2t;
        }
        if (a.trace && lane == 0) {
            atomicAdd(&a.trace[kTrConvWaitRaw], tr0);
            atomicAdd(&a.trace[kTrConvWaitA], tr1);
            atomicAdd(&a.trace[kTrConvWork], tr3);
            atomicAdd(&a.trace[kTrConvFence], tr2 - tr3);
            atomicAdd(&a.trace[kTrConvSt], tr4);
            if (warp == 0) atomicAdd(&a.trace[kTrTiles], (unsigned long long)it);
        }
    } else if (warp < kConvWarps + 4) {
        // ------------------------------------------------ epilogue
        const int q = warp & 3;  // TMEM lane quarter (warps 4..7)
        const float thr = a.thr;
        const float sq = sqrtf(thr);
        constexpr int HB = K / 2;  // bins per half (cos block then sin block)
        // Guard for a per-bin error bound |X^_k - X_k| <= coef * sum|x|.
        // Packed rows: |value| <= c, so sum|x| <= L c.  int8 rows: by
        // Parseval and Cauchy-Schwarz, S = sum|x| satisfies S^2 <= L sum x^2
        // = X_0^2 + 2 sum_{k=1..H} p_k <= X_0^2 + 2H (sqrt(max p^) + coef S)^2
        // (bin L/2 of an even L counted twice: still a bound), so
        // S <= (|X_0| + sqrt(2H max p^)) / (1 - sqrt(2H) coef).
        const float m2h = sqrtf(2.f * (float)(L / 2));
        // per error coefficient: int8 rows d = coef / (1 - sqrt(2H) coef) *
        // (|X_0| + sqrt(2H max p)); packed rows d = coef L c
        struct Coef {
            float sc, dc;
        };
        auto coef_of = [&](float coef) {
            return Coef{coef / (1.f - m2h * coef), coef * (float)L * (float)a.alpha_c};
        };
        // sqrt(pm) <= (pm + T) / (2 sqrt T) (AM-GM; equality at pm = T, the
        // only rows whose verdict the band can change); 1 + 2^-20 covers
        // the rounding of the factor
        const float hs = 0.5f / sq * 1.00000095367431640625f;
        const float m2h_hs = m2h * hs, m2h_hs_t = m2h * hs * thr;
        auto guard = [&](float pm, float x0v, Coef k) {
            float d;
            if constexpr (B == 0)
                d = k.sc * (fmaf(m2h_hs, pm, m2h_hs_t) + fabsf(x0v));
            else
                d = k.dc;
            return fmaxf(a.guard_cfg, fmaf(2.f * sq, d, fmaf(3.f * d, d, 1e-4f)));
        };
        // the hi twiddles alone are within 2^-12 of the exact ones per
        // component: sqrt 2 * 2^-12 = 3.45267e-4 more on the modulus
        const Coef sc_hi = coef_of(a.err_coef + 3.4527e-4f), sc_lo = coef_of(a.err_coef);
        const int mask_words = (int)a.mask_words;
        Ring acc;
        unsigned long long tr0 = 0, tr1 = 0, tr2 = 0, tr3 = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, acc.next(C::NACC)) {
            const int b = acc.slot;
            const uint32_t ph = acc.phase;
            const long long c0t = tclock<TR>();
            if (!mbar_wait(u_acc_full + 8u * b, ph, abort_flag, a.status, 3)) break;
            const long long c1t = tclock<TR>();
            tr0 += c1t - c0t;
            tc_fence_after();
            const int r = q * 32 + lane;
            const int row = t * kTileM + r;
            const bool valid = row < n32;
            const uint32_t taddr = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * C::N);
            // accumulator columns: [0, HB) cos hi, [HB, K) sin hi, [K, K + HB)
            // cos lo, [K + HB, 2K) sin lo; cos column HB - 1 is the row sum X_0.
            // First the hi columns alone, with the wider hi-only guard: a
            // row clearly below or above the bound is decided there.  Only
            // a warp with a row inside that band reads the lo columns too
            // (rare: about 1e-5 of the rows of the int8 workload).
            float pmax = 0.f, x0 = 0.f, g = 0.f;
            long long c_ld = c1t;
            bool exact = WRITE_PSD;
            if constexpr (!WRITE_PSD) {
                psd_hi_all<HB, TR>(taddr, pmax, x0, c_ld);
                g = guard(pmax, x0, sc_hi);
                // only picks the warps that redo the row exactly: the verdict
                // below is taken with the same bounds either way
                const bool near = valid && fabsf(pmax - thr) <= g;
                exact = __any_sync(0xFFFFFFFFu, near);
            }
            if (exact) {
                const float2 px = exact_pass<HB, WRITE_PSD>(taddr, valid ? a.psd_out + (int64_t)row * HB : nullptr);
                pmax = px.x;
                x0 = px.y;
                g = guard(pmax, x0, sc_lo);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(u_acc_empty + 8u * b);
            const long long c_rel = tclock<TR>();
            tr1 += c_ld - c1t;
            const bool sure = valid && pmax < thr - g;
            const bool unsure = valid && !sure && pmax <= thr + g;
            const uint32_t bits = __ballot_sync(0xFFFFFFFFu, sure || unsure);
            const int word = t * 4 + q;
            if (lane == 0 && word < mask_words) a.mask[word] = bits;
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
            const long long c_end = tclock<TR>();
            tr2 += c_end - c1t;
            tr3 += c_end - c_rel;
        }
        if (a.trace && lane == 0) {
            atomicAdd(&a.trace[kTrEpiWaitAcc], tr0);
            atomicAdd(&a.trace[kTrEpiLd], tr1);
            atomicAdd(&a.trace[kTrEpiWork], tr2);
            atomicAdd(&a.trace[kTrEpiTail], tr3);
        }
    } else if (warp == kConvWarps + 4) {
        // ------------------------------------------------ producer
        int64_t it = 0;
        if (lane == 0) {
            mbar_arrive_expect_tx(b_full, C::B_BYTES);
            bulk_g2s(sB, a.bimage, C::B_BYTES, b_full);
            const uint32_t u_raw = smem_u32(sRaw);
            const uint8_t* src = B == 0 ? reinterpret_cast<const uint8_t*>(a.seqs)
                                        : reinterpret_cast<const uint8_t*>(a.words);
            unsigned long long tr0 = 0, tr1 = 0;
            Ring raw;
            for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it, raw.next(RS)) {
                const int rs = raw.slot;
                const uint32_t ph = raw.phase;
                const long long c0 = tclock<TR>();
                if (!mbar_wait(u_raw_empty + 8u * rs, ph ^ 1u, abort_flag, a.status, 4)) break;
                const long long c1 = tclock<TR>();
                tr0 += c1 - c0;
                const bool full_tile = t < nfull;
                if (full_tile) {
                    const uint32_t bytes = (uint32_t)(kTileM * row_bytes);
                    mbar_arrive_expect_tx(u_raw_full + 8u * rs, bytes);
                    bulk_g2s(u_raw + (uint32_t)rs * lay.raw_stride, src + (int64_t)t * kTileM * row_bytes, bytes,
                             u_raw_full + 8u * rs);
                } else {
                    mbar_arrive(u_raw_full + 8u * rs);
                }
                tr1 += tclock<TR>() - c1;
            }
            if (a.trace) {
                atomicAdd(&a.trace[kTrProdWait], tr0);
                atomicAdd(&a.trace[kTrProdIssue], tr1);
            }
            // Do not leave the CTA with copies in flight: wait (bounded, even
            // after an abort) for the last phase issued on every stage.
            const int issued = (int)(it < RS ? it : RS);
            for (int k = 0; k < issued; ++k) {
                const int64_t j = it - 1 - k;
                const int rs = (int)(j % RS);
                const uint32_t ph = (uint32_t)((j / RS) & 1);
                const uint64_t t0 = globaltimer_ns();
                while (!mbar_try_wait(&raw_full[rs], ph)) {
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
            // B descriptor of k-step 0; later steps add to the start-address
            // field (bits 0-13, address >> 4)
            const uint64_t bdesc0 = sdesc_noswizzle(smem_u32(sB), C::B_KSTRIDE, 128);
            bool ok = mbar_wait(b_full, 0, abort_flag, a.status, 5);
            Ring ast, acc;
            unsigned long long tr0 = 0, tr1 = 0, tr2 = 0, tr3 = 0;
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x, ast.next(C::AS), acc.next(C::NACC)) {
                const int as = ast.slot;
                const uint32_t aph = ast.phase;
                const int b = acc.slot;
                const uint32_t bph = acc.phase;
                const long long c0 = tclock<TR>();
                if (!mbar_wait(u_a_full + 8u * as, aph, abort_flag, a.status, 6)) break;
                const long long c1 = tclock<TR>();
                if (!mbar_wait(u_acc_empty + 8u * b, bph ^ 1u, abort_flag, a.status, 9)) break;
                const long long c2 = tclock<TR>();
                tr0 += c1 - c0;
                tr1 += c2 - c1;
                tc_fence_after();
                const uint32_t d = tmem_base + (uint32_t)(b * C::N);
                const uint32_t a0 = tmem_base + (uint32_t)(C::A_COL0 + as * (K / 2));
                // one instruction per 16-wide K step covers the hi and lo
                // twiddles side by side (N = 2K)
#pragma unroll
                for (int ks = 0; ks < C::KSTEPS; ++ks)
                    umma_f16_ts(d, a0 + (uint32_t)(8 * ks), bdesc0 + (uint64_t)((2 * ks * C::B_KSTRIDE) >> 4), idesc,
                                ks != 0 ? 1u : 0u);
                const long long c3 = tclock<TR>();
                if constexpr (C::AS != C::NACC) umma_commit(u_a_empty + 8u * as);
                umma_commit(u_acc_full + 8u * b);
                const long long c4 = tclock<TR>();
                tr2 += c3 - c2;
                tr3 += c4 - c3;
            }
            if (a.trace) {
                atomicAdd(&a.trace[kTrMmaWaitA], tr0);
                atomicAdd(&a.trace[kTrMmaWaitAcc], tr1);
                atomicAdd(&a.trace[kTrMmaIssue], tr2);
                atomicAdd(&a.trace[kTrMmaCommit], tr3);
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

template <int K, int B, bool WP>
cudaError_t launch_kb(const PsdTcArgs& a, int num_sms, cudaStream_t st) {
    using C = TcCfg<K>;
    const SmemLayout lay = smem_layout<K>(B == 0 ? a.L : 16);
    const int64_t ntiles = (a.n + kTileM - 1) / kTileM;
    if (ntiles == 0) return cudaSuccess;
    if (a.n >= (int64_t(1) << 31)) return cudaErrorInvalidValue;  // 32-bit row indices
    // the counting variant exists for the int8 input only (diagnostics)
    auto kern = psd_tc_kernel<K, B, WP, false>;
    if constexpr (B == 0 && !WP)
        if (a.trace) kern = psd_tc_kernel<K, B, WP, true>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.total);
    if (e != cudaSuccess) return e;
    const int per_sm = a.grid_per_sm > 0 && a.grid_per_sm < C::MIN_BLOCKS ? a.grid_per_sm : C::MIN_BLOCKS;
    int64_t grid = (int64_t)num_sms * per_sm;
    if (grid > ntiles) grid = ntiles;
    kern<<<(unsigned)grid, kThreads, lay.total, st>>>(a, lay);
    return cudaGetLastError();
}

template <int K>
cudaError_t launch_k(const PsdTcArgs& a, int num_sms, cudaStream_t st) {
    if (a.words == nullptr) {
        if (a.psd_out) return launch_kb<K, 0, true>(a, num_sms, st);
        return launch_kb<K, 0, false>(a, num_sms, st);
    }
    if (a.psd_out) return cudaErrorInvalidValue;
    switch (a.pack_bits) {
        case 1: return launch_kb<K, 1, false>(a, num_sms, st);
        case 2:
            if constexpr (K <= 80) return launch_kb<K, 2, false>(a, num_sms, st);
            break;
        case 3:
            if constexpr (K <= 48) return launch_kb<K, 3, false>(a, num_sms, st);
            break;
        case 4:
            if constexpr (K <= 48) return launch_kb<K, 4, false>(a, num_sms, st);
            break;
        default: break;
    }
    return cudaErrorInvalidValue;
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


// ------------------------------------------------------------ multi-job filter
// Several jobs' packed rows (different lengths, alphabets and bounds) in one
// persistent launch: the tiles of job j are the global tiles [T_j, T_j+1),
// a tile never straddles jobs, and every tile runs at its own job's padded
// length K_j (16, 32, 48 or 64; the launch is instantiated for the largest).
// Each role looks its tile's job up and takes that job's words, digit
// table, twiddle image, UMMA shape (N = 2 K_j, K_j / 16 steps), bound and
// outputs; the barrier rings and the TMEM layout (sized for the largest K)
// are those of psd_tc_kernel.

struct MultiLayout {
    uint32_t lut_off, raw_off, raw_stride, raw_stages, bar_off, misc_off, total;
};

// b_bytes: the jobs' twiddle images, back to back from offset 0
template <int K>
MultiLayout multi_layout(uint32_t b_bytes, int njobs, uint32_t budget) {
    using C = TcCfg<K>;
    MultiLayout s;
    uint32_t off = (b_bytes + 1023) & ~1023u;
    s.lut_off = off;
    off += (uint32_t)njobs * kLutBytes;
    s.bar_off = off;
    off += (2 * kMaxRawStages + 2 * C::AS + 2 * C::NACC + 2) * 8;
    s.misc_off = off;
    // TMEM slot, abort flag; first tile of each job (+ end); rows, whole
    // tiles, K and image offset of each job
    off += 16 + 4 * (kMaxTcJobs + 1) + 4 * 4 * kMaxTcJobs;
    off = (off + 127) & ~127u;
    s.raw_stride = (uint32_t)((kTileM * 16 + kRawSlack + 127) & ~127);
    s.raw_off = off;
    const uint32_t room = budget > off + 1024 ? budget - off - 1024 : 0;
    int st = (int)(room / s.raw_stride);
    if (st > kMaxRawStages) st = kMaxRawStages;
    s.raw_stages = (uint32_t)(st < 2 ? 0 : st);  // 0: does not fit this budget
    off += (uint32_t)(st < 2 ? 2 : st) * s.raw_stride;
    s.total = off + 1024;
    // at most two CTAs per SM, as in psd_tc_kernel
    if (s.total < 96 * 1024) s.total = 96 * 1024;
    return s;
}

// Calls f(std::integral_constant<int, kj>) for kj in {16, 32, 48, 64}, kj <= KMAX.
template <int KMAX, class F>
__device__ __forceinline__ void dispatch_k(int kj, F&& f) {
    if (kj == 16) {
        f(std::integral_constant<int, 16>{});
    } else if constexpr (KMAX >= 32) {
        if (kj == 32) {
            f(std::integral_constant<int, 32>{});
        } else if constexpr (KMAX >= 48) {
            if (kj == 48) {
                f(std::integral_constant<int, 48>{});
            } else if constexpr (KMAX >= 64) {
                if (kj == 64) f(std::integral_constant<int, 64>{});
            }
        }
    }
}

template <int K>
__global__ void __launch_bounds__(kThreads, TcCfg<K>::MIN_BLOCKS) psd_tc_multi_kernel(PsdTcMultiArgs a,
                                                                                        MultiLayout lay) {
    using C = TcCfg<K>;
    extern __shared__ uint8_t smem_raw_base[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw_base) + 1023) & ~uintptr_t(1023));
    uint8_t* sB = smem;
    uint8_t* sLut = smem + lay.lut_off;
    uint8_t* sRaw = smem + lay.raw_off;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + lay.bar_off);
    uint64_t* raw_full = bars;
    uint64_t* raw_empty = bars + kMaxRawStages;
    uint64_t* a_full = bars + 2 * kMaxRawStages;
    uint64_t* a_empty = a_full + C::AS;
    uint64_t* acc_full = a_empty + C::AS;
    uint64_t* acc_empty = acc_full + C::NACC;
    uint64_t* b_full = acc_empty + C::NACC;
    uint64_t* final_bar = b_full + 1;
    const uint32_t u_raw_full = smem_u32(raw_full), u_raw_empty = smem_u32(raw_empty);
    const uint32_t u_a_full = smem_u32(a_full), u_a_empty = smem_u32(a_empty);
    const uint32_t u_acc_full = smem_u32(acc_full), u_acc_empty = smem_u32(acc_empty);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + lay.misc_off);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + lay.misc_off + 4);
    int* s_tile0 = reinterpret_cast<int*>(smem + lay.misc_off + 16);  // [njobs + 1] first global tile of each job
    int* s_rows = s_tile0 + kMaxTcJobs + 1;                           // rows of each job
    int* s_nfull = s_rows + kMaxTcJobs;  // tiles bulk-copied (whole, from 16-byte aligned words)
    int* s_k = s_nfull + kMaxTcJobs;     // padded length
    int* s_boff = s_k + kMaxTcJobs;      // twiddle image offset in sB

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int nj = a.njobs;
    const int RS = (int)lay.raw_stages;

    if (threadIdx.x == 0) {
        for (int i = 0; i < RS; ++i) {
            mbar_init(&raw_full[i], 1);
            mbar_init(&raw_empty[i], kConvWarps);
        }
        for (int i = 0; i < C::AS; ++i) {
            mbar_init(&a_full[i], kConvWarps);
            mbar_init(&a_empty[i], 1);
        }
        for (int i = 0; i < C::NACC; ++i) {
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], 4);
        }
        mbar_init(b_full, 1);
        mbar_init(final_bar, 1);
        *abort_flag = 0;
        int t = 0, boff = 0;
        for (int j = 0; j < nj; ++j) {
            int64_t n = a.job[j].cap;
            if (a.job[j].n_dev) {
                const int64_t nd = (int64_t)*reinterpret_cast<const volatile unsigned long long*>(a.job[j].n_dev);
                if (nd < n) n = nd;
            }
            s_rows[j] = (int)n;
            const bool aligned = (reinterpret_cast<uintptr_t>(a.job[j].words) & 15) == 0;
            s_nfull[j] = aligned ? (int)(n / kTileM) : 0;
            s_tile0[j] = t;
            t += (int)((n + kTileM - 1) / kTileM);
            s_k[j] = a.job[j].K;
            s_boff[j] = boff;
            boff += 4 * a.job[j].K * a.job[j].K;  // 2K x K fp16: a multiple of 1024 bytes
        }
        s_tile0[nj] = t;
        mbar_fence_init();
    }
    for (int j = 0; j < nj; ++j) build_lut(sLut + j * kLutBytes, a.job[j].bits, a.job[j].alpha_c);
    if (warp == 9) {
        tmem_alloc(tmem_slot, C::TMEM_COLS);
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *reinterpret_cast<volatile uint32_t*>(tmem_slot);
    const int ntiles = s_tile0[nj];
    // the job of global tile t (at most eight jobs: a short scan)
    auto job_of = [&](int t) {
        int j = 0;
        while (j + 1 < nj && s_tile0[j + 1] <= t) ++j;
        return j;
    };

    if (warp < kConvWarps) {
        // ------------------------------------------------ converters
        const int r = threadIdx.x;
        const uint32_t lane_base = tmem_base + ((uint32_t)(warp * 32) << 16) + (uint32_t)C::A_COL0;
        Ring raw, ast;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, raw.next(RS), ast.next(C::AS)) {
            const int rs = raw.slot, as = ast.slot;
            const uint32_t rph = raw.phase, aph = ast.phase;
            if (!mbar_wait(u_raw_full + 8u * rs, rph, abort_flag, a.status, 1)) break;
            if (!mbar_wait((C::AS == C::NACC ? u_acc_full : u_a_empty) + 8u * as, aph ^ 1u, abort_flag, a.status, 2))
                break;
            tc_fence_after();
            const int j = job_of(t);
            const PsdTcJob& jb = a.job[j];
            const int lt = t - s_tile0[j];
            const int row = lt * kTileM + r;
            uint4 wv;
            if (lt < s_nfull[j])
                wv = *reinterpret_cast<const uint4*>(sRaw + rs * lay.raw_stride + r * 16);
            else
                wv = row < s_rows[j] ? jb.words[row] : make_uint4(0, 0, 0, 0);
            uint32_t sw[4];
            shl128(wv, 128 - jb.bits * jb.L, sw);
            const uint8_t* lut = sLut + j * kLutBytes;
            const uint32_t aaddr = lane_base + (uint32_t)(as * (K / 2));
            const int bits = jb.bits;
            dispatch_k<K>(s_k[j], [&](auto kc) {
                constexpr int KJ = decltype(kc)::value;
                uint32_t h[KJ / 2];
                switch (bits) {
                    case 1: packed_row<1, 0, KJ / 8>(sw, lut, h); break;
                    case 2: packed_row<2, 0, KJ / 8>(sw, lut, h); break;
                    case 3:
                        if constexpr (KJ <= 48) packed_row<3, 0, KJ / 8>(sw, lut, h);
                        break;
                    default:
                        if constexpr (KJ <= 48) packed_row<4, 0, KJ / 8>(sw, lut, h);
                        break;
                }
#pragma unroll
                for (int g = 0; g < KJ / 16; ++g) tmem_st8(aaddr + 8 * g, h + 8 * g);
            });
            tmem_wait_st();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(u_a_full + 8u * as);
                mbar_arrive(u_raw_empty + 8u * rs);
            }
        }
    } else if (warp < kConvWarps + 4) {
        // ------------------------------------------------ epilogue
        const int q = warp & 3;
        Ring acc;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, acc.next(C::NACC)) {
            const int b = acc.slot;
            if (!mbar_wait(u_acc_full + 8u * b, acc.phase, abort_flag, a.status, 3)) break;
            tc_fence_after();
            const int j = job_of(t);
            const PsdTcJob& jb = a.job[j];
            const int lt = t - s_tile0[j];
            const int row = lt * kTileM + q * 32 + lane;
            const bool valid = row < s_rows[j];
            const uint32_t taddr = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * C::N);
            const float thr = jb.thr, sq2 = 2.f * sqrtf(thr);
            // packed rows: |value| <= c, so the per-bin error is at most coef L c
            auto guard = [&](float d) { return fmaxf(jb.guard_cfg, fmaf(sq2, d, fmaf(3.f * d, d, 1e-4f))); };
            float pmax = 0.f, g = 0.f;
            dispatch_k<K>(s_k[j], [&](auto kc) {
                constexpr int HB = decltype(kc)::value / 2;
                float x0 = 0.f;
                long long c_ld = 0;
                psd_hi_all<HB, false>(taddr, pmax, x0, c_ld);
                g = guard(jb.dc_hi);
                if (__any_sync(0xFFFFFFFFu, valid && fabsf(pmax - thr) <= g)) {
                    pmax = exact_pass<HB, false>(taddr, nullptr).x;
                    g = guard(jb.dc_lo);
                }
            });
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(u_acc_empty + 8u * b);
            const bool sure = valid && pmax < thr - g;
            const bool unsure = valid && !sure && pmax <= thr + g;
            const uint32_t bits = __ballot_sync(0xFFFFFFFFu, sure || unsure);
            const int word = lt * 4 + q;
            if (lane == 0 && (int64_t)word < ((jb.cap + 31) >> 5)) jb.mask[word] = bits;
            const uint32_t ub = __ballot_sync(0xFFFFFFFFu, unsure);
            if (ub) {
                unsigned long long basei = 0;
                if (lane == 0) basei = atomicAdd(jb.unsure_count, (unsigned long long)__popc(ub));
                basei = __shfl_sync(0xFFFFFFFFu, basei, 0);
                if (unsure) {
                    const unsigned long long pos = basei + __popc(ub & ((1u << lane) - 1u));
                    if ((int64_t)pos < jb.cap)
                        jb.unsure[pos] = (uint32_t)row;
                    else
                        atomicCAS(a.status, 0, GP_KSTATUS_OVERFLOW);
                }
            }
        }
    } else if (warp == kConvWarps + 4) {
        // ------------------------------------------------ producer
        int64_t it = 0;
        if (lane == 0) {
            uint32_t bbytes = 0;
            for (int j = 0; j < nj; ++j) bbytes += 4u * (uint32_t)(s_k[j] * s_k[j]);
            mbar_arrive_expect_tx(b_full, bbytes);
            for (int j = 0; j < nj; ++j)
                bulk_g2s(sB + s_boff[j], a.job[j].bimage, 4u * (uint32_t)(s_k[j] * s_k[j]), b_full);
            const uint32_t u_raw = smem_u32(sRaw);
            Ring raw;
            for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it, raw.next(RS)) {
                const int rs = raw.slot;
                if (!mbar_wait(u_raw_empty + 8u * rs, raw.phase ^ 1u, abort_flag, a.status, 4)) break;
                const int j = job_of(t);
                const int lt = t - s_tile0[j];
                if (lt < s_nfull[j]) {
                    const uint32_t bytes = (uint32_t)(kTileM * 16);
                    mbar_arrive_expect_tx(u_raw_full + 8u * rs, bytes);
                    bulk_g2s(u_raw + (uint32_t)rs * lay.raw_stride,
                             reinterpret_cast<const uint8_t*>(a.job[j].words) + (int64_t)lt * kTileM * 16, bytes,
                             u_raw_full + 8u * rs);
                } else {
                    mbar_arrive(u_raw_full + 8u * rs);
                }
            }
            // no copies left in flight: wait (bounded) for the last phase of every stage
            const int issued = (int)(it < RS ? it : RS);
            for (int k = 0; k < issued; ++k) {
                const int64_t jj = it - 1 - k;
                const int rs = (int)(jj % RS);
                const uint32_t ph = (uint32_t)((jj / RS) & 1);
                const uint64_t t0 = globaltimer_ns();
                while (!mbar_try_wait(&raw_full[rs], ph)) {
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
            bool ok = mbar_wait(b_full, 0, abort_flag, a.status, 5);
            Ring ast, acc;
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x, ast.next(C::AS), acc.next(C::NACC)) {
                const int as = ast.slot, b = acc.slot;
                if (!mbar_wait(u_a_full + 8u * as, ast.phase, abort_flag, a.status, 6)) break;
                if (!mbar_wait(u_acc_empty + 8u * b, acc.phase ^ 1u, abort_flag, a.status, 9)) break;
                tc_fence_after();
                const int j = job_of(t);
                const int kj = s_k[j];
                // the tile's job's shape and twiddle image: N = 2 K_j, K_j / 16 steps
                const uint32_t idesc = idesc_f16_f32(C::M, 2 * kj);
                const uint32_t kstride = (uint32_t)(2 * kj / 8) * 128;
                const uint64_t bdesc0 = sdesc_noswizzle(smem_u32(sB + s_boff[j]), kstride, 128);
                const uint32_t d = tmem_base + (uint32_t)(b * C::N);
                const uint32_t a0 = tmem_base + (uint32_t)(C::A_COL0 + as * (K / 2));
                for (int ks = 0; ks < kj / 16; ++ks)
                    umma_f16_ts(d, a0 + (uint32_t)(8 * ks), bdesc0 + (uint64_t)((2 * ks * kstride) >> 4), idesc,
                                ks != 0 ? 1u : 0u);
                if constexpr (C::AS != C::NACC) umma_commit(u_a_empty + 8u * as);
                umma_commit(u_acc_full + 8u * b);
            }
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
cudaError_t launch_multi_k(const PsdTcMultiArgs& a, int num_sms, cudaStream_t st) {
    using C = TcCfg<K>;
    uint32_t b_bytes = 0;
    for (int j = 0; j < a.njobs; ++j) b_bytes += 4u * (uint32_t)(a.job[j].K * a.job[j].K);
    // two CTAs per SM when every job's twiddle image and digit table fit beside
    // the raw ring in the two-CTA budget, else one
    MultiLayout lay = multi_layout<K>(b_bytes, a.njobs, kSmemBudget2Cta);
    int fit = C::MIN_BLOCKS;
    if (lay.raw_stages == 0 || C::MIN_BLOCKS < 2) {
        lay = multi_layout<K>(b_bytes, a.njobs, kSmemBudget1Cta);
        fit = 1;
    }
    if (lay.raw_stages == 0) return cudaErrorInvalidValue;
    auto kern = psd_tc_multi_kernel<K>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.total);
    if (e != cudaSuccess) return e;
    int64_t cap_tiles = 0;
    for (int j = 0; j < a.njobs; ++j) cap_tiles += (a.job[j].cap + kTileM - 1) / kTileM;
    if (cap_tiles == 0) return cudaSuccess;
    const int per_sm = a.grid_per_sm > 0 && a.grid_per_sm < fit ? a.grid_per_sm : fit;
    int64_t grid = (int64_t)num_sms * per_sm;
    if (grid > cap_tiles) grid = cap_tiles;
    kern<<<(unsigned)grid, kThreads, lay.total, st>>>(a, lay);
    return cudaGetLastError();
}

}  // namespace

// K: L + 1 rounded up to 16, so that the last cosine row is free for the
// row sum (bin K/2 > L/2).
int tc_k_for_len(int L) {
    if (L < 2) return 0;
    const int K = (L + 16) / 16 * 16;
    return K <= kMaxTcK ? K : 0;
}

bool tc_packed_supported(int L, int b) {
    const int K = tc_k_for_len(L);
    if (!K || b < 1 || b > 4 || b * L > 128) return false;
    if (b == 2) return K <= 80;
    if (b == 3 || b == 4) return K <= 48;
    return true;
}

// |X_k - X^_k| <= sum|x| * err_coef:  per component (real or imaginary
// part) the twiddle residual after the hi + lo split (<= 2^-24) plus fp32
// accumulation in the tensor core, bounded generously as 17 roundings of
// relative size 2^-22 per UMMA step (2K/16 steps + the final) applied to
// partial sums no larger than sum|x|; times sqrt 2 for the modulus.
float tc_err_coef(int K) {
    const double steps = 2.0 * K / 16.0 + 1.0;
    return (float)(std::sqrt(2.0) * (std::ldexp(1.0, -24) + steps * 17.0 * std::ldexp(1.0, -22)));
}

size_t build_twiddle_image(int L, int K, void* out) {
    const size_t bytes = (size_t)2 * K * K * 2;
    if (!out) return bytes;
    std::vector<uint16_t> img((size_t)2 * K * K, 0);
    const double two_pi = 6.283185307179586476925286766559;
    for (int nrow = 0; nrow < K; ++nrow) {
        int bin = 0;
        const int kind = tc_row_kind(nrow, L, K, &bin);
        if (kind == 0) continue;
        for (int j = 0; j < L; ++j) {
            const int m = (int)(((long long)j * bin) % L);
            const double w = kind == 3 ? 1.0 : kind == 2 ? std::sin(two_pi * m / L) : std::cos(two_pi * m / L);
            const uint16_t h = half_bits(w);
            const uint16_t l = half_bits(w - half_value(h));
            img[tc_image_index(nrow, j, 0, K)] = h;
            img[tc_image_index(nrow, j, 1, K)] = l;
        }
    }
    std::memcpy(out, img.data(), bytes);
    return bytes;
}

bool tc_multi_supported(int L, int b) { return tc_packed_supported(L, b) && tc_k_for_len(L) <= kMaxMultiK; }

cudaError_t launch_psd_tc_multi(const PsdTcMultiArgs& a, int num_sms, cudaStream_t st) {
    if (a.njobs < 1 || a.njobs > kMaxTcJobs) return cudaErrorInvalidValue;
    int kmax = 0;
    int64_t tiles = 0;
    for (int j = 0; j < a.njobs; ++j) {
        const PsdTcJob& q = a.job[j];
        if (!tc_multi_supported(q.L, q.bits) || q.K != tc_k_for_len(q.L) || q.cap < 0 ||
            q.cap >= (int64_t(1) << 31))
            return cudaErrorInvalidValue;
        kmax = q.K > kmax ? q.K : kmax;
        tiles += (q.cap + kTileM - 1) / kTileM;
    }
    if (tiles >= (int64_t(1) << 31)) return cudaErrorInvalidValue;  // 32-bit global tile index
    switch (kmax) {
        case 16: return launch_multi_k<16>(a, num_sms, st);
        case 32: return launch_multi_k<32>(a, num_sms, st);
        case 48: return launch_multi_k<48>(a, num_sms, st);
        case 64: return launch_multi_k<64>(a, num_sms, st);
        default: return cudaErrorInvalidValue;
    }
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
