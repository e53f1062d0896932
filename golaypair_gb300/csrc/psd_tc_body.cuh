// psd_tc_body.cuh -- the tensor-core PSD filter's persistent CTA body, shared
// by the one-job kernel (psd_tc.cu) and the multi-job kernel
// (psd_tc_multi.cu).  The algorithm and the warp roles are described at the
// top of psd_tc.cu.
#pragma once
#include <cmath>
#include <cstring>
#include <type_traits>

#include "gp_device.cuh"
#include "gp_internal.h"

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
// SH: int8 rows read from the 4-byte boundary at or below their first byte
// (PsdTcArgs::i8_shift; the image carries the wrapped twiddle rows).
// The whole kernel for one job: roles, rings and TMEM of TcCfg<K>, input
// words (B = 1..4) or int8 rows (B = 0), over the tiles first, first +
// stride, ... of the job (the one-job kernel: its CTA index and grid size).
template <int K, int B, bool WRITE_PSD, bool TR, bool SH = false>
__device__ __forceinline__ void tc_body(const PsdTcArgs& a, const SmemLayout& lay, int first, int stride) {
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
        // Without SH, row r's bytes L..K-1 in a full tile are the next
        // row's first bytes: they land in A columns whose B rows are all
        // zero, so they add nothing and are not masked.
        const int r = threadIdx.x;  // row of the tile = TMEM lane
        const int norm = 128 - B * L;  // packed: left shift that puts digit 0 at bit 127
        const uint32_t lane_base = tmem_base + ((uint32_t)(warp * 32) << 16) + (uint32_t)C::A_COL0;
        // SH: the row's bytes sit at columns [s, s + L) of the K bytes read
        // from the 4-byte boundary below it (the tile starts on one, so s is
        // the same for every tile); mk keeps those bytes and clears the
        // neighbouring rows' (a cleared byte converts to 0)
        uint32_t mk[SH ? K / 4 : 1];
        if constexpr (SH) {
            const int s = (r * L) & 3;
#pragma unroll
            for (int i = 0; i < K / 4; ++i) {
                uint32_t m = 0u;
#pragma unroll
                for (int bb = 0; bb < 4; ++bb) {
                    const int col = 4 * i + bb;
                    if (col >= s && col < s + L) m |= 0xFFu << (8 * bb);
                }
                mk[i] = m;
            }
        }
        int it = 0;
        Ring raw, ast;
        unsigned long long tr0 = 0, tr1 = 0, tr2 = 0, tr3 = 0, tr4 = 0;
        for (int t = first; t < ntiles; t += stride, ++it, raw.next(RS), ast.next(C::AS)) {
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
                    if constexpr (SH) {
                        // mask and sign bias in one logic op per word
#pragma unroll
                        for (int c = 0; c < C::KCH; ++c) {
                            biased_u8x4_to_h2x2((wp[2 * c] & mk[2 * c]) ^ 0x80808080u, h[4 * c], h[4 * c + 1]);
                            biased_u8x4_to_h2x2((wp[2 * c + 1] & mk[2 * c + 1]) ^ 0x80808080u, h[4 * c + 2],
                                                h[4 * c + 3]);
                        }
                    } else {
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
        for (int t = first; t < ntiles; t += stride, acc.next(C::NACC)) {
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
            for (int t = first; t < ntiles; t += stride, ++it, raw.next(RS)) {
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
            for (int t = first; ok && t < ntiles; t += stride, ast.next(C::AS), acc.next(C::NACC)) {
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

}  // namespace
}  // namespace gp
