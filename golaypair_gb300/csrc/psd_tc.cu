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
// X never contribute.  The exception: int8 rows of a length whose rows start
// off 4-byte boundaries are read from the boundary below and placed s <= 3
// columns along (s = (row L) mod 4, no byte realignment per row); columns
// j = L .. L + 2 then hold the twiddles of j - L, so the shifted row's X_k
// gains a unit phase and its PSD is unchanged, and the converters clear
// the neighbouring rows' bytes.  K = L + 1 rounded up to 16, so the last cosine row
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
#include <vector>

#include "psd_tc_body.cuh"

namespace gp {

namespace {

template <int K, int B, bool WRITE_PSD, bool TR, bool SH>
__global__ void __launch_bounds__(kThreads, TcCfg<K>::MIN_BLOCKS) psd_tc_kernel(PsdTcArgs a, SmemLayout lay) {
    tc_body<K, B, WRITE_PSD, TR, SH>(a, lay, blockIdx.x, gridDim.x);
}

// largest padded K with shifted int8 loads (one mask register per 4 bytes)
constexpr int kMaxShiftK = 64;

template <int K, int B, bool WP>
cudaError_t launch_kb(const PsdTcArgs& a, int num_sms, cudaStream_t st) {
    using C = TcCfg<K>;
    const SmemLayout lay = smem_layout<K>(B == 0 ? a.L : 16);
    const int64_t ntiles = (a.n + kTileM - 1) / kTileM;
    if (ntiles == 0) return cudaSuccess;
    if (a.n >= (int64_t(1) << 31)) return cudaErrorInvalidValue;  // 32-bit row indices
    if (a.i8_shift && (B != 0 || !tc_i8_shifted(a.L))) return cudaErrorInvalidValue;
    // the counting variant exists for the int8 input only (diagnostics)
    auto kern = psd_tc_kernel<K, B, WP, false, false>;
    if constexpr (B == 0 && K <= kMaxShiftK)
        if (a.i8_shift) kern = psd_tc_kernel<K, B, WP, false, true>;
    if constexpr (B == 0 && !WP) {
        if (a.trace) kern = psd_tc_kernel<K, B, WP, true, false>;
        if constexpr (K <= kMaxShiftK)
            if (a.trace && a.i8_shift) kern = psd_tc_kernel<K, B, WP, true, true>;
    }
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


}  // namespace

// K: L + 1 rounded up to 16, so that the last cosine row is free for the
// row sum (bin K/2 > L/2).
int tc_k_for_len(int L) {
    if (L < 2) return 0;
    const int K = (L + 16) / 16 * 16;
    return K <= kMaxTcK ? K : 0;
}

namespace {
int i8_max_shift(int L) { return L % 4 == 0 ? 0 : L % 2 == 0 ? 2 : 3; }
}  // namespace

bool tc_i8_shifted(int L) {
    const int K = tc_k_for_len(L);
    return K != 0 && K <= kMaxShiftK && L + i8_max_shift(L) <= K;
}

int tc_i8_wrap_rows(int L) { return tc_i8_shifted(L) ? i8_max_shift(L) : 0; }

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

size_t build_twiddle_image(int L, int K, void* out, int wrap) {
    const size_t bytes = (size_t)2 * K * K * 2;
    if (!out) return bytes;
    std::vector<uint16_t> img((size_t)2 * K * K, 0);
    const double two_pi = 6.283185307179586476925286766559;
    const int jend = L + wrap < K ? L + wrap : K;
    for (int nrow = 0; nrow < K; ++nrow) {
        int bin = 0;
        const int kind = tc_row_kind(nrow, L, K, &bin);
        if (kind == 0) continue;
        for (int j = 0; j < jend; ++j) {
            const int m = (int)(((long long)(j % L) * bin) % L);
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
