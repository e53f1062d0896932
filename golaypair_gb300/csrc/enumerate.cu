// enumerate.cu -- rank-window necklace enumerator (kernel (a)).
//
// Restates generate_necklaces_prefix / generate_necklaces_wrapper
// (src/utils/lyndon.cpp:47-121) and the row-sum gate of generate_hybrid
// (src/core/generate/generate_hybrid.cpp:35-41,139-154) for the GPU.
//
// The reference walks the FKM recursion over the sorted alphabet and sees
// every prenecklace of length L in lexicographic order, keeping those whose
// period divides L (necklaces).  Here the word space is cut into rank
// windows; each thread starts at the first prenecklace >= its window's first
// word and steps the FKM successor
//     i = last position whose digit is not maximal; a_i += 1;
//     a_j = a_{j-i} for j > i  (period i)
// until it leaves the window.  Words are packed (see rows.cuh), so the
// successor is a handful of 128-bit bit operations.  Necklaces whose digit
// sum matches a decomposition's row sum are appended (warp-aggregated) to a
// candidate buffer with their A/B role bits.  A thread that meets the
// buffer's soft capacity saves its position; the host drains the buffer
// and relaunches.
#include "gp_device.cuh"
#include "enumerate.h"

namespace gp {

namespace {

struct W128 {
    uint64_t lo, hi;
};
__device__ __forceinline__ W128 w128(const decltype(EnumArgs::maxpat)& v) { return {v.lo, v.hi}; }

__device__ __forceinline__ W128 shr(W128 a, int s) {
    if (s <= 0) return a;
    if (s >= 128) return {0, 0};
    if (s >= 64) return {a.hi >> (s - 64), 0};
    return {(a.lo >> s) | (a.hi << (64 - s)), a.hi >> s};
}
__device__ __forceinline__ W128 shl(W128 a, int s) {
    if (s <= 0) return a;
    if (s >= 128) return {0, 0};
    if (s >= 64) return {0, a.lo << (s - 64)};
    return {a.lo << s, (a.hi << s) | (a.lo >> (64 - s))};
}
__device__ __forceinline__ W128 band(W128 a, W128 b) { return {a.lo & b.lo, a.hi & b.hi}; }
__device__ __forceinline__ W128 bor(W128 a, W128 b) { return {a.lo | b.lo, a.hi | b.hi}; }
__device__ __forceinline__ W128 bxor(W128 a, W128 b) { return {a.lo ^ b.lo, a.hi ^ b.hi}; }
__device__ __forceinline__ bool is_zero(W128 a) { return (a.lo | a.hi) == 0; }
__device__ __forceinline__ bool lt(W128 a, W128 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ W128 low_mask(int bits) {  // 2^bits - 1
    if (bits >= 128) return {~0ull, ~0ull};
    if (bits >= 64) return {~0ull, bits == 64 ? 0ull : ((1ull << (bits - 64)) - 1ull)};
    return {bits == 0 ? 0ull : ((1ull << bits) - 1ull), 0ull};
}
__device__ __forceinline__ int ctz128(W128 a) {
    return a.lo ? __ffsll((long long)a.lo) - 1 : 64 + __ffsll((long long)a.hi) - 1;
}
__device__ __forceinline__ int digit(W128 w, int b, int L, int j) {
    const W128 s = shr(w, b * (L - 1 - j));
    return (int)(s.lo & ((1ull << b) - 1ull));
}

// Keeps the first p digits and repeats them with period p over L digits.
__device__ __forceinline__ W128 periodic_fill(W128 w, int b, int L, int p) {
    W128 x = band(w, bxor(low_mask(b * L), low_mask(b * (L - p))));
    for (int len = p; len < L; len <<= 1) x = bor(x, shr(x, b * len));
    return band(x, low_mask(b * L));
}

// First prenecklace >= w (w a word of L digits); returns its period.
__device__ __forceinline__ int first_prenecklace(W128& w, int b, int L) {
    int p = 1;
    for (int i = 1; i < L; ++i) {
        const int d = digit(w, b, L, i), e = digit(w, b, L, i - p);
        if (d > e) {
            p = i + 1;
        } else if (d < e) {
            w = periodic_fill(w, b, L, p);
            return p;
        }
    }
    return p;
}

// FKM successor; returns the new period, or 0 when w was the last word.
__device__ __forceinline__ int fkm_next(W128& w, const EnumArgs& a) {
    const W128 x = band(bxor(w, w128(a.maxpat)), low_mask(a.b * a.L));
    if (is_zero(x)) return 0;
    const int r = ctz128(x) / a.b;  // digits after the incremented one
    const int j = a.L - 1 - r;
    w = bor(band(w, bxor(low_mask(a.b * a.L), low_mask(a.b * r))), {0, 0});
    // increment digit j (it is below the maximum, so no carry)
    const W128 one = shl({1ull, 0ull}, a.b * r);
    w.lo += one.lo;
    w.hi += one.hi + (w.lo < one.lo ? 1ull : 0ull);
    const int p = j + 1;
    w = periodic_fill(w, a.b, a.L, p);
    return p;
}

__device__ __forceinline__ int digit_sum(W128 w, const EnumArgs& a) {
    int s = 0;
    for (int t = 0; t < a.b; ++t) {
        const W128 m = band(w, W128{a.plane[t].lo, a.plane[t].hi});
        s += (__popcll(m.lo) + __popcll(m.hi)) << t;
    }
    return s;
}

__global__ void __launch_bounds__(256) enumerate_kernel(EnumArgs a) {
    __shared__ uint8_t role_tab[kMaxDigitSum + 1];
    for (int i = threadIdx.x; i <= kMaxDigitSum; i += blockDim.x) role_tab[i] = a.roles[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    int64_t win = tid;                   // this thread's current window
    bool active = win < a.nwin;
    W128 w = {0, 0}, end = {0, 0};
    int p = 0;
    bool have = false;                   // w is a valid prenecklace to process
    unsigned long long necklaces = 0;
    bool stop = false;
    int step = 0;
    for (;;) {
        // (re)load a window when idle
        if (active && !have) {
            const uint4 c = a.cur[win];
            const uint4 e = a.end[win];
            w = {((uint64_t)c.y << 32) | c.x, ((uint64_t)c.w << 32) | c.z};
            end = {((uint64_t)e.y << 32) | e.x, ((uint64_t)e.w << 32) | e.z};
            if (lt(w, end)) {
                p = first_prenecklace(w, a.b, a.L);
                have = lt(w, end);
            }
            if (!have) {
                a.cur[win] = a.end[win];  // window finished
                win += nthreads;
                active = win < a.nwin;
            }
        }
        const bool any = __any_sync(0xFFFFFFFFu, active);
        if (!any) break;
        uint8_t role = 0;
        W128 cand = w;
        if (active && have) {
            if (a.L % p == 0) {
                ++necklaces;
                role = role_tab[digit_sum(w, a)];
            }
            const int np = fkm_next(w, a);
            if (np == 0 || !lt(w, end)) {
                have = false;
                a.cur[win] = a.end[win];
                win += nthreads;
                active = win < a.nwin;
            } else {
                p = np;
            }
        }
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, role != 0);
        if (bal) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(a.count, (unsigned long long)__popc(bal));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (role) {
                const unsigned long long pos = base + __popc(bal & ((1u << lane) - 1u));
                if ((int64_t)pos < a.cap) {
                    a.words[pos] = make_uint4((uint32_t)cand.lo, (uint32_t)(cand.lo >> 32), (uint32_t)cand.hi,
                                              (uint32_t)(cand.hi >> 32));
                    a.out_roles[pos] = role;
                } else {
                    atomicCAS(a.status, 0, GP_KSTATUS_OVERFLOW);
                }
            }
        }
        if ((++step & 7) == 0) {
            unsigned long long cnt = 0;
            if (lane == 0) cnt = *reinterpret_cast<volatile unsigned long long*>(a.count);
            cnt = __shfl_sync(0xFFFFFFFFu, cnt, 0);
            if ((int64_t)cnt >= a.soft_cap) {
                stop = true;
                break;
            }
        }
    }
    if (stop) {
        // save the position of the unfinished window; later windows of this
        // thread are untouched and still hold their starting words
        if (active && have) {
            a.cur[win] = make_uint4((uint32_t)w.lo, (uint32_t)(w.lo >> 32), (uint32_t)w.hi, (uint32_t)(w.hi >> 32));
        }
        *a.incomplete = 1;
    }
    if (necklaces) atomicAdd(a.necklaces, necklaces);
}

}  // namespace

cudaError_t launch_enumerate(const EnumArgs& a, int num_sms, cudaStream_t st) {
    if (a.nwin <= 0) return cudaSuccess;
    int64_t blocks = (a.nwin + 255) / 256;
    const int64_t maxb = (int64_t)num_sms * 8;
    if (blocks > maxb) blocks = maxb;
    enumerate_kernel<<<(unsigned)blocks, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace gp
