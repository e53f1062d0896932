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
//     a_j = a_{j-(i+1)} for j > i  (period i + 1)
// until it leaves the window.  Words are packed (see rows.cuh), so the
// successor is a handful of 64- or 128-bit bit operations.  One step takes a
// block: the successors that only change the last two digits follow a fixed
// pattern (rows of Lyndon words, see the kernel), so a block's necklaces are
// counted row by row without visiting them.  Necklaces whose digit sum
// matches a decomposition's row sum are appended (warp-aggregated) to a
// candidate buffer with their A/B role bits.
//
// One launch serves several jobs (orders / compressions, each with its own
// length, alphabet, row-sum table and candidate buffer): every window names
// its job.  A window whose job's buffer has met its soft capacity is left
// with its position saved; the host drains the buffers and relaunches.
#include "gp_device.cuh"
#include "enumerate.h"

namespace gp {

namespace {

struct W128 {
    uint64_t lo, hi;
};
__device__ __forceinline__ W128 w128(const U128p& v) { return {v.lo, v.hi}; }

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

// The layout of the job a thread is enumerating, held in registers.
struct JobView {
    int L, b;
    bool narrow;              // b * L <= 64: the word fits its low 64 bits
    uint32_t inv_b;           // floor(x / b) = (x * inv_b) >> 8 for 0 <= x < 128
    W128 maxpat, full;        // full = low_mask(b * L)
    W128 ones;                // bit 0 of every digit; bit t of every digit = ones << t
    W128 divisors;            // bit p set iff p divides L (the necklace test, no division)
};

__device__ __forceinline__ JobView job_view(const EnumJob& j) {
    JobView v;
    v.L = j.L;
    v.b = j.b;
    v.maxpat = w128(j.maxpat);
    v.full = low_mask(j.b * j.L);
    v.ones = w128(j.plane[0]);
    v.inv_b = (256u + (uint32_t)j.b - 1u) / (uint32_t)j.b;
    v.narrow = j.b * j.L <= 64;
    v.divisors = {0, 0};
    for (int p = 1; p <= j.L; ++p)
        if (j.L % p == 0) v.divisors = bor(v.divisors, shl({1ull, 0ull}, p));
    return v;
}

__device__ __forceinline__ bool divides_L(const JobView& a, int p) {
    return ((p < 64 ? (a.divisors.lo >> p) : (a.divisors.hi >> (p - 64))) & 1ull) != 0;
}

// FKM successor; returns the new period, or 0 when w was the last word.
__device__ __forceinline__ int fkm_next(W128& w, const JobView& a) {
    const W128 x = band(bxor(w, a.maxpat), a.full);
    if (is_zero(x)) return 0;
    const int r = (int)(((uint32_t)ctz128(x) * a.inv_b) >> 8);  // digits after the incremented one
    const int j = a.L - 1 - r;
    w = band(w, bxor(a.full, low_mask(a.b * r)));
    // increment digit j (it is below the maximum, so no carry)
    const W128 one = shl({1ull, 0ull}, a.b * r);
    w.lo += one.lo;
    w.hi += one.hi + (w.lo < one.lo ? 1ull : 0ull);
    const int p = j + 1;
    w = periodic_fill(w, a.b, a.L, p);
    return p;
}

// The same successor on words of at most 64 bits (native 64-bit shifts; no
// shift below reaches 64: b * len, b * r < b * L <= 64).
__device__ __forceinline__ uint64_t mask64(int bits) { return bits >= 64 ? ~0ull : ((1ull << bits) - 1ull); }

__device__ __forceinline__ int fkm_next64(uint64_t& w, const JobView& a) {
    const uint64_t x = (w ^ a.maxpat.lo) & a.full.lo;
    if (!x) return 0;
    const int r = (int)(((uint32_t)(__ffsll((long long)x) - 1) * a.inv_b) >> 8);
    const int p = a.L - r;  // the incremented digit is L - 1 - r; the new period is its index + 1
    w = (w & (a.full.lo ^ mask64(a.b * r))) + (1ull << (a.b * r));
    uint64_t y = w & (a.full.lo ^ mask64(a.b * r));
    for (int len = p; len < a.L; len <<= 1) y |= y >> (a.b * len);
    w = y & a.full.lo;
    return p;
}

__device__ __forceinline__ int digit_sum64(uint64_t w, const JobView& a) {
    int s = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t)
        if (t < a.b) s += __popcll(w & (a.ones.lo << t)) << t;
    return s;
}

__device__ __forceinline__ int digit_sum(W128 w, const JobView& a) {
    int s = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        if (t < a.b) {
            const W128 m = band(w, shl(a.ones, t));
            s += (__popcll(m.lo) + __popcll(m.hi)) << t;
        }
    }
    return s;
}

__device__ __forceinline__ uint4 to_u4(W128 w) {
    return make_uint4((uint32_t)w.lo, (uint32_t)(w.lo >> 32), (uint32_t)w.hi, (uint32_t)(w.hi >> 32));
}
__device__ __forceinline__ W128 from_u4(uint4 v) {
    return {((uint64_t)v.y << 32) | v.x, ((uint64_t)v.w << 32) | v.z};
}
__device__ __forceinline__ bool job_full(const EnumJob& j) {
    return (int64_t)*reinterpret_cast<volatile unsigned long long*>(j.count) >= j.soft_cap;
}

// Bits lo .. lo + n - 1 (n <= 16) of a job's digit-sum bitset, as bits 0 .. n - 1.
__device__ __forceinline__ uint64_t role_bits(const unsigned long long* tb, int lo, int n) {
    const int wi = lo >> 6, sh = lo & 63;
    uint64_t x = tb[wi] >> sh;
    if (sh) x |= tb[wi + 1] << (64 - sh);
    return x & ((1ull << n) - 1ull);
}

// Each thread takes windows from a global counter.  A window whose job
// has reached its soft capacity is left (position saved) and the thread goes
// on with its next window, so one full job does not idle the others.
// MINB = 3: 72 registers, no spills (3 CTAs of 256 per SM);
// MINB = 4: at most 64 registers (4 CTAs of 256 per SM); MINB = 8: capped
// at 32 registers for full occupancy (some spills).  The tuner picks.
//
// Candidates go to a per-warp queue in shared memory first; the warp writes
// them out when kFlushAt or more are queued, with one counter atomic per
// job present.  (An atomic per step, whose returned offset the whole warp waits
// for, made the kernel memory-latency bound.)  A job's soft capacity is
// checked on a count loaded at the previous check, so the load's latency
// overlaps the steps in between.
constexpr int kFlushAt = kEnumQueue - 32;
constexpr int kQueue = kEnumQueue;  // per warp: < kFlushAt queued + 32 from one step

// NARROW: every job's words fit 63 bits, so a word and its window end are
// 64-bit values (the high halves are zero and drop out of the registers).
template <int MINB, bool NARROW>
__global__ void __launch_bounds__(256, MINB) enumerate_kernel(EnumArgs a) {
    __shared__ uint8_t role_tab[kMaxEnumJobs][kMaxDigitSum + 1];
    __shared__ EnumJob jobs[kMaxEnumJobs];
    __shared__ uint4 q_word[8][kQueue];
    __shared__ uint8_t q_role[8][kQueue];
    __shared__ uint8_t q_job[8][kQueue];
    // bit s of tbits[j]: digit sum s has a role in job j (one spare word so
    // that a 64-bit window starting below bit 1024 stays inside)
    __shared__ unsigned long long tbits[kMaxEnumJobs][(kMaxDigitSum + 1) / 64 + 1];
    for (int i = threadIdx.x; i < kMaxEnumJobs * ((kMaxDigitSum + 1) / 64 + 1); i += blockDim.x)
        (&tbits[0][0])[i] = 0ull;
    __syncthreads();
    for (int i = threadIdx.x; i < a.njobs * (kMaxDigitSum + 1); i += blockDim.x) {
        const int jj = i / (kMaxDigitSum + 1), ds = i % (kMaxDigitSum + 1);
        role_tab[jj][ds] = a.roles[i];
        if (a.roles[i]) atomicOr(&tbits[jj][ds >> 6], 1ull << (ds & 63));
    }
    if (threadIdx.x < a.njobs) jobs[threadIdx.x] = a.jobs[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int wq = threadIdx.x >> 5;  // this warp's queue
    const uint32_t lt_mask = (1u << lane) - 1u;
    int qlen = 0;                     // queued candidates (the same in every lane)
    // writes the warp's queue out (every lane of the warp calls it)
    auto flush = [&]() {
        __syncwarp();
        for (int base = 0; base < qlen; base += 32) {
            const int e = base + lane;
            const bool has = e < qlen;
            const uint32_t hm = __ballot_sync(0xFFFFFFFFu, has);
            if (has) {
                const int jb = q_job[wq][e];
                const uint32_t grp = __match_any_sync(hm, jb);
                const int leader = __ffs(grp) - 1;
                const EnumJob& J = jobs[jb];
                unsigned long long pos0 = 0;
                if (lane == leader) pos0 = atomicAdd(J.count, (unsigned long long)__popc(grp));
                pos0 = __shfl_sync(grp, pos0, leader);
                const unsigned long long pos = pos0 + __popc(grp & lt_mask);
                if ((int64_t)pos < J.cap) {
                    J.words[pos] = q_word[wq][e];
                    J.out_roles[pos] = q_role[wq][e];
                } else {
                    atomicCAS(a.status, 0, GP_KSTATUS_OVERFLOW);
                }
            }
        }
        qlen = 0;
        __syncwarp();
    };
    unsigned long long seen_count = 0;  // count of job seen_job, loaded at the previous check
    int seen_job = -1;
    // windows are handed out dynamically: a thread takes the next unvisited
    // one from a global counter when it needs work (long windows do not
    // hold up a statically assigned share)
    // The index of the window after the current one is fetched when the
    // current one starts, so the atomic's latency is hidden by its steps.
    int64_t pref = -1;
    auto take = [&]() -> int64_t {
        const int64_t w0 = pref >= 0 ? pref : (int64_t)atomicAdd(a.next_win, 1ull);
        pref = -1;
        return w0;
    };
    int64_t win = take();  // current window
    bool active = win < a.nwin;
    W128 w = {0, 0}, end = {0, 0};
    JobView jv{};
    int job = 0;
    int p = 0;
    bool have = false;  // w is a valid prenecklace to process
    bool parked_any = false;
    unsigned long long necklaces = 0;  // of job `job`, flushed when the job changes
    for (int step = 1;; ++step) {
        // (re)load a window when idle; skip windows whose job is full
        while (active && !have) {
            const int nj = a.win_job[win];
            if (nj != job && necklaces) {
                atomicAdd(jobs[job].necklaces, necklaces);
                necklaces = 0;
            }
            job = nj;
            if (job_full(jobs[job])) {
                parked_any = true;  // window untouched: it keeps its position
            } else {
                w = from_u4(a.cur[win]);
                end = from_u4(a.end[win]);
                if constexpr (NARROW) {
                    w.hi = 0;
                    end.hi = 0;
                }
                jv = job_view(jobs[job]);
                if (lt(w, end)) {
                    p = first_prenecklace(w, jv.b, jv.L);
                    have = lt(w, end);
                }
                if (have && pref < 0) pref = (int64_t)atomicAdd(a.next_win, 1ull);
                if (!have) a.cur[win] = a.end[win];  // window finished
            }
            if (!have) {
                win = take();
                active = win < a.nwin;
            }
        }
        if (!__any_sync(0xFFFFFFFFu, active)) break;
        // One step takes a block of words that differ from the prenecklace w
        // only in the last two digits (v, d), in FKM order:
        //  * the rest of w's row: FKM's successor of a word whose last digit
        //    is below the maximum K is the word with that digit raised by
        //    one, with period L (a Lyndon word, so a necklace);
        //  * when the last digit reaches K and the second-to-last v is below
        //    K: the successor raises v and sets the last digit to the first
        //    digit a_0 (period L - 1), then raises the last digit again
        //    (period L) up to K; and so on up to v = K (L >= 3, so a_0 is not
        //    the raised digit, and k^2 <= 64 for the candidate mask);
        // up to the window's end.  The block's necklaces are counted without
        // visiting them one by one, its candidates are the words whose digit
        // sum has a role, and one successor follows the whole block.
        W128 w0 = w;
        uint64_t cmask = 0;  // bit (v - v0) * k + d: that word is a candidate
        int spre = 0, v0 = 0, kk = 1;
        if (active) {
            const int b = jv.b;
            const uint64_t dmask = (1ull << b) - 1ull;
            const int K = (int)(jv.maxpat.lo & dmask);
            kk = K + 1;
            const int d0 = (int)(w.lo & dmask);
            v0 = (int)((w.lo >> b) & dmask);
            const bool two = jv.L >= 3 && kk * kk <= 64;
            const int vmax = two ? K : v0;
            // words at or past the window's end are cut: x = (v << b) | d below xend
            uint32_t xend = 0xFFFFFFFFu;
            const uint64_t m2 = (1ull << (2 * b)) - 1ull;
            if ((NARROW || end.hi == w.hi) && (end.lo & ~m2) == (w.lo & ~m2)) xend = (uint32_t)(end.lo & m2);
            const int a0 = (NARROW || jv.narrow) ? (int)((w.lo >> (b * (jv.L - 1))) & dmask) : digit(w, b, jv.L, 0);
            const int s0 = (NARROW || jv.narrow) ? digit_sum64(w.lo, jv) : digit_sum(w, jv);
            spre = s0 - v0 - d0;
            const bool neck_first = divides_L(jv, p), neck_row = divides_L(jv, jv.L - 1);
            int lastv = v0, lastd = d0;
            for (int v = v0; v <= vmax; ++v) {
                // row v: words (v, dlo .. dhi); every one a necklace but
                // perhaps the first; candidates: the digit sums with a role
                const int dlo = v == v0 ? d0 : a0;
                int dhi = K;
                bool cut = false;
                const int64_t lim = (int64_t)xend - ((int64_t)v << b) - 1;  // xend = 2^32 - 1: no cut
                if (lim < (int64_t)dhi) {
                    dhi = (int)lim;
                    cut = true;
                }
                if (dhi < dlo) break;
                const int n = dhi - dlo + 1;
                const bool first_neck = v == v0 ? neck_first : neck_row;
                necklaces += (unsigned long long)(n - (first_neck ? 0 : 1));
                uint64_t rm = role_bits(tbits[job], spre + v + dlo, n);
                if (!first_neck) rm &= ~1ull;
                cmask |= rm << ((v - v0) * kk + dlo);
                lastv = v;
                lastd = dhi;
                if (cut) break;
            }
            // the block's last word, then its successor
            w.lo = (w.lo & ~m2) | ((uint64_t)lastv << b) | (uint64_t)lastd;
            int np;
            if (NARROW || jv.narrow) {
                uint64_t wl = w.lo;
                np = fkm_next64(wl, jv);
                w.lo = wl;
            } else {
                np = fkm_next(w, jv);
            }
            if (np == 0 || !(NARROW ? w.lo < end.lo : lt(w, end))) {
                have = false;
                a.cur[win] = a.end[win];
                win = take();
                active = win < a.nwin;
            } else {
                p = np;
            }
        }
        // queue the block's candidates, one per lane per round; write the
        // queue out from kFlushAt
        while (__any_sync(0xFFFFFFFFu, cmask != 0)) {
            const bool has = cmask != 0;
            const int t = has ? __ffsll((long long)cmask) - 1 : 0;
            cmask &= cmask - 1ull;
            const uint32_t want = __ballot_sync(0xFFFFFFFFu, has);
            if (has) {
                const int slot = qlen + __popc(want & lt_mask);
                const int v = v0 + t / kk, d = t % kk;
                W128 cand = w0;
                const int b = jv.b;
                const uint64_t m2 = (1ull << (2 * b)) - 1ull;
                cand.lo = (cand.lo & ~m2) | ((uint64_t)v << b) | (uint64_t)d;
                q_word[wq][slot] = to_u4(cand);
                q_role[wq][slot] = role_tab[job][spre + v + d];
                q_job[wq][slot] = (uint8_t)job;
            }
            qlen += __popc(want);
            if (qlen >= kFlushAt) flush();
        }
        // every kCapCheck steps: leave a window whose job reached its soft
        // capacity (by the count loaded kCapCheck steps ago), then load the
        // count afresh
        if ((step & (kCapCheck - 1)) == 0 && active && have) {
            if (seen_job == job && (int64_t)seen_count >= jobs[job].soft_cap) {
                a.cur[win] = to_u4(w);
                have = false;
                parked_any = true;
                win = take();
                active = win < a.nwin;
            } else {
                seen_count = *reinterpret_cast<volatile unsigned long long*>(jobs[job].count);
                seen_job = job;
            }
        }
    }
    flush();
    if (parked_any) *a.incomplete = 1;
    if (necklaces) atomicAdd(jobs[job].necklaces, necklaces);
}

template <bool NARROW>
cudaError_t launch_enumerate_t(const EnumArgs& a, int num_sms, cudaStream_t st, int variant) {
    // one wave of resident blocks: windows are handed out dynamically
    static int resident[3] = {0, 0, 0};
    const int vi = variant == 1 ? 1 : variant == 2 ? 2 : 0;
    int& per_sm = resident[vi];
    if (per_sm == 0) {
        cudaError_t e = vi == 1   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, enumerate_kernel<8, NARROW>, 256, 0)
                        : vi == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, enumerate_kernel<3, NARROW>, 256, 0)
                                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, enumerate_kernel<4, NARROW>, 256, 0);
        if (e != cudaSuccess || per_sm < 1) per_sm = 1;
    }
    int64_t blocks = (a.nwin + 255) / 256;
    const int64_t maxb = (int64_t)num_sms * per_sm;
    if (blocks > maxb) blocks = maxb;
    if (vi == 1)
        enumerate_kernel<8, NARROW><<<(unsigned)blocks, 256, 0, st>>>(a);
    else if (vi == 2)
        enumerate_kernel<3, NARROW><<<(unsigned)blocks, 256, 0, st>>>(a);
    else
        enumerate_kernel<4, NARROW><<<(unsigned)blocks, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_enumerate(const EnumArgs& a, int num_sms, cudaStream_t st, int variant) {
    if (a.nwin <= 0) return cudaSuccess;
    if (a.njobs < 1 || a.njobs > kMaxEnumJobs) return cudaErrorInvalidValue;
    return a.narrow ? launch_enumerate_t<true>(a, num_sms, st, variant)
                    : launch_enumerate_t<false>(a, num_sms, st, variant);
}

}  // namespace gp
