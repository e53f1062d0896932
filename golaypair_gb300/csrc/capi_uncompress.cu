// capi_uncompress.cu -- uncompression stage (kernel (d), first half).
//
// Replaces uncompress_pipeline / uncompress_recursive
// (src/core/uncompression/uncompression.cpp:32-210) and the GPU stub it can
// dispatch to (src/core/uncompression/gpu/uncompress_gpu.cpp:17-92, whose
// kernel computes nothing).  The reference, per compressed pair (a, b):
// expands each side to every sequence of the new compression (entry i's
// partition fills positions i, i+L, i+2L, ...), keeps the expansions whose
// PSD passes the filter, writes them with their signatures to two scratch
// files, sorts both and merge-joins them on the signature string with an
// exact PAF check.  Here many pairs are uncompressed per launch sequence:
//
// 1. Plan (uncompression.cpp:88-142): one partition table per letter and the
//    first entry's partitions reduced to rotation/reversal minima (host, once
//    per level); the reference's rotation of each side, its rows and counts
//    (ux_plan_kernel, one thread per side).  A side is a mixed-radix number
//    over its positions; the expansion of rank t has digit d_i at position i.
//
// 2. ux_scan_kernel (fused expansion + PSD filter).  The DFT of an expansion
//    is a sum of per-position terms, X_k = sum_i C_i(d_i, k) with
//    C_i(d, k) = sum_q v_q(d) w^((i + L q) k), w = exp(-2 pi i / L').  Bins
//    k that are multiples of the ratio r = c / c' do not depend on the
//    expansion (they are the compressed sequence's DFT) and are checked once
//    per side when it is planned.  For the other bins a thread adds the terms of the
//    side's leading free positions once (its "prefix"), then walks a table of
//    precomputed sums over the trailing free positions (the "suffix", up to a
//    few hundred combinations in shared memory): one packed fp32 add per bin
//    and |X|^2 per expansion.  A rigorous bound of the fp32 rounding error
//    sorts every expansion into sure pass, sure reject, or unsure.  A batch
//    scans each distinct side once: a side repeats in the pairs of its
//    signature group, and its survivors do not depend on the pair or role.
// 3. ux_recheck_kernel: unsure expansions in FP64 (one warp per expansion,
//    lanes over bins), the reference's filter psd[k] <= 2n - paf + 0.001.
// 4. The join.  For a complementary pair, PAF_a(s) + PAF_b(s) = paf * c'
//    (src/utils/golay.cpp:27-44) implies psd_a(k) + psd_b(k) = 2n - paf at
//    every k != 0, so the a-side's inverted signature equals the b-side's
//    plain one: every pair the reference writes joins on the exact integer
//    PAF vectors (a: paf*c' - PAF_a, b: PAF_b).  ux_key_kernel hashes those
//    vectors and buckets the survivors by (pair, hash bits), one entry per
//    pair and role that uses the survivor's side;
//    ux_join_kernel matches each bucket in a shared-memory hash table and
//    verifies the PAF sums exactly.  No signature is computed on the device.
// 5. Host: the few matched pairs get their FP64 signatures; a pair is kept
//    when the two signature strings are equal (the reference's join key),
//    and the pairs of each input pair are written in the order of the
//    reference's sorted files (a line, then b line), input pairs in order.
#include <algorithm>
#include <stdexcept>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <type_traits>
#include <vector>

#include "ctx.h"
#include "host_math.h"
#include "prims.h"

namespace {

constexpr int kMaxL = 64;          // compressed length
constexpr int kMaxLnew = 128;      // uncompressed length
constexpr int kMaxRows = 32;       // letters + first-entry lists
constexpr int kScanThreads = 256;  // prefixes per scan unit
constexpr int kRankBits = 40;      // survivor word: side << 40 | rank (the batch's distinct side)
constexpr uint64_t kRankMask = (uint64_t(1) << kRankBits) - 1;
constexpr int kMaxSidesPerBatch = 1 << 23;
constexpr int kBucketTarget = 512;  // survivors per join bucket (mean)
constexpr int kJoinTab = 4096;      // shared hash slots of the join kernel
constexpr int kJoinMaxB = kJoinTab / 2;
constexpr size_t kScanSmemBudget = 96 * 1024;

// ------------------------------------------------------------ device side

struct LevelDev {
    int L, r, Lnew, H, nrows, dmax, np;  // np: bin pairs of the scan's template
    int nb;                               // varying bins
    int one_bit;                          // new alphabet is {-1, 1} and Lnew <= 64
    int target;                           // paf * c'
    const int* cnt;                       // [nrows] choices per row
    const int8_t* vals;                   // [nrows][dmax][r] values of each choice
    const float4* ctab;                   // [L][nrows][dmax][np]: (re 2p, re 2p+1, im 2p, im 2p+1)
    const double2* ctab64;                // [L][nrows][dmax][2 np]
    const uint8_t* side_rows;             // [sides][L] row of each position
};

__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// digits of a rank: position L-1 least significant, positions with one
// choice contribute nothing
__device__ __forceinline__ void decode_rank(uint64_t rank, const uint8_t* rows, const int* cnt, int L, uint8_t* d) {
    for (int i = L - 1; i >= 0; --i) {
        const uint32_t c = (uint32_t)cnt[rows[i]];
        if (c == 1) {
            d[i] = 0;
        } else if (rank >> 32) {
            d[i] = (uint8_t)(rank % c);
            rank /= c;
        } else {
            const uint32_t q = (uint32_t)rank / c;
            d[i] = (uint8_t)((uint32_t)rank - q * c);
            rank = q;
        }
    }
}

struct ScanArgs {
    LevelDev lv;
    const uint64_t* unit_begin;    // [sides + 1]
    const uint64_t* prefix_count;  // [sides]
    const uint32_t* nsuf;          // [sides] free positions in the suffix table
    int n_sides;
    uint64_t n_units;
    float thr_lo, thr_hi;          // sure pass below, sure reject above
    uint64_t* surv;
    uint64_t surv_cap;
    uint64_t* unsure;
    uint64_t unsure_cap;
    unsigned long long* counters;  // [0] survivors [1] unsure [2] matches
    uint32_t* side_count;          // survivors per side
    int* status;
};

__device__ __forceinline__ void flag_overflow(int* status) { atomicCAS(status, 0, GP_KSTATUS_OVERFLOW); }

// CTAs per SM the registers are capped for.  Up to 8 varying bins (one
// phase): 64 registers, four CTAs.  Two phases (below), up to 24 bins: three
// CTAs, 80 registers, no spills (at order 57, 20 bins: 8.5-8.6 s for the
// whole file against 9.7-9.8 s at four CTAs with spills, and 9.9 s for the
// one-phase scan at four CTAs).  Wider prefix sums need more registers.
constexpr int scan_min_ctas(int np) { return np <= 4 ? 4 : np <= 12 ? 3 : np <= 24 ? 2 : 1; }

template <int V>
using Int = std::integral_constant<int, V>;

// NA: bin pairs of the scan's first phase (0: one phase over all NP)
template <int NP, int NA>
__global__ void __launch_bounds__(kScanThreads, scan_min_ctas(NP)) ux_scan_kernel(ScanArgs a) {
    extern __shared__ float4 smem[];
    // the queue of phase B, per warp: (suffix | lane << 16) and the phase-A max
    __shared__ uint32_t s_qitem[kScanThreads / 32][NA ? 96 : 1];
    __shared__ float s_qmax[kScanThreads / 32][NA ? 96 : 1];
    __shared__ int s_nfree, s_npre;
    __shared__ uint32_t s_scount;
    __shared__ int s_pos[kMaxL], s_cnt[kMaxL], s_coff[kMaxL];
    __shared__ float4 s_F[NP];
    const LevelDev& lv = a.lv;
    float4* s_S = smem;  // [scount][NP] suffix sums, then the free positions' terms
    float4* s_C = smem;  // placed after the suffix table when a side starts
    const int tid = threadIdx.x, lane = tid & 31;
    // a contiguous share of the units per CTA: consecutive units mostly
    // belong to one side, so its tables are built once and no barrier
    // separates the units of a side
    const uint64_t u_begin = a.n_units * blockIdx.x / gridDim.x;
    const uint64_t u_end = a.n_units * (blockIdx.x + 1) / gridDim.x;
    int side = -1;  // the same in every thread of the CTA
    uint32_t scount = 1;
    int npre = 0;
    for (uint64_t u = u_begin; u < u_end; ++u) {
        // the side of unit u: the last side whose first unit is <= u
        int sd = side;
        if (sd < 0) {
            int lo = 0, hi = a.n_sides - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (a.unit_begin[mid] <= u)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            sd = lo;
        }
        while (sd + 1 < a.n_sides && a.unit_begin[sd + 1] <= u) ++sd;
        const uint8_t* rows = lv.side_rows + (size_t)sd * lv.L;
        if (sd != side) {
            __syncthreads();  // every thread is done with the previous side's tables
            side = sd;
            if (tid == 0) {
                int nfree = 0, off = 0;
                for (int i = 0; i < lv.L; ++i) {
                    const int c = lv.cnt[rows[i]];
                    if (c > 1) {
                        s_pos[nfree] = i;
                        s_cnt[nfree] = c;
                        s_coff[nfree] = off;
                        off += c * NP;
                        ++nfree;
                    }
                }
                const int nsuf = (int)a.nsuf[side];
                uint32_t sc = 1;
                for (int f = nfree - nsuf; f < nfree; ++f) sc *= (uint32_t)s_cnt[f];
                s_nfree = nfree;
                s_npre = nfree - nsuf;
                s_scount = sc;
            }
            __syncthreads();
            scount = s_scount;
            npre = s_npre;
            s_C = smem + (size_t)scount * NP;
            const int nfree = s_nfree;
            // the free positions' terms, then the fixed positions' sum
            for (int f = 0; f < nfree; ++f) {
                const int i = s_pos[f], c = s_cnt[f];
                const float4* src = lv.ctab + ((size_t)(i * lv.nrows + rows[i]) * lv.dmax) * NP;
                for (int k = tid; k < c * NP; k += kScanThreads) s_C[s_coff[f] + k] = src[k];
            }
            if (tid < NP) {
                float4 F = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int i = 0; i < lv.L; ++i) {
                    if (lv.cnt[rows[i]] != 1) continue;
                    const float4 t = lv.ctab[((size_t)(i * lv.nrows + rows[i]) * lv.dmax) * NP + tid];
                    F.x += t.x;
                    F.y += t.y;
                    F.z += t.z;
                    F.w += t.w;
                }
                s_F[tid] = F;
            }
            __syncthreads();
            // suffix table: every combination of the trailing free positions
            for (uint32_t k = tid; k < scount * NP; k += kScanThreads) {
                const uint32_t j = k / NP, p = k - j * NP;
                uint32_t rem = j;
                float4 S = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int f = nfree - 1; f >= npre; --f) {
                    const uint32_t c = (uint32_t)s_cnt[f];
                    const uint32_t q = rem / c;
                    const uint32_t d = rem - q * c;
                    rem = q;
                    const float4 t = s_C[s_coff[f] + d * NP + p];
                    S.x += t.x;
                    S.y += t.y;
                    S.z += t.z;
                    S.w += t.w;
                }
                s_S[j * NP + p] = S;
            }
            __syncthreads();
        }
        const uint64_t pidx = (u - a.unit_begin[side]) * (uint64_t)kScanThreads + (uint64_t)tid;
        const bool active = pidx < a.prefix_count[side];
        float2 Pr[NP], Pi[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const float4 F = s_F[p];
            Pr[p] = make_float2(F.x, F.y);
            Pi[p] = make_float2(F.z, F.w);
        }
        if (active) {  // the prefix: digits of pidx over the leading free positions
            uint64_t rem = pidx;
            for (int f = npre - 1; f >= 0; --f) {
                const uint32_t c = (uint32_t)s_cnt[f];
                uint32_t d;
                if (rem >> 32) {
                    d = (uint32_t)(rem % c);
                    rem /= c;
                } else {
                    const uint32_t q = (uint32_t)rem / c;
                    d = (uint32_t)rem - q * c;
                    rem = q;
                }
                const float4* tp = s_C + s_coff[f] + d * NP;
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    const float4 v = tp[p];
                    Pr[p] = __fadd2_rn(Pr[p], make_float2(v.x, v.y));
                    Pi[p] = __fadd2_rn(Pi[p], make_float2(v.z, v.w));
                }
            }
        }
        const uint64_t unit_pidx0 = (u - a.unit_begin[side]) * (uint64_t)kScanThreads + (uint64_t)(tid & ~31);
        const float init = active ? 0.f : __int_as_float(0x7f800000);
        // max p over bin pairs [P0, P1) of prefix + suffix j
        auto eval_range = [&](uint32_t j, auto p0c, auto p1c, float m0, float m1) {
            constexpr int P0 = decltype(p0c)::value, P1 = decltype(p1c)::value;
            const float4* S = s_S + j * NP;
#pragma unroll
            for (int p = P0; p < P1; ++p) {
                const float4 s = S[p];
                const float2 xr = __fadd2_rn(Pr[p], make_float2(s.x, s.y));
                const float2 xi = __fadd2_rn(Pi[p], make_float2(s.z, s.w));
                const float2 q = __ffma2_rn(xr, xr, __fmul2_rn(xi, xi));
                if (p & 1)
                    m1 = max3f(m1, q.x, q.y);
                else
                    m0 = max3f(m0, q.x, q.y);
            }
            return fmaxf(m0, m1);
        };
        // survivors (sure passes) and the band around the bound (unsure),
        // appended with one atomic per warp and list; rank: the expansion's
        // rank within its side
        auto emit = [&](float m, uint64_t rank) {
            const bool cand = m <= a.thr_hi;
            const unsigned bal = __ballot_sync(0xFFFFFFFFu, cand);
            if (!bal) return;
            const bool sure = cand && m < a.thr_lo;
            const unsigned bs = __ballot_sync(0xFFFFFFFFu, sure);
            const unsigned bu = bal & ~bs;
            unsigned long long base_s = 0, base_u = 0;
            if (lane == 0) {
                if (bs) {
                    base_s = atomicAdd(&a.counters[0], (unsigned long long)__popc(bs));
                    atomicAdd(&a.side_count[side], (uint32_t)__popc(bs));
                }
                if (bu) base_u = atomicAdd(&a.counters[1], (unsigned long long)__popc(bu));
            }
            base_s = __shfl_sync(0xFFFFFFFFu, base_s, 0);
            base_u = __shfl_sync(0xFFFFFFFFu, base_u, 0);
            if (cand) {
                const unsigned lt = (1u << lane) - 1u;
                const uint64_t val = ((uint64_t)side << kRankBits) | rank;
                if (sure) {
                    const unsigned long long pos = base_s + __popc(bs & lt);
                    if (pos < a.surv_cap)
                        a.surv[pos] = val;
                    else
                        flag_overflow(a.status);
                } else {
                    const unsigned long long pos = base_u + __popc(bu & lt);
                    if (pos < a.unsure_cap)
                        a.unsure[pos] = val;
                    else
                        flag_overflow(a.status);
                }
            }
        };
        if constexpr (NA == 0) {
            const uint64_t rank0 = pidx * (uint64_t)scount;
            uint32_t j = 0;
            for (; j + 2 <= scount; j += 2) {  // two independent suffixes per step
                const float ma = eval_range(j, Int<0>{}, Int<NP>{}, init, init);
                const float mb = eval_range(j + 1, Int<0>{}, Int<NP>{}, init, init);
                if (__any_sync(0xFFFFFFFFu, ma <= a.thr_hi || mb <= a.thr_hi)) {
                    emit(ma, rank0 + j);
                    emit(mb, rank0 + j + 1);
                }
            }
            if (j < scount) emit(eval_range(j, Int<0>{}, Int<NP>{}, init, init), rank0 + j);
        } else {
            // Two phases.  Phase A: the first NA bin pairs of every (prefix,
            // suffix); most expansions are already above the bound there.
            // The others are queued per warp as (suffix, lane); phase B takes
            // 32 queued expansions at a time, one per lane, fetches the
            // prefix's remaining bin pairs from the queuing lane's registers
            // by shuffle and finishes the max.  Same max, same verdicts.
            uint32_t* qi = s_qitem[tid >> 5];
            float* qm = s_qmax[tid >> 5];
            int qn = 0;  // queued entries (the same in every lane)
            auto phase_b = [&](int n) {
                const bool have = lane < n;
                const uint32_t item = have ? qi[lane] : (uint32_t)lane << 16;
                const uint32_t j = item & 0xFFFFu;
                const int src = (int)(item >> 16);
                float m0 = have ? qm[lane] : __int_as_float(0x7f800000), m1 = m0;
                const float4* S = s_S + j * NP;
#pragma unroll
                for (int p = NA; p < NP; ++p) {
                    const float2 pr = make_float2(__shfl_sync(0xFFFFFFFFu, Pr[p].x, src),
                                                  __shfl_sync(0xFFFFFFFFu, Pr[p].y, src));
                    const float2 pi = make_float2(__shfl_sync(0xFFFFFFFFu, Pi[p].x, src),
                                                  __shfl_sync(0xFFFFFFFFu, Pi[p].y, src));
                    const float4 sv = S[p];
                    const float2 xr = __fadd2_rn(pr, make_float2(sv.x, sv.y));
                    const float2 xi = __fadd2_rn(pi, make_float2(sv.z, sv.w));
                    const float2 q = __ffma2_rn(xr, xr, __fmul2_rn(xi, xi));
                    if (p & 1)
                        m1 = max3f(m1, q.x, q.y);
                    else
                        m0 = max3f(m0, q.x, q.y);
                }
                emit(fmaxf(m0, m1), (unit_pidx0 + (uint64_t)src) * scount + j);
            };
            auto push = [&](float m, uint32_t j) {
                const bool c = m <= a.thr_hi;
                const unsigned b = __ballot_sync(0xFFFFFFFFu, c);
                if (c) {
                    const int slot = qn + __popc(b & ((1u << lane) - 1u));
                    qi[slot] = j | ((uint32_t)lane << 16);
                    qm[slot] = m;
                }
                qn += __popc(b);
            };
            auto drain = [&]() {  // phase B over the first 32 entries; the rest move to the front
                __syncwarp();
                phase_b(32);
                __syncwarp();
                const int rest = qn - 32;
                uint32_t i0 = 0, i1 = 0;
                float m0 = 0.f, m1 = 0.f;
                if (lane < rest) {
                    i0 = qi[32 + lane];
                    m0 = qm[32 + lane];
                }
                if (lane + 32 < rest) {
                    i1 = qi[64 + lane];
                    m1 = qm[64 + lane];
                }
                __syncwarp();
                if (lane < rest) {
                    qi[lane] = i0;
                    qm[lane] = m0;
                }
                if (lane + 32 < rest) {
                    qi[32 + lane] = i1;
                    qm[32 + lane] = m1;
                }
                qn = rest;
                __syncwarp();
            };
            uint32_t j = 0;
            for (; j + 2 <= scount; j += 2) {  // two independent suffixes per step
                const float ma = eval_range(j, Int<0>{}, Int<NA>{}, init, init);
                const float mb = eval_range(j + 1, Int<0>{}, Int<NA>{}, init, init);
                push(ma, j);
                push(mb, j + 1);
                while (qn >= 32) drain();  // below 32 again: the next step's 64 pushes fit the 96 slots
            }
            if (j < scount) {
                push(eval_range(j, Int<0>{}, Int<NA>{}, init, init), j);
                while (qn >= 32) drain();
            }
            if (qn > 0) {
                __syncwarp();
                phase_b(qn);
                qn = 0;
                __syncwarp();
            }
        }
    }
}

// The unsure expansions in FP64: each lane decodes one expansion's digits
// into shared memory, then the warp takes its 32 expansions in turn with
// lanes over the bins (the reference's filter, fourier.cpp:45-52).
struct RecheckArgs {
    LevelDev lv;
    double thr;
    const uint64_t* unsure;
    uint64_t unsure_cap;
    uint64_t* surv;
    uint64_t surv_cap;
    unsigned long long* counters;
    uint32_t* side_count;
    int* status;
};

constexpr int kRecheckWarps = 4;

__global__ void __launch_bounds__(kRecheckWarps * 32) ux_recheck_kernel(RecheckArgs a) {
    __shared__ uint8_t s_dig[kRecheckWarps][32][kMaxL];
    const LevelDev& lv = a.lv;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t n = min((uint64_t)a.counters[1], a.unsure_cap);
    const uint64_t gw = (uint64_t)blockIdx.x * kRecheckWarps + warp, nw = (uint64_t)gridDim.x * kRecheckWarps;
    for (uint64_t base = gw * 32; base < n; base += nw * 32) {
        uint64_t val = 0;
        if (base + lane < n) {
            val = a.unsure[base + lane];
            decode_rank(val & kRankMask, lv.side_rows + (size_t)(val >> kRankBits) * lv.L, lv.cnt, lv.L,
                        s_dig[warp][lane]);
        }
        __syncwarp();
        const int m = (int)min((uint64_t)32, n - base);
        for (int e = 0; e < m; ++e) {
            const uint64_t v = __shfl_sync(0xFFFFFFFFu, val, e);
            const int side = (int)(v >> kRankBits);
            const uint8_t* rows = lv.side_rows + (size_t)side * lv.L;
            double pmax = 0.0;
            for (int b = lane; b < lv.nb; b += 32) {
                double re = 0.0, im = 0.0;
                for (int i = 0; i < lv.L; ++i) {
                    const double2 t =
                        lv.ctab64[((size_t)(i * lv.nrows + rows[i]) * lv.dmax + s_dig[warp][e][i]) * (2 * lv.np) + b];
                    re += t.x;
                    im += t.y;
                }
                pmax = fmax(pmax, re * re + im * im);
            }
            for (int o = 16; o; o >>= 1) pmax = fmax(pmax, __shfl_xor_sync(0xFFFFFFFFu, pmax, o));
            if (lane == 0 && pmax <= a.thr) {
                const unsigned long long pos = atomicAdd(&a.counters[0], 1ull);
                atomicAdd(&a.side_count[side], 1u);
                if (pos < a.surv_cap)
                    a.surv[pos] = v;
                else
                    flag_overflow(a.status);
            }
        }
        __syncwarp();
    }
}

// Values of an expansion at its Lnew positions.
__device__ __forceinline__ void expand_values(const LevelDev& lv, uint64_t val, int8_t* x) {
    uint8_t d[kMaxL];
    const uint8_t* rows = lv.side_rows + (size_t)(val >> kRankBits) * lv.L;
    decode_rank(val & kRankMask, rows, lv.cnt, lv.L, d);
    for (int i = 0; i < lv.L; ++i) {
        const int8_t* v = lv.vals + ((size_t)rows[i] * lv.dmax + d[i]) * lv.r;
        for (int q = 0; q < lv.r; ++q) x[i + lv.L * q] = v[q];
    }
}

// PAF(s), s = 1 .. H, of an expansion (src/utils/golay.cpp:27-33).
__device__ __forceinline__ void expansion_paf(const LevelDev& lv, uint64_t val, int* paf) {
    int8_t x[kMaxLnew];
    expand_values(lv, val, x);
    const int N = lv.Lnew;
    if (lv.one_bit) {
        uint64_t w = 0;
        for (int j = 0; j < N; ++j) w |= (uint64_t)(x[j] > 0) << j;
        const uint64_t mask = N == 64 ? ~0ull : ((1ull << N) - 1ull);
        for (int s = 1; s <= lv.H; ++s) {
            const uint64_t rot = ((w >> s) | (w << (N - s))) & mask;  // bit j = bit j + s of w
            paf[s - 1] = N - 2 * __popcll(w ^ rot);
        }
        return;
    }
    for (int s = 1; s <= lv.H; ++s) {
        int acc = 0, j2 = s;
        for (int j = 0; j < N; ++j) {
            acc += (int)x[j] * (int)x[j2];
            if (++j2 == N) j2 = 0;
        }
        paf[s - 1] = acc;
    }
}

__device__ __forceinline__ uint64_t mix64(uint64_t h) {
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    h *= 0xc4ceb9fe1a85ec53ull;
    h ^= h >> 33;
    return h;
}

// join key of a survivor's PAF vector in its role: as the a-side of a pair
// it hashes paf*c' - PAF_a(s), as the b-side PAF_b(s); complementary pairs
// have equal keys
__device__ __forceinline__ uint64_t join_key(const LevelDev& lv, const int* paf, bool is_a) {
    uint64_t h = 0x243f6a8885a308d3ull;
    for (int s = 0; s < lv.H; ++s) {
        const int v = is_a ? lv.target - paf[s] : paf[s];
        h = (h ^ (uint64_t)(uint32_t)v) * 0x100000001b3ull;
    }
    return mix64(h);
}

// Survivor words carry the batch's unique side index: equal compressed
// sides (a side repeats in the pairs of its signature group) are expanded
// and filtered once.  Each survivor yields one join entry per use of its
// side, a use being (pair, role) with role 1 for the b-side.
struct KeyArgs {
    LevelDev lv;
    const uint64_t* surv;
    uint64_t n;
    const uint32_t* use_beg;    // [unique sides + 1] first use of each side
    const uint32_t* uses;       // pair << 1 | role
    const uint8_t* pair_lg;     // [pairs] log2 buckets of the pair (255: pair skipped)
    const uint32_t* pair_base;  // [pairs] first bucket of the pair
    uint64_t* keys;             // [entries]
    uint32_t* bucket;           // [entries]
    uint32_t* eidx;             // [entries] survivor index | role << 31
    uint64_t entry_cap;
    unsigned long long* ecount;
    uint32_t* bcount;
    int* status;
};

// Entry i is survivor i's first use (bucket ~0 when its side has none in a
// pair that can match); further uses, rare, take slots from n on, reserved
// once per warp.
__global__ void ux_key_kernel(KeyArgs a) {
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < a.n; i0 += stride) {
        const uint64_t i = i0 + lane;
        uint64_t v = 0;
        uint32_t j0 = 0, j1 = 0, cnt = 0;
        if (i < a.n) {
            v = a.surv[i];
            const uint32_t u = (uint32_t)(v >> kRankBits);
            j0 = a.use_beg[u];
            j1 = a.use_beg[u + 1];
            for (uint32_t j = j0; j < j1; ++j) cnt += a.pair_lg[a.uses[j] >> 1] != 255 ? 1u : 0u;
        }
        uint64_t extra = 0;  // slot of this lane's second use
        if (__any_sync(0xFFFFFFFFu, cnt > 1)) {
            const uint32_t mine = cnt > 1 ? cnt - 1 : 0u;
            uint32_t incl = mine;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
                if (lane >= d) incl += t;
            }
            const uint32_t tot = __shfl_sync(0xFFFFFFFFu, incl, 31);
            unsigned long long base = 0;
            if (lane == 31) base = atomicAdd(a.ecount, (unsigned long long)tot);
            base = __shfl_sync(0xFFFFFFFFu, base, 31);
            extra = a.n + base + (incl - mine);
        }
        if (i >= a.n) continue;
        if (!cnt) {
            a.bucket[i] = 0xFFFFFFFFu;
            continue;
        }
        int paf[kMaxLnew / 2];
        expansion_paf(a.lv, v, paf);
        uint64_t e = i;
        for (uint32_t j = j0; j < j1; ++j) {
            const uint32_t code = a.uses[j], pair = code >> 1, role = code & 1u;
            const int lg = a.pair_lg[pair];
            if (lg == 255) continue;
            if (e >= a.entry_cap) {
                flag_overflow(a.status);
                break;
            }
            const uint64_t h = join_key(a.lv, paf, role == 0);
            const uint32_t b = a.pair_base[pair] + (lg ? (uint32_t)(h >> (64 - lg)) : 0u);
            a.keys[e] = h;
            a.bucket[e] = b;
            a.eidx[e] = (uint32_t)i | (role << 31);
            atomicAdd(&a.bcount[b], 1u);
            e = e == i ? extra : e + 1;
        }
    }
}

__global__ void ux_scatter_kernel(const uint64_t* keys, const uint32_t* bucket, const uint32_t* eidx, uint64_t n,
                                  const uint32_t* boff, uint32_t* bcur, uint64_t* ent_h, uint32_t* ent_i) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = bucket[e];
        if (b == 0xFFFFFFFFu) continue;
        const uint32_t pos = boff[b] + atomicAdd(&bcur[b], 1u);
        ent_h[pos] = keys[e];
        ent_i[pos] = eidx[e];  // bit 31: b-side
    }
}

struct JoinArgs {
    LevelDev lv;
    const uint64_t* surv;
    const uint64_t* ent_h;
    const uint32_t* ent_i;
    const uint32_t* boff;
    const uint32_t* bcount;
    uint32_t n_buckets;
    const uint32_t* pair_base;  // [pairs] first bucket (non-decreasing; a skipped pair has none)
    uint32_t n_pairs;
    uint64_t* matches;  // (a survivor word, b survivor word), side fields 2 pair and 2 pair + 1
    uint64_t match_cap;
    unsigned long long* counters;
    int* status;
};

// the pair that owns bucket bk: the last pair whose first bucket is <= bk
// (a skipped pair shares its base with the next pair and owns no bucket)
__device__ __forceinline__ uint32_t bucket_pair(const JoinArgs& a, uint32_t bk) {
    uint32_t lo = 0, hi = a.n_pairs;  // answer in [lo, hi)
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (a.pair_base[mid] <= bk)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void verify_and_emit(const JoinArgs& a, uint32_t ia, uint32_t ib, uint32_t pair) {
    int pa[kMaxLnew / 2], pb[kMaxLnew / 2];
    const uint64_t va = a.surv[ia], vb = a.surv[ib];
    expansion_paf(a.lv, va, pa);
    expansion_paf(a.lv, vb, pb);
    for (int s = 0; s < a.lv.H; ++s)
        if (pa[s] + pb[s] != a.lv.target) return;
    const unsigned long long pos = atomicAdd(&a.counters[2], 1ull);
    if (pos < a.match_cap) {
        a.matches[2 * pos] = ((uint64_t)(2 * pair) << kRankBits) | (va & kRankMask);
        a.matches[2 * pos + 1] = ((uint64_t)(2 * pair + 1) << kRankBits) | (vb & kRankMask);
    } else {
        flag_overflow(a.status);
    }
}

// One bucket per block iteration: b-side entries into a shared hash table
// keyed by the low hash bits (the bucket came from the high ones), a-side
// entries probe it.  A bucket too large for the table is joined pairwise.
__global__ void __launch_bounds__(256) ux_join_kernel(JoinArgs a) {
    __shared__ uint32_t tab[kJoinTab];
    for (uint32_t bk = blockIdx.x; bk < a.n_buckets; bk += gridDim.x) {
        const uint32_t n = a.bcount[bk], base = a.boff[bk];
        const uint32_t pair = n ? bucket_pair(a, bk) : 0u;
        __syncthreads();
        if (n > kJoinMaxB) {  // rare: quadratic over the bucket
            for (uint64_t w = threadIdx.x; w < (uint64_t)n * n; w += blockDim.x) {
                const uint32_t e = (uint32_t)(w / n), f = (uint32_t)(w % n);
                const uint32_t ie = a.ent_i[base + e], jf = a.ent_i[base + f];
                if ((ie >> 31) || !(jf >> 31) || a.ent_h[base + e] != a.ent_h[base + f]) continue;
                verify_and_emit(a, ie & 0x7FFFFFFFu, jf & 0x7FFFFFFFu, pair);
            }
            continue;
        }
        for (int k = threadIdx.x; k < kJoinTab; k += blockDim.x) tab[k] = 0;
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
            if (!(a.ent_i[base + e] >> 31)) continue;
            uint32_t slot = (uint32_t)a.ent_h[base + e] & (kJoinTab - 1);
            while (atomicCAS(&tab[slot], 0u, e + 1) != 0u) slot = (slot + 1) & (kJoinTab - 1);
        }
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
            const uint32_t ie = a.ent_i[base + e];
            if (ie >> 31) continue;
            const uint64_t h = a.ent_h[base + e];
            uint32_t slot = (uint32_t)h & (kJoinTab - 1);
            for (uint32_t t; (t = tab[slot]) != 0u; slot = (slot + 1) & (kJoinTab - 1))
                if (a.ent_h[base + t - 1] == h) verify_and_emit(a, ie, a.ent_i[base + t - 1] & 0x7FFFFFFFu, pair);
        }
    }
}

// ------------------------------------------------------------ side planning
// uncompression.cpp:107-142, one thread per side of a compressed pair:
//  * the rotation: the first distinct letter (ascending value) with the most
//    partitions; the sequence is rotated left by i whenever position i holds
//    that letter, on the already rotated sequence (the reference's loop);
//  * the rows: the letter's index at every position, plus A at position 0
//    (the first entry's partitions reduced to rotation/reversal minima);
//  * the bins that are multiples of r: the compressed sequence's DFT, the
//    same for every expansion, checked once in FP64 (no fused multiply-add,
//    as the host's loop);
//  * the expansion count and the split into scan prefixes and the suffix
//    table (the trailing free positions whose combinations fit smax).
struct PlanOut {
    uint64_t total;         // expansions (0: none can pass)
    uint64_t prefix_count;  // total / suffix_count
    uint32_t nsuf, suffix_count, free_choices, overflow;
};

struct PlanArgs {
    const uint8_t* seqs;     // [sides][L] letter indices (validated on the host)
    int n_sides, L, A, Lnew, n_cbins, smax;
    const int* cbins;        // [n_cbins]
    const int* cnt;          // [2A] choices per row
    const double2* tw;       // [Lnew] (cos, sin)(2 pi m / Lnew)
    const int8_t* letter;    // [A] value of each letter index
    const uint8_t* asc;      // [A] letter indices by ascending value
    double thr;
    uint8_t* rows;           // [sides][L]
    PlanOut* out;            // [sides]
};

__global__ void __launch_bounds__(128) ux_plan_kernel(PlanArgs a) {
    const int64_t sid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (sid >= a.n_sides) return;
    const int L = a.L;
    uint8_t x[kMaxL], y[kMaxL];
    uint32_t present = 0;
    for (int i = 0; i < L; ++i) {
        x[i] = a.seqs[sid * L + i];
        present |= 1u << x[i];
    }
    int best = x[0], best_n = 0;
    for (int t = 0; t < a.A; ++t) {
        const int e = a.asc[t];
        if (!((present >> e) & 1u)) continue;
        if (a.cnt[e] > best_n) {
            best_n = a.cnt[e];
            best = e;
        }
    }
    for (int i = 0; i < L; ++i) {
        if (x[i] != best) continue;
        for (int j = 0; j < L; ++j) y[j] = x[j + i < L ? j + i : j + i - L];
        for (int j = 0; j < L; ++j) x[j] = y[j];
    }
    uint8_t* rows = a.rows + sid * L;
    for (int i = 0; i < L; ++i) rows[i] = (uint8_t)(x[i] + (i == 0 ? a.A : 0));
    PlanOut o{0, 0, 0, 1, 0, 0};
    bool pass = true;
    for (int b = 0; b < a.n_cbins && pass; ++b) {
        const int k = a.cbins[b];
        double re = 0.0, im = 0.0;
        for (int i = 0; i < L; ++i) {
            const int m = (int)(((long long)i * k) % a.Lnew);
            const double v = (double)a.letter[x[i]];
            re = __dadd_rn(re, __dmul_rn(v, a.tw[m].x));
            im = __dsub_rn(im, __dmul_rn(v, a.tw[m].y));
        }
        pass = !(__dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im)) > a.thr);
    }
    if (pass) {
        uint64_t total = 1;
        for (int i = 0; i < L && total; ++i) {
            const uint64_t n = (uint64_t)a.cnt[rows[i]];
            if (n == 0) {
                total = 0;
            } else if (total > (kRankMask >> 1) / n) {
                o.overflow = 1;
                total = 0;
            } else {
                total *= n;
            }
        }
        if (total) {
            uint32_t sc = 1, nsuf = 0, fc = 0;
            bool fits = true;
            for (int i = L - 1; i >= 0; --i) {
                const uint32_t n = (uint32_t)a.cnt[rows[i]];
                if (n <= 1) continue;
                fc += n;
                if (fits && (uint64_t)sc * n <= (uint64_t)a.smax) {
                    sc *= n;
                    ++nsuf;
                } else {
                    fits = false;
                }
            }
            o.total = total;
            o.nsuf = nsuf;
            o.suffix_count = sc;
            o.free_choices = fc;
            o.prefix_count = total / sc;
        }
    }
    a.out[sid] = o;
}

// ------------------------------------------------------------ host side

// src/utils/array.cpp:131-160: non-decreasing sequences of length len
void combinations(int len, const std::vector<int>& alpha, std::vector<std::vector<int>>& out) {
    std::vector<int> idx(len, 0);
    const int k = (int)alpha.size();
    for (;;) {
        std::vector<int> v(len);
        for (int i = 0; i < len; ++i) v[i] = alpha[idx[i]];
        out.push_back(v);
        int p = len - 1;
        while (p >= 0 && idx[p] == k - 1) --p;
        if (p < 0) break;
        idx[p]++;
        for (int q = p + 1; q < len; ++q) idx[q] = idx[p];
    }
}

// One uncompression level (order, c -> c') with its tables.
struct Level {
    int order = 0, c = 0, cn = 0, paf = 0, L = 0, r = 0, Lnew = 0, H = 0, nb = 0, np = 0;
    int A = 0, nrows = 0, dmax = 0, smax = 0;
    std::vector<int> alpha, nalpha;
    std::map<int, int> letter_index;  // letter value -> index into alpha
    std::vector<uint8_t> asc;         // letter indices by ascending value
    std::vector<std::vector<std::vector<int>>> rowparts;  // [row][choice] -> r values
    std::vector<int> bins;     // varying bins
    std::vector<int> cbins;    // bins that are multiples of r (constant per side)
    double thr = 0;            // 2n - paf + 0.001
    float thr_lo = 0, thr_hi = 0;
    std::vector<double> cs, sn;  // cos / sin (2 pi m / Lnew)
};

// The reference's partition table and first-entry reduction
// (uncompression.cpp:88-142): rows 0..A-1 hold every ordered partition of
// letter a into r new letters (next_permutation order of each sorted
// combination); rows A..2A-1 the rotation/reversal minima of those
// partitions, the choices of a side's first entry.
int build_level(gp_ctx* c, Level& lv, int order, int compress, int new_compress, int paf) {
    lv.order = order;
    lv.c = compress;
    lv.cn = new_compress;
    lv.paf = paf;
    lv.L = order / compress;
    lv.r = compress / new_compress;
    lv.Lnew = lv.L * lv.r;
    lv.H = lv.Lnew / 2;
    lv.alpha = gp::alphabet(compress);
    lv.nalpha = gp::alphabet(new_compress);
    lv.A = (int)lv.alpha.size();
    if (lv.L > kMaxL || lv.Lnew > kMaxLnew || 2 * lv.A > kMaxRows)
        return c->fail(GP_ERR_UNSUPPORTED, "uncompress: length %d -> %d over %d letters", lv.L, lv.Lnew, lv.A);
    const int r = lv.r;
    std::vector<std::vector<int>> parts;
    combinations(r, lv.nalpha, parts);
    lv.rowparts.assign(2 * lv.A, {});
    for (int a = 0; a < lv.A; ++a) {
        const int letter = lv.alpha[a];
        lv.letter_index[letter] = a;
        std::vector<std::vector<int>> list;
        for (auto part : parts) {
            int sum = 0;
            for (int v : part) sum += v;
            if (sum != letter) continue;
            do {
                list.push_back(part);
            } while (std::next_permutation(part.begin(), part.end()));
        }
        std::set<std::vector<int>> first;
        for (auto& perm : list) {
            std::vector<int> mn = perm;
            for (int rev = 0; rev < 2; ++rev)
                for (int s = 0; s < r; ++s) {
                    std::vector<int> cand(r);
                    for (int i = 0; i < r; ++i) {
                        const int src = (i + s) % r;
                        cand[i] = rev ? perm[r - 1 - src] : perm[src];
                    }
                    if (cand < mn) mn = cand;
                }
            first.insert(mn);
        }
        lv.rowparts[a] = list;
        lv.rowparts[lv.A + a] = std::vector<std::vector<int>>(first.begin(), first.end());
    }
    for (auto& kv : lv.letter_index) lv.asc.push_back((uint8_t)kv.second);  // std::map: ascending values
    lv.nrows = 2 * lv.A;
    lv.dmax = 1;
    for (auto& row : lv.rowparts) lv.dmax = std::max<int>(lv.dmax, (int)row.size());
    for (int k = 1; k <= lv.H; ++k) (k % r ? lv.bins : lv.cbins).push_back(k);
    lv.nb = (int)lv.bins.size();
    // bin pairs of the scan kernel's template
    const int want = (lv.nb + 1) / 2;
    static const int kNp[] = {2, 4, 6, 8, 10, 12, 16, 24, 32};
    lv.np = 0;
    for (int p : kNp)
        if (p >= want) {
            lv.np = p;
            break;
        }
    if (!lv.np) return c->fail(GP_ERR_UNSUPPORTED, "uncompress: %d varying bins", lv.nb);
    const size_t ctab_bytes = (size_t)lv.L * lv.dmax * lv.np * 16;
    if (ctab_bytes + 16 * lv.np > kScanSmemBudget / 2)
        return c->fail(GP_ERR_UNSUPPORTED, "uncompress: partition tables too large (%zu bytes)", ctab_bytes);
    lv.smax = (int)std::min<size_t>(729, (kScanSmemBudget - ctab_bytes) / ((size_t)lv.np * 16));
    lv.thr = 2.0 * order - paf + 0.001;
    // rigorous fp32 error of |X_k|^2: terms and partial sums per component are
    // at most L r max|v|; table rounding and at most L + 1 additions each add
    // a relative 2^-24 of that; the square and sum two more roundings
    const double u = std::ldexp(1.0, -24);
    const double comp = (double)lv.L * r * new_compress;
    const double eps = std::sqrt(2.0) * (2.0 * lv.L + 2.0) * u * comp;
    const double delta = 2.0 * (2.0 * std::sqrt(lv.thr + 1.0) * eps + 3.0 * eps * eps + 4.0 * u * (lv.thr + 1.0));
    lv.thr_lo = std::nextafter((float)(lv.thr - delta), 0.f);
    lv.thr_hi = std::nextafter((float)(lv.thr + delta), 1e30f);
    lv.cs.resize(lv.Lnew);
    lv.sn.resize(lv.Lnew);
    for (int m = 0; m < lv.Lnew; ++m) {  // the FP64 DFT's table: angle 2 pi m / L' in double
        const double ang = 6.283185307179586476925286766559 * (double)m / (double)lv.Lnew;
        lv.cs[m] = std::cos(ang);
        lv.sn[m] = std::sin(ang);
    }
    return GP_OK;
}

// Device copies of a level's tables (context scratch ux[0..3]).
int upload_level(gp_ctx* c, const Level& lv, LevelDev& d, cudaStream_t s) {
    const int np = lv.np, NB = 2 * np;
    std::vector<int> cnt(lv.nrows);
    std::vector<int8_t> vals((size_t)lv.nrows * lv.dmax * lv.r, 0);
    std::vector<float4> ct((size_t)lv.L * lv.nrows * lv.dmax * np, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<double2> ct64((size_t)lv.L * lv.nrows * lv.dmax * NB, make_double2(0.0, 0.0));
    for (int row = 0; row < lv.nrows; ++row) {
        cnt[row] = (int)lv.rowparts[row].size();
        for (int d = 0; d < cnt[row]; ++d)
            for (int q = 0; q < lv.r; ++q) vals[((size_t)row * lv.dmax + d) * lv.r + q] = (int8_t)lv.rowparts[row][d][q];
    }
    for (int i = 0; i < lv.L; ++i)
        for (int row = 0; row < lv.nrows; ++row)
            for (int d = 0; d < cnt[row]; ++d) {
                const size_t at = ((size_t)i * lv.nrows + row) * lv.dmax + d;
                for (int b = 0; b < lv.nb; ++b) {
                    const int k = lv.bins[b];
                    long double re = 0, im = 0;
                    for (int q = 0; q < lv.r; ++q) {
                        const int m = (int)(((long long)(i + lv.L * q) * k) % lv.Lnew);
                        const long double ang = 6.283185307179586476925286766559L * (long double)m / (long double)lv.Lnew;
                        re += (long double)lv.rowparts[row][d][q] * cosl(ang);
                        im -= (long double)lv.rowparts[row][d][q] * sinl(ang);
                    }
                    ct64[at * NB + b] = make_double2((double)re, (double)im);
                    float4& f = ct[at * np + b / 2];
                    if (b & 1) {
                        f.y = (float)re;
                        f.w = (float)im;
                    } else {
                        f.x = (float)re;
                        f.z = (float)im;
                    }
                }
            }
    DevBuf &dcnt = c->ux[0], &dvals = c->ux[1], &dct = c->ux[2], &dct64 = c->ux[3];
    if (!dcnt.ensure(cnt.size() * 4) || !dvals.ensure(vals.size() + 16) || !dct.ensure(ct.size() * 16) ||
        !dct64.ensure(ct64.size() * 16))
        return c->fail(GP_ERR_NOMEM, "uncompress: level tables");
    GP_CUDA_TRY(c, cudaMemcpyAsync(dcnt.p, cnt.data(), cnt.size() * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dvals.p, vals.data(), vals.size(), cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dct.p, ct.data(), ct.size() * 16, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dct64.p, ct64.data(), ct64.size() * 16, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));  // the host vectors go out of scope
    d.L = lv.L;
    d.r = lv.r;
    d.Lnew = lv.Lnew;
    d.H = lv.H;
    d.nrows = lv.nrows;
    d.dmax = lv.dmax;
    d.np = np;
    d.nb = lv.nb;
    d.one_bit = lv.cn == 1 && lv.Lnew <= 64;
    d.target = lv.paf * lv.cn;
    d.cnt = dcnt.as<int>();
    d.vals = dvals.as<int8_t>();
    d.ctab = dct.as<float4>();
    d.ctab64 = dct64.as<double2>();
    return GP_OK;
}

// One side of a compressed pair, planned.
struct Side {
    std::vector<uint8_t> rows;  // row of each position
    uint64_t total = 0;         // expansions (0: none can pass)
    uint64_t prefix_count = 0;
    uint32_t nsuf = 0;
    uint32_t suffix_count = 1;  // combinations in the suffix table
    uint32_t free_choices = 0;  // choices summed over the free positions (the scan's term table)
};

// Plans every side on the device (ux_plan_kernel) from the sides' letter
// indices (2 per pair), and copies the plans back: the host batches the
// pairs by expansion count and sizes the scan's shared memory from them.
int plan_sides(gp_ctx* c, const Level& lv, const std::vector<uint8_t>& seqs, std::vector<Side>& sides,
               cudaStream_t s) {
    const int L = lv.L;
    const int64_t ns = (int64_t)seqs.size() / L;
    sides.assign(ns, Side{});
    if (ns == 0) return GP_OK;
    if (ns > INT32_MAX) return c->fail(GP_ERR_UNSUPPORTED, "uncompress: %lld sides", (long long)ns);
    std::vector<double2> tw(lv.Lnew);
    for (int m = 0; m < lv.Lnew; ++m) tw[m] = make_double2(lv.cs[m], lv.sn[m]);
    std::vector<int8_t> letter(lv.A);
    for (int i = 0; i < lv.A; ++i) letter[i] = (int8_t)lv.alpha[i];
    DevBuf &dseq = c->ux[23], &drows = c->ux[24], &dout = c->ux[25], &dcb = c->ux[26], &dtw = c->ux[27],
           &dlet = c->ux[28], &dasc = c->ux[29], &dcnt = c->ux[30];
    std::vector<int> cnt(lv.nrows);
    for (int row = 0; row < lv.nrows; ++row) cnt[row] = (int)lv.rowparts[row].size();
    if (!dseq.ensure(seqs.size()) || !drows.ensure(seqs.size()) || !dout.ensure((size_t)ns * sizeof(PlanOut)) ||
        !dcb.ensure(lv.cbins.size() * 4 + 4) || !dtw.ensure(tw.size() * 16) || !dlet.ensure(16) ||
        !dasc.ensure(16) || !dcnt.ensure(cnt.size() * 4))
        return c->fail(GP_ERR_NOMEM, "uncompress: planning buffers");
    GP_CUDA_TRY(c, cudaMemcpyAsync(dseq.p, seqs.data(), seqs.size(), cudaMemcpyHostToDevice, s));
    if (!lv.cbins.empty())
        GP_CUDA_TRY(c, cudaMemcpyAsync(dcb.p, lv.cbins.data(), lv.cbins.size() * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dtw.p, tw.data(), tw.size() * 16, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dlet.p, letter.data(), letter.size(), cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dasc.p, lv.asc.data(), lv.asc.size(), cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dcnt.p, cnt.data(), cnt.size() * 4, cudaMemcpyHostToDevice, s));
    PlanArgs pa{};
    pa.seqs = dseq.as<uint8_t>();
    pa.n_sides = (int)ns;
    pa.L = L;
    pa.A = lv.A;
    pa.Lnew = lv.Lnew;
    pa.n_cbins = (int)lv.cbins.size();
    pa.smax = lv.smax;
    pa.cbins = dcb.as<int>();
    pa.cnt = dcnt.as<int>();
    pa.tw = dtw.as<double2>();
    pa.letter = dlet.as<int8_t>();
    pa.asc = dasc.as<uint8_t>();
    pa.thr = lv.thr;
    pa.rows = drows.as<uint8_t>();
    pa.out = dout.as<PlanOut>();
    ux_plan_kernel<<<(unsigned)((ns + 127) / 128), 128, 0, s>>>(pa);
    GP_CUDA_TRY(c, cudaGetLastError());
    std::vector<uint8_t> rows(seqs.size());
    std::vector<PlanOut> po(ns);
    GP_CUDA_TRY(c, cudaMemcpyAsync(rows.data(), drows.p, rows.size(), cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(po.data(), dout.p, (size_t)ns * sizeof(PlanOut), cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    for (int64_t k = 0; k < ns; ++k) {
        if (po[k].overflow) return c->fail(GP_ERR_UNSUPPORTED, "uncompress: more than 2^39 expansions of one side");
        Side& sd = sides[k];
        sd.rows.assign(rows.begin() + k * L, rows.begin() + (k + 1) * L);
        sd.total = po[k].total;
        sd.prefix_count = po[k].prefix_count;
        sd.nsuf = po[k].nsuf;
        sd.suffix_count = po[k].suffix_count;
        sd.free_choices = po[k].free_choices;
    }
    return GP_OK;
}

void put_uint(std::string& s, unsigned v) {
    char tmp[12];
    int n = 0;
    do {
        tmp[n++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    while (n) s.push_back(tmp[--n]);
}

void put_int(std::string& s, int v) {
    if (v < 0) {
        s.push_back('-');
        put_uint(s, (unsigned)(-v));
    } else {
        put_uint(s, (unsigned)v);
    }
}

// The expansion of a survivor word, on the host.
void host_expand(const Level& lv, const Side& sd, uint64_t rank, std::vector<int>& x) {
    std::vector<int> d(lv.L, 0);
    for (int i = lv.L - 1; i >= 0; --i) {
        const uint64_t c = lv.rowparts[sd.rows[i]].size();
        d[i] = (int)(rank % c);
        rank /= c;
    }
    x.assign(lv.Lnew, 0);
    for (int i = 0; i < lv.L; ++i)
        for (int q = 0; q < lv.r; ++q) x[i + lv.L * q] = lv.rowparts[sd.rows[i]][d[i]][q];
}

// "PSD" + signature + " " + sequence (src/utils/io.cpp:14-36; the a-side
// writes bound - rint(psd)), the line the reference's scratch files hold.
void candidate_line(const Level& lv, const std::vector<int>& x, bool invert, std::string& line, std::string& seq) {
    const int N = lv.Lnew, bound = 2 * lv.order - lv.paf;
    line = "PSD";
    for (int k = 1; k < N; ++k) {
        double re = 0, im = 0;
        for (int j = 0, m = 0; j < N; ++j, m += k, m -= m >= N ? N : 0) {
            re += x[j] * lv.cs[m];
            im -= x[j] * lv.sn[m];
        }
        const int p = (int)std::nearbyint(re * re + im * im);
        put_int(line, invert ? bound - p : p);
    }
    seq.clear();
    for (int v : x) {
        put_int(seq, v);
        seq.push_back(' ');
    }
    line.push_back(' ');
    line += seq;
}

std::string signature_token(const std::string& line) { return line.substr(0, line.find(' ')); }

bool slurp(const char* path, std::string& out) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    out.resize(sz > 0 ? (size_t)sz : 0);
    size_t got = sz > 0 ? fread(&out[0], 1, (size_t)sz, f) : 0;
    fclose(f);
    out.resize(got);
    return true;
}

using ScanKernel = void (*)(ScanArgs);

ScanKernel scan_kernel_for(int np) {
    switch (np) {
        case 2: return ux_scan_kernel<2, 0>;
        case 4: return ux_scan_kernel<4, 0>;
        // phase A over about 3/5 of the bin pairs (order 57, 10 pairs, whole
        // file: 6 pairs 8.5-8.6 s, 7 pairs 8.7 s, 5 pairs 8.9 s, 8 pairs 8.9 s,
        // 4 pairs 9.4 s, 9 pairs 9.3-9.4 s)
        case 6: return ux_scan_kernel<6, 3>;
        case 8: return ux_scan_kernel<8, 4>;
        case 10: return ux_scan_kernel<10, 6>;
        case 12: return ux_scan_kernel<12, 7>;
        case 16: return ux_scan_kernel<16, 9>;
        case 24: return ux_scan_kernel<24, 14>;
        case 32: return ux_scan_kernel<32, 19>;
    }
    return nullptr;
}

unsigned grid_for(uint64_t n, unsigned cap) {
    uint64_t g = (n + 255) / 256;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(g, cap));
}

// A matched pair of expansions: its two candidate lines (the reference's
// sorted scratch files' order), the output line and the two sequences.
struct Match {
    std::string la, lb, line;
    std::vector<int> xa, xb;
};

// The engine over consecutive pairs [p0, p1): device scratch in ux[4..].
struct Batcher {
    gp_ctx* c;
    const Level& lv;
    const LevelDev& ld;
    const std::vector<Side>& sides;    // 2 per pair: a, b
    const std::vector<uint8_t>& seqs;  // the sides' letter indices, L per side
    cudaStream_t s;
    ScanKernel scan;
    int scan_blocks = 0;
    size_t smem = 0;
    // the matched pairs of each pair of the batch, in output order
    std::vector<std::vector<Match>> out;

    // Runs the batch; on overflow of a device list returns GP_ERR_OVERFLOW
    // with *overflowed set, so the caller can halve the batch.
    int run(int64_t p0, int64_t p1, bool* overflowed);
};

int Batcher::run(int64_t p0, int64_t p1, bool* overflowed) {
    *overflowed = false;
    const int L = lv.L;
    const int64_t np_ = p1 - p0, ns = 2 * np_;
    // the batch's distinct sides (equal letters expand and filter the same
    // way, whatever the pair or role): scanned once each
    std::vector<uint32_t> uid(ns);
    std::vector<int64_t> urep;  // unique side -> its first batch side
    {
        std::unordered_map<std::string, uint32_t> seen;
        seen.reserve((size_t)ns * 2);
        for (int64_t k = 0; k < ns; ++k) {
            std::string key(reinterpret_cast<const char*>(&seqs[(size_t)(2 * p0 + k) * L]), L);
            auto it = seen.emplace(std::move(key), (uint32_t)urep.size());
            if (it.second) urep.push_back(k);
            uid[k] = it.first->second;
        }
    }
    const int64_t nu = (int64_t)urep.size();
    // uses of each unique side: pair << 1 | role, in batch-side order
    std::vector<uint32_t> use_beg(nu + 1, 0), uses(ns);
    for (int64_t k = 0; k < ns; ++k) ++use_beg[uid[k] + 1];
    for (int64_t u = 0; u < nu; ++u) use_beg[u + 1] += use_beg[u];
    {
        std::vector<uint32_t> fill(use_beg.begin(), use_beg.end() - 1);
        for (int64_t k = 0; k < ns; ++k) uses[fill[uid[k]]++] = (uint32_t)k;  // k = 2 pair + role
    }
    std::vector<uint8_t> rows((size_t)nu * L);
    std::vector<uint64_t> ubeg(nu + 1), pcnt(nu);
    std::vector<uint32_t> nsuf(nu);
    uint64_t units = 0, total = 0;
    for (int64_t u = 0; u < nu; ++u) {
        const Side& sd = sides[2 * p0 + urep[u]];
        memcpy(&rows[(size_t)u * L], sd.rows.data(), L);
        ubeg[u] = units;
        pcnt[u] = sd.total ? sd.prefix_count : 0;
        nsuf[u] = sd.nsuf;
        if (sd.total) {
            units += (sd.prefix_count + kScanThreads - 1) / kScanThreads;
            total += sd.total;
        }
    }
    ubeg[nu] = units;
    out.assign(np_, {});
    if (units == 0) return GP_OK;
    // capacities: every expansion could pass at small sizes; at large ones
    // a pass rate of 1/8 (order 57: under 1 %), at most 2^30 survivors (8 GB;
    // the join packs survivor indices into 31 bits); unsure 1/64 of that.
    // A batch that overflows is split in two and run again.
    const uint64_t surv_cap = std::max<uint64_t>(
        1024, std::min<uint64_t>(uint64_t(1) << 30, std::min<uint64_t>(total, std::max<uint64_t>(total / 8, 1 << 20))));
    const uint64_t unsure_cap = std::max<uint64_t>(1024, surv_cap / 64);
    DevBuf &drows = c->ux[4], &dubeg = c->ux[5], &dpcnt = c->ux[6], &dnsuf = c->ux[7], &dcnt = c->ux[8],
           &dsurv = c->ux[9], &duns = c->ux[10], &dside = c->ux[11];
    if (!drows.ensure(rows.size()) || !dubeg.ensure(ubeg.size() * 8) || !dpcnt.ensure(pcnt.size() * 8) ||
        !dnsuf.ensure(nsuf.size() * 4) || !dcnt.ensure(64) || !dsurv.ensure(surv_cap * 8) ||
        !duns.ensure(unsure_cap * 8) || !dside.ensure((size_t)nu * 4))
        return c->fail(GP_ERR_NOMEM, "uncompress: batch buffers");
    GP_CUDA_TRY(c, cudaMemcpyAsync(drows.p, rows.data(), rows.size(), cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dubeg.p, ubeg.data(), ubeg.size() * 8, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dpcnt.p, pcnt.data(), pcnt.size() * 8, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dnsuf.p, nsuf.data(), nsuf.size() * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemsetAsync(dcnt.p, 0, 64, s));
    GP_CUDA_TRY(c, cudaMemsetAsync(dside.p, 0, (size_t)nu * 4, s));
    unsigned long long* counters = dcnt.as<unsigned long long>();
    LevelDev d = ld;
    d.side_rows = drows.as<uint8_t>();
    ScanArgs sa{};
    sa.lv = d;
    sa.unit_begin = dubeg.as<uint64_t>();
    sa.prefix_count = dpcnt.as<uint64_t>();
    sa.nsuf = dnsuf.as<uint32_t>();
    sa.n_sides = (int)nu;
    sa.n_units = units;
    sa.thr_lo = lv.thr_lo;
    sa.thr_hi = lv.thr_hi;
    sa.surv = dsurv.as<uint64_t>();
    sa.surv_cap = surv_cap;
    sa.unsure = duns.as<uint64_t>();
    sa.unsure_cap = unsure_cap;
    sa.counters = counters;
    sa.side_count = dside.as<uint32_t>();
    sa.status = c->status.as<int>();
    const unsigned sgrid = (unsigned)std::min<uint64_t>(units, (uint64_t)scan_blocks);
    scan<<<sgrid, kScanThreads, smem, s>>>(sa);
    GP_CUDA_TRY(c, cudaGetLastError());
    RecheckArgs ra{};
    ra.lv = d;
    ra.thr = lv.thr;
    ra.unsure = sa.unsure;
    ra.unsure_cap = unsure_cap;
    ra.surv = sa.surv;
    ra.surv_cap = surv_cap;
    ra.counters = counters;
    ra.side_count = sa.side_count;
    ra.status = sa.status;
    ux_recheck_kernel<<<(unsigned)c->num_sms * 8, kRecheckWarps * 32, 0, s>>>(ra);
    GP_CUDA_TRY(c, cudaGetLastError());
    std::vector<unsigned long long> hc(8);
    std::vector<uint32_t> side_count(nu);
    GP_CUDA_TRY(c, cudaMemcpyAsync(hc.data(), counters, 64, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(side_count.data(), sa.side_count, (size_t)nu * 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    if (hc[0] > surv_cap || hc[1] > unsure_cap) {
        cudaMemset(c->status.p, 0, sizeof(int));
        *overflowed = true;
        return GP_ERR_OVERFLOW;
    }
    int rc = c->check_status("uncompress");
    if (rc) return rc;
    const uint64_t nsurv = hc[0];
    // buckets: a pair with no survivor on one side cannot match; its base
    // is the next pair's (bases stay non-decreasing for the join's search)
    std::vector<uint8_t> lg(np_, 255);
    std::vector<uint32_t> pbase(np_, 0);
    uint64_t nbk = 0;
    std::vector<uint32_t> uses_ok(nu, 0);  // uses of each distinct side in pairs that can match
    for (int64_t p = 0; p < np_; ++p) {
        const uint64_t na = side_count[uid[2 * p]], nbb = side_count[uid[2 * p + 1]];
        pbase[p] = (uint32_t)std::min<uint64_t>(nbk, UINT32_MAX);
        if (!na || !nbb) continue;
        int l = 0;
        while (((uint64_t)kBucketTarget << l) < na + nbb && l < 30) ++l;
        lg[p] = (uint8_t)l;
        nbk += uint64_t(1) << l;
        ++uses_ok[uid[2 * p]];
        ++uses_ok[uid[2 * p + 1]];
    }
    if (nbk == 0 || nsurv == 0) return GP_OK;
    // join entries: one slot per survivor (its first use), then the further uses
    uint64_t entries = nsurv;
    for (int64_t u = 0; u < nu; ++u)
        if (uses_ok[u] > 1) entries += (uint64_t)side_count[u] * (uses_ok[u] - 1);
    if (nbk >= (uint64_t(1) << 31)) return c->fail(GP_ERR_UNSUPPORTED, "uncompress: %llu join buckets", (unsigned long long)nbk);
    if (entries >= (uint64_t(1) << 32)) return c->fail(GP_ERR_UNSUPPORTED, "uncompress: %llu join entries", (unsigned long long)entries);
    DevBuf &dlg = c->ux[12], &dpb = c->ux[13], &dkeys = c->ux[14], &dbkt = c->ux[15], &dbc = c->ux[16],
           &dbo = c->ux[17], &dbcur = c->ux[18], &dscan = c->ux[19], &deh = c->ux[20], &dei = c->ux[21],
           &dm = c->ux[22], &dub = c->ux[31], &duse = c->ux[32], &deix = c->ux[33];
    const uint64_t match_cap = std::max<uint64_t>(1 << 16, entries / 16);
    if (!dlg.ensure(np_) || !dpb.ensure((size_t)np_ * 4) || !dkeys.ensure(entries * 8) || !dbkt.ensure(entries * 4) ||
        !deix.ensure(entries * 4) || !dub.ensure(use_beg.size() * 4) || !duse.ensure(uses.size() * 4) ||
        !dbc.ensure(nbk * 4) || !dbo.ensure(nbk * 4 + 4) || !dbcur.ensure(nbk * 4) ||
        !dscan.ensure(gp::scan_tmp_bytes((int64_t)nbk)) || !deh.ensure(entries * 8) || !dei.ensure(entries * 4) ||
        !dm.ensure(match_cap * 16))
        return c->fail(GP_ERR_NOMEM, "uncompress: join buffers");
    GP_CUDA_TRY(c, cudaMemcpyAsync(dlg.p, lg.data(), np_, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dpb.p, pbase.data(), (size_t)np_ * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dub.p, use_beg.data(), use_beg.size() * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(duse.p, uses.data(), uses.size() * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemsetAsync(dbc.p, 0, nbk * 4, s));
    GP_CUDA_TRY(c, cudaMemsetAsync(dbcur.p, 0, nbk * 4, s));
    KeyArgs ka{};
    ka.lv = d;
    ka.surv = sa.surv;
    ka.n = nsurv;
    ka.use_beg = dub.as<uint32_t>();
    ka.uses = duse.as<uint32_t>();
    ka.pair_lg = dlg.as<uint8_t>();
    ka.pair_base = dpb.as<uint32_t>();
    ka.keys = dkeys.as<uint64_t>();
    ka.bucket = dbkt.as<uint32_t>();
    ka.eidx = deix.as<uint32_t>();
    ka.entry_cap = entries;
    ka.ecount = counters + 3;
    ka.bcount = dbc.as<uint32_t>();
    ka.status = sa.status;
    ux_key_kernel<<<grid_for(nsurv, (unsigned)c->num_sms * 16), 256, 0, s>>>(ka);
    GP_CUDA_TRY(c, cudaGetLastError());
    GP_CUDA_TRY(c, gp::exclusive_scan_u32(dbc.as<uint32_t>(), dbo.as<uint32_t>(), (int64_t)nbk, dscan.as<uint32_t>(), s));
    ux_scatter_kernel<<<grid_for(entries, (unsigned)c->num_sms * 16), 256, 0, s>>>(
        ka.keys, ka.bucket, ka.eidx, entries, dbo.as<uint32_t>(), dbcur.as<uint32_t>(), deh.as<uint64_t>(),
        dei.as<uint32_t>());
    GP_CUDA_TRY(c, cudaGetLastError());
    JoinArgs ja{};
    ja.lv = d;
    ja.surv = sa.surv;
    ja.ent_h = deh.as<uint64_t>();
    ja.ent_i = dei.as<uint32_t>();
    ja.boff = dbo.as<uint32_t>();
    ja.bcount = dbc.as<uint32_t>();
    ja.n_buckets = (uint32_t)nbk;
    ja.pair_base = dpb.as<uint32_t>();
    ja.n_pairs = (uint32_t)np_;
    ja.matches = dm.as<uint64_t>();
    ja.match_cap = match_cap;
    ja.counters = counters;
    ja.status = sa.status;
    ux_join_kernel<<<(unsigned)std::min<uint64_t>(nbk, (uint64_t)c->num_sms * 8), 256, 0, s>>>(ja);
    GP_CUDA_TRY(c, cudaGetLastError());
    GP_CUDA_TRY(c, cudaMemcpyAsync(hc.data(), counters, 64, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    if (hc[2] > match_cap) {
        cudaMemset(c->status.p, 0, sizeof(int));
        *overflowed = true;
        return GP_ERR_OVERFLOW;
    }
    rc = c->check_status("uncompress join");
    if (rc) return rc;
    const uint64_t nm = hc[2];
    if (nm == 0) return GP_OK;
    std::vector<uint64_t> hm(nm * 2);
    GP_CUDA_TRY(c, cudaMemcpy(hm.data(), dm.p, nm * 16, cudaMemcpyDeviceToHost));
    // signatures of the matched expansions; the reference joins on the
    // signature string, which the PAF condition implies up to FP64 rounding
    std::vector<Match> items(nm);
    std::vector<char> keep(nm, 0);
    std::vector<int64_t> pair_of(nm);
    auto work = [&](uint64_t lo, uint64_t hi) {
        std::vector<int> xa, xb;
        std::string la, sa_, lb, sb_;
        for (uint64_t m = lo; m < hi; ++m) {
            const uint64_t va = hm[2 * m], vb = hm[2 * m + 1];
            const int64_t side_a = (int64_t)(va >> kRankBits), side_b = (int64_t)(vb >> kRankBits);
            host_expand(lv, sides[2 * p0 + side_a], va & kRankMask, xa);
            host_expand(lv, sides[2 * p0 + side_b], vb & kRankMask, xb);
            candidate_line(lv, xa, true, la, sa_);
            candidate_line(lv, xb, false, lb, sb_);
            pair_of[m] = side_a >> 1;
            if (signature_token(la) != signature_token(lb)) continue;
            keep[m] = 1;
            items[m] = Match{la, lb, sa_ + " " + sb_ + "\n", xa, xb};
        }
    };
    const unsigned nt = (unsigned)std::min<uint64_t>(16, (nm + 63) / 64);
    if (nt <= 1) {
        work(0, nm);
    } else {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t) th.emplace_back(work, nm * t / nt, nm * (t + 1) / nt);
        for (auto& t : th) t.join();
    }
    for (uint64_t m = 0; m < nm; ++m)
        if (keep[m]) out[pair_of[m]].push_back(std::move(items[m]));
    for (auto& v : out)
        std::sort(v.begin(), v.end(),
                  [](const Match& p, const Match& q) { return p.la != q.la ? p.la < q.la : p.lb < q.lb; });
    return GP_OK;
}

// The selected lines of a pair file as letter indices, 2L per pair.
// io.cpp:52-55: a line of the wrong length is an error, the pairs before it
// are still uncompressed and written (format_rc).  A value that is not a
// letter of the compression is an error before anything is written.
int parse_pairs(gp_ctx* c, const Level& lv, const std::string& text, int64_t first, int64_t end_line, int64_t step,
                std::vector<uint8_t>& seqs, int& format_rc) {
    const int L = lv.L;
    const char* p = text.data();
    const char* end = p + text.size();
    int64_t line_no = 0;
    std::vector<int> vals;
    while (p < end) {
        const char* nl = (const char*)memchr(p, '\n', (size_t)(end - p));
        if (!nl) nl = end;
        const int64_t this_line = line_no;
        if (this_line < first || this_line >= end_line || (this_line - first) % step != 0) {
            ++line_no;
            p = nl + 1;
            if (this_line >= end_line) break;
            continue;
        }
        vals.clear();
        const char* q = p;
        while (q < nl) {
            while (q < nl && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
            if (q >= nl) break;
            char* e2;
            const long v = strtol(q, &e2, 10);
            if (e2 == q) break;
            vals.push_back((int)v);
            q = e2;
        }
        p = nl + 1;
        if ((int)vals.size() != 2 * L) {
            format_rc = c->fail(GP_ERR_FORMAT, "PairReader: input line %lld: length is %zu. Expected %d",
                                (long long)line_no, vals.size(), 2 * L);
            break;
        }
        ++line_no;
        for (int v : vals) {
            const auto it = lv.letter_index.find(v);
            if (it == lv.letter_index.end())
                return c->fail(GP_ERR_FORMAT, "uncompress: value %d is not a letter of compression %d", v, lv.c);
            seqs.push_back((uint8_t)it->second);
        }
    }
    return GP_OK;
}

// One level over the pairs in seqs (letter indices, 2L per pair): plans the
// sides on the device, runs the engine in batches of consecutive pairs,
// writes the matched pairs to out and, when next is set, appends their
// sequences (values, 2 L' per pair, in output order) for the next level.
int run_level(gp_ctx* c, const Level& lv, const std::vector<uint8_t>& seqs, FILE* out, std::vector<int8_t>* next) {
    cudaStream_t s = c->s_comp;
    std::vector<Side> sides;
    int rc = plan_sides(c, lv, seqs, sides, s);
    if (rc) return rc;
    const int64_t npairs = (int64_t)sides.size() / 2;
    if (npairs == 0) return GP_OK;
    LevelDev ld{};
    rc = upload_level(c, lv, ld, s);
    if (rc) return rc;
    Batcher bt{c, lv, ld, sides, seqs, s, scan_kernel_for(lv.np), 0, 0, {}};
    {
        // shared memory of the scan: the largest suffix table and term table
        // any side of this call needs (a few tens of KB: several CTAs per SM)
        uint64_t max_sc = 1, max_fc = 0;
        for (const Side& sd : sides) {
            if (!sd.total) continue;
            max_sc = std::max<uint64_t>(max_sc, sd.suffix_count);
            max_fc = std::max<uint64_t>(max_fc, sd.free_choices);
        }
        bt.smem = (size_t)(max_sc + max_fc) * lv.np * 16;
        cudaError_t e = cudaFuncSetAttribute(bt.scan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bt.smem);
        int per_sm = 0;
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bt.scan, kScanThreads, bt.smem);
        if (e != cudaSuccess || per_sm < 1)
            return c->fail(GP_ERR_CUDA, "uncompress: scan kernel occupancy (%s)", cudaGetErrorString(e));
        bt.scan_blocks = c->num_sms * std::max(1, per_sm);
    }
    // batches of consecutive pairs, by expansions; a batch whose device
    // lists overflow is split in half and run again
    constexpr uint64_t kBatchExpansions = uint64_t(1) << 35;
    std::vector<std::pair<int64_t, int64_t>> todo;
    for (int64_t p = 0; p < npairs;) {
        int64_t q = p;
        uint64_t tot = 0;
        while (q < npairs && (q == p || (tot + sides[2 * q].total + sides[2 * q + 1].total <= kBatchExpansions &&
                                         q - p < kMaxSidesPerBatch / 2))) {
            tot += sides[2 * q].total + sides[2 * q + 1].total;
            ++q;
        }
        todo.emplace_back(p, q);
        p = q;
    }
    std::reverse(todo.begin(), todo.end());
    std::string buf;
    while (!todo.empty()) {
        const auto [p0, p1] = todo.back();
        todo.pop_back();
        bool over = false;
        rc = bt.run(p0, p1, &over);
        if (rc == GP_ERR_OVERFLOW && over && p1 - p0 > 1) {
            const int64_t mid = p0 + (p1 - p0) / 2;
            todo.emplace_back(mid, p1);
            todo.emplace_back(p0, mid);
            continue;
        }
        if (rc == GP_ERR_OVERFLOW && over) return c->fail(GP_ERR_OVERFLOW, "uncompress: one pair overflows the device lists");
        if (rc) return rc;
        buf.clear();
        for (auto& v : bt.out)
            for (auto& m : v) {
                buf += m.line;
                if (next) {
                    for (int x : m.xa) next->push_back((int8_t)x);
                    for (int x : m.xb) next->push_back((int8_t)x);
                }
            }
        if (!buf.empty() && fwrite(buf.data(), 1, buf.size(), out) != buf.size())
            return c->fail(GP_ERR_IO, "uncompress: write failed");
    }
    return GP_OK;
}

// The levels compress[0] -> compress[1] -> ... of one chain (src/main.cpp:
// 117-139 runs uncompress_pipeline once per level, each reading the file
// the previous one wrote).  Level 0 reads the selected lines of in_pairs;
// each later level takes the previous level's pairs from memory, in the
// order they were written, so its input equals the file the previous level
// wrote.  Every level's file is written.
int uncompress_chain_impl(gp_ctx* c, int order, const int* compress, int ncomp, int paf, const char* in_pairs,
                                 const char* const* out_pairs, int64_t first, int64_t end_line, int64_t step) {
    StageRange nvtx_range("gp_uncompress");
    if (!c || !compress || ncomp < 2 || !in_pairs || !out_pairs) return GP_ERR_ARG;
    for (int i = 0; i + 1 < ncomp; ++i)
        if (!out_pairs[i]) return GP_ERR_ARG;
    if (first < 0 || step < 1) return c->fail(GP_ERR_ARG, "uncompress: bad line range (first %lld, step %lld)",
                                              (long long)first, (long long)step);
    cudaSetDevice(c->device);
    std::vector<int8_t> carried;  // the previous level's pairs (values), 2 L per pair
    bool have_input = true;
    for (int lvl = 0; lvl + 1 < ncomp; ++lvl) {
        const int cc = compress[lvl], cn = compress[lvl + 1];
        // the reference constructs its PairReader / PairWriter before the
        // pipeline runs (src/main.cpp:122-123): the output is truncated even
        // when nothing is uncompressed
        FILE* out = fopen(out_pairs[lvl], "w");
        if (!out) return c->fail(GP_ERR_IO, "uncompress: cannot open %s", out_pairs[lvl]);
        struct Closer {
            FILE* f;
            ~Closer() { fclose(f); }
        } closer{out};
        std::vector<int8_t> next;
        if (cc <= 1) {  // uncompression.cpp:42
            carried.clear();
            continue;
        }
        if (cn < 1 || cc % cn || order % cc)
            return c->fail(GP_ERR_ARG, "uncompress: compression %d -> %d of order %d", cc, cn, order);
        Level lv;
        int rc = build_level(c, lv, order, cc, cn, paf);
        if (rc) return rc;
        std::vector<uint8_t> seqs;
        int format_rc = GP_OK;
        if (lvl == 0) {
            std::string text;
            // an unreadable input yields no pairs (the reader is simply not good)
            have_input = slurp(in_pairs, text);
            if (have_input) rc = parse_pairs(c, lv, text, first, end_line, step, seqs, format_rc);
            if (rc) return rc;
        } else {
            seqs.reserve(carried.size());
            for (int8_t v : carried) {
                const auto it = lv.letter_index.find(v);
                if (it == lv.letter_index.end())
                    return c->fail(GP_ERR_FORMAT, "uncompress: value %d is not a letter of compression %d", v, cc);
                seqs.push_back((uint8_t)it->second);
            }
        }
        const bool more = lvl + 2 < ncomp;
        rc = run_level(c, lv, seqs, out, more ? &next : nullptr);
        if (rc) return rc;
        if (format_rc) return format_rc;  // the chain stops at a malformed input line
        carried.swap(next);
    }
    return GP_OK;
}

}  // namespace

extern "C" {

int gp_uncompress(gp_ctx* c, int order, int compress, int new_compress, int paf, const char* in_pairs,
                  const char* out_pairs, const char* work_dir, const char* prefix) {
    return gp_uncompress_lines(c, order, compress, new_compress, paf, in_pairs, out_pairs, work_dir, prefix, 0,
                               INT64_MAX, 1);
}

static int gp_uncompress_lines_impl(gp_ctx* c, int order, int compress, int new_compress, int paf, const char* in_pairs,
                                    const char* out_pairs, const char* work_dir, const char* prefix, int64_t first,
                                    int64_t end_line, int64_t step) {
    (void)work_dir;
    (void)prefix;
    if (!c || !in_pairs || !out_pairs) return GP_ERR_ARG;
    const int comps[2] = {compress, new_compress};
    const char* outs[1] = {out_pairs};
    return uncompress_chain_impl(c, order, comps, 2, paf, in_pairs, outs, first, end_line, step);
}

// No C++ exception (an allocation failure on a huge input) crosses the C ABI.
int gp_uncompress_lines(gp_ctx* c, int order, int compress, int new_compress, int paf, const char* in_pairs, const char* out_pairs,
                        const char* work_dir, const char* prefix, int64_t first, int64_t end_line, int64_t step) {
    try {
        return gp_uncompress_lines_impl(c, order, compress, new_compress, paf, in_pairs, out_pairs, work_dir, prefix, first, end_line, step);
    } catch (const std::exception& e) {
        return c ? c->fail(GP_ERR_NOMEM, "uncompress: %s", e.what()) : GP_ERR_NOMEM;
    }
}

int gp_uncompress_chain(gp_ctx* c, int order, const int* compress, int ncomp, int paf, const char* in_pairs,
                        const char* const* out_pairs, int64_t first, int64_t end_line, int64_t step) {
    try {
        return uncompress_chain_impl(c, order, compress, ncomp, paf, in_pairs, out_pairs, first, end_line, step);
    } catch (const std::exception& e) {
        return c ? c->fail(GP_ERR_NOMEM, "uncompress: %s", e.what()) : GP_ERR_NOMEM;
    }
}

}  // extern "C"
