// capi_equiv.cu -- equivalence filter (kernel (d), second half).
//
// Replaces cache_filter (src/core/filter/filter.cpp:18-163).  The generator
// set is the closure of the index pair ({1..L}, {L+1..2L}) under the
// reference's pair operations (src/utils/equivalence.cpp:46-95,146-277):
// rotate b by 1..L-1, swap a and b, reverse b, decimate both by every unit,
// and (compression 1, even L only) negate the odd positions of both.  It is
// built on the host, as the reference builds it once per run.
//
// Per pair the filter needs its class size and the input pairs in its
// class.  For L >= 3, canon_kernel finds both from canonical forms: every
// group element is an affine map per half (the description below, checked
// against the closure by gp_debug_pair_group_check), so a pair's least image
// over the group takes O(4 phi(L) L^2) work; pairs with equal least images
// are in one class, and the class size is the group order over the number
// of elements that fix the pair (orbit-stabiliser).  For L < 3 class_kernel
// applies every element of the closure with the reference's application
// rule (equivalence.cpp:97-144), hashing the images of several pairs per
// pass over the transposed table and looking them up in a hash set of the
// input pairs.  Either way the host then replays the reference's in-order
// erase loop (filter.cpp:117-144) on those class sizes and member lists.
#include <algorithm>
#include <chrono>
#include <stdexcept>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "ctx.h"

namespace {

constexpr int kMaxW = 256;  // 2L entries per pair

// Entry o of the image of the pair under generator g: the generator table
// is stored transposed (srcT[o * ng + g], signed 1-based source position),
// so that a warp's consecutive generators read consecutive entries.
__device__ __forceinline__ int image_at(const int16_t* srcT, int64_t ng, int64_t g, const int8_t* sx, int o) {
    const int s = srcT[(int64_t)o * ng + g];
    const int v = sx[(s < 0 ? -s : s) - 1];
    return s < 0 ? -v : v;
}

constexpr int kPairsPerCta = 8;  // pairs whose images one pass over the generator table hashes

// FNV-1a over the entries as bytes (value mod 256), folded; the host hashes
// the input pairs with the same steps
__host__ __device__ __forceinline__ uint32_t fnv_step(uint32_t h, int v) { return (h ^ (uint8_t)v) * 16777619u; }
__host__ __device__ __forceinline__ uint32_t fnv_fold(uint32_t h) { return h ^ (h >> 15); }
constexpr uint32_t kFnvBasis = 2166136261u;

// the image of the pair sx under generator g equals target (W entries)
__device__ __forceinline__ bool image_equals(const int16_t* srcT, int64_t ng, int64_t g, const int8_t* sx,
                                             const int8_t* target, int W) {
    for (int o = 0; o < W; ++o)
        if (image_at(srcT, ng, g, sx, o) != target[o]) return false;
    return true;
}

struct ClassArgs {
    const int16_t* srcT;      // generator table, transposed: srcT[o * ng + g]
    int64_t ng;
    int64_t group0;           // first pair group of the launch
    const int8_t* pairs;      // np x W, sorted (the reference's set order)
    int64_t np;
    int W;
    const uint32_t* set_h;    // hash set of the pairs: folded hash, pair index (EMPTY: 0xFFFFFFFF)
    const uint32_t* set_i;
    uint32_t set_mask;
    uint32_t* stab;           // per pair: generators that fix it
    uint32_t* members;        // (pair, member) index pairs
    unsigned long long* nmembers;
    int64_t mcap;
    int* status;
};

// CTA b: pairs of group b / splits (kPairsPerCta consecutive pairs) and the
// generators of share b % splits.
__global__ void __launch_bounds__(256) class_kernel(ClassArgs a, int splits) {
    constexpr int PG = kPairsPerCta;
    __shared__ int8_t sx[PG][kMaxW];
    __shared__ uint32_t self_h[PG];
    const int64_t group = a.group0 + blockIdx.x / splits;
    const int part = blockIdx.x % splits;
    const int64_t x0 = group * PG;
    const int npg = (int)min((int64_t)PG, a.np - x0);
    const int W = a.W;
    for (int k = threadIdx.x; k < PG * W; k += blockDim.x) {
        const int p = k / W, o = k - p * W;
        sx[p][o] = p < npg ? a.pairs[(x0 + p) * W + o] : 0;
    }
    __syncthreads();
    if (threadIdx.x < PG) {
        uint32_t h = kFnvBasis;
        for (int o = 0; o < W; ++o) h = fnv_step(h, sx[threadIdx.x][o]);
        self_h[threadIdx.x] = fnv_fold(h);
    }
    __syncthreads();
    uint32_t stab[PG];
#pragma unroll
    for (int p = 0; p < PG; ++p) stab[p] = 0;
    const int64_t step = (int64_t)splits * blockDim.x;
    for (int64_t g = (int64_t)part * blockDim.x + threadIdx.x; g < a.ng; g += step) {
        uint32_t h[PG];
#pragma unroll
        for (int p = 0; p < PG; ++p) h[p] = kFnvBasis;
        for (int o = 0; o < W; ++o) {  // one read of the generator's entry serves every pair of the group
            const int sgn = a.srcT[(int64_t)o * a.ng + g];
            const int idx = (sgn < 0 ? -sgn : sgn) - 1;
#pragma unroll
            for (int p = 0; p < PG; ++p) {
                const int v = sx[p][idx];
                h[p] = fnv_step(h[p], sgn < 0 ? -v : v);
            }
        }
#pragma unroll
        for (int p = 0; p < PG; ++p) {
            if (p >= npg) continue;
            const uint32_t hp = fnv_fold(h[p]);
            if (hp == self_h[p] && image_equals(a.srcT, a.ng, g, sx[p], sx[p], W)) ++stab[p];
            for (uint32_t slot = hp & a.set_mask;; slot = (slot + 1) & a.set_mask) {
                const uint32_t m = a.set_i[slot];
                if (m == 0xFFFFFFFFu) break;
                if (a.set_h[slot] != hp || !image_equals(a.srcT, a.ng, g, sx[p], a.pairs + (int64_t)m * W, W))
                    continue;
                const unsigned long long pos = atomicAdd(a.nmembers, 1ull);
                if ((int64_t)pos < a.mcap) {
                    a.members[2 * pos] = (uint32_t)(x0 + p);
                    a.members[2 * pos + 1] = m;
                } else {
                    atomicCAS(a.status, 0, GP_KSTATUS_OVERFLOW);
                }
            }
        }
    }
#pragma unroll
    for (int p = 0; p < PG; ++p) {
        const uint32_t t = __reduce_add_sync(0xFFFFFFFFu, stab[p]);
        if ((threadIdx.x & 31) == 0 && t && p < npg) atomicAdd(&a.stab[x0 + p], t);
    }
}

// ------------------------------------------------------------ canonical forms
// For L >= 3 every element of the pair group is, on each half of the
// result, an affine map of one source half: optionally swap the halves,
// then
//     a'[i] = (-1)^(alpha i + beta_a) * src_a[(u i + s_a) mod L]
//     b'[i] = (-1)^(alpha i + beta_b) * src_b[(e u i + s_b) mod L]
// with u a unit mod L, e = +-1, s_a, s_b any shifts, and the signs only
// where the alternating negation is a generator (alpha, beta_a, beta_b:
// 8 patterns).  These 2 * 2 * phi(L) * L^2 (* 8) maps are all in the group
// (decimation by u, reversal of b, shifts of b and their conjugates by the
// swap, and the negation of one half, which the alternating negation and an
// odd shift give) and as many as its order, so they are the group;
// gp_debug_pair_group_check compares them with the closure.  Two pairs are
// in one class iff they have the same least image (lexicographic, entries as
// signed integers), and the class size is the group order over the number of
// elements that fix the pair.  Per (swap, e, signs, u) the least image takes
// the least shift of each half separately, so a pair costs
// O(4 phi(L) (8) L^2) instead of O(|G| L).
struct CanonArgs {
    const int8_t* pairs;   // np x W
    int64_t np;
    int L;
    const int16_t* units;  // every unit mod L
    int nu;
    int alt;               // 1: the 8 sign patterns
    int8_t* canon;         // np x W: least image
    uint32_t* fixers;      // elements fixing the pair
};

struct Combo {
    int ha, hb;  // source half of a' and b' (offset 0 or L)
    int ma, mb;  // multipliers
    int pa, pb;  // sign pattern: bit 0 alpha, bit 1 beta
};

__device__ __forceinline__ Combo combo_of(const CanonArgs& a, int c) {
    const int swap = c & 1;
    c >>= 1;
    const int e = c & 1;
    c >>= 1;
    int alpha = 0, ba = 0, bb = 0;
    if (a.alt) {
        alpha = c & 1;
        ba = (c >> 1) & 1;
        bb = (c >> 2) & 1;
        c >>= 3;
    }
    const int u = a.units[c];
    Combo k;
    k.ha = swap ? a.L : 0;
    k.hb = swap ? 0 : a.L;
    k.ma = u;
    k.mb = e ? a.L - u : u;
    k.pa = alpha | (ba << 1);
    k.pb = alpha | (bb << 1);
    return k;
}

// (-1)^(alpha i + beta) for pattern pat
__device__ __forceinline__ int sign_of(int pat, int i) { return (((pat & 1) & i) ^ (pat >> 1)) ? -1 : 1; }

// Entry o of the image of x under (combo, s_a, s_b).
__device__ __forceinline__ int image_entry(const int8_t* x, int L, const Combo& k, int sa, int sb, int o) {
    if (o < L) return sign_of(k.pa, o) * x[k.ha + (int)(((long long)k.ma * o + sa) % L)];
    const int i = o - L;
    return sign_of(k.pb, i) * x[k.hb + (int)(((long long)k.mb * i + sb) % L)];
}

// The least shift of one half, H(s)[i] = sign(i) x[h + (m i + s) mod L],
// and how many shifts give exactly target.
__device__ void least_shift(const int8_t* x, int L, int h, int m, int pat, const int8_t* target, int& s_best,
                            int& n_fix) {
    s_best = 0;
    n_fix = 0;
    for (int s = 0; s < L; ++s) {
        int cmp = 0;  // sign of H(s) - H(s_best) at the first difference
        bool eq = true;
        int i1 = s, i2 = s_best;
        for (int i = 0; i < L; ++i) {
            const int sg = sign_of(pat, i);
            const int v = sg * x[h + i1];
            if (cmp == 0 && s > 0) {
                const int w = sg * x[h + i2];
                if (v != w) cmp = v < w ? -1 : 1;
            }
            if (eq && v != target[i]) eq = false;
            if (!eq && (cmp != 0 || s == 0)) break;
            i1 += m;
            i1 -= i1 >= L ? L : 0;
            i2 += m;
            i2 -= i2 >= L ? L : 0;
        }
        if (cmp < 0) s_best = s;
        n_fix += eq ? 1 : 0;
    }
}

// -1, 0, 1: image (c1, sa1, sb1) against image (c2, sa2, sb2)
__device__ int compare_images(const CanonArgs& a, const int8_t* x, int c1, int sa1, int sb1, int c2, int sa2,
                              int sb2) {
    const Combo k1 = combo_of(a, c1), k2 = combo_of(a, c2);
    for (int o = 0; o < 2 * a.L; ++o) {
        const int v = image_entry(x, a.L, k1, sa1, sb1, o), w = image_entry(x, a.L, k2, sa2, sb2, o);
        if (v != w) return v < w ? -1 : 1;
    }
    return 0;
}

constexpr int kCanonThreads = 128;

__global__ void __launch_bounds__(kCanonThreads) canon_kernel(CanonArgs a) {
    __shared__ int8_t x[kMaxW];
    __shared__ int s_c[kCanonThreads], s_sa[kCanonThreads], s_sb[kCanonThreads];
    __shared__ unsigned s_fix[kCanonThreads / 32];
    const int L = a.L, W = 2 * L;
    const int ncombo = 4 * a.nu * (a.alt ? 8 : 1);
    for (int64_t pr = blockIdx.x; pr < a.np; pr += gridDim.x) {
        __syncthreads();
        for (int o = threadIdx.x; o < W; o += blockDim.x) x[o] = a.pairs[pr * W + o];
        __syncthreads();
        int bc = -1, bsa = 0, bsb = 0;
        unsigned fix = 0;
        for (int c = threadIdx.x; c < ncombo; c += blockDim.x) {
            const Combo k = combo_of(a, c);
            int sa, sb, fa, fb;
            least_shift(x, L, k.ha, k.ma, k.pa, x, sa, fa);
            least_shift(x, L, k.hb, k.mb, k.pb, x + L, sb, fb);
            fix += (unsigned)(fa * fb);
            if (bc < 0 || compare_images(a, x, c, sa, sb, bc, bsa, bsb) < 0) {
                bc = c;
                bsa = sa;
                bsb = sb;
            }
        }
        s_c[threadIdx.x] = bc;
        s_sa[threadIdx.x] = bsa;
        s_sb[threadIdx.x] = bsb;
        fix = __reduce_add_sync(0xFFFFFFFFu, fix);
        if ((threadIdx.x & 31) == 0) s_fix[threadIdx.x >> 5] = fix;
        __syncthreads();
        for (int stride = kCanonThreads / 2; stride > 0; stride >>= 1) {
            if (threadIdx.x < stride) {
                const int o = threadIdx.x + stride;
                if (s_c[o] >= 0 &&
                    (s_c[threadIdx.x] < 0 || compare_images(a, x, s_c[o], s_sa[o], s_sb[o], s_c[threadIdx.x],
                                                            s_sa[threadIdx.x], s_sb[threadIdx.x]) < 0)) {
                    s_c[threadIdx.x] = s_c[o];
                    s_sa[threadIdx.x] = s_sa[o];
                    s_sb[threadIdx.x] = s_sb[o];
                }
            }
            __syncthreads();
        }
        const Combo k = combo_of(a, s_c[0]);
        for (int o = threadIdx.x; o < W; o += blockDim.x)
            a.canon[pr * W + o] = (int8_t)image_entry(x, L, k, s_sa[0], s_sb[0], o);
        if (threadIdx.x == 0) {
            unsigned t = 0;
            for (int w = 0; w < kCanonThreads / 32; ++w) t += s_fix[w];
            a.fixers[pr] = t;
        }
    }
}

std::vector<int16_t> all_units(int L) {
    std::vector<int16_t> u;
    for (int v = 1; v < L; ++v)
        if (std::gcd(v, L) == 1) u.push_back((int16_t)v);
    return u;
}

// Units that generate the group of units mod L (greedy: each one added is
// not yet in the subgroup generated by the ones before).
std::vector<int> unit_generators(int L) {
    std::vector<char> in(L, 0);
    std::vector<int> sub = {1 % L}, gens;
    if (L > 1) in[1] = 1;
    for (int u = 2; u < L; ++u) {
        if (std::gcd(u, L) != 1 || in[u]) continue;
        gens.push_back(u);
        for (size_t at = 0; at < sub.size(); ++at)  // closure of sub under multiplication by the generators
            for (int g : gens) {
                const int v = (int)((long long)sub[at] * g % L);
                if (!in[v]) {
                    in[v] = 1;
                    sub.push_back(v);
                }
            }
    }
    return gens;
}

// Closure of the identity pair under the reference's pair operations
// (filter.cpp:70-87: every shift of b, swap, reverse b, every decimation,
// and the alternating negation).  The closure is the group those operations
// generate, so it is built from a generating subset: shift by 1, swap,
// reverse, decimation by generators of the unit group, alternating
// negation.  Same set, about 15x less work at length 57.
// Returns the items flat: count x W entries.
//
// Every generator maps each half affinely (position i takes +-entry
// u*i + s of one half, one u for both halves up to sign, the sign set by the
// parity of i), and so does every product of them.  An element is therefore
// fixed by the entries at positions 0, 1, L and L+1: with by_key the closure
// compares those 64 bits instead of all 2L entries.  The items are built by
// applying generators, never inferred, so when that closure reaches the
// group's known size it is the group; pair_generators checks exactly that
// and otherwise redoes the closure comparing whole items.
uint64_t pair_group_size(int L, int compress);
extern const uint64_t kMaxGroupBytes;

std::vector<int16_t> pair_closure(int L, int compress, bool by_key) {
    const int W = 2 * L;
    const bool use_alt = !(compress > 1 || L % 2 == 1);  // filter.cpp:83-87
    const std::vector<int> units = unit_generators(L);
    std::vector<int16_t> out;            // items, W entries each
    std::vector<uint32_t> slot(1u << 10, UINT32_MAX);  // open addressing: item index per slot
    std::vector<uint64_t> keys;  // by_key: every item's key
    size_t count = 0;
    auto key_of = [&](const int16_t* v) {
        return (uint64_t)(uint16_t)v[0] | (uint64_t)(uint16_t)v[1] << 16 | (uint64_t)(uint16_t)v[L] << 32 |
               (uint64_t)(uint16_t)v[L + 1] << 48;
    };
    auto mix = [](uint64_t h) {  // MurmurHash3's 64-bit finaliser
        h ^= h >> 33;
        h *= 0xff51afd7ed558ccdULL;
        h ^= h >> 33;
        h *= 0xc4ceb9fe1a85ec53ULL;
        return h ^ (h >> 33);
    };
    auto hash = [&](const int16_t* v) {
        uint64_t h = 1469598103934665603ULL;  // FNV-1a over the whole item
        for (int i = 0; i < W; ++i) {
            h ^= (uint16_t)v[i];
            h *= 1099511628211ULL;
        }
        return h ^ (h >> 29);
    };
    auto grow = [&]() {
        std::vector<uint32_t> ns(slot.size() * 2, UINT32_MAX);
        const size_t mask = ns.size() - 1;
        for (size_t i = 0; i < count; ++i) {
            size_t h = (by_key ? mix(keys[i]) : hash(out.data() + i * W)) & mask;
            while (ns[h] != UINT32_MAX) h = (h + 1) & mask;
            ns[h] = (uint32_t)i;
        }
        slot.swap(ns);
    };
    auto add = [&](const int16_t* v) {
        if (2 * (count + 1) > slot.size()) grow();
        const size_t mask = slot.size() - 1;
        const uint64_t k = by_key ? key_of(v) : 0;
        size_t h = (by_key ? mix(k) : hash(v)) & mask;
        while (slot[h] != UINT32_MAX) {
            if (by_key ? keys[slot[h]] == k : std::memcmp(out.data() + (size_t)slot[h] * W, v, (size_t)W * 2) == 0)
                return;
            h = (h + 1) & mask;
        }
        slot[h] = (uint32_t)count++;
        out.insert(out.end(), v, v + W);
        if (by_key) keys.push_back(k);
    };
    auto find_key = [&](uint64_t k) {
        const size_t mask = slot.size() - 1;
        for (size_t h = mix(k) & mask; slot[h] != UINT32_MAX; h = (h + 1) & mask)
            if (keys[slot[h]] == k) return true;
        return false;
    };
    // the generators as maps: output position j takes (neg[j] ? -1 : 1) * input[src[j]]
    struct Gen {
        std::vector<int> src;
        std::vector<char> neg;
    };
    std::vector<Gen> gens;
    auto identity = [&]() {
        Gen g{std::vector<int>(W), std::vector<char>(W, 0)};
        for (int j = 0; j < W; ++j) g.src[j] = j;
        return g;
    };
    if (L > 1) {  // shift_pair by 1: rotate b left by 1
        Gen g = identity();
        for (int i = 0; i < L; ++i) g.src[L + i] = L + (i + 1) % L;
        gens.push_back(g);
    }
    {  // swap_pair
        Gen g = identity();
        for (int i = 0; i < L; ++i) {
            g.src[i] = L + i;
            g.src[L + i] = i;
        }
        gens.push_back(g);
    }
    {  // reverse_pair: reverse b
        Gen g = identity();
        for (int i = 0; i < L; ++i) g.src[L + i] = L + L - 1 - i;
        gens.push_back(g);
    }
    for (int u : units) {  // decimate_pair: both parts, new[i] = old[i*u mod L]
        Gen g = identity();
        for (int i = 0; i < L; ++i) {
            g.src[i] = (int)(((long long)i * u) % L);
            g.src[L + i] = L + g.src[i];
        }
        gens.push_back(g);
    }
    if (use_alt) {  // altnegative_pair: negate odd positions of both
        Gen g = identity();
        for (int i = 1; i < L; i += 2) g.neg[i] = g.neg[L + i] = 1;
        gens.push_back(g);
    }
    const uint64_t expect = pair_group_size(L, compress);
    if (expect * (uint64_t)W * 2 <= kMaxGroupBytes) out.reserve((size_t)expect * W);
    std::vector<int16_t> cur(W), n(W);
    auto at = [&](const Gen& g, int j) { return g.neg[j] ? (int16_t)-cur[g.src[j]] : cur[g.src[j]]; };
    for (int i = 0; i < L; ++i) {
        cur[i] = (int16_t)(i + 1);
        cur[L + i] = (int16_t)(L + i + 1);
    }
    add(cur.data());
    for (size_t item = 0; item < count; ++item) {
        std::memcpy(cur.data(), out.data() + item * W, (size_t)W * 2);
        for (const Gen& g : gens) {
            if (by_key) {  // look the image up by its key; write it out only when new
                const uint64_t k = (uint64_t)(uint16_t)at(g, 0) | (uint64_t)(uint16_t)at(g, 1) << 16 |
                                   (uint64_t)(uint16_t)at(g, L) << 32 | (uint64_t)(uint16_t)at(g, L + 1) << 48;
                if (find_key(k)) continue;
            }
            for (int j = 0; j < W; ++j) n[j] = at(g, j);
            add(n.data());
        }
    }
    return out;
}

std::vector<int16_t> pair_generators(int L, int compress) {
    if (L >= 3) {
        std::vector<int16_t> g = pair_closure(L, compress, true);
        if (g.size() == pair_group_size(L, compress) * (uint64_t)(2 * L)) return g;
    }
    return pair_closure(L, compress, false);
}

// Rewrites a generator item as "output position o takes +-input[src]" over
// the concatenated pair (a then b), following equivalence.cpp:108-136.
std::vector<int16_t> as_sources(const int16_t* item, int L) {
    std::vector<int16_t> out(2 * L);
    const int a0 = item[0];
    const bool swapped = (a0 < 0 && -a0 > L) || (a0 > 0 && a0 > L);
    for (int i = 0; i < L; ++i) {
        const int ia = item[i], ib = item[L + i];
        const int pa = ((ia < 0 ? -ia : ia) - 1) % L, pb = ((ib < 0 ? -ib : ib) - 1) % L;
        if (swapped) {
            // new b[i] = +-a[pa], new a[i] = +-b[pb]
            out[L + i] = (int16_t)((ia < 0 ? -1 : 1) * (pa + 1));
            out[i] = (int16_t)((ib < 0 ? -1 : 1) * (L + pb + 1));
        } else {
            out[i] = (int16_t)((ia < 0 ? -1 : 1) * (pa + 1));
            out[L + i] = (int16_t)((ib < 0 ? -1 : 1) * (L + pb + 1));
        }
    }
    return out;
}

uint64_t pair_group_size(int L, int compress);

// Class sizes and members of the pairs P (sorted, distinct) by canonical
// forms on the device (canon_kernel): member_list[span[i].first ..
// span[i].second) are the pairs with the same least image as pair i (itself
// included), csize[i] is the group order over the number of elements fixing
// pair i.  L >= 3.
int canonical_classes(gp_ctx* c, int L, int compress, const std::vector<std::vector<int8_t>>& P,
                      std::vector<unsigned long long>& csize, std::vector<uint32_t>& member_list,
                      std::vector<std::pair<uint32_t, uint32_t>>& span) {
    const int W = 2 * L;
    const int64_t np = (int64_t)P.size();
    const std::vector<int16_t> units = all_units(L);
    std::vector<int8_t> pairs((size_t)np * W);
    for (int64_t i = 0; i < np; ++i) std::memcpy(&pairs[(size_t)i * W], P[i].data(), W);
    cudaStream_t s = c->s_comp;
    DevBuf dp, du, dc, df;
    if (!dp.ensure(pairs.size()) || !du.ensure(units.size() * 2) || !dc.ensure(pairs.size()) ||
        !df.ensure((size_t)np * 4))
        return c->fail(GP_ERR_NOMEM, "equivalence filter: device allocation");
    GP_CUDA_TRY(c, cudaMemcpyAsync(dp.p, pairs.data(), pairs.size(), cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(du.p, units.data(), units.size() * 2, cudaMemcpyHostToDevice, s));
    CanonArgs ca{};
    ca.pairs = dp.as<int8_t>();
    ca.np = np;
    ca.L = L;
    ca.units = du.as<int16_t>();
    ca.nu = (int)units.size();
    ca.alt = !(compress > 1 || L % 2 == 1) ? 1 : 0;  // filter.cpp:83-87
    ca.canon = dc.as<int8_t>();
    ca.fixers = df.as<uint32_t>();
    const int64_t grid = std::min<int64_t>(np, (int64_t)c->num_sms * 16);
    canon_kernel<<<(unsigned)grid, kCanonThreads, 0, s>>>(ca);
    GP_CUDA_TRY(c, cudaGetLastError());
    std::vector<int8_t> canon(pairs.size());
    std::vector<uint32_t> fixers(np);
    GP_CUDA_TRY(c, cudaMemcpyAsync(canon.data(), dc.p, canon.size(), cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(fixers.data(), df.p, (size_t)np * 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    const uint64_t G = pair_group_size(L, compress);
    for (int64_t i = 0; i < np; ++i) {
        if (fixers[i] == 0 || G % fixers[i] != 0)
            return c->fail(GP_ERR_CUDA, "equivalence filter: %u of %llu elements fix pair %lld", fixers[i],
                           (unsigned long long)G, (long long)i);
        csize[i] = G / fixers[i];
    }
    // the classes: runs of equal least images
    std::vector<uint32_t> ord(np);
    for (int64_t i = 0; i < np; ++i) ord[i] = (uint32_t)i;
    auto row = [&](uint32_t i) { return canon.data() + (size_t)i * W; };
    std::sort(ord.begin(), ord.end(), [&](uint32_t x, uint32_t y) {
        const int d = std::memcmp(row(x), row(y), (size_t)W);
        return d != 0 ? d < 0 : x < y;
    });
    for (int64_t r0 = 0; r0 < np;) {
        int64_t r1 = r0 + 1;
        while (r1 < np && std::memcmp(row(ord[r0]), row(ord[r1]), (size_t)W) == 0) ++r1;
        for (int64_t k = r0; k < r1; ++k) span[ord[k]] = {(uint32_t)r0, (uint32_t)r1};
        r0 = r1;
    }
    member_list.swap(ord);
    return GP_OK;
}

// Size of the generator group: 4 phi(L) L^2, times 8 sign patterns with the
// alternating negation (exact for L >= 3, an upper bound at L = 2).
uint64_t pair_group_size(int L, int compress) {
    uint64_t phi = 0;
    for (int u = 1; u <= L; ++u)
        if (std::gcd(u, L) == 1) ++phi;
    const bool use_alt = !(compress > 1 || L % 2 == 1);
    return 4 * phi * (uint64_t)L * (uint64_t)L * (use_alt ? 8 : 1);
}

// The group's items take 2L int16 each on the host and again on the device.
extern const uint64_t kMaxGroupBytes = uint64_t(1) << 32;

}  // namespace

extern "C" {

// 1 when the affine parametrisation the canonical-form kernel enumerates
// (swap, e, signs, u, s_a, s_b) gives exactly the closure's group of length
// L at this compression, 0 when not, -1 when not applicable (L < 3 or too
// large).  Host only; a test hook.
int gp_debug_pair_group_check(int L, int compress) {
    if (L < 3 || 2 * L > kMaxW || compress < 1) return -1;
    if (pair_group_size(L, compress) * (uint64_t)(4 * L) > kMaxGroupBytes) return -1;
    const int W = 2 * L;
    const bool alt = !(compress > 1 || L % 2 == 1);
    const std::vector<int16_t> units = all_units(L);
    std::vector<std::vector<int16_t>> mine, closure;
    for (int swap = 0; swap < 2; ++swap)
        for (int e = 0; e < 2; ++e)
            for (int pat = 0; pat < (alt ? 8 : 1); ++pat)
                for (int16_t u : units)
                    for (int sa = 0; sa < L; ++sa)
                        for (int sb = 0; sb < L; ++sb) {
                            const int ha = swap ? L : 0, hb = swap ? 0 : L, ma = u, mb = e ? L - u : u;
                            const int alpha = pat & 1, ba = (pat >> 1) & 1, bb = (pat >> 2) & 1;
                            std::vector<int16_t> item(W);
                            for (int i = 0; i < L; ++i) {
                                const int sga = ((alpha & i) ^ ba) & 1 ? -1 : 1, sgb = ((alpha & i) ^ bb) & 1 ? -1 : 1;
                                item[i] = (int16_t)(sga * (ha + (int)(((long long)ma * i + sa) % L) + 1));
                                item[L + i] = (int16_t)(sgb * (hb + (int)(((long long)mb * i + sb) % L) + 1));
                            }
                            mine.push_back(std::move(item));
                        }
    const std::vector<int16_t> g = pair_generators(L, compress);
    for (size_t i = 0; i + W <= g.size(); i += W) closure.emplace_back(g.begin() + i, g.begin() + i + W);
    std::sort(mine.begin(), mine.end());
    std::sort(closure.begin(), closure.end());
    return mine == closure ? 1 : 0;
}

int64_t gp_debug_pair_generator_count(int L, int compress) {
    if (L < 1 || 2 * L > kMaxW || compress < 1) return -1;
    if (pair_group_size(L, compress) * (uint64_t)(4 * L) > kMaxGroupBytes) return -1;
    return (int64_t)(pair_generators(L, compress).size() / (size_t)(2 * L));
}

static int gp_equiv_filter_impl(gp_ctx* c, int order, int compress, const char* in_path, const char* out_path) {
    StageRange nvtx_range("gp_equiv_filter");
    if (!c || !in_path || !out_path) return GP_ERR_ARG;
    if (compress < 1 || order % compress) return c->fail(GP_ERR_ARG, "order %d not divisible by %d", order, compress);
    cudaSetDevice(c->device);
    const int L = order / compress;
    const int W = 2 * L;
    if (W > kMaxW) return c->fail(GP_ERR_UNSUPPORTED, "equivalence filter: length %d", L);
    if (L < 3 && pair_group_size(L, compress) * (uint64_t)(2 * W) > kMaxGroupBytes)  // the table path only
        return c->fail(GP_ERR_UNSUPPORTED, "equivalence filter: %llu generators at length %d exceed %llu bytes",
                       (unsigned long long)pair_group_size(L, compress), L, (unsigned long long)kMaxGroupBytes);
    // GP_EQUIV_TIMING=1 in the environment prints the phase times to stderr (diagnostics)
    static const bool timing = getenv("GP_EQUIV_TIMING") != nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    auto lap = [&](const char* what) {
        if (timing)
            fprintf(stderr, "[equiv] %s %.4f s\n", what,
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    };
    FILE* out = fopen(out_path, "w");  // filter.cpp:24 opens the output first
    FILE* in = fopen(in_path, "rb");
    if (!in) {
        if (out) fclose(out);
        return GP_OK;  // filter.cpp:33-37: "Bad File." and success
    }
    // the generator group depends only on (L, compression): built on a host
    // thread while the pairs are read and sorted
    std::vector<int16_t> gens;
    bool group_failed = false;
    std::thread group_thread;
    if (L < 3)  // the table of every element (longer lengths use canonical forms)
        group_thread = std::thread([&] {
            try {
                gens = pair_generators(L, compress);
            } catch (const std::exception&) {
                group_failed = true;
            }
        });
    struct Joiner {
        std::thread& t;
        ~Joiner() {
            if (t.joinable()) t.join();
        }
    } joiner{group_thread};
    // filter.cpp:45-62: L values for a, then (if the stream is still good) L
    // for b: whitespace-separated integers up to the first token that is not
    // one, W per pair, a trailing partial pair dropped
    std::vector<std::vector<int8_t>> P;
    {
        std::string text;
        fseek(in, 0, SEEK_END);
        const long sz = ftell(in);
        fseek(in, 0, SEEK_SET);
        text.resize(sz > 0 ? (size_t)sz : 0);
        text.resize(sz > 0 ? fread(&text[0], 1, (size_t)sz, in) : 0);
        fclose(in);
        std::vector<int8_t> cur;
        const char* q = text.c_str();
        for (;;) {
            char* e;
            const long v = strtol(q, &e, 10);
            if (e == q) break;
            q = e;
            cur.push_back((int8_t)v);
            if ((int)cur.size() == W) {
                P.push_back(cur);
                cur.clear();
            }
        }
    }
    lap("read");
    std::sort(P.begin(), P.end());
    P.erase(std::unique(P.begin(), P.end()), P.end());
    const int64_t np = (int64_t)P.size();
    std::vector<char> alive(np, 1);
    if (np > 0) {
        std::vector<unsigned long long> csize(np);
        // the input pairs of each pair's class: member_list[span[i].first .. span[i].second)
        std::vector<uint32_t> member_list;
        std::vector<std::pair<uint32_t, uint32_t>> span(np);
        if (L >= 3) {
            lap("sort");
            int rc = canonical_classes(c, L, compress, P, csize, member_list, span);
            if (rc) {
                if (out) fclose(out);
                return rc;
            }
            lap("classes");
        } else {
            lap("sort");
            group_thread.join();
            if (group_failed) {
                if (out) fclose(out);
                return c->fail(GP_ERR_NOMEM, "equivalence filter: generator group of length %d", L);
            }
            lap("group");
            const int64_t ng = (int64_t)(gens.size() / (size_t)W);
            std::vector<int16_t> items((size_t)ng * W);  // transposed: items[o * ng + g]
            {
                const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
                std::vector<std::thread> th;
                for (unsigned t = 0; t < nt; ++t)
                    th.emplace_back([&, t] {
                        // blocks of 64 generators: each thread writes whole cache lines of every row
                        for (int64_t g0 = (int64_t)t * 64; g0 < ng; g0 += (int64_t)nt * 64)
                            for (int64_t g = g0; g < std::min<int64_t>(g0 + 64, ng); ++g) {
                                const auto s = as_sources(gens.data() + (size_t)g * W, L);
                                for (int o = 0; o < W; ++o) items[(size_t)o * ng + g] = s[o];
                            }
                    });
                for (auto& x : th) x.join();
            }
            lap("table");
            std::vector<int8_t> pairs((size_t)np * W);
            for (int64_t i = 0; i < np; ++i)
                for (int j = 0; j < W; ++j) pairs[i * W + j] = P[i][j];
            // hash set of the pairs (the image lookup), same hash as the kernel's
            uint32_t set_size = 1;
            while (set_size < 2 * (uint64_t)np) set_size <<= 1;
            std::vector<uint32_t> set_h(set_size, 0), set_i(set_size, 0xFFFFFFFFu);
            for (int64_t i = 0; i < np; ++i) {
                uint32_t h = kFnvBasis;
                for (int j = 0; j < W; ++j) h = fnv_step(h, P[i][j]);
                h = fnv_fold(h);
                uint32_t slot = h & (set_size - 1);
                while (set_i[slot] != 0xFFFFFFFFu) slot = (slot + 1) & (set_size - 1);
                set_h[slot] = h;
                set_i[slot] = (uint32_t)i;
            }
            const int64_t mcap = std::max<int64_t>(np * 64, 1 << 20);
            cudaStream_t s = c->s_comp;
            DevBuf di, dp, dsh, dsi, dst, dm, dmisc;
            if (!di.ensure(items.size() * 2) || !dp.ensure(pairs.size()) || !dsh.ensure((size_t)set_size * 4) ||
                !dsi.ensure((size_t)set_size * 4) || !dst.ensure(np * 4) || !dm.ensure((size_t)mcap * 8) ||
                !dmisc.ensure(64))
                return c->fail(GP_ERR_NOMEM, "equivalence filter: device allocation");
            GP_CUDA_TRY(c, cudaMemcpyAsync(di.p, items.data(), items.size() * 2, cudaMemcpyHostToDevice, s));
            GP_CUDA_TRY(c, cudaMemcpyAsync(dp.p, pairs.data(), pairs.size(), cudaMemcpyHostToDevice, s));
            GP_CUDA_TRY(c, cudaMemcpyAsync(dsh.p, set_h.data(), (size_t)set_size * 4, cudaMemcpyHostToDevice, s));
            GP_CUDA_TRY(c, cudaMemcpyAsync(dsi.p, set_i.data(), (size_t)set_size * 4, cudaMemcpyHostToDevice, s));
            GP_CUDA_TRY(c, cudaMemsetAsync(dst.p, 0, np * 4, s));
            GP_CUDA_TRY(c, cudaMemsetAsync(dmisc.p, 0, 64, s));
            ClassArgs ca{};
            ca.srcT = di.as<int16_t>();
            ca.ng = ng;
            ca.pairs = dp.as<int8_t>();
            ca.np = np;
            ca.W = W;
            ca.set_h = dsh.as<uint32_t>();
            ca.set_i = dsi.as<uint32_t>();
            ca.set_mask = set_size - 1;
            ca.stab = dst.as<uint32_t>();
            ca.members = dm.as<uint32_t>();
            ca.nmembers = dmisc.as<unsigned long long>();
            ca.mcap = mcap;
            ca.status = c->status.as<int>();
            const int64_t groups = (np + kPairsPerCta - 1) / kPairsPerCta;
            // generator shares per group: enough CTAs for eight per SM, each share
            // at least one generator per thread
            const int64_t want = std::max<int64_t>(1, (8 * (int64_t)c->num_sms + groups - 1) / groups);
            const int splits = (int)std::max<int64_t>(1, std::min<int64_t>(want, (ng + 255) / 256));
            for (int64_t g0 = 0; g0 < groups; g0 += (int64_t(1) << 20)) {  // grids of at most 2^20 groups
                const int64_t gn = std::min<int64_t>(groups - g0, int64_t(1) << 20);
                ClassArgs cb = ca;
                cb.group0 = g0;
                class_kernel<<<(unsigned)(gn * splits), 256, 0, s>>>(cb, splits);
            }
            GP_CUDA_TRY(c, cudaGetLastError());
            GP_CUDA_TRY(c, cudaStreamSynchronize(s));
            lap("classes");
            int rc = c->check_status("equivalence filter");
            if (rc) {
                if (out) fclose(out);
                return rc;
            }
            std::vector<uint32_t> stab(np);
            unsigned long long nmem = 0;
            GP_CUDA_TRY(c, cudaMemcpy(stab.data(), dst.p, np * 4, cudaMemcpyDeviceToHost));
            GP_CUDA_TRY(c, cudaMemcpy(&nmem, dmisc.p, 8, cudaMemcpyDeviceToHost));
            // orbit-stabiliser: class size = group order / generators fixing the pair
            for (int64_t i = 0; i < np; ++i) {
                if (stab[i] == 0 || ng % stab[i] != 0) {
                    if (out) fclose(out);
                    return c->fail(GP_ERR_CUDA, "equivalence filter: stabiliser of pair %lld is %u of %lld generators",
                                   (long long)i, stab[i], (long long)ng);
                }
                csize[i] = (unsigned long long)(ng / stab[i]);
            }
            std::vector<uint32_t> mem((size_t)nmem * 2);
            if (nmem) GP_CUDA_TRY(c, cudaMemcpy(mem.data(), dm.p, mem.size() * 4, cudaMemcpyDeviceToHost));
            std::vector<std::vector<uint32_t>> members(np);
            for (unsigned long long i = 0; i < nmem; ++i) members[mem[2 * i]].push_back(mem[2 * i + 1]);
            for (int64_t i = 0; i < np; ++i) {
                span[i].first = (uint32_t)member_list.size();
                member_list.insert(member_list.end(), members[i].begin(), members[i].end());
                span[i].second = (uint32_t)member_list.size();
            }
        }
        // filter.cpp:117-144, in set order
        int64_t n_alive = np;
        for (int64_t it = 0; it < np; ++it) {
            if (!alive[it]) continue;
            const uint32_t* mb = member_list.data() + span[it].first;
            const uint32_t* me = member_list.data() + span[it].second;
            if ((int64_t)csize[it] > n_alive) {
                for (const uint32_t* m = mb; m < me; ++m)
                    if ((int64_t)*m > it && alive[*m]) {
                        alive[*m] = 0;
                        --n_alive;
                    }
            } else {
                for (const uint32_t* m = mb; m < me; ++m)
                    if (alive[*m]) {
                        alive[*m] = 0;
                        --n_alive;
                    }
                if (!alive[it]) {
                    alive[it] = 1;
                    ++n_alive;
                }
            }
        }
    }
    lap("erase");
    if (out) {
        // "%d " per entry of a, " ", "%d " per entry of b, newline
        std::string buf;
        buf.reserve((size_t)np * (3 * W + 2));
        auto put = [&](int v) {
            if (v < 0) {
                buf.push_back('-');
                v = -v;
            }
            char tmp[8];
            int n = 0;
            do {
                tmp[n++] = (char)('0' + v % 10);
                v /= 10;
            } while (v);
            while (n) buf.push_back(tmp[--n]);
            buf.push_back(' ');
        };
        for (int64_t i = 0; i < np; ++i) {
            if (!alive[i]) continue;
            for (int k = 0; k < L; ++k) put(P[i][k]);
            buf.push_back(' ');
            for (int k = 0; k < L; ++k) put(P[i][L + k]);
            buf.push_back('\n');
        }
        const bool ok = buf.empty() || fwrite(buf.data(), 1, buf.size(), out) == buf.size();
        if (fclose(out) != 0 || !ok) return c->fail(GP_ERR_IO, "equivalence filter: write failed: %s", out_path);
    }
    lap("written");
    return GP_OK;
}

// No C++ exception (an allocation failure on a huge input) crosses the C ABI.
int gp_equiv_filter(gp_ctx* c, int order, int compress, const char* in_path, const char* out_path) {
    try {
        return gp_equiv_filter_impl(c, order, compress, in_path, out_path);
    } catch (const std::exception& e) {
        return c ? c->fail(GP_ERR_NOMEM, "equivalence filter: %s", e.what()) : GP_ERR_NOMEM;
    }
}

}  // extern "C"
