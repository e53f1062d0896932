// capi_equiv.cu -- equivalence filter (kernel (d), second half).
//
// Replaces cache_filter (src/core/filter/filter.cpp:18-163).  The generator
// set is the closure of the index pair ({1..L}, {L+1..2L}) under the
// reference's pair operations (src/utils/equivalence.cpp:46-95,146-277):
// rotate b by 1..L-1, swap a and b, reverse b, decimate both by every unit,
// and (compression 1, even L only) negate the odd positions of both.  It is
// built on the host, as the reference builds it once per run.
//
// class_kernel (several CTAs per pair, each a share of the generators)
// applies every generator to the pair with the reference's application rule
// (equivalence.cpp:97-144), counts the distinct images in a per-pair
// open-addressing table (generator ids; images are recomputed entry by
// entry, never stored) and looks every distinct image up in the sorted pair
// set.  The host then replays the reference's in-order erase loop
// (filter.cpp:117-144) on those class sizes and member lists.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
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

__device__ __forceinline__ uint32_t image_hash(const int16_t* srcT, int64_t ng, int64_t g, const int8_t* sx, int W) {
    uint32_t h = 2166136261u;
    for (int o = 0; o < W; ++o) {
        h ^= (uint8_t)image_at(srcT, ng, g, sx, o);
        h *= 16777619u;
    }
    return h ^ (h >> 15);
}

__device__ __forceinline__ bool same_image(const int16_t* srcT, int64_t ng, int64_t g1, int64_t g2, const int8_t* sx,
                                           int W) {
    for (int o = 0; o < W; ++o)
        if (image_at(srcT, ng, g1, sx, o) != image_at(srcT, ng, g2, sx, o)) return false;
    return true;
}

// keys: sorted pairs, W bytes each (value + 128, so byte order = int order);
// the image of generator g is compared entry by entry as it is computed
__device__ __forceinline__ int64_t find_image(const uint8_t* keys, int64_t np, int W, const int16_t* srcT, int64_t ng,
                                              int64_t g, const int8_t* sx) {
    int64_t lo = 0, hi = np - 1;
    while (lo <= hi) {
        const int64_t mid = (lo + hi) >> 1;
        const uint8_t* k = keys + mid * W;
        int c = 0;
        for (int i = 0; i < W; ++i) {
            const int a = k[i], b = image_at(srcT, ng, g, sx, i) + 128;
            if (a != b) {
                c = a < b ? -1 : 1;
                break;
            }
        }
        if (c == 0) return mid;
        if (c < 0)
            lo = mid + 1;
        else
            hi = mid - 1;
    }
    return -1;
}

// CTA b handles pair p0 + b / splits and the generators of its share
// (b % splits): the CTAs of one pair share its open-addressing table of
// generator ids, so each distinct image is counted once.
__global__ void class_kernel(const int16_t* srcT, int64_t ng, const int8_t* pairs, const uint8_t* keys, int64_t np,
                             int W, int64_t p0, int splits, int32_t* tables, int64_t tsize,
                             unsigned long long* class_size, uint32_t* members, unsigned long long* nmembers,
                             int64_t mcap, int* status) {
    const int64_t local = blockIdx.x / splits;
    const int part = blockIdx.x % splits;
    const int64_t x = p0 + local;
    const int8_t* xs = pairs + x * W;
    int32_t* tab = tables + local * tsize;
    __shared__ int8_t sx[kMaxW];
    for (int i = threadIdx.x; i < W; i += blockDim.x) sx[i] = xs[i];
    __syncthreads();
    unsigned distinct = 0;
    const int64_t step = (int64_t)splits * blockDim.x;
    for (int64_t g = (int64_t)part * blockDim.x + threadIdx.x; g < ng; g += step) {
        int64_t h = (int64_t)(image_hash(srcT, ng, g, sx, W) & (uint32_t)(tsize - 1));
        bool inserted = false;
        for (int64_t probe = 0; probe < tsize; ++probe) {
            const int32_t old = atomicCAS(&tab[h], -1, (int32_t)g);
            if (old == -1) {
                inserted = true;
                break;
            }
            if (same_image(srcT, ng, g, old, sx, W)) break;
            h = (h + 1) & (tsize - 1);
        }
        if (!inserted) continue;
        ++distinct;
        const int64_t m = find_image(keys, np, W, srcT, ng, g, sx);
        if (m >= 0) {
            const unsigned long long pos = atomicAdd(nmembers, 1ull);
            if ((int64_t)pos < mcap) {
                members[2 * pos] = (uint32_t)x;
                members[2 * pos + 1] = (uint32_t)m;
            } else {
                atomicCAS(status, 0, GP_KSTATUS_OVERFLOW);
            }
        }
    }
    distinct = __reduce_add_sync(0xFFFFFFFFu, distinct);
    if ((threadIdx.x & 31) == 0 && distinct) atomicAdd(&class_size[x], (unsigned long long)distinct);
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

int64_t gp_debug_pair_generator_count(int L, int compress) {
    if (L < 1 || 2 * L > kMaxW || compress < 1) return -1;
    if (pair_group_size(L, compress) * (uint64_t)(4 * L) > kMaxGroupBytes) return -1;
    return (int64_t)(pair_generators(L, compress).size() / (size_t)(2 * L));
}

int gp_equiv_filter(gp_ctx* c, int order, int compress, const char* in_path, const char* out_path) {
    StageRange nvtx_range("gp_equiv_filter");
    if (!c || !in_path || !out_path) return GP_ERR_ARG;
    if (compress < 1 || order % compress) return c->fail(GP_ERR_ARG, "order %d not divisible by %d", order, compress);
    cudaSetDevice(c->device);
    const int L = order / compress;
    const int W = 2 * L;
    if (W > kMaxW) return c->fail(GP_ERR_UNSUPPORTED, "equivalence filter: length %d", L);
    if (pair_group_size(L, compress) * (uint64_t)(2 * W) > kMaxGroupBytes)
        return c->fail(GP_ERR_UNSUPPORTED, "equivalence filter: %llu generators at length %d exceed %llu bytes",
                       (unsigned long long)pair_group_size(L, compress), L, (unsigned long long)kMaxGroupBytes);
    FILE* out = fopen(out_path, "w");  // filter.cpp:24 opens the output first
    FILE* in = fopen(in_path, "rb");
    if (!in) {
        if (out) fclose(out);
        return GP_OK;  // filter.cpp:33-37: "Bad File." and success
    }
    // filter.cpp:45-62: L values for a, then (if the stream is still good) L for b
    std::vector<std::vector<int8_t>> P;
    {
        std::vector<int8_t> cur;
        long v;
        while (fscanf(in, "%ld", &v) == 1) {
            cur.push_back((int8_t)v);
            if ((int)cur.size() == W) {
                P.push_back(cur);
                cur.clear();
            }
        }
        fclose(in);
    }
    std::sort(P.begin(), P.end());
    P.erase(std::unique(P.begin(), P.end()), P.end());
    const int64_t np = (int64_t)P.size();
    std::vector<char> alive(np, 1);
    if (np > 0) {
        const auto gens = pair_generators(L, compress);
        const int64_t ng = (int64_t)(gens.size() / (size_t)W);
        std::vector<int16_t> items((size_t)ng * W);  // transposed: items[o * ng + g]
        for (int64_t g = 0; g < ng; ++g) {
            const auto s = as_sources(gens.data() + (size_t)g * W, L);
            for (int o = 0; o < W; ++o) items[(size_t)o * ng + g] = s[o];
        }
        std::vector<int8_t> pairs((size_t)np * W);
        std::vector<uint8_t> keys((size_t)np * W);
        for (int64_t i = 0; i < np; ++i)
            for (int j = 0; j < W; ++j) {
                pairs[i * W + j] = P[i][j];
                keys[i * W + j] = (uint8_t)(P[i][j] + 128);
            }
        int64_t tsize = 1;
        while (tsize < 2 * ng) tsize <<= 1;
        int64_t batch = std::max<int64_t>(1, std::min<int64_t>(np, (int64_t(1) << 28) / (tsize * 4)));
        const int64_t mcap = std::max<int64_t>(np * 64, 1 << 20);
        cudaStream_t s = c->s_comp;
        DevBuf di, dp, dk, dt, dcs, dm, dmisc;
        if (!di.ensure(items.size() * 2) || !dp.ensure(pairs.size()) || !dk.ensure(keys.size()) ||
            !dt.ensure((size_t)batch * tsize * 4) || !dcs.ensure(np * 8) || !dm.ensure((size_t)mcap * 8) ||
            !dmisc.ensure(64))
            return c->fail(GP_ERR_NOMEM, "equivalence filter: device allocation");
        GP_CUDA_TRY(c, cudaMemcpyAsync(di.p, items.data(), items.size() * 2, cudaMemcpyHostToDevice, s));
        GP_CUDA_TRY(c, cudaMemcpyAsync(dp.p, pairs.data(), pairs.size(), cudaMemcpyHostToDevice, s));
        GP_CUDA_TRY(c, cudaMemcpyAsync(dk.p, keys.data(), keys.size(), cudaMemcpyHostToDevice, s));
        GP_CUDA_TRY(c, cudaMemsetAsync(dcs.p, 0, np * 8, s));
        GP_CUDA_TRY(c, cudaMemsetAsync(dmisc.p, 0, 64, s));
        for (int64_t p0 = 0; p0 < np; p0 += batch) {
            const int64_t nb = std::min(batch, np - p0);
            // CTAs per pair: enough for four CTAs per SM, each with at least
            // one generator per thread
            const int64_t want = std::max<int64_t>(1, (4 * (int64_t)c->num_sms + nb - 1) / nb);
            const int splits = (int)std::max<int64_t>(1, std::min<int64_t>(want, (ng + 255) / 256));
            GP_CUDA_TRY(c, cudaMemsetAsync(dt.p, 0xFF, (size_t)nb * tsize * 4, s));
            class_kernel<<<(unsigned)(nb * splits), 256, 0, s>>>(
                di.as<int16_t>(), ng, dp.as<int8_t>(), dk.as<uint8_t>(), np, W, p0, splits, dt.as<int32_t>(), tsize,
                dcs.as<unsigned long long>(), dm.as<uint32_t>(), dmisc.as<unsigned long long>(), mcap,
                c->status.as<int>());
            GP_CUDA_TRY(c, cudaGetLastError());
        }
        GP_CUDA_TRY(c, cudaStreamSynchronize(s));
        int rc = c->check_status("equivalence filter");
        if (rc) {
            if (out) fclose(out);
            return rc;
        }
        std::vector<unsigned long long> csize(np);
        unsigned long long nmem = 0;
        GP_CUDA_TRY(c, cudaMemcpy(csize.data(), dcs.p, np * 8, cudaMemcpyDeviceToHost));
        GP_CUDA_TRY(c, cudaMemcpy(&nmem, dmisc.p, 8, cudaMemcpyDeviceToHost));
        std::vector<uint32_t> mem((size_t)nmem * 2);
        if (nmem) GP_CUDA_TRY(c, cudaMemcpy(mem.data(), dm.p, mem.size() * 4, cudaMemcpyDeviceToHost));
        std::vector<std::vector<uint32_t>> members(np);
        for (unsigned long long i = 0; i < nmem; ++i) members[mem[2 * i]].push_back(mem[2 * i + 1]);
        // filter.cpp:117-144, in set order
        int64_t n_alive = np;
        for (int64_t it = 0; it < np; ++it) {
            if (!alive[it]) continue;
            if ((int64_t)csize[it] > n_alive) {
                for (uint32_t m : members[it])
                    if ((int64_t)m > it && alive[m]) {
                        alive[m] = 0;
                        --n_alive;
                    }
            } else {
                for (uint32_t m : members[it])
                    if (alive[m]) {
                        alive[m] = 0;
                        --n_alive;
                    }
                if (!alive[it]) {
                    alive[it] = 1;
                    ++n_alive;
                }
            }
        }
    }
    if (out) {
        for (int64_t i = 0; i < np; ++i) {
            if (!alive[i]) continue;
            for (int k = 0; k < L; ++k) fprintf(out, "%d ", P[i][k]);
            fprintf(out, " ");
            for (int k = 0; k < L; ++k) fprintf(out, "%d ", P[i][L + k]);
            fprintf(out, "\n");
        }
        fclose(out);
    }
    return GP_OK;
}

}  // extern "C"
