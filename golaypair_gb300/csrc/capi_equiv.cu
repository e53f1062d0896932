// capi_equiv.cu -- equivalence filter (kernel (d), second half).
//
// Replaces cache_filter (src/core/filter/filter.cpp:18-163).  The generator
// set is the closure of the index pair ({1..L}, {L+1..2L}) under the
// reference's pair operations (src/utils/equivalence.cpp:46-95,146-277):
// rotate b by 1..L-1, swap a and b, reverse b, decimate both by every unit,
// and (compression 1, even L only) negate the odd positions of both.  It is
// built on the host, as the reference builds it once per run.
//
// class_kernel (one CTA per pair) applies every generator to the pair with
// the reference's application rule (equivalence.cpp:97-144), counts the
// distinct images in a per-pair open-addressing table (generator ids, images
// compared by recomputation) and looks every distinct image up in the sorted
// pair set.  The host then replays the reference's in-order erase loop
// (filter.cpp:117-144) on those class sizes and member lists.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <unordered_set>
#include <vector>

#include "ctx.h"

namespace {

constexpr int kMaxW = 256;  // 2L entries per pair

__device__ __forceinline__ void apply_item(const int16_t* item, const int8_t* x, int W, int8_t* y) {
    for (int o = 0; o < W; ++o) {
        const int s = item[o];
        const int v = x[(s < 0 ? -s : s) - 1];
        y[o] = (int8_t)(s < 0 ? -v : v);
    }
}

__device__ __forceinline__ uint32_t hash_bytes(const int8_t* y, int W) {
    uint32_t h = 2166136261u;
    for (int i = 0; i < W; ++i) {
        h ^= (uint8_t)y[i];
        h *= 16777619u;
    }
    return h ^ (h >> 15);
}

// keys: sorted pairs, W bytes each (value + 128, so byte order = int order)
__device__ __forceinline__ int64_t find_pair(const uint8_t* keys, int64_t np, int W, const int8_t* y) {
    int64_t lo = 0, hi = np - 1;
    while (lo <= hi) {
        const int64_t mid = (lo + hi) >> 1;
        const uint8_t* k = keys + mid * W;
        int c = 0;
        for (int i = 0; i < W; ++i) {
            const int a = k[i], b = (int)(uint8_t)(y[i] + 128);
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

__global__ void class_kernel(const int16_t* items, int64_t nitems, const int8_t* pairs, const uint8_t* keys, int64_t np,
                             int W, int64_t p0, int32_t* tables, int64_t tsize, unsigned long long* class_size,
                             uint32_t* members, unsigned long long* nmembers, int64_t mcap, int* status) {
    const int64_t x = p0 + blockIdx.x;
    const int8_t* xs = pairs + x * W;
    int32_t* tab = tables + (int64_t)blockIdx.x * tsize;
    __shared__ int8_t sx[kMaxW];
    for (int i = threadIdx.x; i < W; i += blockDim.x) sx[i] = xs[i];
    __syncthreads();
    int8_t y[kMaxW], z[kMaxW];
    unsigned long long distinct = 0;
    for (int64_t g = threadIdx.x; g < nitems; g += blockDim.x) {
        apply_item(items + g * W, sx, W, y);
        int64_t h = (int64_t)(hash_bytes(y, W) & (uint32_t)(tsize - 1));
        bool inserted = false;
        for (int64_t probe = 0; probe < tsize; ++probe) {
            const int32_t old = atomicCAS(&tab[h], -1, (int32_t)g);
            if (old == -1) {
                inserted = true;
                break;
            }
            apply_item(items + (int64_t)old * W, sx, W, z);
            bool same = true;
            for (int i = 0; i < W; ++i)
                if (z[i] != y[i]) {
                    same = false;
                    break;
                }
            if (same) break;
            h = (h + 1) & (tsize - 1);
        }
        if (!inserted) continue;
        ++distinct;
        const int64_t m = find_pair(keys, np, W, y);
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
    if (distinct) atomicAdd(&class_size[x], distinct);
}

struct VecHash {
    size_t operator()(const std::vector<int16_t>& v) const {
        uint64_t h = 1469598103934665603ULL;
        for (int16_t x : v) {
            h ^= (uint16_t)x;
            h *= 1099511628211ULL;
        }
        return (size_t)h;
    }
};

// Closure of the identity pair under the reference's pair operations.
std::vector<std::vector<int16_t>> pair_generators(int L, int compress) {
    const int W = 2 * L;
    const bool use_alt = !(compress > 1 || L % 2 == 1);  // filter.cpp:83-87
    std::vector<int> units;
    for (int u = 1; u < L; ++u)
        if (std::gcd(u, L) == 1) units.push_back(u);
    std::vector<std::vector<int16_t>> out;
    std::unordered_set<std::vector<int16_t>, VecHash> seen;
    std::vector<int16_t> id(W);
    for (int i = 0; i < L; ++i) {
        id[i] = (int16_t)(i + 1);
        id[L + i] = (int16_t)(L + i + 1);
    }
    seen.insert(id);
    out.push_back(id);
    auto add = [&](std::vector<int16_t>&& v) {
        if (seen.insert(v).second) out.push_back(std::move(v));
    };
    for (size_t at = 0; at < out.size(); ++at) {
        const std::vector<int16_t> cur = out[at];
        for (int s = 1; s <= L - 1; ++s) {  // shift_pair: rotate b left by s
            std::vector<int16_t> n = cur;
            for (int i = 0; i < L; ++i) n[L + i] = cur[L + (i + s) % L];
            add(std::move(n));
        }
        {  // swap_pair
            std::vector<int16_t> n(W);
            for (int i = 0; i < L; ++i) {
                n[i] = cur[L + i];
                n[L + i] = cur[i];
            }
            add(std::move(n));
        }
        {  // reverse_pair: reverse b
            std::vector<int16_t> n = cur;
            for (int i = 0; i < L; ++i) n[L + i] = cur[L + L - 1 - i];
            add(std::move(n));
        }
        for (int u : units) {  // decimate_pair: both parts, new[i] = old[i*u mod L]
            std::vector<int16_t> n(W);
            for (int i = 0; i < L; ++i) {
                const int src = (int)(((long long)i * u) % L);
                n[i] = cur[src];
                n[L + i] = cur[L + src];
            }
            add(std::move(n));
        }
        if (use_alt) {  // altnegative_pair: negate odd positions of both
            std::vector<int16_t> n = cur;
            for (int i = 1; i < L; i += 2) {
                n[i] = (int16_t)-n[i];
                n[L + i] = (int16_t)-n[L + i];
            }
            add(std::move(n));
        }
    }
    return out;
}

// Rewrites a generator item as "output position o takes +-input[src]" over
// the concatenated pair (a then b), following equivalence.cpp:108-136.
std::vector<int16_t> as_sources(const std::vector<int16_t>& item, int L) {
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

}  // namespace

extern "C" {

int gp_equiv_filter(gp_ctx* c, int order, int compress, const char* in_path, const char* out_path) {
    if (!c || !in_path || !out_path) return GP_ERR_ARG;
    if (compress < 1 || order % compress) return c->fail(GP_ERR_ARG, "order %d not divisible by %d", order, compress);
    cudaSetDevice(c->device);
    const int L = order / compress;
    const int W = 2 * L;
    if (W > kMaxW) return c->fail(GP_ERR_UNSUPPORTED, "equivalence filter: length %d", L);
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
        const int64_t ng = (int64_t)gens.size();
        std::vector<int16_t> items((size_t)ng * W);
        for (int64_t g = 0; g < ng; ++g) {
            const auto s = as_sources(gens[g], L);
            std::copy(s.begin(), s.end(), items.begin() + g * W);
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
            GP_CUDA_TRY(c, cudaMemsetAsync(dt.p, 0xFF, (size_t)nb * tsize * 4, s));
            class_kernel<<<(unsigned)nb, 256, 0, s>>>(di.as<int16_t>(), ng, dp.as<int8_t>(), dk.as<uint8_t>(), np, W, p0,
                                                     dt.as<int32_t>(), tsize, dcs.as<unsigned long long>(),
                                                     dm.as<uint32_t>(), dmisc.as<unsigned long long>(), mcap,
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
