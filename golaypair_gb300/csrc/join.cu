// join.cu -- device-resident signature join for the uncompression stage.
//
// The reference writes every PSD-passing expansion of a and of b to text,
// sorts both files and merge-joins them on the first token, the signature
// string (src/core/uncompression/uncompression.cpp:195-218,
// src/core/match/match_pairs.cpp:15-121).  A pair of an order-57 search
// expands to ~10^8 candidates per side, so here the records never leave the
// device:
//   sig_hash_kernel   64-bit FNV-1a of each record's signature string (the
//                     decimal digits the reference would print)
//   radix sort        both sides by that hash (prims.cu)
//   join_count_kernel per A record, the range of B records with the same hash
//   pair_check_kernel every candidate pair: exact signature-string equality
//                     (the reference joins on the string, so different
//                     vectors with equal concatenations do meet), then exact
//                     integer PAF (src/utils/golay.cpp:27-44)
// The few matched pairs are ordered on the host by their line text, which is
// the order the reference's sorted files and cross products produce.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "ctx.h"
#include "join.h"
#include "prims.h"
#include "rows.cuh"

namespace gp {

namespace {

unsigned grid_for(int64_t n, int cap_blocks = 65535 * 4) {
    int64_t g = (n + 255) / 256;
    if (g > cap_blocks) g = cap_blocks;
    return (unsigned)(g < 1 ? 1 : g);
}

__device__ __forceinline__ int ndigits(unsigned v) { return v >= 100 ? (v >= 1000 ? (v >= 10000 ? 5 : 4) : 3) : (v >= 10 ? 2 : 1); }

__global__ void sig_hash_kernel(const uint16_t* sig, int64_t n, int S, uint32_t* keys) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t h = 14695981039346656037ull;
        const uint16_t* s = sig + i * S;
        for (int k = 0; k < S; ++k) {
            const unsigned v = s[k];
            const int nd = ndigits(v);
            unsigned p = 1;
            for (int d = 1; d < nd; ++d) p *= 10;
            for (int d = 0; d < nd; ++d) {
                h ^= (uint64_t)('0' + (v / p) % 10);
                h *= 1099511628211ull;
                p /= 10;
            }
        }
        keys[2 * i] = (uint32_t)(h >> 32);
        keys[2 * i + 1] = (uint32_t)h;
    }
}

__global__ void paf_from_words_kernel(const uint4* words, int64_t n, int L, int b, int c, int H, int16_t* paf) {
    int8_t x[kMaxTcK];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint4 w = words[i];
        const uint64_t lo = ((uint64_t)w.y << 32) | w.x, hi = ((uint64_t)w.w << 32) | w.z;
        for (int j = 0; j < L; ++j) x[j] = (int8_t)(2 * word_digit(lo, hi, b, L, j) - c);
        for (int s = 1; s <= H; ++s) {
            int r = 0, j2 = s;
            for (int j = 0; j < L; ++j) {
                r += (int)x[j] * (int)x[j2];
                if (++j2 == L) j2 = 0;
            }
            paf[i * H + (s - 1)] = (int16_t)r;
        }
    }
}

__global__ void gather_keys_kernel(const uint32_t* keys, const uint32_t* idx, int64_t n, uint64_t* out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t r = idx[i];
        out[i] = ((uint64_t)keys[2 * r] << 32) | keys[2 * r + 1];
    }
}

__global__ void join_count_kernel(const uint64_t* ha, int64_t na, const uint64_t* hb, int64_t nb, uint32_t* lb,
                                  uint32_t* cnt) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < na; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t h = ha[i];
        int64_t lo = 0, hi = nb;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (hb[mid] < h)
                lo = mid + 1;
            else
                hi = mid;
        }
        int64_t e = lo;
        while (e < nb && hb[e] == h) ++e;
        lb[i] = (uint32_t)lo;
        cnt[i] = (uint32_t)(e - lo);
    }
}

// true when the decimal concatenations of two signatures are the same string
__device__ bool same_sig_string(const uint16_t* a, const uint16_t* b, int S) {
    int ia = 0, ib = 0;      // value index
    int da = -1, db = -1;    // digit position inside the current value (-1: load next)
    unsigned pa = 0, pb = 0, va = 0, vb = 0;
    for (;;) {
        if (da < 0) {
            if (ia == S) break;
            va = a[ia++];
            da = ndigits(va) - 1;
            pa = 1;
            for (int d = 0; d < da; ++d) pa *= 10;
        }
        if (db < 0) {
            if (ib == S) return false;
            vb = b[ib++];
            db = ndigits(vb) - 1;
            pb = 1;
            for (int d = 0; d < db; ++d) pb *= 10;
        }
        if ((va / pa) % 10 != (vb / pb) % 10) return false;
        pa /= 10;
        pb /= 10;
        --da;
        --db;
    }
    return db < 0 && ib == S;
}

__global__ void pair_check_kernel(const uint32_t* off, const uint32_t* lb, int64_t na, uint64_t total,
                                  const uint32_t* idxa, const uint32_t* idxb, const uint16_t* siga,
                                  const uint16_t* sigb, int S, const int16_t* pafa, const int16_t* pafb, int H,
                                  int target, uint32_t* out, unsigned long long* nout, int64_t cap, int* status) {
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total;
         w += (uint64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = na - 1;  // last A position with off <= w
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if ((uint64_t)off[mid] <= w)
                lo = mid;
            else
                hi = mid - 1;
        }
        const uint32_t ra = idxa[lo];
        const uint32_t rb = idxb[lb[lo] + (uint32_t)(w - off[lo])];
        const int16_t* pa = pafa + (int64_t)ra * H;
        const int16_t* pb = pafb + (int64_t)rb * H;
        bool ok = true;
        for (int s = 0; s < H && ok; ++s) ok = pa[s] + pb[s] == target;
        if (ok) ok = same_sig_string(siga + (int64_t)ra * S, sigb + (int64_t)rb * S, S);
        if (ok) {
            const unsigned long long pos = atomicAdd(nout, 1ull);
            if ((int64_t)pos < cap) {
                out[2 * pos] = ra;
                out[2 * pos + 1] = rb;
            } else {
                atomicCAS(status, 0, GP_KSTATUS_OVERFLOW);
            }
        }
    }
}

}  // namespace

int device_join(gp_ctx* c, const JoinSide& A, const JoinSide& B, int L, int pack_bits, int alpha_c, int target,
                std::vector<std::pair<uint32_t, uint32_t>>& matches) {
    matches.clear();
    if (A.n == 0 || B.n == 0) return GP_OK;
    cudaStream_t s = c->s_comp;
    const int S = L - 1, H = L / 2;
    const int64_t na = A.n, nb = B.n;
    DevBuf &ka = c->ux[14], &kb = c->ux[15], &ia = c->ux[16], &ib = c->ux[17], &tmp = c->ux[18], &ha = c->ux[19],
           &hb = c->ux[20], &pa = c->ux[21], &pb = c->ux[22], &lb = c->ux[23], &cnt = c->ux[24], &off = c->ux[25],
           &stmp = c->ux[26], &outp = c->ux[27], &misc = c->ux[28];
    const int64_t nmax = std::max(na, nb);
    if (!ka.ensure(na * 8) || !kb.ensure(nb * 8) || !ia.ensure(na * 4) || !ib.ensure(nb * 4) ||
        !tmp.ensure(radix_sort_tmp_bytes(nmax)) || !ha.ensure(na * 8) || !hb.ensure(nb * 8) ||
        !pa.ensure(na * H * 2 + 16) || !pb.ensure(nb * H * 2 + 16) || !lb.ensure(na * 4) || !cnt.ensure(na * 4) ||
        !off.ensure(na * 4 + 4) || !stmp.ensure(scan_tmp_bytes(na)) || !misc.ensure(64))
        return c->fail(GP_ERR_NOMEM, "join: device allocation");
    sig_hash_kernel<<<grid_for(na), 256, 0, s>>>(A.sig, na, S, ka.as<uint32_t>());
    sig_hash_kernel<<<grid_for(nb), 256, 0, s>>>(B.sig, nb, S, kb.as<uint32_t>());
    paf_from_words_kernel<<<grid_for(na, 4096), 256, 0, s>>>(A.words, na, L, pack_bits, alpha_c, H, pa.as<int16_t>());
    paf_from_words_kernel<<<grid_for(nb, 4096), 256, 0, s>>>(B.words, nb, L, pack_bits, alpha_c, H, pb.as<int16_t>());
    GP_CUDA_TRY(c, cudaGetLastError());
    GP_CUDA_TRY(c, iota_u32(ia.as<uint32_t>(), na, s));
    GP_CUDA_TRY(c, iota_u32(ib.as<uint32_t>(), nb, s));
    GP_CUDA_TRY(c, radix_sort_keys(ka.as<uint32_t>(), 2, 2, ia.as<uint32_t>(), na, tmp.p, s));
    GP_CUDA_TRY(c, radix_sort_keys(kb.as<uint32_t>(), 2, 2, ib.as<uint32_t>(), nb, tmp.p, s));
    gather_keys_kernel<<<grid_for(na), 256, 0, s>>>(ka.as<uint32_t>(), ia.as<uint32_t>(), na, ha.as<uint64_t>());
    gather_keys_kernel<<<grid_for(nb), 256, 0, s>>>(kb.as<uint32_t>(), ib.as<uint32_t>(), nb, hb.as<uint64_t>());
    join_count_kernel<<<grid_for(na), 256, 0, s>>>(ha.as<uint64_t>(), na, hb.as<uint64_t>(), nb, lb.as<uint32_t>(),
                                                   cnt.as<uint32_t>());
    GP_CUDA_TRY(c, cudaGetLastError());
    GP_CUDA_TRY(c, exclusive_scan_u32(cnt.as<uint32_t>(), off.as<uint32_t>(), na, stmp.as<uint32_t>(), s));
    uint32_t last_off = 0, last_cnt = 0;
    GP_CUDA_TRY(c, cudaMemcpyAsync(&last_off, off.as<uint32_t>() + na - 1, 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(&last_cnt, cnt.as<uint32_t>() + na - 1, 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    const uint64_t total = (uint64_t)last_off + last_cnt;
    if (total == 0) return GP_OK;
    if (total >= (uint64_t(1) << 32)) return c->fail(GP_ERR_UNSUPPORTED, "join: %llu candidate pairs", (unsigned long long)total);
    const int64_t cap = std::max<int64_t>(1 << 16, std::min<int64_t>((int64_t)total, int64_t(1) << 26));
    if (!outp.ensure((size_t)cap * 8)) return c->fail(GP_ERR_NOMEM, "join: output");
    GP_CUDA_TRY(c, cudaMemsetAsync(misc.p, 0, 64, s));
    pair_check_kernel<<<grid_for((int64_t)total), 256, 0, s>>>(
        off.as<uint32_t>(), lb.as<uint32_t>(), na, total, ia.as<uint32_t>(), ib.as<uint32_t>(), A.sig, B.sig, S,
        pa.as<int16_t>(), pb.as<int16_t>(), H, target, outp.as<uint32_t>(), misc.as<unsigned long long>(), cap,
        c->status.as<int>());
    GP_CUDA_TRY(c, cudaGetLastError());
    unsigned long long nm = 0;
    GP_CUDA_TRY(c, cudaMemcpyAsync(&nm, misc.p, 8, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    int rc = c->check_status("join");
    if (rc) return rc;
    std::vector<uint32_t> h((size_t)nm * 2);
    if (nm) GP_CUDA_TRY(c, cudaMemcpy(h.data(), outp.p, h.size() * 4, cudaMemcpyDeviceToHost));
    for (unsigned long long i = 0; i < nm; ++i) matches.emplace_back(h[2 * i], h[2 * i + 1]);
    return GP_OK;
}

}  // namespace gp
