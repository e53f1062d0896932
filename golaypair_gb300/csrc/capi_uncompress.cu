// capi_uncompress.cu -- uncompression stage (kernel (d), first half).
//
// Replaces uncompress_pipeline / uncompress_recursive
// (src/core/uncompression/uncompression.cpp:32-210) and the GPU stub it can
// dispatch to (src/core/uncompression/gpu/uncompress_gpu.cpp:17-92, whose
// kernel computes nothing).  For every compressed pair (a, b):
//   host    partition table per letter, the reference's rotation of the
//           sequence, the first entry's partitions reduced to their
//           rotation/reversal minima (uncompression.cpp:88-142);
//   device  expand_kernel: mixed-radix rank -> uncompressed word (entry i's
//           partition fills positions i, i+L, i+2L, ...; uncompression.cpp:
//           144-165), then the tensor-core PSD filter at the new length,
//           then finalize_kernel (exact FP64 PSD and signatures: a-side
//           inverted, b-side plain, uncompression.cpp:195-207);
//   device  sort + match of the two candidate sets (gp_sort_text /
//           gp_match_texts), pairs appended in input-pair order.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "ctx.h"
#include "finalize.h"
#include "host_math.h"

int gp_sort_text(gp_ctx* c, const std::string& text, std::string& out);
int gp_match_texts(gp_ctx* c, int L, int compress, int paf, const std::string& ta, const std::string& tb,
                   std::string& out, int64_t* n_pairs);

namespace {

constexpr int kMaxPos = 128;

struct ExpandArgs {
    int L;          // compressed length
    int r;          // parts per entry
    int Lnew;       // L * r
    int b;          // bits per new digit
    int cnew;       // new alphabet offset: digit = (value + cnew) / 2
    uint64_t rank0;
    int64_t n;
    const int* cnt;     // choices per position
    const int* off;     // offset of position i's table in vals (entries)
    const int8_t* vals; // choice values, r per choice
    uint4* words;
};

__global__ void expand_kernel(ExpandArgs a) {
    __shared__ int s_cnt[kMaxPos], s_off[kMaxPos];
    for (int i = threadIdx.x; i < a.L; i += blockDim.x) {
        s_cnt[i] = a.cnt[i];
        s_off[i] = a.off[i];
    }
    __syncthreads();
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.n; t += (int64_t)gridDim.x * blockDim.x) {
        uint64_t rank = a.rank0 + (uint64_t)t;
        uint64_t lo = 0, hi = 0;
        for (int i = a.L - 1; i >= 0; --i) {
            const uint64_t c = (uint64_t)s_cnt[i];
            const int d = (int)(rank % c);
            rank /= c;
            const int8_t* v = a.vals + (int64_t)(s_off[i] + d) * a.r;
            for (int q = 0; q < a.r; ++q) {
                const int p = i + a.L * q;
                const uint64_t digit = (uint64_t)((v[q] + a.cnew) >> 1);
                const int pos = a.b * (a.Lnew - 1 - p);
                if (pos >= 64)
                    hi |= digit << (pos - 64);
                else {
                    lo |= digit << pos;
                    if (pos + a.b > 64 && pos > 0) hi |= digit >> (64 - pos);
                }
            }
        }
        a.words[t] = make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
    }
}

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

struct Expansion {
    std::vector<int> cnt, off;
    std::vector<int8_t> vals;
    uint64_t total = 1;
    bool overflow = false;
};

// src/core/uncompression/uncompression.cpp:88-142 (orig is rotated in place)
Expansion plan_expansion(std::vector<int>& orig, int compress, int new_compress) {
    const std::vector<int> alpha = gp::alphabet(compress), nalpha = gp::alphabet(new_compress);
    const int r = compress / new_compress;
    std::vector<std::vector<int>> parts;
    combinations(r, nalpha, parts);
    std::map<int, std::vector<std::vector<int>>> partitions;
    for (int letter : alpha) {
        std::vector<std::vector<int>> list;
        for (auto part : parts) {
            int sum = 0;
            for (int v : part) sum += v;
            if (sum != letter) continue;
            do {
                list.push_back(part);
            } while (std::next_permutation(part.begin(), part.end()));
        }
        partitions[letter] = list;
    }
    // first distinct element (ascending) with the most partitions
    std::set<int> distinct(orig.begin(), orig.end());
    size_t best_n = 0;
    int best = orig[0];
    for (int e : distinct) {
        auto it = partitions.find(e);
        const size_t n = it == partitions.end() ? 0 : it->second.size();
        if (n > best_n) {
            best_n = n;
            best = e;
        }
    }
    // rotate left by i whenever orig[i] == best, on the already rotated sequence
    for (size_t i = 0; i < orig.size(); ++i)
        if (orig[i] == best) std::rotate(orig.begin(), orig.begin() + i, orig.end());
    // first entry: minima of each partition under rotation and reversal
    std::set<std::vector<int>> first;
    for (auto& perm : partitions[orig[0]]) {
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
    Expansion e;
    const int L = (int)orig.size();
    auto add = [&](const std::vector<std::vector<int>>& list) {
        e.off.push_back((int)(e.vals.size() / r));
        e.cnt.push_back((int)list.size());
        for (auto& v : list)
            for (int x : v) e.vals.push_back((int8_t)x);
        const uint64_t c = list.size();
        if (c == 0) {
            e.total = 0;
        } else if (e.total > (uint64_t(1) << 62) / c) {
            e.overflow = true;
        } else {
            e.total *= c;
        }
    };
    add(std::vector<std::vector<int>>(first.begin(), first.end()));
    for (int i = 1; i < L; ++i) add(partitions[orig[i]]);
    return e;
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

// Expands one compressed sequence on the device; appends the candidate lines
// of every expansion that passes the PSD filter to `text`.
int expand_one(gp_ctx* c, std::vector<int> orig, int order, int compress, int new_compress, int paf, bool invert,
               std::string& text, int64_t* n_exp) {
    const int L = (int)orig.size();
    Expansion e = plan_expansion(orig, compress, new_compress);
    if (e.overflow) return c->fail(GP_ERR_UNSUPPORTED, "uncompress: more than 2^62 expansions");
    const int r = compress / new_compress;
    const int Lnew = L * r;
    const std::vector<int> nalpha = gp::alphabet(new_compress);
    const int b = gp::bits_for((int)nalpha.size());
    if (L > kMaxPos || b * Lnew > 128 || !gp::tc_packed_supported(Lnew, b))
        return c->fail(GP_ERR_UNSUPPORTED, "uncompress: length %d over %d letters", Lnew, (int)nalpha.size());
    *n_exp += (int64_t)e.total;
    if (e.total == 0) return GP_OK;
    cudaStream_t s = c->s_comp;
    DevBuf dcnt, doff, dvals, dwords, dmask, dunsure, didx, dmisc, drec;
    const int64_t chunk = (int64_t)std::min<uint64_t>(e.total, uint64_t(1) << 24);
    if (!dcnt.ensure(L * 4) || !doff.ensure(L * 4) || !dvals.ensure(e.vals.size() + 16) || !dwords.ensure(chunk * 16) ||
        !dmask.ensure((chunk + 31) / 32 * 4) || !dunsure.ensure(chunk * 4) || !didx.ensure(chunk * 4) ||
        !dmisc.ensure(64))
        return c->fail(GP_ERR_NOMEM, "uncompress: device allocation");
    GP_CUDA_TRY(c, cudaMemcpyAsync(dcnt.p, e.cnt.data(), L * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(doff.p, e.off.data(), L * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dvals.p, e.vals.data(), e.vals.size(), cudaMemcpyHostToDevice, s));
    unsigned long long* misc = dmisc.as<unsigned long long>();  // [0] unsure [1] survivors [2] records [3] passes
    const gp::RowSrc src{nullptr, dwords.as<uint4>(), Lnew, b, new_compress};
    const double* tw = c->twiddle64(Lnew);
    if (!tw) return c->fail(GP_ERR_NOMEM, "twiddles");
    const int bound = 2 * order - paf;
    for (uint64_t r0 = 0; r0 < e.total; r0 += (uint64_t)chunk) {
        const int64_t n = (int64_t)std::min<uint64_t>((uint64_t)chunk, e.total - r0);
        ExpandArgs ea{L, r, Lnew, b, new_compress, r0, n, dcnt.as<int>(), doff.as<int>(), dvals.as<int8_t>(),
                      dwords.as<uint4>()};
        int64_t blocks = (n + 255) / 256;
        if (blocks > (int64_t)c->num_sms * 16) blocks = (int64_t)c->num_sms * 16;
        expand_kernel<<<(unsigned)blocks, 256, 0, s>>>(ea);
        GP_CUDA_TRY(c, cudaGetLastError());
        GP_CUDA_TRY(c, cudaMemsetAsync(misc, 0, 64, s));
        int rc = c->enqueue_filter(src, n, order, paf, GP_PSD_TC_GUARDED, dmask.as<uint32_t>(), dunsure.as<uint32_t>(),
                                   misc + 0, s);
        if (rc) return rc;
        GP_CUDA_TRY(c, gp::launch_mask_to_list(dmask.as<uint32_t>(), n, didx.as<uint32_t>(), misc + 1, n,
                                               c->status.as<int>(), c->num_sms, s));
        unsigned long long surv = 0;
        GP_CUDA_TRY(c, cudaMemcpyAsync(&surv, misc + 1, 8, cudaMemcpyDeviceToHost, s));
        GP_CUDA_TRY(c, cudaStreamSynchronize(s));
        rc = c->check_status("uncompress filter");
        if (rc) return rc;
        if (!surv) continue;
        const size_t rec_bytes = (size_t)surv * (16 + 1 + 2 * (Lnew - 1)) + 64;
        if (!drec.ensure(rec_bytes)) return c->fail(GP_ERR_NOMEM, "uncompress: records");
        uint8_t* rb = drec.as<uint8_t>();
        gp::FinalizeArgs fa;
        fa.src = src;
        fa.roles = nullptr;
        fa.fixed_role = 1;
        fa.idx = didx.as<uint32_t>();
        fa.n_idx = misc + 1;
        fa.idx_cap = n;
        fa.tw = tw;
        fa.thr = 2.0 * order - paf + 0.001;
        fa.bound = bound;
        fa.invert_roles = invert ? 1 : 0;
        fa.check_canonical = 0;
        fa.units = nullptr;
        fa.n_units = 0;
        fa.rec_words = reinterpret_cast<uint4*>(rb);
        fa.rec_role = rb + surv * 16;
        fa.rec_sig = reinterpret_cast<uint16_t*>(rb + surv * 17 + ((surv * 17) & 1));
        fa.rec_src = nullptr;
        fa.rec_count = misc + 2;
        fa.rec_cap = (int64_t)surv;
        fa.psd_pass = misc + 3;
        fa.status = c->status.as<int>();
        GP_CUDA_TRY(c, gp::launch_finalize(fa, (int64_t)surv, c->num_sms, s));
        unsigned long long nrec = 0;
        GP_CUDA_TRY(c, cudaMemcpyAsync(&nrec, misc + 2, 8, cudaMemcpyDeviceToHost, s));
        GP_CUDA_TRY(c, cudaStreamSynchronize(s));
        rc = c->check_status("uncompress finalize");
        if (rc) return rc;
        if (!nrec) continue;
        std::vector<uint4> w(nrec);
        std::vector<uint16_t> sg(nrec * (Lnew - 1));
        GP_CUDA_TRY(c, cudaMemcpy(w.data(), fa.rec_words, nrec * 16, cudaMemcpyDeviceToHost));
        GP_CUDA_TRY(c, cudaMemcpy(sg.data(), fa.rec_sig, sg.size() * 2, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nrec; ++i) {
            const gp::u128 word = ((gp::u128)w[i].w << 96) | ((gp::u128)w[i].z << 64) | ((gp::u128)w[i].y << 32) | w[i].x;
            text += "PSD";
            for (int k = 0; k < Lnew - 1; ++k) put_uint(text, sg[i * (Lnew - 1) + k]);
            text.push_back(' ');
            for (int j = 0; j < Lnew; ++j) {
                const int v = nalpha[gp::word_digit_h(word, b, Lnew, j)];
                if (v < 0) {
                    text.push_back('-');
                    put_uint(text, (unsigned)(-v));
                } else {
                    put_uint(text, (unsigned)v);
                }
                text.push_back(' ');
            }
            text.push_back('\n');
        }
    }
    return GP_OK;
}

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

}  // namespace

extern "C" {

int gp_uncompress(gp_ctx* c, int order, int compress, int new_compress, int paf, const char* in_pairs,
                  const char* out_pairs, const char* work_dir, const char* prefix) {
    if (!c || !in_pairs || !out_pairs) return GP_ERR_ARG;
    (void)work_dir;
    (void)prefix;
    cudaSetDevice(c->device);
    // the reference constructs its PairReader / PairWriter before the
    // pipeline runs (src/main.cpp:122-123): the output is truncated even
    // when nothing is uncompressed
    FILE* out = fopen(out_pairs, "w");
    if (!out) return c->fail(GP_ERR_IO, "uncompress: cannot open %s", out_pairs);
    if (compress <= 1) {  // uncompression.cpp:42
        fclose(out);
        return GP_OK;
    }
    if (new_compress < 1 || compress % new_compress || order % compress) {
        fclose(out);
        return c->fail(GP_ERR_ARG, "uncompress: compression %d -> %d of order %d", compress, new_compress, order);
    }
    std::string text;
    if (!slurp(in_pairs, text)) {
        fclose(out);
        return GP_OK;  // an unreadable input yields no pairs (the reader is simply not good)
    }
    const int L = order / compress;
    const char* p = text.data();
    const char* end = p + text.size();
    long line_no = 0;
    int rc = GP_OK;
    while (p < end && rc == GP_OK) {
        const char* nl = (const char*)memchr(p, '\n', (size_t)(end - p));
        if (!nl) nl = end;
        std::vector<int> vals;
        std::string line(p, nl);
        const char* q = line.c_str();
        while (*q) {
            while (*q == ' ' || *q == '\t' || *q == '\r') ++q;
            if (!*q) break;
            char* e2;
            const long v = strtol(q, &e2, 10);
            if (e2 == q) break;
            vals.push_back((int)v);
            q = e2;
        }
        p = nl + 1;
        // io.cpp:52-55: a line of the wrong length is an error
        if ((int)vals.size() != 2 * L) {
            rc = c->fail(GP_ERR_FORMAT, "PairReader: input line %ld: length is %zu. Expected %d", line_no, vals.size(),
                         2 * L);
            break;
        }
        ++line_no;
        std::vector<int> a(vals.begin(), vals.begin() + L), b(vals.begin() + L, vals.end());
        std::string ta, tb, sa, sb, pairs;
        int64_t na = 0, nb = 0;
        rc = expand_one(c, a, order, compress, new_compress, paf, true, ta, &na);
        if (rc) break;
        rc = expand_one(c, b, order, compress, new_compress, paf, false, tb, &nb);
        if (rc) break;
        rc = gp_sort_text(c, ta, sa);
        if (rc) break;
        rc = gp_sort_text(c, tb, sb);
        if (rc) break;
        int64_t np = 0;
        const int mrc = gp_match_texts(c, order / new_compress, new_compress, paf, sa, sb, pairs, &np);
        if (mrc < 0) {
            rc = mrc;
            break;
        }
        fwrite(pairs.data(), 1, pairs.size(), out);
    }
    fclose(out);
    return rc;
}

}  // extern "C"
