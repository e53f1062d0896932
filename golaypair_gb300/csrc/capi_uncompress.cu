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
//   device  the signature join of the two candidate sets (join.cu) with
//           exact PAF verification; only the matched pairs come back to
//           the host, where they are put in the reference's line order
//           (sorted a-line, then b-line) and appended in input-pair order.
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
#include "join.h"

namespace {

constexpr int kMaxPos = 128;
// context scratch buffers of the two sides' expansions (c->ux[slot .. slot+8]),
// two sets so that one pair expands while the previous one is joined (join.cu
// and the gather below use ux[8 .. 28])
constexpr int kSlotA[2] = {30, 48}, kSlotB[2] = {39, 57};

struct ExpandArgs {
    int L;          // compressed length
    int r;          // parts per entry
    int Lnew;       // L * r
    int b;          // bits per new digit
    int cnew;       // new alphabet offset: digit = (value + cnew) / 2
    uint64_t rank0;
    int64_t n;          // ranks rank0 .. rank0 + n - 1, n <= 2^24
    int d0[kMaxPos];    // mixed-radix digits of rank0 (position L-1 least significant)
    const uint64_t* inv;  // ceil(2^40 / cnt[i]): t / cnt[i] = t * inv[i] >> 40 for t < 2^24
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
    __shared__ uint64_t s_inv[kMaxPos];
    __shared__ int s_d0[kMaxPos];
    for (int i = threadIdx.x; i < a.L; i += blockDim.x) {
        s_inv[i] = a.inv[i];
        s_d0[i] = a.d0[i];
    }
    __syncthreads();
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.n; t += (int64_t)gridDim.x * blockDim.x) {
        // digits of rank0 + t: the digits of t (exact reciprocal division,
        // t < 2^24) added to those of rank0 with carry
        uint32_t rest = (uint32_t)t;
        int carry = 0;
        uint64_t lo = 0, hi = 0;
        for (int i = a.L - 1; i >= 0; --i) {
            const int c = s_cnt[i];
            const uint32_t q = (uint32_t)(((uint64_t)rest * s_inv[i]) >> 40);
            int d = (int)(rest - q * (uint32_t)c) + s_d0[i] + carry;
            rest = q;
            carry = d >= c;
            if (carry) d -= c;
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

// Device records of one side: packed words and signatures.
struct Side {
    DevBuf words, sig;
    int64_t n = 0, cap = 0;
    unsigned long long* nrec = nullptr;  // pinned: record count, copied back by the expansion's stream
    bool pending = false;                // enqueued, count not read yet
};

__global__ void gather_records_kernel(const uint4* words, const uint16_t* sig, int S, const uint32_t* rows, int64_t n,
                                      uint4* ow, uint16_t* os) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t r = rows[i];
        ow[i] = words[r];
        for (int k = 0; k < S; ++k) os[i * S + k] = sig[(int64_t)r * S + k];
    }
}

// Enqueues on stream s the expansion of one compressed sequence, keeping in
// `side` every expansion that passes the PSD filter, with its signature
// (uncompression.cpp:195-207; invert selects bound - rint(psd)).  Device
// scratch: the nine context buffers from c->ux[slot].  finish_side reads the
// record count once the stream is done.
int expand_side(gp_ctx* c, std::vector<int> orig, int order, int compress, int new_compress, int paf, bool invert,
                Side& side, int64_t* n_exp, cudaStream_t s, int slot) {
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
    side.n = 0;
    side.pending = false;
    if (e.total == 0) return GP_OK;
    DevBuf* ux = c->ux + slot;
    DevBuf &dcnt = ux[0], &doff = ux[1], &dvals = ux[2], &dwords = ux[3], &dmask = ux[4], &dunsure = ux[5],
           &didx = ux[6], &dmisc = ux[7], &dinv = ux[8];
    const int64_t chunk = (int64_t)std::min<uint64_t>(e.total, uint64_t(1) << 24);
    if (!dcnt.ensure(L * 4) || !doff.ensure(L * 4) || !dvals.ensure(e.vals.size() + 16) || !dwords.ensure(chunk * 16) ||
        !dmask.ensure((chunk + 31) / 32 * 4) || !dunsure.ensure(chunk * 4) || !didx.ensure(chunk * 4) ||
        !dmisc.ensure(64))
        return c->fail(GP_ERR_NOMEM, "uncompress: device allocation");
    // record arena: every expansion could pass; capped at 2^26 records
    side.cap = (int64_t)std::min<uint64_t>(e.total, uint64_t(1) << 26);
    if (!side.words.ensure((size_t)side.cap * 16) || !side.sig.ensure((size_t)side.cap * 2 * (Lnew - 1) + 16))
        return c->fail(GP_ERR_NOMEM, "uncompress: record arena");
    // exact for offsets below 2^24 while every count is at most 2^16
    for (int i = 0; i < L; ++i)
        if (e.cnt[i] > (1 << 16)) return c->fail(GP_ERR_UNSUPPORTED, "uncompress: %d choices for one entry", e.cnt[i]);
    std::vector<uint64_t> inv(L);
    for (int i = 0; i < L; ++i) inv[i] = ((uint64_t(1) << 40) + (uint64_t)e.cnt[i] - 1) / (uint64_t)e.cnt[i];
    if (!dinv.ensure(L * 8)) return c->fail(GP_ERR_NOMEM, "uncompress: device allocation");
    GP_CUDA_TRY(c, cudaMemcpyAsync(dinv.p, inv.data(), L * 8, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dcnt.p, e.cnt.data(), L * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(doff.p, e.off.data(), L * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dvals.p, e.vals.data(), e.vals.size(), cudaMemcpyHostToDevice, s));
    unsigned long long* misc = dmisc.as<unsigned long long>();  // [0] unsure [1] survivors [2] records [3] passes
    GP_CUDA_TRY(c, cudaMemsetAsync(misc, 0, 64, s));
    const gp::RowSrc src{nullptr, dwords.as<uint4>(), Lnew, b, new_compress};
    const double* tw = c->twiddle64(Lnew);
    if (!tw) return c->fail(GP_ERR_NOMEM, "twiddles");
    for (uint64_t r0 = 0; r0 < e.total; r0 += (uint64_t)chunk) {
        const int64_t n = (int64_t)std::min<uint64_t>((uint64_t)chunk, e.total - r0);
        ExpandArgs ea{};
        ea.L = L;
        ea.r = r;
        ea.Lnew = Lnew;
        ea.b = b;
        ea.cnew = new_compress;
        ea.rank0 = r0;
        ea.n = n;
        {
            uint64_t q = r0;  // digits of r0, position L-1 least significant
            for (int i = L - 1; i >= 0; --i) {
                ea.d0[i] = (int)(q % (uint64_t)e.cnt[i]);
                q /= (uint64_t)e.cnt[i];
            }
        }
        ea.inv = dinv.as<uint64_t>();
        ea.cnt = dcnt.as<int>();
        ea.off = doff.as<int>();
        ea.vals = dvals.as<int8_t>();
        ea.words = dwords.as<uint4>();
        int64_t blocks = (n + 255) / 256;
        if (blocks > (int64_t)c->num_sms * 16) blocks = (int64_t)c->num_sms * 16;
        expand_kernel<<<(unsigned)blocks, 256, 0, s>>>(ea);
        GP_CUDA_TRY(c, cudaGetLastError());
        GP_CUDA_TRY(c, cudaMemsetAsync(misc + 1, 0, 8, s));
        int rc = c->enqueue_filter(src, n, order, paf, GP_PSD_TC_GUARDED, dmask.as<uint32_t>(), dunsure.as<uint32_t>(),
                                   misc + 0, s);
        if (rc) return rc;
        GP_CUDA_TRY(c, gp::launch_mask_to_list(dmask.as<uint32_t>(), n, didx.as<uint32_t>(), misc + 1, n,
                                               c->status.as<int>(), c->num_sms, s));
        gp::FinalizeArgs fa;
        fa.src = src;
        fa.roles = nullptr;
        fa.fixed_role = 1;
        fa.idx = didx.as<uint32_t>();
        fa.n_idx = misc + 1;
        fa.idx_cap = n;
        fa.tw = tw;
        fa.thr = 2.0 * order - paf + 0.001;
        fa.bound = 2 * order - paf;
        fa.invert_roles = invert ? 1 : 0;
        fa.check_canonical = 0;
        fa.units = nullptr;
        fa.n_units = 0;
        fa.rec_words = side.words.as<uint4>();
        fa.rec_role = nullptr;
        fa.rec_sig = side.sig.as<uint16_t>();
        fa.rec_src = nullptr;
        fa.rec_count = misc + 2;  // accumulates over chunks
        fa.rec_cap = side.cap;
        fa.psd_pass = misc + 3;
        fa.status = c->status.as<int>();
        GP_CUDA_TRY(c, gp::launch_finalize(fa, n, c->num_sms, s));
    }
    GP_CUDA_TRY(c, cudaMemcpyAsync(side.nrec, misc + 2, 8, cudaMemcpyDeviceToHost, s));
    side.pending = true;
    return GP_OK;
}

// Waits for a side's expansion on stream s and takes its record count.
int finish_side(gp_ctx* c, Side& side, cudaStream_t s) {
    if (!side.pending) return GP_OK;
    side.pending = false;
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    int rc = c->check_status("uncompress");
    if (rc) return rc;
    side.n = (int64_t)std::min<unsigned long long>(*side.nrec, (unsigned long long)side.cap);
    return GP_OK;
}

void put_seq(std::string& t, const std::vector<int>& alpha, gp::u128 word, int b, int L) {
    for (int j = 0; j < L; ++j) {
        const int v = alpha[gp::word_digit_h(word, b, L, j)];
        if (v < 0) {
            t.push_back('-');
            put_uint(t, (unsigned)(-v));
        } else {
            put_uint(t, (unsigned)v);
        }
        t.push_back(' ');
    }
}

// Joins the two sides and appends the matched pairs, in the reference's
// order, to `out`.
int join_sides(gp_ctx* c, Side& A, Side& B, int Lnew, int new_compress, int paf, std::string& out) {
    const std::vector<int> nalpha = gp::alphabet(new_compress);
    const int b = gp::bits_for((int)nalpha.size());
    std::vector<std::pair<uint32_t, uint32_t>> m;
    int rc = gp::device_join(c, gp::JoinSide{A.words.as<uint4>(), A.sig.as<uint16_t>(), A.n},
                             gp::JoinSide{B.words.as<uint4>(), B.sig.as<uint16_t>(), B.n}, Lnew, b, new_compress,
                             paf * new_compress, m);
    if (rc || m.empty()) return rc;
    const int S = Lnew - 1;
    const int64_t nm = (int64_t)m.size();
    std::vector<uint32_t> ra(nm), rb(nm);
    for (int64_t i = 0; i < nm; ++i) {
        ra[i] = m[i].first;
        rb[i] = m[i].second;
    }
    cudaStream_t s = c->s_comp;
    DevBuf &dra = c->ux[8], &drb = c->ux[9], &wa = c->ux[10], &wb = c->ux[11], &sa = c->ux[12], &sb = c->ux[13];
    if (!dra.ensure(nm * 4) || !drb.ensure(nm * 4) || !wa.ensure(nm * 16) || !wb.ensure(nm * 16) ||
        !sa.ensure(nm * S * 2 + 16) || !sb.ensure(nm * S * 2 + 16))
        return c->fail(GP_ERR_NOMEM, "uncompress: gather");
    GP_CUDA_TRY(c, cudaMemcpyAsync(dra.p, ra.data(), nm * 4, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(drb.p, rb.data(), nm * 4, cudaMemcpyHostToDevice, s));
    const unsigned g = (unsigned)std::min<int64_t>((nm + 255) / 256, 4096);
    gather_records_kernel<<<g, 256, 0, s>>>(A.words.as<uint4>(), A.sig.as<uint16_t>(), S, dra.as<uint32_t>(), nm,
                                            wa.as<uint4>(), sa.as<uint16_t>());
    gather_records_kernel<<<g, 256, 0, s>>>(B.words.as<uint4>(), B.sig.as<uint16_t>(), S, drb.as<uint32_t>(), nm,
                                            wb.as<uint4>(), sb.as<uint16_t>());
    GP_CUDA_TRY(c, cudaGetLastError());
    std::vector<uint4> hwa(nm), hwb(nm);
    std::vector<uint16_t> hsa((size_t)nm * S), hsb((size_t)nm * S);
    GP_CUDA_TRY(c, cudaMemcpyAsync(hwa.data(), wa.p, nm * 16, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(hwb.data(), wb.p, nm * 16, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(hsa.data(), sa.p, hsa.size() * 2, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(hsb.data(), sb.p, hsb.size() * 2, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    auto word_of = [](const uint4& w) {
        return ((gp::u128)w.w << 96) | ((gp::u128)w.z << 64) | ((gp::u128)w.y << 32) | w.x;
    };
    struct Item {
        std::string a_line, b_line, pair_line;
    };
    std::vector<Item> items(nm);
    for (int64_t i = 0; i < nm; ++i) {
        Item& it = items[i];
        const gp::u128 x = word_of(hwa[i]), y = word_of(hwb[i]);
        std::string sa_txt, sb_txt;
        put_seq(sa_txt, nalpha, x, b, Lnew);
        put_seq(sb_txt, nalpha, y, b, Lnew);
        it.a_line = "PSD";
        for (int k = 0; k < S; ++k) put_uint(it.a_line, hsa[i * S + k]);
        it.a_line.push_back(' ');
        it.a_line += sa_txt;
        it.b_line = "PSD";
        for (int k = 0; k < S; ++k) put_uint(it.b_line, hsb[i * S + k]);
        it.b_line.push_back(' ');
        it.b_line += sb_txt;
        it.pair_line = sa_txt + " " + sb_txt + "\n";
    }
    std::sort(items.begin(), items.end(), [](const Item& p, const Item& q) {
        return p.a_line != q.a_line ? p.a_line < q.a_line : p.b_line < q.b_line;
    });
    for (auto& it : items) out += it.pair_line;
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
    return gp_uncompress_lines(c, order, compress, new_compress, paf, in_pairs, out_pairs, work_dir, prefix, 0,
                               INT64_MAX, 1);
}

int gp_uncompress_lines(gp_ctx* c, int order, int compress, int new_compress, int paf, const char* in_pairs,
                        const char* out_pairs, const char* work_dir, const char* prefix, int64_t first, int64_t end_line,
                        int64_t step) {
    StageRange nvtx_range("gp_uncompress");
    if (!c || !in_pairs || !out_pairs) return GP_ERR_ARG;
    if (first < 0 || step < 1) return c->fail(GP_ERR_ARG, "uncompress: bad line range (first %lld, step %lld)",
                                              (long long)first, (long long)step);
    (void)work_dir;
    (void)prefix;
    cudaSetDevice(c->device);
    if (!c->ensure_job_streams() || !c->h_ux.ensure(64))
        return c->fail(GP_ERR_CUDA, "uncompress: streams / pinned counts");
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
    // Pairs alternate between two sets of sides, scratch and streams: pair
    // i+1 expands on the device while pair i is joined and formatted.  The
    // join leaves no device work behind, so a set is free again once its
    // pair is written; output stays in input-pair order.
    struct PairSet {
        Side a, b;
        cudaStream_t sa, sb;
        bool busy = false;
    };
    PairSet set[2];
    for (int k = 0; k < 2; ++k) {
        set[k].sa = c->s_jobs[2 * k];
        set[k].sb = c->s_jobs[2 * k + 1];
        set[k].a.nrec = c->h_ux.as<unsigned long long>() + 2 * k;
        set[k].b.nrec = c->h_ux.as<unsigned long long>() + 2 * k + 1;
    }
    auto retire = [&](PairSet& ps) -> int {
        if (!ps.busy) return GP_OK;
        ps.busy = false;
        int r = finish_side(c, ps.a, ps.sa);
        if (r) return r;
        r = finish_side(c, ps.b, ps.sb);
        if (r) return r;
        std::string pairs;
        r = join_sides(c, ps.a, ps.b, order / new_compress, new_compress, paf, pairs);
        if (!r && !pairs.empty()) fwrite(pairs.data(), 1, pairs.size(), out);
        return r;
    };
    int cur = 0;
    while (p < end && rc == GP_OK) {
        const char* nl = (const char*)memchr(p, '\n', (size_t)(end - p));
        if (!nl) nl = end;
        // lines outside [first, end_line) or off the step are left out
        const int64_t this_line = line_no;
        if (this_line < first || this_line >= end_line || (this_line - first) % step != 0) {
            ++line_no;
            p = nl + 1;
            if (this_line >= end_line) break;
            continue;
        }
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
        // io.cpp:52-55: a line of the wrong length is an error (the pairs
        // before it are still written)
        if ((int)vals.size() != 2 * L) {
            rc = retire(set[cur ^ 1]);
            if (!rc)
                rc = c->fail(GP_ERR_FORMAT, "PairReader: input line %ld: length is %zu. Expected %d", line_no,
                             vals.size(), 2 * L);
            break;
        }
        ++line_no;
        std::vector<int> a(vals.begin(), vals.begin() + L), b(vals.begin() + L, vals.end());
        int64_t na = 0, nb = 0;
        PairSet& ps = set[cur];
        ps.busy = true;
        // the two sides expand on two streams, each with its own scratch
        rc = expand_side(c, a, order, compress, new_compress, paf, true, ps.a, &na, ps.sa, kSlotA[cur]);
        if (rc) break;
        rc = expand_side(c, b, order, compress, new_compress, paf, false, ps.b, &nb, ps.sb, kSlotB[cur]);
        if (rc) break;
        rc = retire(set[cur ^ 1]);  // the previous pair, while this one expands
        cur ^= 1;
    }
    if (rc == GP_OK) rc = retire(set[cur ^ 1]);
    for (auto& ps : set) {  // nothing of this call stays in flight, also after an error
        cudaStreamSynchronize(ps.sa);
        cudaStreamSynchronize(ps.sb);
    }
    fclose(out);
    return rc;
}

}  // extern "C"
