// capi_sortmatch.cu -- sort and match stages.
//
// gp_sort replaces GNU_sort (src/core/sort/sort.cpp:7-22), i.e.
// `sort -S 2G -T dir files | uniq > out` in the C locale: every line becomes
// a fixed-width key (4 bits per character for the candidate alphabet
// ' ' '-' '0'-'9' 'D' 'P' 'S', else 8 bits per byte; the pad code sorts
// below every character, so a prefix sorts first as in a byte compare), the
// keys are radix-sorted on the device (stable LSD, prims.cu) and adjacent
// duplicates are dropped.
//
// gp_match replaces match_pairs (src/core/match/match_pairs.cpp:15-121):
// the sorted files are grouped by their first token, equal tokens of A and
// B are joined, and every pair of the cross product is checked on the device
// by exact integer PAF (src/utils/golay.cpp:27-44) using per-line PAF
// vectors.  Pairs are written in the reference's order: token order, then A
// line order, then B line order.
#include <algorithm>
#include <stdexcept>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "prims.h"
#include "host_par.h"
#include "survivors.h"

namespace {

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

// 4-bit codes preserving byte order; 0 = padding
__host__ __device__ inline int code4(unsigned char ch) {
    switch (ch) {
        case ' ': return 1;
        case '-': return 2;
        case 'D': return 13;
        case 'P': return 14;
        case 'S': return 15;
        default: return (ch >= '0' && ch <= '9') ? 3 + (ch - '0') : -1;
    }
}

__global__ void build_keys_kernel(const char* text, const uint64_t* start, const uint32_t* len, int64_t n, int W,
                                  int nibble, uint32_t* keys) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const char* s = text + start[i];
        const uint32_t l = len[i];
        uint32_t* k = keys + i * W;
        const int per = nibble ? 8 : 4;
        const int bits = nibble ? 4 : 8;
        for (int w = 0; w < W; ++w) {
            uint32_t v = 0;
            for (int c = 0; c < per; ++c) {
                const uint32_t pos = (uint32_t)(w * per + c);
                uint32_t code = 0;
                if (pos < l) {
                    const unsigned char ch = (unsigned char)s[pos];
                    code = nibble ? (uint32_t)code4(ch) : (uint32_t)ch;
                }
                v = (v << bits) | code;
            }
            k[w] = v;
        }
    }
}

// PAF(s) = sum_i x_i x_{(i+s) mod L}, s = 1..L/2 (src/utils/golay.cpp:27-33)
__global__ void paf_kernel(const int8_t* seqs, int64_t n, int L, int H, int* paf) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int8_t* x = seqs + i * L;
        for (int s = 1; s <= H; ++s) {
            int r = 0;
            int j2 = s;
            for (int j = 0; j < L; ++j) {
                r += (int)x[j] * (int)x[j2];
                if (++j2 == L) j2 = 0;
            }
            paf[i * H + (s - 1)] = r;
        }
    }
}

struct GroupPair {
    uint32_t a0, na, b0, nb;
    uint64_t first;  // index of this group's first pair in the flattened product
};

// one thread per candidate pair; flags[w] = 1 if the pair is complementary
__global__ void pair_check_kernel(const GroupPair* gps, int64_t ng, uint64_t total, const int* pafa, const int* pafb,
                                  int H, int target, uint32_t* flags) {
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total;
         w += (uint64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = ng - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (gps[mid].first <= w)
                lo = mid;
            else
                hi = mid - 1;
        }
        const GroupPair g = gps[lo];
        const uint64_t off = w - g.first;
        const uint32_t ia = g.a0 + (uint32_t)(off / g.nb);
        const uint32_t ib = g.b0 + (uint32_t)(off % g.nb);
        const int* pa = pafa + (int64_t)ia * H;
        const int* pb = pafb + (int64_t)ib * H;
        uint32_t ok = 1;
        for (int s = 0; s < H; ++s)
            if (pa[s] + pb[s] != target) {
                ok = 0;
                break;
            }
        flags[w] = ok;
    }
}

unsigned grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    if (g > 65535 * 8) g = 65535 * 8;
    return (unsigned)(g < 1 ? 1 : g);
}

struct Cand {
    std::vector<uint32_t> tok_off, tok_len;  // first token in the text
    std::vector<int8_t> seqs;                // L per line
    size_t n = 0;
};

// Parses candidate lines: a first token, then exactly L integers.  Chunks
// of whole lines are parsed by host threads, then joined in order.
bool parse_candidates(const std::string& text, int L, Cand& out, std::string& err) {
    const char* base = text.data();
    const char* tend = base + text.size();
    const std::vector<size_t> cut = gp::line_chunks(base, text.size(), std::min<size_t>(4 * gp::host_threads(), text.size() / (1 << 18) + 1));
    const size_t nc = cut.size() - 1;
    std::vector<Cand> part(nc);
    std::vector<char> bad(nc, 0);
    gp::par_for(nc, [&](size_t k) {
        Cand& o = part[k];
        const char* p = base + cut[k];
        const char* end = base + cut[k + 1];
        while (p < end) {
            const char* nl = (const char*)memchr(p, '\n', (size_t)(end - p));
            if (!nl) nl = end;
            const char* q = p;
            while (q < nl && *q == ' ') ++q;
            if (q < nl) {
                const char* t = q;
                while (q < nl && *q != ' ') ++q;
                o.tok_off.push_back((uint32_t)(t - base));
                o.tok_len.push_back((uint32_t)(q - t));
                int got = 0;
                while (got < L) {
                    while (q < nl && *q == ' ') ++q;
                    if (q >= nl) break;
                    const char* e;
                    const long v = gp::read_long(q, tend, &e);
                    if (e == q) break;
                    o.seqs.push_back((int8_t)v);
                    ++got;
                    q = e;
                }
                if (got != L) {
                    bad[k] = 1;
                    return;
                }
                o.n++;
            }
            p = nl + 1;
        }
    });
    for (size_t k = 0; k < nc; ++k)
        if (bad[k]) {
            err = "candidate line with fewer than L values";
            return false;
        }
    size_t n = 0, ns = 0;
    for (const Cand& o : part) {
        n += o.n;
        ns += o.seqs.size();
    }
    out.tok_off.reserve(n);
    out.tok_len.reserve(n);
    out.seqs.reserve(ns);
    for (const Cand& o : part) {
        out.tok_off.insert(out.tok_off.end(), o.tok_off.begin(), o.tok_off.end());
        out.tok_len.insert(out.tok_len.end(), o.tok_len.begin(), o.tok_len.end());
        out.seqs.insert(out.seqs.end(), o.seqs.begin(), o.seqs.end());
        out.n += o.n;
    }
    return true;
}

// src/io.cpp PairWriter line: a entries, one more space, b entries
void put_pair(std::string& s, const int8_t* a, const int8_t* b, int L) {
    for (int i = 0; i < L; ++i) gp::put_int_sp(s, a[i]);
    s.push_back(' ');
    for (int i = 0; i < L; ++i) gp::put_int_sp(s, b[i]);
    s.push_back('\n');
}

}  // namespace

// Shared with the uncompression stage: match two sorted candidate texts and
// append the pairs to `out`.  Returns GP_EMPTY_INPUT if either is empty.
int gp_match_texts(gp_ctx* c, int L, int compress, int paf, const std::string& ta, const std::string& tb,
                   std::string& out, int64_t* n_pairs) {
    if (ta.empty() || tb.empty()) return GP_EMPTY_INPUT;
    Cand A, B;
    std::string err;
    if (!parse_candidates(ta, L, A, err) || !parse_candidates(tb, L, B, err)) return c->fail(GP_ERR_FORMAT, "match: %s", err.c_str());
    // group boundaries and the merge on the first token (std::string order)
    auto tok = [](const std::string& t, const Cand& x, size_t i) {
        return std::string_view(t.data() + x.tok_off[i], x.tok_len[i]);
    };
    std::vector<GroupPair> gps;
    uint64_t total = 0;
    size_t i = 0, j = 0;
    while (i < A.n && j < B.n) {
        const auto x = tok(ta, A, i), y = tok(tb, B, j);
        const int cmp = x.compare(y);
        if (cmp == 0) {
            size_t i2 = i, j2 = j;
            while (i2 < A.n && tok(ta, A, i2) == x) ++i2;
            while (j2 < B.n && tok(tb, B, j2) == y) ++j2;
            gps.push_back({(uint32_t)i, (uint32_t)(i2 - i), (uint32_t)j, (uint32_t)(j2 - j), total});
            total += (uint64_t)(i2 - i) * (j2 - j);
            i = i2;
            j = j2;
        } else if (cmp < 0) {
            ++i;
        } else {
            ++j;
        }
    }
    if (n_pairs) *n_pairs = 0;
    if (total == 0) return GP_OK;
    cudaStream_t s = c->s_comp;
    const int H = L / 2;
    DevBuf da, db, dpa, dpb, dg, df, dpos, dscan, dlist;
    const int64_t need_flags = (int64_t)total;
    if (!da.ensure(A.seqs.size() + 16) || !db.ensure(B.seqs.size() + 16) || !dpa.ensure(A.n * (H + 1) * 4) ||
        !dpb.ensure(B.n * (H + 1) * 4) || !dg.ensure(gps.size() * sizeof(GroupPair)) || !df.ensure(need_flags * 4) ||
        !dpos.ensure(need_flags * 4) || !dscan.ensure(gp::scan_tmp_bytes(need_flags)) || !dlist.ensure(need_flags * 4 + 4))
        return c->fail(GP_ERR_NOMEM, "match: device allocation");
    GP_CUDA_TRY(c, cudaMemcpyAsync(da.p, A.seqs.data(), A.seqs.size(), cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(db.p, B.seqs.data(), B.seqs.size(), cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dg.p, gps.data(), gps.size() * sizeof(GroupPair), cudaMemcpyHostToDevice, s));
    if (H > 0) {
        paf_kernel<<<grid_for((int64_t)A.n), 256, 0, s>>>(da.as<int8_t>(), (int64_t)A.n, L, H, dpa.as<int>());
        paf_kernel<<<grid_for((int64_t)B.n), 256, 0, s>>>(db.as<int8_t>(), (int64_t)B.n, L, H, dpb.as<int>());
    }
    pair_check_kernel<<<grid_for((int64_t)total), 256, 0, s>>>(dg.as<GroupPair>(), (int64_t)gps.size(), total,
                                                               dpa.as<int>(), dpb.as<int>(), H, paf * compress,
                                                               df.as<uint32_t>());
    GP_CUDA_TRY(c, cudaGetLastError());
    uint32_t* d_cnt = dlist.as<uint32_t>() + need_flags;
    GP_CUDA_TRY(c, gp::compact_flags(df.as<uint32_t>(), nullptr, dlist.as<uint32_t>(), need_flags, dpos.as<uint32_t>(),
                                     dscan.as<uint32_t>(), d_cnt, s));
    uint32_t nk = 0;
    GP_CUDA_TRY(c, cudaMemcpyAsync(&nk, d_cnt, 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    std::vector<uint32_t> keep(nk);
    if (nk) GP_CUDA_TRY(c, cudaMemcpy(keep.data(), dlist.p, (size_t)nk * 4, cudaMemcpyDeviceToHost));
    // pair lines in order, formatted in blocks by host threads
    const size_t per = 1 << 14;
    const size_t nblk = (keep.size() + per - 1) / per;
    std::vector<std::string> blk(nblk);
    gp::par_for(nblk, [&](size_t bi) {
        const size_t lo = bi * per, hi = std::min(keep.size(), lo + per);
        std::string& o = blk[bi];
        o.reserve((hi - lo) * (size_t)(6 * L + 2));
        size_t g = (size_t)(std::upper_bound(gps.begin(), gps.end(), (uint64_t)keep[lo],
                                             [](uint64_t w, const GroupPair& x) { return w < x.first; }) -
                            gps.begin()) - 1;
        for (size_t k = lo; k < hi; ++k) {
            const uint32_t w = keep[k];
            while (g + 1 < gps.size() && gps[g + 1].first <= w) ++g;
            const uint64_t off = w - gps[g].first;
            const uint32_t ia = gps[g].a0 + (uint32_t)(off / gps[g].nb);
            const uint32_t ib = gps[g].b0 + (uint32_t)(off % gps[g].nb);
            put_pair(o, A.seqs.data() + (size_t)ia * L, B.seqs.data() + (size_t)ib * L, L);
        }
    });
    for (const std::string& o : blk) out += o;
    if (n_pairs) *n_pairs = nk;
    return GP_OK;
}

// The sort's tuner: per key width, times whole sorts with 8- and 4-bit
// passes on (up to) the first 2^18 keys, twice each (the first round warms
// up), and keeps the faster; cached in the context.  Leaves di scrambled.
int sort_radix_bits(gp_ctx* c, const uint32_t* dk, int Wk, int64_t n, uint32_t* di, void* tmp, cudaStream_t s,
                    int* bits) {
    const std::string key = "sort:W" + std::to_string(Wk);
    auto it = c->tuned.find(key);
    if (it != c->tuned.end()) {
        *bits = (int)it->second[0];
        return GP_OK;
    }
    *bits = 8;
    if (n < (1 << 14)) return GP_OK;  // too small to time: default, not cached
    const int64_t m = std::min<int64_t>(n, 1 << 18);
    double best = 1e300;
    const int order[4] = {8, 4, 8, 4};
    for (int r = 0; r < 4; ++r) {
        GP_CUDA_TRY(c, gp::iota_u32(di, m, s));
        GP_CUDA_TRY(c, cudaStreamSynchronize(s));
        const auto t0 = std::chrono::steady_clock::now();
        GP_CUDA_TRY(c, gp::radix_sort_keys(dk, Wk, Wk, di, m, tmp, s, order[r]));
        GP_CUDA_TRY(c, cudaStreamSynchronize(s));
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (r >= 2 && el < best) {
            best = el;
            *bits = order[r];
        }
    }
    c->tuned[key] = {*bits, (int64_t)(best * 1e6)};
    return GP_OK;
}

// Sorted, de-duplicated lines of `text` (byte order).
int gp_sort_text(gp_ctx* c, const std::string& text, std::string& out) {
    std::vector<uint64_t> start;
    std::vector<uint32_t> len;
    size_t maxlen = 0;
    bool nibble = true;
    {
        // lines and the character check, by chunks of whole lines on host
        // threads, joined in order
        const char* base = text.data();
        const std::vector<size_t> cut = gp::line_chunks(base, text.size(), std::min<size_t>(4 * gp::host_threads(), text.size() / (1 << 18) + 1));
        const size_t nc = cut.size() - 1;
        std::vector<std::vector<uint64_t>> ps(nc);
        std::vector<std::vector<uint32_t>> pl(nc);
        std::vector<size_t> pmax(nc, 0);
        std::vector<char> pnib(nc, 1);
        gp::par_for(nc, [&](size_t k) {
            const char* p = base + cut[k];
            const char* end = base + cut[k + 1];
            for (const char* q = p; q < end; ++q)
                if (*q != '\n' && code4((unsigned char)*q) < 0) {
                    pnib[k] = 0;
                    break;
                }
            while (p < end) {
                const char* nl = (const char*)memchr(p, '\n', (size_t)(end - p));
                const size_t l = nl ? (size_t)(nl - p) : (size_t)(end - p);
                ps[k].push_back((uint64_t)(p - base));
                pl[k].push_back((uint32_t)l);
                pmax[k] = std::max(pmax[k], l);
                p += l + 1;
            }
        });
        size_t tot = 0;
        for (size_t k = 0; k < nc; ++k) tot += ps[k].size();
        start.reserve(tot);
        len.reserve(tot);
        for (size_t k = 0; k < nc; ++k) {
            start.insert(start.end(), ps[k].begin(), ps[k].end());
            len.insert(len.end(), pl[k].begin(), pl[k].end());
            maxlen = std::max(maxlen, pmax[k]);
            nibble = nibble && pnib[k];
        }
    }
    const int64_t n = (int64_t)start.size();
    out.clear();
    if (n == 0) return GP_OK;
    const int per = nibble ? 8 : 4;
    const int W = (int)((maxlen + per - 1) / per) + 0;
    const int Wk = W < 1 ? 1 : W;
    cudaStream_t s = c->s_comp;
    DevBuf dt, ds, dl, dk, di, dtmp, dflag, dpos, dscan, dout;
    if (!dt.ensure(text.size() + 16) || !ds.ensure(n * 8) || !dl.ensure(n * 4) || !dk.ensure((size_t)n * Wk * 4) ||
        !di.ensure(n * 4) || !dtmp.ensure(gp::radix_sort_tmp_bytes(n)) || !dflag.ensure(n * 4) || !dpos.ensure(n * 4) ||
        !dscan.ensure(gp::scan_tmp_bytes(n)) || !dout.ensure(n * 4 + 4))
        return c->fail(GP_ERR_NOMEM, "sort: device allocation");
    GP_CUDA_TRY(c, cudaMemcpyAsync(dt.p, text.data(), text.size(), cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(ds.p, start.data(), n * 8, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(dl.p, len.data(), n * 4, cudaMemcpyHostToDevice, s));
    build_keys_kernel<<<grid_for(n), 256, 0, s>>>(dt.as<char>(), ds.as<uint64_t>(), dl.as<uint32_t>(), n, Wk,
                                                  nibble ? 1 : 0, dk.as<uint32_t>());
    GP_CUDA_TRY(c, cudaGetLastError());
    int bits = 8;
    int rc = sort_radix_bits(c, dk.as<uint32_t>(), Wk, n, di.as<uint32_t>(), dtmp.p, s, &bits);
    if (rc) return rc;
    GP_CUDA_TRY(c, gp::iota_u32(di.as<uint32_t>(), n, s));
    GP_CUDA_TRY(c, gp::radix_sort_keys(dk.as<uint32_t>(), Wk, Wk, di.as<uint32_t>(), n, dtmp.p, s, bits));
    GP_CUDA_TRY(c, gp::mark_unique(dk.as<uint32_t>(), Wk, di.as<uint32_t>(), n, Wk, dflag.as<uint32_t>(), s));
    uint32_t* d_cnt = dout.as<uint32_t>() + n;
    GP_CUDA_TRY(c, gp::compact_flags(dflag.as<uint32_t>(), di.as<uint32_t>(), dout.as<uint32_t>(), n, dpos.as<uint32_t>(),
                                     dscan.as<uint32_t>(), d_cnt, s));
    uint32_t nu = 0;
    GP_CUDA_TRY(c, cudaMemcpyAsync(&nu, d_cnt, 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    std::vector<uint32_t> order(nu);
    if (nu) GP_CUDA_TRY(c, cudaMemcpy(order.data(), dout.p, (size_t)nu * 4, cudaMemcpyDeviceToHost));
    // output: each kept line and its newline at a prefix-sum offset, copied
    // by host threads
    std::vector<size_t> at(nu + 1, 0);
    for (uint32_t k = 0; k < nu; ++k) at[k + 1] = at[k] + len[order[k]] + 1;
    out.resize(at[nu]);
    const size_t lines_per = 1 << 15;
    gp::par_for((nu + lines_per - 1) / lines_per, [&](size_t bi) {
        const size_t lo = bi * lines_per, hi = std::min<size_t>(nu, lo + lines_per);
        for (size_t k = lo; k < hi; ++k) {
            const uint32_t i = order[k];
            std::memcpy(&out[at[k]], text.data() + start[i], len[i]);
            out[at[k] + len[i]] = '\n';
        }
    });
    return GP_OK;
}

// ------------------------------------------------ binary survivor inputs
// Every input a binary survivor file of one job: the records go to the
// device as they are, the device formats their lines (the text the
// generation call would have written, survivors.h), sorts them with the
// same keys as text input and gathers the kept lines in order; the host
// only reads the files and writes the sorted text.

struct SurvGeom {
    int L, bits, k, sig_bytes, word_bytes, rec_bytes;
    int alpha[16];
};

__device__ __forceinline__ int ndigits_u(unsigned v) {
    int n = 1;
    while (v >= 10) {
        v /= 10;
        ++n;
    }
    return n;
}

__device__ __forceinline__ void rec_word(const uint8_t* r, int word_bytes, uint64_t& lo, uint64_t& hi) {
    lo = hi = 0;
    for (int i = 0; i < word_bytes; ++i) {
        const uint64_t b = r[i];
        if (i < 8)
            lo |= b << (8 * i);
        else
            hi |= b << (8 * (i - 8));
    }
}

__device__ __forceinline__ int rec_digit(uint64_t lo, uint64_t hi, int bits, int L, int j) {
    const int pos = bits * (L - 1 - j);
    const uint64_t m = (1ull << bits) - 1ull;
    if (pos >= 64) return (int)((hi >> (pos - 64)) & m);
    uint64_t v = lo >> pos;
    if (pos + bits > 64 && pos > 0) v |= hi << (64 - pos);
    return (int)(v & m);
}

__device__ __forceinline__ unsigned rec_sig(const uint8_t* r, const SurvGeom& g, int k) {
    const uint8_t* s = r + g.word_bytes;
    return g.sig_bytes == 1 ? s[k] : (unsigned)(s[2 * k] | (s[2 * k + 1] << 8));
}

// line length (newline included) of every record; a digit past the
// alphabet or bits above the word make the input malformed
__global__ void surv_len_kernel(const uint8_t* recs, int64_t n, SurvGeom g, uint32_t* len, unsigned* maxlen,
                                int* bad) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t* r = recs + i * g.rec_bytes;
        uint64_t lo, hi;
        rec_word(r, g.word_bytes, lo, hi);
        const int used = g.bits * g.L;
        const bool high = used < 64 ? (lo >> used) != 0 || hi != 0 : (used < 128 && (hi >> (used - 64)) != 0);
        uint32_t l = 3 + 1 + 1;  // "PSD", the space after the signature, the newline
        for (int k = 0; k < g.L - 1; ++k) l += (uint32_t)ndigits_u(rec_sig(r, g, k));
        bool ok = !high;
        for (int j = 0; j < g.L; ++j) {
            const int d = rec_digit(lo, hi, g.bits, g.L, j);
            if (d >= g.k) {
                ok = false;
                break;
            }
            const int v = g.alpha[d];
            l += (uint32_t)(ndigits_u((unsigned)(v < 0 ? -v : v)) + (v < 0) + 1);
        }
        if (!ok) atomicExch(bad, 1);
        len[i] = l;
        atomicMax(maxlen, l - 1);
    }
}

__device__ __forceinline__ char* put_dec(char* o, unsigned v) {
    char tmp[10];
    int n = 0;
    do {
        tmp[n++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    while (n) *o++ = tmp[--n];
    return o;
}

// each record's line (src/utils/io.cpp:14-36) at its offset
__global__ void surv_format_kernel(const uint8_t* recs, int64_t n, SurvGeom g, const uint32_t* off, char* text,
                                   uint64_t* start, uint32_t* len) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t* r = recs + i * g.rec_bytes;
        uint64_t lo, hi;
        rec_word(r, g.word_bytes, lo, hi);
        char* o = text + off[i];
        char* const o0 = o;
        *o++ = 'P';
        *o++ = 'S';
        *o++ = 'D';
        for (int k = 0; k < g.L - 1; ++k) o = put_dec(o, rec_sig(r, g, k));
        *o++ = ' ';
        for (int j = 0; j < g.L; ++j) {
            const int v = g.alpha[rec_digit(lo, hi, g.bits, g.L, j)];
            if (v < 0) *o++ = '-';
            o = put_dec(o, (unsigned)(v < 0 ? -v : v));
            *o++ = ' ';
        }
        *o = '\n';
        start[i] = off[i];
        len[i] = (uint32_t)(o - o0);  // without the newline, as the text path's line lengths
    }
}

__global__ void gather_len_kernel(const uint32_t* len, const uint32_t* order, int64_t n, uint32_t* out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = len[order[i]] + 1;
}

// one warp per kept line: its bytes and newline at the line's output offset
__global__ void gather_lines_kernel(const char* text, const uint64_t* start, const uint32_t* len,
                                    const uint32_t* order, const uint32_t* out_off, int64_t n, char* out) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = w0; k < n; k += nw) {
        const uint32_t i = order[k];
        const char* src = text + start[i];
        char* dst = out + out_off[k];
        const uint32_t l = len[i] + 1;  // the newline follows the line in the formatted text
        for (uint32_t c = lane; c < l; c += 32) dst[c] = src[c];
    }
}

// Sorted, de-duplicated lines of the records (all of one geometry).
// Returns GP_ERR_FORMAT on a malformed record.
int gp_sort_records(gp_ctx* c, const SurvGeom& g, const std::vector<uint8_t>& recs, int64_t n, std::string& out) {
    out.clear();
    if (n == 0) return GP_OK;
    cudaStream_t s = c->s_comp;
    DevBuf dr, dl, dlen2, doff, dscan, dmisc, dt, ds, dk, di, dtmp, dflag, dpos, dord, dooff, dout;
    if (!dr.ensure(recs.size() + 16) || !dl.ensure(n * 4 + 4) || !doff.ensure(n * 4 + 4) ||
        !dscan.ensure(gp::scan_tmp_bytes(n)) || !dmisc.ensure(64) || !ds.ensure(n * 8))
        return c->fail(GP_ERR_NOMEM, "sort: device allocation");
    GP_CUDA_TRY(c, cudaMemcpyAsync(dr.p, recs.data(), recs.size(), cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemsetAsync(dmisc.p, 0, 64, s));
    unsigned* d_maxlen = dmisc.as<unsigned>();
    int* d_bad = dmisc.as<int>() + 1;
    surv_len_kernel<<<grid_for(n), 256, 0, s>>>(dr.as<uint8_t>(), n, g, dl.as<uint32_t>(), d_maxlen, d_bad);
    GP_CUDA_TRY(c, cudaGetLastError());
    GP_CUDA_TRY(c, gp::exclusive_scan_u32(dl.as<uint32_t>(), doff.as<uint32_t>(), n, dscan.as<uint32_t>(), s));
    uint32_t last_off = 0, last_len = 0;
    unsigned hm[2] = {0, 0};
    GP_CUDA_TRY(c, cudaMemcpyAsync(&last_off, doff.as<uint32_t>() + n - 1, 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(&last_len, dl.as<uint32_t>() + n - 1, 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(hm, dmisc.p, 8, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    if (hm[1]) return c->fail(GP_ERR_FORMAT, "sort: malformed survivor record");
    const uint64_t total = (uint64_t)last_off + last_len;
    if (total >= (uint64_t(1) << 32)) return c->fail(GP_ERR_UNSUPPORTED, "sort: %llu bytes of lines", (unsigned long long)total);
    const int Wk = std::max(1, (int)((hm[0] + 7) / 8));
    if (!dt.ensure(total + 16) || !dk.ensure((size_t)n * Wk * 4) || !di.ensure(n * 4) ||
        !dtmp.ensure(gp::radix_sort_tmp_bytes(n)) || !dflag.ensure(n * 4) || !dpos.ensure(n * 4) ||
        !dord.ensure(n * 4 + 4) || !dlen2.ensure(n * 4) || !dooff.ensure(n * 4))
        return c->fail(GP_ERR_NOMEM, "sort: device allocation");
    surv_format_kernel<<<grid_for(n), 256, 0, s>>>(dr.as<uint8_t>(), n, g, doff.as<uint32_t>(), dt.as<char>(),
                                                   ds.as<uint64_t>(), dl.as<uint32_t>());
    build_keys_kernel<<<grid_for(n), 256, 0, s>>>(dt.as<char>(), ds.as<uint64_t>(), dl.as<uint32_t>(), n, Wk, 1,
                                                  dk.as<uint32_t>());
    GP_CUDA_TRY(c, cudaGetLastError());
    int bits = 8;
    int rc = sort_radix_bits(c, dk.as<uint32_t>(), Wk, n, di.as<uint32_t>(), dtmp.p, s, &bits);
    if (rc) return rc;
    GP_CUDA_TRY(c, gp::iota_u32(di.as<uint32_t>(), n, s));
    GP_CUDA_TRY(c, gp::radix_sort_keys(dk.as<uint32_t>(), Wk, Wk, di.as<uint32_t>(), n, dtmp.p, s, bits));
    GP_CUDA_TRY(c, gp::mark_unique(dk.as<uint32_t>(), Wk, di.as<uint32_t>(), n, Wk, dflag.as<uint32_t>(), s));
    uint32_t* d_cnt = dord.as<uint32_t>() + n;
    GP_CUDA_TRY(c, gp::compact_flags(dflag.as<uint32_t>(), di.as<uint32_t>(), dord.as<uint32_t>(), n,
                                     dpos.as<uint32_t>(), dscan.as<uint32_t>(), d_cnt, s));
    uint32_t nu = 0;
    GP_CUDA_TRY(c, cudaMemcpyAsync(&nu, d_cnt, 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    if (nu == 0) return GP_OK;
    gather_len_kernel<<<grid_for(nu), 256, 0, s>>>(dl.as<uint32_t>(), dord.as<uint32_t>(), nu, dlen2.as<uint32_t>());
    GP_CUDA_TRY(c, cudaGetLastError());
    GP_CUDA_TRY(c, gp::exclusive_scan_u32(dlen2.as<uint32_t>(), dooff.as<uint32_t>(), nu, dscan.as<uint32_t>(), s));
    uint32_t o_last = 0, l_last = 0;
    GP_CUDA_TRY(c, cudaMemcpyAsync(&o_last, dooff.as<uint32_t>() + nu - 1, 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(&l_last, dlen2.as<uint32_t>() + nu - 1, 4, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    const uint64_t out_bytes = (uint64_t)o_last + l_last;
    if (!dout.ensure(out_bytes + 16)) return c->fail(GP_ERR_NOMEM, "sort: device allocation");
    gather_lines_kernel<<<(unsigned)std::min<int64_t>((nu + 7) / 8, 65535 * 8), 256, 0, s>>>(
        dt.as<char>(), ds.as<uint64_t>(), dl.as<uint32_t>(), dord.as<uint32_t>(), dooff.as<uint32_t>(), nu,
        dout.as<char>());
    GP_CUDA_TRY(c, cudaGetLastError());
    out.resize(out_bytes);
    GP_CUDA_TRY(c, cudaMemcpyAsync(&out[0], dout.p, out_bytes, cudaMemcpyDeviceToHost, s));
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    return GP_OK;
}

extern "C" {

int gp_tuned_settings(const gp_ctx* c, char* buf, int cap) {
    if (!c) return GP_ERR_ARG;
    std::string t;
    for (const auto& kv : c->tuned) {
        t += kv.first;
        for (int64_t v : kv.second) t += " " + std::to_string(v);
        t += "\n";
    }
    if (buf && cap > 0) {
        const size_t k = std::min(t.size(), (size_t)cap - 1);
        std::memcpy(buf, t.data(), k);
        buf[k] = 0;
    }
    return (int)t.size() + 1;
}

static int gp_sort_impl(gp_ctx* c, const char** in_paths, int n_in, const char* out_path) {
    StageRange nvtx_range("gp_sort");
    if (!c || (!in_paths && n_in > 0) || !out_path) return GP_ERR_ARG;
    cudaSetDevice(c->device);
    // every input is read once
    std::vector<std::string> texts(n_in);
    for (int i = 0; i < n_in; ++i)
        if (!slurp(in_paths[i], texts[i])) return c->fail(GP_ERR_IO, "sort: cannot read %s", in_paths[i]);
    {
        // all inputs binary survivor files of one job: the records are
        // formatted and sorted on the device
        std::vector<uint8_t> recs;
        SurvGeom g{};
        int64_t n = 0;
        bool binary = n_in > 0;
        gp::SurvHeader h0{};
        for (int i = 0; i < n_in && binary; ++i) {
            gp::SurvHeader h;
            const uint8_t* body = nullptr;
            const int kind = gp::surv_parse(texts[i], h, &body);
            if (kind < 0) return c->fail(GP_ERR_FORMAT, "sort: malformed survivor file %s", in_paths[i]);
            if (kind == 0 || (i > 0 && (h.L != h0.L || h.bits != h0.bits || h.k != h0.k || h.sig_bytes != h0.sig_bytes ||
                                        std::memcmp(h.alpha, h0.alpha, 16) != 0))) {
                binary = false;
                break;
            }
            if (i == 0) h0 = h;
            recs.insert(recs.end(), body, body + h.count * gp::surv_record_bytes(h));
            n += (int64_t)h.count;
        }
        if (binary) {
            g.L = h0.L;
            g.bits = h0.bits;
            g.k = h0.k;
            g.sig_bytes = h0.sig_bytes;
            g.word_bytes = h0.word_bytes;
            g.rec_bytes = (int)gp::surv_record_bytes(h0);
            for (int a = 0; a < 16; ++a) g.alpha[a] = h0.alpha[a];
            std::string sorted;
            int rc = gp_sort_records(c, g, recs, n, sorted);
            if (rc) return rc;
            FILE* f = fopen(out_path, "w");
            if (!f) return c->fail(GP_ERR_IO, "sort: cannot write %s", out_path);
            fwrite(sorted.data(), 1, sorted.size(), f);
            return fclose(f) == 0 ? GP_OK : c->fail(GP_ERR_IO, "sort: write failed");
        }
    }
    std::string all;
    for (int i = 0; i < n_in; ++i) {
        std::string& one = texts[i];
        gp::SurvHeader h;
        const uint8_t* body = nullptr;
        const int kind = gp::surv_parse(one, h, &body);
        if (kind < 0 || (kind > 0 && !gp::surv_to_text(h, body, all)))
            return c->fail(GP_ERR_FORMAT, "sort: malformed survivor file %s", in_paths[i]);
        if (kind > 0) continue;
        if (all.empty())
            all.swap(one);  // the first text input: no copy
        else
            all += one;
        if (!all.empty() && all.back() != '\n') all.push_back('\n');
        std::string().swap(one);
    }
    std::string sorted;
    int rc = gp_sort_text(c, all, sorted);
    if (rc) return rc;
    FILE* f = fopen(out_path, "w");
    if (!f) return c->fail(GP_ERR_IO, "sort: cannot write %s", out_path);
    fwrite(sorted.data(), 1, sorted.size(), f);
    return fclose(f) == 0 ? GP_OK : c->fail(GP_ERR_IO, "sort: write failed");
}

// No C++ exception (an allocation failure on a huge input) crosses the C ABI.
int gp_sort(gp_ctx* c, const char** in_paths, int n_in, const char* out_path) {
    try {
        return gp_sort_impl(c, in_paths, n_in, out_path);
    } catch (const std::exception& e) {
        return c ? c->fail(GP_ERR_NOMEM, "sort: %s", e.what()) : GP_ERR_NOMEM;
    }
}

static int gp_match_impl(gp_ctx* c, int order, int compress, int paf, const char* path_a, const char* path_b, const char* out_path,
             int append, int64_t* n_pairs) {
    StageRange nvtx_range("gp_match");
    if (!c || !path_a || !path_b || !out_path) return GP_ERR_ARG;
    if (compress < 1 || order % compress) return c->fail(GP_ERR_ARG, "order %d not divisible by %d", order, compress);
    cudaSetDevice(c->device);
    // the reference opens the pair writer (truncating unless appending)
    // before looking at the inputs (src/main.cpp:97-101)
    FILE* f = fopen(out_path, append ? "a" : "w");
    if (!f) return c->fail(GP_ERR_IO, "match: cannot open %s", out_path);
    std::string ta, tb, out;
    const bool okA = slurp(path_a, ta), okB = slurp(path_b, tb);
    if (n_pairs) *n_pairs = 0;
    if (!okA || !okB || ta.empty() || tb.empty()) {
        fclose(f);
        return GP_EMPTY_INPUT;
    }
    int rc = gp_match_texts(c, order / compress, compress, paf, ta, tb, out, n_pairs);
    fwrite(out.data(), 1, out.size(), f);
    fclose(f);
    return rc;
}

// No C++ exception (an allocation failure on a huge input) crosses the C ABI.
int gp_match(gp_ctx* c, int order, int compress, int paf, const char* path_a, const char* path_b, const char* out_path,
             int append, int64_t* n_pairs) {
    try {
        return gp_match_impl(c, order, compress, paf, path_a, path_b, out_path, append, n_pairs);
    } catch (const std::exception& e) {
        return c ? c->fail(GP_ERR_NOMEM, "match: %s", e.what()) : GP_ERR_NOMEM;
    }
}

}  // extern "C"
