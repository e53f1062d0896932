// capi_gen.cu -- candidate generation stage (replaces generate_hybrid,
// src/core/generate/generate_hybrid.cpp:107-163, and its job split,
// src/utils/lyndon.cpp:87-121).
//
// Device pipeline per batch:
//   enumerate_kernel   rank windows -> row-sum-gated necklaces (packed words)
//   psd_tc_kernel      guarded FP32 tensor-core PSD filter (+ FP64 recheck)
//   mask_to_list       surviving rows
//   finalize_kernel    exact FP64 PSD, canonical check, signature records
// The host then orders each role's records by word (the reference's FKM
// order) and writes the candidate files.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "enumerate.h"
#include "finalize.h"
#include "host_math.h"

namespace {

struct Record {
    gp::u128 word;
    std::vector<uint16_t> sig;
};

struct GenPlan {
    int order, compress, paf, L, k, b;
    std::vector<int> alpha;
    std::vector<std::pair<int, int>> dec;
};

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
        put_uint(s, (unsigned)(-(long long)v));
    } else {
        put_uint(s, (unsigned)v);
    }
}

// src/utils/io.cpp:14-36 line format
void format_line(std::string& out, const GenPlan& p, gp::u128 word, const uint16_t* sig) {
    out += "PSD";
    for (int k = 0; k < p.L - 1; ++k) put_uint(out, sig[k]);
    out.push_back(' ');
    for (int j = 0; j < p.L; ++j) {
        put_int(out, p.alpha[gp::word_digit_h(word, p.b, p.L, j)]);
        out.push_back(' ');
    }
    out.push_back('\n');
}

int write_records(gp_ctx* c, const GenPlan& p, std::vector<Record>& recs, const char* path) {
    std::sort(recs.begin(), recs.end(), [](const Record& x, const Record& y) { return x.word < y.word; });
    FILE* f = fopen(path, "w");
    if (!f) return c->fail(GP_ERR_IO, "cannot open %s for writing", path);
    std::string buf;
    buf.reserve(1 << 20);
    for (const Record& r : recs) {
        format_line(buf, p, r.word, r.sig.data());
        if (buf.size() > (1u << 20)) {
            fwrite(buf.data(), 1, buf.size(), f);
            buf.clear();
        }
    }
    fwrite(buf.data(), 1, buf.size(), f);
    const bool ok = fclose(f) == 0;
    return ok ? GP_OK : c->fail(GP_ERR_IO, "write failed: %s", path);
}

// Runs the device pipeline over rank ranges [lo, hi) of the word space.
int run_generation(gp_ctx* c, const GenPlan& p, const std::vector<std::pair<gp::u128, gp::u128>>& ranges,
                   std::vector<Record>& rec_a, std::vector<Record>& rec_b, gp_gen_stats* st) {
    const int L = p.L, b = p.b, k = p.k;
    cudaStream_t s = c->s_comp;
    // ---- windows
    gp::u128 total = 0;
    for (auto& r : ranges) total += r.second - r.first;
    const int64_t target = (int64_t)c->num_sms * 256 * 8;
    gp::u128 wsize = total / (gp::u128)target;
    if (wsize < 1) wsize = 1;
    const gp::u128 space = gp::upow(k, L);
    const gp::u128 maxw = gp::rank_to_word(space - 1, k, b, L);
    std::vector<uint4> cur, end;
    auto to_u4 = [](gp::u128 w) {
        return make_uint4((uint32_t)w, (uint32_t)(w >> 32), (uint32_t)(w >> 64), (uint32_t)(w >> 96));
    };
    for (auto& r : ranges) {
        for (gp::u128 lo = r.first; lo < r.second; lo += wsize) {
            gp::u128 hi = lo + wsize < r.second ? lo + wsize : r.second;
            cur.push_back(to_u4(gp::rank_to_word(lo, k, b, L)));
            end.push_back(to_u4(hi >= space ? maxw + 1 : gp::rank_to_word(hi, k, b, L)));
        }
    }
    const int64_t nwin = (int64_t)cur.size();
    // ---- roles by digit sum: rowsum = -c L + 2 * digitsum
    std::vector<uint8_t> roles(gp::kMaxDigitSum + 1, 0);
    for (int ds = 0; ds <= L * (k - 1) && ds <= gp::kMaxDigitSum; ++ds) {
        const int rs = -p.compress * L + 2 * ds;
        for (auto& d : p.dec) {
            if (rs == d.first) roles[ds] |= 1;
            if (rs == d.second) roles[ds] |= 2;
        }
    }
    // ---- device buffers
    const int64_t cap = std::min<int64_t>(int64_t(1) << 25, std::max<int64_t>(1 << 16, (int64_t)std::min<gp::u128>(total, (gp::u128)1 << 40)));
    const int64_t slack = (int64_t)c->num_sms * 8 * 256 / 32 * 256 + 4096;
    const int64_t hard = cap + slack;
    DevBuf& d_cur = c->scratch[5];
    DevBuf& d_end = c->scratch[6];
    DevBuf& d_words = c->scratch[7];
    DevBuf& d_roles = c->scratch[8];
    DevBuf& d_mask = c->scratch[9];
    DevBuf& d_unsure = c->scratch[10];
    DevBuf& d_idx = c->scratch[11];
    DevBuf& d_rtab = c->scratch[12];
    DevBuf& d_misc = c->scratch[13];  // counters
    DevBuf& d_rec = c->scratch[14];
    DevBuf& d_units = c->scratch[15];
    if (!d_cur.ensure(nwin * 16) || !d_end.ensure(nwin * 16) || !d_words.ensure(hard * 16) || !d_roles.ensure(hard) ||
        !d_mask.ensure((hard + 31) / 32 * 4) || !d_unsure.ensure(hard * 4) || !d_idx.ensure(hard * 4) ||
        !d_rtab.ensure(roles.size()) || !d_misc.ensure(64 * 8) || !d_units.ensure(2 * (L + 1)))
        return c->fail(GP_ERR_NOMEM, "generate: device allocation failed");
    GP_CUDA_TRY(c, cudaMemcpyAsync(d_cur.p, cur.data(), nwin * 16, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(d_end.p, end.data(), nwin * 16, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(d_rtab.p, roles.data(), roles.size(), cudaMemcpyHostToDevice, s));
    std::vector<int16_t> units;
    for (int u = 1; u < L; ++u)
        if (std::gcd(u, L) == 1) units.push_back((int16_t)u);
    if (units.empty()) units.push_back(1);
    GP_CUDA_TRY(c, cudaMemcpyAsync(d_units.p, units.data(), units.size() * 2, cudaMemcpyHostToDevice, s));
    unsigned long long* misc = d_misc.as<unsigned long long>();
    // misc: [0] candidates, [1] necklaces, [2] incomplete(int), [3] unsure count,
    //       [4] survivors, [5] records, [6] psd passes
    gp::EnumArgs ea;
    ea.L = L;
    ea.b = b;
    gp::u128 mp = 0;
    for (int j = 0; j < L; ++j) mp |= (gp::u128)(k - 1) << (b * j);
    ea.maxpat.lo = (uint64_t)mp;
    ea.maxpat.hi = (uint64_t)(mp >> 64);
    for (int t = 0; t < 4; ++t) {
        gp::u128 pl = 0;
        if (t < b)
            for (int j = 0; j < L; ++j) pl |= (gp::u128)1 << (b * j + t);
        ea.plane[t].lo = (uint64_t)pl;
        ea.plane[t].hi = (uint64_t)(pl >> 64);
    }
    ea.roles = d_rtab.as<uint8_t>();
    ea.cur = d_cur.as<uint4>();
    ea.end = d_end.as<uint4>();
    ea.nwin = nwin;
    ea.words = d_words.as<uint4>();
    ea.out_roles = d_roles.as<uint8_t>();
    ea.count = misc + 0;
    ea.cap = hard;
    ea.soft_cap = cap;
    ea.necklaces = misc + 1;
    ea.incomplete = reinterpret_cast<int*>(misc + 2);
    ea.status = c->status.as<int>();

    gp::RowSrc src{nullptr, d_words.as<uint4>(), L, b, p.compress};
    GP_CUDA_TRY(c, cudaMemsetAsync(misc, 0, 64 * 8, s));
    for (int iter = 0;; ++iter) {
        GP_CUDA_TRY(c, cudaMemsetAsync(misc + 0, 0, 8, s));
        GP_CUDA_TRY(c, cudaMemsetAsync(misc + 2, 0, 8, s));
        GP_CUDA_TRY(c, cudaMemsetAsync(misc + 4, 0, 8, s));
        GP_CUDA_TRY(c, cudaMemsetAsync(misc + 5, 0, 8, s));
        GP_CUDA_TRY(c, gp::launch_enumerate(ea, c->num_sms, s));
        unsigned long long h[8];
        GP_CUDA_TRY(c, cudaMemcpyAsync(h, misc, sizeof h, cudaMemcpyDeviceToHost, s));
        GP_CUDA_TRY(c, cudaStreamSynchronize(s));
        int rc = c->check_status("enumerate");
        if (rc) return rc;
        const int64_t n = (int64_t)h[0];
        const bool incomplete = h[2] != 0;
        if (n > 0) {
            st->candidates += n;
            rc = c->enqueue_filter(src, n, p.order, p.paf, GP_PSD_TC_GUARDED, d_mask.as<uint32_t>(),
                                   d_unsure.as<uint32_t>(), misc + 3, s);
            if (rc) return rc;
            GP_CUDA_TRY(c, gp::launch_mask_to_list(d_mask.as<uint32_t>(), n, d_idx.as<uint32_t>(), misc + 4, hard,
                                                   c->status.as<int>(), c->num_sms, s));
            unsigned long long hs[2];
            GP_CUDA_TRY(c, cudaMemcpyAsync(hs, misc + 3, 16, cudaMemcpyDeviceToHost, s));
            GP_CUDA_TRY(c, cudaStreamSynchronize(s));
            rc = c->check_status("psd filter");
            if (rc) return rc;
            st->unsure += (int64_t)hs[0];
            const int64_t surv = (int64_t)hs[1];
            if (surv > 0) {
                const int64_t rcap = 2 * surv;
                const size_t rec_bytes = (size_t)rcap * (16 + 1 + 2 * (L - 1)) + 64;
                if (!d_rec.ensure(rec_bytes)) return c->fail(GP_ERR_NOMEM, "generate: record buffer");
                uint8_t* rb = d_rec.as<uint8_t>();
                gp::FinalizeArgs fa;
                fa.src = src;
                fa.roles = d_roles.as<uint8_t>();
                fa.fixed_role = 0;
                fa.idx = d_idx.as<uint32_t>();
                fa.n_idx = misc + 4;
                fa.idx_cap = hard;
                fa.tw = c->twiddle64(L);
                fa.thr = 2.0 * p.order - p.paf + 0.001;
                fa.bound = 2 * p.order - p.paf;
                fa.invert_roles = 2;  // B lines carry bound - rint(psd) (io.cpp:26-36)
                fa.check_canonical = 1;
                fa.units = d_units.as<int16_t>();
                fa.n_units = (int)units.size();
                fa.rec_words = reinterpret_cast<uint4*>(rb);
                fa.rec_role = rb + (size_t)rcap * 16;
                fa.rec_sig = reinterpret_cast<uint16_t*>(rb + (size_t)rcap * 17 + ((rcap * 17) & 1));
                fa.rec_src = nullptr;
                fa.rec_count = misc + 5;
                fa.rec_cap = rcap;
                fa.psd_pass = misc + 6;
                fa.status = c->status.as<int>();
                GP_CUDA_TRY(c, gp::launch_finalize(fa, surv, c->num_sms, s));
                unsigned long long nrec = 0;
                GP_CUDA_TRY(c, cudaMemcpyAsync(&nrec, misc + 5, 8, cudaMemcpyDeviceToHost, s));
                GP_CUDA_TRY(c, cudaStreamSynchronize(s));
                rc = c->check_status("finalize");
                if (rc) return rc;
                if (nrec) {
                    std::vector<uint4> w(nrec);
                    std::vector<uint8_t> ro(nrec);
                    std::vector<uint16_t> sg(nrec * (L - 1));
                    GP_CUDA_TRY(c, cudaMemcpy(w.data(), fa.rec_words, nrec * 16, cudaMemcpyDeviceToHost));
                    GP_CUDA_TRY(c, cudaMemcpy(ro.data(), fa.rec_role, nrec, cudaMemcpyDeviceToHost));
                    GP_CUDA_TRY(c, cudaMemcpy(sg.data(), fa.rec_sig, sg.size() * 2, cudaMemcpyDeviceToHost));
                    for (size_t i = 0; i < nrec; ++i) {
                        Record r;
                        r.word = ((gp::u128)w[i].w << 96) | ((gp::u128)w[i].z << 64) | ((gp::u128)w[i].y << 32) | w[i].x;
                        r.sig.assign(sg.begin() + i * (L - 1), sg.begin() + (i + 1) * (L - 1));
                        (ro[i] == 1 ? rec_a : rec_b).push_back(std::move(r));
                    }
                }
            }
        }
        if (!incomplete) break;
    }
    unsigned long long h2[8];
    GP_CUDA_TRY(c, cudaMemcpy(h2, misc, sizeof h2, cudaMemcpyDeviceToHost));
    st->necklaces += (int64_t)h2[1];
    st->psd_pass += (int64_t)h2[6];
    return GP_OK;
}

int plan_for(gp_ctx* c, int order, int compress, int paf, GenPlan& p) {
    if (compress < 1 || order < 1 || order % compress != 0)
        return c->fail(GP_ERR_ARG, "order %d is not divisible by compression %d", order, compress);
    p.order = order;
    p.compress = compress;
    p.paf = paf;
    p.L = order / compress;
    p.alpha = gp::alphabet(compress);
    p.k = (int)p.alpha.size();
    p.b = gp::bits_for(p.k);
    p.dec = gp::decomps(gp::sum_constant(order, paf));
    if (p.b * p.L > 126 || p.L * (p.k - 1) > gp::kMaxDigitSum)
        return c->fail(GP_ERR_UNSUPPORTED, "generation: length %d over %d letters exceeds a 126-bit word", p.L, p.k);
    if (!gp::tc_packed_supported(p.L, p.b))
        return c->fail(GP_ERR_UNSUPPORTED, "generation: length %d not supported by the tensor-core filter", p.L);
    return GP_OK;
}

int finish(gp_ctx* c, const GenPlan& p, std::vector<Record>& ra, std::vector<Record>& rb, const char* path_a,
           const char* path_b, gp_gen_stats* st) {
    int rc = write_records(c, p, ra, path_a);
    if (rc) return rc;
    rc = write_records(c, p, rb, path_b);
    if (rc) return rc;
    st->written_a = (int64_t)ra.size();
    st->written_b = (int64_t)rb.size();
    return GP_OK;
}

}  // namespace

extern "C" {

int gp_generate(gp_ctx* c, int order, int compress, int paf, int proc_id, int proc_num, const char* path_a,
                const char* path_b, gp_gen_stats* stats) {
    if (!c || !path_a || !path_b) return GP_ERR_ARG;
    if (proc_num < 1 || proc_id < 0 || proc_id >= proc_num)
        return c->fail(GP_ERR_ARG, "bad job split %d of %d", proc_id, proc_num);
    const auto t0 = std::chrono::steady_clock::now();
    cudaSetDevice(c->device);
    GenPlan p;
    int rc = plan_for(c, order, compress, paf, p);
    if (rc) return rc;
    gp_gen_stats st;
    std::memset(&st, 0, sizeof st);
    if (p.dec.empty()) {
        c->fail(GP_NO_DECOMPOSITION, "Order %d cannot be decomposed into a sum of squares", order);
        // the reference opens (truncates) both files before giving up
        FILE* fa = fopen(path_a, "w");
        FILE* fb = fopen(path_b, "w");
        if (fa) fclose(fa);
        if (fb) fclose(fb);
        return GP_NO_DECOMPOSITION;
    }
    const int L = p.L, k = p.k;
    // job split of src/utils/lyndon.cpp:93-106: prenecklace prefixes of the
    // first length i with at least proc_num * 10000 necklaces, dealt out
    // round robin (1-based count), each covering the words that extend it
    std::vector<std::pair<gp::u128, gp::u128>> ranges;
    int i = 1;
    for (; i <= L; ++i)
        if (gp::necklace_count(i, k) >= (gp::u128)proc_num * 10000) break;
    if (proc_num > 1 && i < L) {
        const gp::u128 span = gp::upow(k, L - i);
        int64_t count = 0;
        gp::prenecklaces(i, k, [&](const std::vector<int>& pre, int) {
            ++count;
            if (count % proc_num != proc_id) return;
            gp::u128 r = 0;
            for (int d : pre) r = r * (gp::u128)k + (gp::u128)d;
            ranges.emplace_back(r * span, (r + 1) * span);
        });
    } else {
        ranges.emplace_back(0, gp::upow(k, L));
    }
    std::vector<Record> ra, rb;
    rc = run_generation(c, p, ranges, ra, rb, &st);
    if (rc) return rc;
    rc = finish(c, p, ra, rb, path_a, path_b, &st);
    if (rc) return rc;
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = st;
    return GP_OK;
}

int gp_generate_window(gp_ctx* c, int order, int compress, int paf, uint64_t begin_hi, uint64_t begin_lo,
                       uint64_t end_hi, uint64_t end_lo, const char* path_a, const char* path_b,
                       gp_gen_stats* stats) {
    if (!c || !path_a || !path_b) return GP_ERR_ARG;
    const auto t0 = std::chrono::steady_clock::now();
    cudaSetDevice(c->device);
    GenPlan p;
    int rc = plan_for(c, order, compress, paf, p);
    if (rc) return rc;
    gp_gen_stats st;
    std::memset(&st, 0, sizeof st);
    if (p.dec.empty()) return c->fail(GP_NO_DECOMPOSITION, "Order %d cannot be decomposed", order);
    gp::u128 lo = ((gp::u128)begin_hi << 64) | begin_lo;
    gp::u128 hi = ((gp::u128)end_hi << 64) | end_lo;
    const gp::u128 space = gp::upow(p.k, p.L);
    if (hi > space) hi = space;
    std::vector<std::pair<gp::u128, gp::u128>> ranges;
    if (lo < hi) ranges.emplace_back(lo, hi);
    std::vector<Record> ra, rb;
    rc = run_generation(c, p, ranges, ra, rb, &st);
    if (rc) return rc;
    rc = finish(c, p, ra, rb, path_a, path_b, &st);
    if (rc) return rc;
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = st;
    return GP_OK;
}

}  // extern "C"
