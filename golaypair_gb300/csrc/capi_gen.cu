// capi_gen.cu -- candidate generation stage (replaces generate_hybrid,
// src/core/generate/generate_hybrid.cpp:107-163, and its job split,
// src/utils/lyndon.cpp:87-121).
//
// Device pipeline per iteration (the batch engine below):
//   enumerate_kernel   rank windows -> row-sum-gated necklaces (packed words)
//   psd_tc_kernel      guarded FP32 tensor-core PSD filter (+ FP64 recheck)
//   mask_to_list       surviving rows
//   finalize_kernel    exact FP64 PSD, canonical check, signature records
// The host then orders each role's records by word (the reference's FKM
// order) and writes the candidate files.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "ctx.h"
#include "enumerate.h"
#include "finalize.h"
#include "host_math.h"
#include "survivors.h"

namespace {

// Survivor records of one role: packed words and their (L-1) signature
// values, in flat arrays.
struct RecordSet {
    std::vector<gp::u128> words;
    std::vector<uint16_t> sigs;
    size_t size() const { return words.size(); }
};

struct GenPlan {
    int order, compress, paf, L, k, b;
    std::vector<int> alpha;
    std::vector<std::pair<int, int>> dec;
};

// src/utils/io.cpp:14-36 line format
void format_line(std::string& out, const GenPlan& p, gp::u128 word, const uint16_t* sig) {
    gp::format_survivor_line(out, p.L, p.b, p.alpha.data(), word, sig);
}

// Writes the records in word order (the reference's FKM order).  Lines
// are formatted by several host threads into per-thread buffers, then
// written in order.
int write_records_binary(gp_ctx* c, const GenPlan& p, const RecordSet& recs, const std::vector<uint32_t>& order,
                         int role, const char* path);

// Sorts v with cmp: host threads sort equal chunks, then merge them pairwise
// in rounds (every merge of a round on its own thread).
template <class T, class Cmp>
void parallel_sort(std::vector<T>& v, Cmp cmp) {
    const size_t n = v.size();
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < (size_t(1) << 16) || hw == 1) {
        std::sort(v.begin(), v.end(), cmp);
        return;
    }
    std::vector<size_t> bounds;
    for (unsigned t = 0; t <= hw; ++t) bounds.push_back(n * t / hw);
    {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < hw; ++t)
            th.emplace_back([&, t] { std::sort(v.begin() + bounds[t], v.begin() + bounds[t + 1], cmp); });
        for (auto& x : th) x.join();
    }
    std::vector<T> tmp(n);
    while (bounds.size() > 2) {
        std::vector<size_t> nb;
        std::vector<std::thread> th;
        for (size_t i = 0; i + 1 < bounds.size(); i += 2) {
            const size_t lo = bounds[i], mid = bounds[i + 1], hi = i + 2 < bounds.size() ? bounds[i + 2] : mid;
            nb.push_back(lo);
            th.emplace_back([&, lo, mid, hi] {
                std::merge(v.begin() + lo, v.begin() + mid, v.begin() + mid, v.begin() + hi, tmp.begin() + lo, cmp);
            });
        }
        nb.push_back(n);
        for (auto& x : th) x.join();
        v.swap(tmp);
        bounds.swap(nb);
    }
}

int write_records(gp_ctx* c, const GenPlan& p, const RecordSet& recs, int role, const char* path) {
    const size_t n = recs.size();
    const int S = p.L - 1;
    std::vector<uint32_t> order(n);
    for (size_t i = 0; i < n; ++i) order[i] = (uint32_t)i;
    parallel_sort(order, [&](uint32_t x, uint32_t y) { return recs.words[x] < recs.words[y]; });
    if (c->out_format == GP_FORMAT_BINARY) return write_records_binary(c, p, recs, order, role, path);
    FILE* f = fopen(path, "w");
    if (!f) return c->fail(GP_ERR_IO, "cannot open %s for writing", path);
    const size_t per_block = 1 << 13;  // lines per formatting task
    const size_t nblocks = (n + per_block - 1) / per_block;
    unsigned nthreads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (nblocks < nthreads) nthreads = (unsigned)std::max<size_t>(1, nblocks);
    bool ok = true;
    // rounds of nthreads blocks: format in parallel, write in order; the
    // next round is formatted while this one is written
    std::vector<std::string> bufs[2] = {std::vector<std::string>(nthreads), std::vector<std::string>(nthreads)};
    auto format_round = [&](size_t b0, std::vector<std::string>& bs) {
        std::vector<std::thread> th;
        const unsigned m = (unsigned)std::min<size_t>(nthreads, nblocks - b0);
        for (unsigned t = 0; t < m; ++t) {
            th.emplace_back([&, t, b0] {
                std::string& out = bs[t];
                out.clear();
                const size_t lo = (b0 + t) * per_block, hi = std::min(n, lo + per_block);
                out.reserve((hi - lo) * (size_t)(4 * p.L + 8));
                for (size_t i = lo; i < hi; ++i) {
                    const uint32_t r = order[i];
                    format_line(out, p, recs.words[r], recs.sigs.data() + (size_t)r * S);
                }
            });
        }
        return th;
    };
    if (nblocks) {
        std::vector<std::thread> th = format_round(0, bufs[0]);
        for (size_t b0 = 0, r = 0; b0 < nblocks; b0 += nthreads, r ^= 1) {
            for (auto& x : th) x.join();
            const unsigned m = (unsigned)std::min<size_t>(nthreads, nblocks - b0);
            th = b0 + nthreads < nblocks ? format_round(b0 + nthreads, bufs[r ^ 1]) : std::vector<std::thread>();
            for (unsigned t = 0; t < m && ok; ++t)
                if (fwrite(bufs[r][t].data(), 1, bufs[r][t].size(), f) != bufs[r][t].size()) ok = false;
        }
        for (auto& x : th) x.join();
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? GP_OK : c->fail(GP_ERR_IO, "write failed: %s", path);
}

// The same records as a binary survivor file (survivors.h), in the same
// order.
int write_records_binary(gp_ctx* c, const GenPlan& p, const RecordSet& recs, const std::vector<uint32_t>& order,
                         int role, const char* path) {
    const size_t n = recs.size();
    const int S = p.L - 1;
    gp::SurvHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, gp::kSurvMagic, 8);
    h.version = 1;
    h.order = p.order;
    h.compress = p.compress;
    h.paf = p.paf;
    h.L = p.L;
    h.k = p.k;
    h.bits = p.b;
    h.role = role;
    uint16_t mx = 0;
    for (uint16_t v : recs.sigs) mx = std::max(mx, v);
    h.sig_bytes = mx <= 255 ? 1 : 2;
    h.word_bytes = (p.b * p.L + 7) / 8;
    h.count = n;
    for (int i = 0; i < p.k && i < 16; ++i) h.alpha[i] = (int8_t)p.alpha[i];
    const size_t rb = gp::surv_record_bytes(h);
    std::vector<uint8_t> body(n * rb);
    for (size_t i = 0; i < n; ++i) {
        const uint32_t r = order[i];
        gp::surv_put_record(body.data() + i * rb, h, recs.words[r], recs.sigs.data() + (size_t)r * S);
    }
    FILE* f = fopen(path, "wb");
    if (!f) return c->fail(GP_ERR_IO, "cannot open %s for writing", path);
    bool ok = fwrite(&h, sizeof h, 1, f) == 1;
    if (n) ok = ok && fwrite(body.data(), 1, body.size(), f) == body.size();
    ok = (fclose(f) == 0) && ok;
    return ok ? GP_OK : c->fail(GP_ERR_IO, "write failed: %s", path);
}

// ------------------------------------------------------------ batch engine
//
// One engine serves gp_generate (one job) and gp_generate_batch (up to
// kMaxEnumJobs jobs of different orders / compressions).  Per iteration:
//
//   memset   per-iteration counters
//   enumerate_kernel          all jobs' rank windows, one launch
//   per job, on its own stream branch:
//     psd_tc_kernel           row count read on the device
//     psd_recheck_kernel      FP64 recheck of the unsure rows
//     mask_to_list_kernel     surviving rows
//     finalize_kernel         FP64 PSD, canonical check, records (accumulate)
//   copy     counters -> pinned host
//
// Nothing in that sequence depends on a host-side count, so it is captured
// once as a CUDA graph and replayed until every window is finished.  The
// host reads the counters after each replay, drains a job's records when
// its record buffer could not take another iteration, and stops when no
// window is left unfinished.

constexpr int kIterSlots = 4;   // per job: [0] candidates, [1] unsure, [2] survivors
constexpr int kCumSlots = 4;    // per job: [0] necklaces, [1] records, [2] psd passes
constexpr int kIncomplete = kIterSlots * gp::kMaxEnumJobs;          // u64 slot of the flag
constexpr int kNextWin = kIncomplete + 1;                          // window handout counter
constexpr int kNextWinWide = kIncomplete + 2;                      // the same for the wide jobs' launch
constexpr int kIterWords = kIncomplete + 3;
constexpr int kCumBase = 40;                                        // u64 offset of the cumulative block
constexpr int kCounterWords = kCumBase + kCumSlots * gp::kMaxEnumJobs;

struct BatchCfg {
    int enum_variant = 0;        // enumerator kernel variant (see launch_enumerate)
    int windows_per_thread = 1;  // rank windows per enumerator thread
    int64_t cand_cap = int64_t(1) << 22;  // candidates per job per iteration (soft)
    int tc_ctas_per_sm = 0;      // tensor-core filter CTAs per SM (0 = as many as fit)
    int use_graph = 1;
    // 1: one launch per kernel and iteration over every job (filter,
    // recheck, listing, finalize); 0: per-job launches on the jobs' own
    // streams
    int multi_launch = 0;
};


struct JobRun {
    GenPlan p;
    std::vector<std::pair<gp::u128, gp::u128>> ranges;
    int64_t soft = 0, hard = 0, rcap = 0, rec_bytes = 0;
    size_t off_words = 0, off_roles = 0, off_mask = 0, off_unsure = 0, off_idx = 0, off_rec = 0, off_units = 0;
    std::vector<int16_t> units;
    RecordSet ra, rb;
    gp_gen_stats st{};
    // set when the engine stopped early: the word ranks still to search
    std::vector<std::pair<gp::u128, gp::u128>> remaining;
};

// True when one filter launch takes every job (lengths up to 63).
bool multi_launch_ok(const std::vector<JobRun>& jobs) {
    for (auto& j : jobs)
        if (!gp::tc_multi_supported(j.p.L, j.p.b)) return false;
    return (int)jobs.size() <= gp::kMaxTcJobs;
}

// Early stop of the engine (checkpointed searches): after an iteration that
// reaches max_iterations (> 0) or max_seconds (> 0) with windows left, the
// engine drains its records, stores each job's unfinished rank ranges in
// JobRun::remaining and returns with stopped = true.
struct StopCtl {
    int max_iterations = 0;
    double max_seconds = 0;
    std::chrono::steady_clock::time_point start = std::chrono::steady_clock::now();
    bool stopped = false;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

gp::u128 range_words(const JobRun& j) {
    gp::u128 t = 0;
    for (auto& r : j.ranges) t += r.second - r.first;
    return t;
}

uint4 to_u4(gp::u128 w) {
    return make_uint4((uint32_t)w, (uint32_t)(w >> 32), (uint32_t)(w >> 64), (uint32_t)(w >> 96));
}

// Copies job j's records to the host and appends them to its A/B lists.
int drain_records(gp_ctx* c, JobRun& j, uint8_t* arena, int64_t nrec) {
    if (nrec <= 0) return GP_OK;
    const int L = j.p.L;
    uint8_t* rb = arena + j.off_rec;
    const int64_t rcap = j.rcap;
    std::vector<uint4> w(nrec);
    std::vector<uint8_t> ro(nrec);
    std::vector<uint16_t> sg((size_t)nrec * (L - 1));
    GP_CUDA_TRY(c, cudaMemcpy(w.data(), rb, nrec * 16, cudaMemcpyDeviceToHost));
    GP_CUDA_TRY(c, cudaMemcpy(ro.data(), rb + (size_t)rcap * 16, nrec, cudaMemcpyDeviceToHost));
    GP_CUDA_TRY(c, cudaMemcpy(sg.data(), rb + align_up((size_t)rcap * 17, 16), sg.size() * 2, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < nrec; ++i) {
        RecordSet& rs = ro[i] == 1 ? j.ra : j.rb;
        rs.words.push_back(((gp::u128)w[i].w << 96) | ((gp::u128)w[i].z << 64) | ((gp::u128)w[i].y << 32) | w[i].x);
        rs.sigs.insert(rs.sigs.end(), sg.begin() + i * (L - 1), sg.begin() + (i + 1) * (L - 1));
    }
    return GP_OK;
}

int64_t rec_region_bytes(int64_t rcap, int L) {
    return (int64_t)align_up((size_t)rcap * 17, 16) + rcap * 2 * (int64_t)(L - 1);
}

// Runs the batch engine over the jobs' ranges; records land in the jobs'
// A/B lists, counts in their stats.
// GP_GEN_TIMING=1 in the environment prints the engine's phase times to
// stderr (diagnostics).
double since(std::chrono::steady_clock::time_point t) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
}

int run_batch(gp_ctx* c, std::vector<JobRun>& jobs, const BatchCfg& cfg, int* iterations, StopCtl* stop = nullptr) {
    StageRange nvtx_range("generate");
    static const bool timing = getenv("GP_GEN_TIMING") != nullptr;
    const auto tb = std::chrono::steady_clock::now();
    double t_win = 0, t_setup = 0, t_capture = 0, t_iter = 0;
    const int nj = (int)jobs.size();
    if (nj < 1 || nj > gp::kMaxEnumJobs) return c->fail(GP_ERR_ARG, "batch of %d jobs (1..%d)", nj, gp::kMaxEnumJobs);
    cudaStream_t s = c->s_comp;
    if (!c->ensure_job_streams()) return c->fail(GP_ERR_CUDA, "cannot create job streams");
    // ---- rank windows, shared out over the jobs by words in range
    const int64_t threads = (int64_t)c->num_sms * 8 * 256;
    const int64_t target = threads * std::max(1, cfg.windows_per_thread);
    double total_words = 0;
    for (auto& j : jobs) total_words += (double)range_words(j);
    // Each range is cut into windows of wsize words (the last one shorter);
    // the windows are laid out job by job, range by range, and built by
    // host threads over chunks of consecutive windows (each chunk steps its
    // own rank counter from its first window).
    struct Chunk {
        int ji;
        gp::u128 r0, r1, wsize;  // the range and the job's window size
        int64_t w0, nw;          // first window of the chunk (in its range), count
        int64_t out;             // index of its first window in cur / end / wjob
    };
    std::vector<Chunk> chunks;
    int64_t nwin = 0, nwin_narrow = 0;
    constexpr int64_t kChunkWindows = 8192;
    // the windows of jobs whose words fit 63 bits first: they go to the
    // enumerator's 64-bit instantiation, the others to a second launch
    auto narrow_job = [&](int ji) { return jobs[ji].p.b * jobs[ji].p.L <= 63; };
    for (int pass = 0; pass < 2; ++pass)
    for (int ji = 0; ji < nj; ++ji) {
        if (narrow_job(ji) != (pass == 0)) continue;
        JobRun& j = jobs[ji];
        const gp::u128 words = range_words(j);
        if (words == 0) continue;
        int64_t nw = (int64_t)((double)target * ((double)words / total_words));
        if (nw < 256) nw = 256;
        gp::u128 wsize = words / (gp::u128)nw;
        if (wsize < 1) wsize = 1;
        for (auto& r : j.ranges) {
            if (r.first >= r.second) continue;
            const int64_t n = (int64_t)((r.second - r.first + wsize - 1) / wsize);
            for (int64_t w0 = 0; w0 < n; w0 += kChunkWindows) {
                chunks.push_back({ji, r.first, r.second, wsize, w0, std::min(kChunkWindows, n - w0), nwin});
                nwin += std::min(kChunkWindows, n - w0);
            }
        }
        if (pass == 0) nwin_narrow = nwin;
    }
    std::vector<uint4> cur(nwin), end(nwin);
    std::vector<uint8_t> wjob(nwin);
    {
        std::atomic<size_t> next{0};
        auto work = [&]() {
            for (size_t ci = next++; ci < chunks.size(); ci = next++) {
                const Chunk& ch = chunks[ci];
                const GenPlan& p = jobs[ch.ji].p;
                const gp::u128 space = gp::upow(p.k, p.L);
                const gp::u128 maxw = gp::rank_to_word(space - 1, p.k, p.b, p.L);
                gp::u128 lo = ch.r0 + (gp::u128)ch.w0 * ch.wsize;
                gp::RankStepper step(lo, ch.wsize < space ? ch.wsize : space, p.k, p.b, p.L);
                for (int64_t i = 0; i < ch.nw; ++i, lo += ch.wsize) {
                    const bool whole = lo + ch.wsize <= ch.r1;  // the window ends wsize words on
                    const gp::u128 hi = whole ? lo + ch.wsize : ch.r1;
                    const int64_t o = ch.out + i;
                    cur[o] = to_u4(step.word());
                    step.advance();
                    if (hi >= space)
                        end[o] = to_u4(maxw + 1);
                    else if (whole)
                        end[o] = to_u4(step.word());
                    else
                        end[o] = to_u4(gp::rank_to_word(hi, p.k, p.b, p.L));
                    wjob[o] = (uint8_t)ch.ji;
                }
            }
        };
        const unsigned nt = (unsigned)std::min<size_t>(chunks.size(), std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
        std::vector<std::thread> th;
        for (unsigned t = 1; t < nt; ++t) th.emplace_back(work);
        work();
        for (auto& t : th) t.join();
    }
    t_win = since(tb);
    // ---- capacities and the device arena
    // appends after a job met its soft cap: a lane sees the count at most
    // 2 kCapCheck steps late, and a step (a block of the words that differ
    // from a prenecklace in its last two digits: k rows of up to k words)
    // appends at most one candidate per row and row sum with a role; plus a
    // warp's queue
    auto slack_for = [&](const GenPlan& p) {
        std::vector<int> sums;
        for (auto& d : p.dec) {
            sums.push_back(d.first);
            sums.push_back(d.second);
        }
        std::sort(sums.begin(), sums.end());
        const int64_t nsums = std::unique(sums.begin(), sums.end()) - sums.begin();
        const int64_t per_step = std::max<int64_t>(1, (int64_t)p.k * std::min<int64_t>(p.k, nsums));
        return threads * 2 * gp::kCapCheck * per_step + threads / 32 * gp::kEnumQueue + 4096;
    };
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    const size_t off_ctr = take(kCounterWords * 8);
    const size_t off_ejobs = take(sizeof(gp::EnumJob) * nj);
    const size_t off_rtab = take((size_t)nj * (gp::kMaxDigitSum + 1));
    const size_t off_cur = take((size_t)nwin * 16);
    const size_t off_end = take((size_t)nwin * 16);
    const size_t off_wjob = take((size_t)nwin);
    for (auto& j : jobs) {
        const gp::u128 words = range_words(j);
        if (words < (gp::u128)cfg.cand_cap) {
            j.soft = (int64_t)words + 1;  // never met: the job cannot park
            j.hard = j.soft;
        } else {
            j.soft = cfg.cand_cap;
            j.hard = cfg.cand_cap + slack_for(j.p);
        }
        // one iteration adds at most 2 records per candidate (x == y: A and B)
        j.rcap = 2 * j.hard + std::max<int64_t>(j.hard / 2, 4096);
        j.units.clear();
        for (int u = 1; u < j.p.L; ++u)
            if (std::gcd(u, j.p.L) == 1) j.units.push_back((int16_t)u);
        if (j.units.empty()) j.units.push_back(1);
        j.off_words = take((size_t)j.hard * 16);
        j.off_roles = take((size_t)j.hard);
        j.off_mask = take((size_t)(j.hard + 31) / 32 * 4);
        j.off_unsure = take((size_t)j.hard * 4);
        j.off_idx = take((size_t)j.hard * 4);
        j.off_rec = take((size_t)rec_region_bytes(j.rcap, j.p.L));
        j.off_units = take(j.units.size() * 2);
    }
    DevBuf& arena = c->scratch[7];
    HostPinned& hbuf = c->hscratch[3];
    if (!arena.ensure(off) || !hbuf.ensure(kCounterWords * 8))
        return c->fail(GP_ERR_NOMEM, "batch generation: cannot allocate %zu bytes of device memory", off);
    uint8_t* A = arena.as<uint8_t>();
    unsigned long long* ctr = reinterpret_cast<unsigned long long*>(A + off_ctr);
    unsigned long long* hctr = hbuf.as<unsigned long long>();
    // ---- job tables
    std::vector<gp::EnumJob> ej(nj);
    std::vector<uint8_t> rtab((size_t)nj * (gp::kMaxDigitSum + 1), 0);
    for (int ji = 0; ji < nj; ++ji) {
        JobRun& j = jobs[ji];
        const GenPlan& p = j.p;
        gp::EnumJob& e = ej[ji];
        e.L = p.L;
        e.b = p.b;
        gp::u128 mp = 0;
        for (int q = 0; q < p.L; ++q) mp |= (gp::u128)(p.k - 1) << (p.b * q);
        e.maxpat = {(uint64_t)mp, (uint64_t)(mp >> 64)};
        for (int t = 0; t < 4; ++t) {
            gp::u128 pl = 0;
            if (t < p.b)
                for (int q = 0; q < p.L; ++q) pl |= (gp::u128)1 << (p.b * q + t);
            e.plane[t] = {(uint64_t)pl, (uint64_t)(pl >> 64)};
        }
        e.words = reinterpret_cast<uint4*>(A + j.off_words);
        e.out_roles = A + j.off_roles;
        e.count = ctr + ji * kIterSlots + 0;
        e.cap = j.hard;
        e.soft_cap = j.soft;
        e.necklaces = ctr + kCumBase + ji * kCumSlots + 0;
        // roles by digit sum: row sum = -c L + 2 * digit sum
        for (int ds = 0; ds <= p.L * (p.k - 1) && ds <= gp::kMaxDigitSum; ++ds) {
            const int rs = -p.compress * p.L + 2 * ds;
            uint8_t& r = rtab[(size_t)ji * (gp::kMaxDigitSum + 1) + ds];
            for (auto& d : p.dec) {
                if (rs == d.first) r |= 1;
                if (rs == d.second) r |= 2;
            }
        }
        // (built before any graph capture: the tables are copied synchronously)
        if (!c->twiddle_image(p.L) || !c->twiddle64(p.L))
            return c->fail(GP_ERR_NOMEM, "batch generation: twiddle tables for length %d", p.L);
        GP_CUDA_TRY(c, cudaMemcpyAsync(A + j.off_units, j.units.data(), j.units.size() * 2, cudaMemcpyHostToDevice, s));
    }
    GP_CUDA_TRY(c, cudaMemcpyAsync(A + off_ejobs, ej.data(), sizeof(gp::EnumJob) * nj, cudaMemcpyHostToDevice, s));
    GP_CUDA_TRY(c, cudaMemcpyAsync(A + off_rtab, rtab.data(), rtab.size(), cudaMemcpyHostToDevice, s));
    if (nwin) {
        GP_CUDA_TRY(c, cudaMemcpyAsync(A + off_cur, cur.data(), (size_t)nwin * 16, cudaMemcpyHostToDevice, s));
        GP_CUDA_TRY(c, cudaMemcpyAsync(A + off_end, end.data(), (size_t)nwin * 16, cudaMemcpyHostToDevice, s));
        GP_CUDA_TRY(c, cudaMemcpyAsync(A + off_wjob, wjob.data(), (size_t)nwin, cudaMemcpyHostToDevice, s));
    }
    GP_CUDA_TRY(c, cudaMemsetAsync(ctr, 0, kCounterWords * 8, s));
    gp::EnumArgs ea;
    ea.jobs = reinterpret_cast<const gp::EnumJob*>(A + off_ejobs);
    ea.njobs = nj;
    ea.roles = A + off_rtab;
    ea.cur = reinterpret_cast<uint4*>(A + off_cur);
    ea.end = reinterpret_cast<const uint4*>(A + off_end);
    ea.win_job = A + off_wjob;
    ea.nwin = nwin;
    ea.incomplete = reinterpret_cast<int*>(ctr + kIncomplete);
    ea.next_win = ctr + kNextWin;
    ea.status = c->status.as<int>();
    // two launches per iteration when the batch mixes job widths: windows
    // [0, nwin_narrow) on the 64-bit enumerator, the rest on the 128-bit one
    gp::EnumArgs ea_wide = ea;
    ea.nwin = nwin_narrow;
    ea.narrow = 1;
    ea_wide.cur += nwin_narrow;
    ea_wide.end += nwin_narrow;
    ea_wide.win_job += nwin_narrow;
    ea_wide.nwin = nwin - nwin_narrow;
    ea_wide.next_win = ctr + kNextWinWide;
    ea_wide.narrow = 0;

    // ---- one iteration of the pipeline on stream s
    const bool multi = cfg.multi_launch && multi_launch_ok(jobs);
    auto row_src = [&](int ji) {
        const JobRun& j = jobs[ji];
        return gp::RowSrc{nullptr, reinterpret_cast<const uint4*>(A + j.off_words), j.p.L, j.p.b, j.p.compress};
    };
    auto finalize_args = [&](int ji) {
        JobRun& j = jobs[ji];
        const GenPlan& p = j.p;
        unsigned long long* it = ctr + ji * kIterSlots;
        uint8_t* rb = A + j.off_rec;
        gp::FinalizeArgs fa;
        fa.src = row_src(ji);
        fa.roles = A + j.off_roles;
        fa.fixed_role = 0;
        fa.idx = reinterpret_cast<uint32_t*>(A + j.off_idx);
        fa.n_idx = it + 2;
        fa.idx_cap = j.hard;
        fa.tw = c->twiddle64(p.L);
        fa.thr = 2.0 * p.order - p.paf + 0.001;
        fa.bound = 2 * p.order - p.paf;
        fa.invert_roles = 2;  // B lines carry bound - rint(psd) (io.cpp:26-36)
        fa.check_canonical = 1;
        fa.units = reinterpret_cast<const int16_t*>(A + j.off_units);
        fa.n_units = (int)j.units.size();
        fa.rec_words = reinterpret_cast<uint4*>(rb);
        fa.rec_role = rb + (size_t)j.rcap * 16;
        fa.rec_sig = reinterpret_cast<uint16_t*>(rb + align_up((size_t)j.rcap * 17, 16));
        fa.rec_src = nullptr;
        fa.rec_count = ctr + kCumBase + ji * kCumSlots + 1;
        fa.rec_cap = j.rcap;
        fa.psd_pass = ctr + kCumBase + ji * kCumSlots + 2;
        fa.status = c->status.as<int>();
        fa.prune_tab = c->spectral_prune && fa.bound < kPruneTab ? c->prune_tab.as<uint8_t>() : nullptr;
        return fa;
    };
    // every job in one launch per kernel, all on s
    auto enqueue_multi = [&]() -> int {
        gp::RowSrc src[gp::kMaxTcJobs];
        int64_t cap[gp::kMaxTcJobs];
        const unsigned long long* ndev[gp::kMaxTcJobs];
        int order[gp::kMaxTcJobs], paf[gp::kMaxTcJobs];
        uint32_t *mask[gp::kMaxTcJobs], *unsure[gp::kMaxTcJobs];
        unsigned long long* ucount[gp::kMaxTcJobs];
        gp::ListMultiArgs la{};
        gp::FinalizeMultiArgs fm{};
        la.njobs = fm.njobs = nj;
        la.status = c->status.as<int>();
        for (int ji = 0; ji < nj; ++ji) {
            JobRun& j = jobs[ji];
            unsigned long long* it = ctr + ji * kIterSlots;
            src[ji] = row_src(ji);
            cap[ji] = j.hard;
            ndev[ji] = it + 0;
            order[ji] = j.p.order;
            paf[ji] = j.p.paf;
            mask[ji] = reinterpret_cast<uint32_t*>(A + j.off_mask);
            unsure[ji] = reinterpret_cast<uint32_t*>(A + j.off_unsure);
            ucount[ji] = it + 1;
            la.job[ji] = gp::ListJob{mask[ji], j.hard, it + 0, reinterpret_cast<uint32_t*>(A + j.off_idx), it + 2,
                                     j.hard};
            fm.job[ji] = finalize_args(ji);
        }
        int rc = c->enqueue_filter_multi(src, cap, ndev, order, paf, mask, unsure, ucount, nj, cfg.tc_ctas_per_sm, s);
        if (rc) return rc;
        GP_CUDA_TRY(c, gp::launch_mask_to_list_multi(la, c->num_sms, s));
        GP_CUDA_TRY(c, gp::launch_finalize_multi(fm, cap, c->num_sms, s));
        return GP_OK;
    };
    auto enqueue_iteration = [&]() -> int {
        GP_CUDA_TRY(c, cudaMemsetAsync(ctr, 0, kIterWords * 8, s));
        if (ea.nwin > 0 && ea_wide.nwin > 0) {
            // both launches side by side (a branch of the graph): the wide
            // jobs' blocks take the SMs the narrow launch's finished blocks free
            cudaStream_t sw = c->s_jobs[gp_ctx::kJobStreams - 1];
            cudaEvent_t done = c->ev_join[gp_ctx::kJobStreams - 1];
            GP_CUDA_TRY(c, cudaEventRecord(c->ev_fork, s));
            GP_CUDA_TRY(c, cudaStreamWaitEvent(sw, c->ev_fork, 0));
            GP_CUDA_TRY(c, gp::launch_enumerate(ea, c->num_sms, s, cfg.enum_variant));
            GP_CUDA_TRY(c, gp::launch_enumerate(ea_wide, c->num_sms, sw, cfg.enum_variant));
            GP_CUDA_TRY(c, cudaEventRecord(done, sw));
            GP_CUDA_TRY(c, cudaStreamWaitEvent(s, done, 0));
        } else {  // one of the two has no windows (a no-op)
            GP_CUDA_TRY(c, gp::launch_enumerate(ea, c->num_sms, s, cfg.enum_variant));
            GP_CUDA_TRY(c, gp::launch_enumerate(ea_wide, c->num_sms, s, cfg.enum_variant));
        }
        if (multi) {
            const int rc = enqueue_multi();
            if (rc) return rc;
            GP_CUDA_TRY(c, cudaMemcpyAsync(hctr, ctr, kCounterWords * 8, cudaMemcpyDeviceToHost, s));
            return GP_OK;
        }
        // branches per job
        GP_CUDA_TRY(c, cudaEventRecord(c->ev_fork, s));
        for (int ji = 0; ji < nj; ++ji) {
            JobRun& j = jobs[ji];
            const GenPlan& p = j.p;
            cudaStream_t sj = c->s_jobs[ji];
            GP_CUDA_TRY(c, cudaStreamWaitEvent(sj, c->ev_fork, 0));
            unsigned long long* it = ctr + ji * kIterSlots;
            const gp::RowSrc src = row_src(ji);
            uint32_t* mask = reinterpret_cast<uint32_t*>(A + j.off_mask);
            uint32_t* idx = reinterpret_cast<uint32_t*>(A + j.off_idx);
            int rc = c->enqueue_filter_dev(src, j.hard, it + 0, p.order, p.paf, mask,
                                           reinterpret_cast<uint32_t*>(A + j.off_unsure), it + 1, cfg.tc_ctas_per_sm, sj);
            if (rc) return rc;
            GP_CUDA_TRY(c, gp::launch_mask_to_list(mask, j.hard, idx, it + 2, j.hard, c->status.as<int>(), c->num_sms,
                                                   sj, it + 0));
            const gp::FinalizeArgs fa = finalize_args(ji);
            GP_CUDA_TRY(c, gp::launch_finalize(fa, j.hard, c->num_sms, sj));
            GP_CUDA_TRY(c, cudaEventRecord(c->ev_join[ji], sj));
            GP_CUDA_TRY(c, cudaStreamWaitEvent(s, c->ev_join[ji], 0));
        }
        GP_CUDA_TRY(c, cudaMemcpyAsync(hctr, ctr, kCounterWords * 8, cudaMemcpyDeviceToHost, s));
        return GP_OK;
    };
    t_setup = since(tb) - t_win;
    // ---- capture it once
    cudaGraphExec_t exec = nullptr;
    if (cfg.use_graph) {
        GP_CUDA_TRY(c, cudaStreamSynchronize(s));
        GP_CUDA_TRY(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
        const int rc = enqueue_iteration();
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(s, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return rc;
        }
        if (e != cudaSuccess) return c->cuda_fail(e, "batch generation: graph capture");
        const cudaError_t e2 = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (e2 != cudaSuccess) return c->cuda_fail(e2, "batch generation: graph instantiation");
    }
    struct ExecGuard {
        cudaGraphExec_t& x;
        ~ExecGuard() {
            if (x) cudaGraphExecDestroy(x);
        }
    } guard{exec};
    t_capture = since(tb) - t_win - t_setup;
    // ---- iterate until no window is left unfinished
    int iters = 0;
    int stalled = 0;
    for (;;) {
        if (exec) {
            GP_CUDA_TRY(c, cudaGraphLaunch(exec, s));
        } else {
            const int rc = enqueue_iteration();
            if (rc) return rc;
        }
        GP_CUDA_TRY(c, cudaStreamSynchronize(s));
        int rc = c->check_status("batch generation");
        if (rc) return rc;
        ++iters;
        int64_t added = 0;
        for (int ji = 0; ji < nj; ++ji) {
            JobRun& j = jobs[ji];
            const int64_t cand = (int64_t)hctr[ji * kIterSlots + 0];
            added += cand;
            j.st.candidates += cand;
            j.st.unsure += (int64_t)hctr[ji * kIterSlots + 1];
            const int64_t nrec = (int64_t)hctr[kCumBase + ji * kCumSlots + 1];
            if (nrec > j.rcap - 2 * j.hard) {
                rc = drain_records(c, j, A, nrec);
                if (rc) return rc;
                GP_CUDA_TRY(c, cudaMemsetAsync(ctr + kCumBase + ji * kCumSlots + 1, 0, 8, s));
                hctr[kCumBase + ji * kCumSlots + 1] = 0;
            }
        }
        if (!hctr[kIncomplete]) break;
        // a window is left only when its job met its soft cap, so every
        // unfinished iteration appends candidates
        stalled = added ? 0 : stalled + 1;
        if (stalled > 2) return c->fail(GP_ERR_CUDA, "batch generation: no progress");
        if (stop && ((stop->max_iterations > 0 && iters >= stop->max_iterations) ||
                     (stop->max_seconds > 0 && std::chrono::duration<double>(std::chrono::steady_clock::now() -
                                                                             stop->start).count() >= stop->max_seconds))) {
            // unfinished windows hold the next word to visit (a finished
            // window holds its end): [rank(cur), rank(end)) is still to do
            std::vector<uint4> hcur(nwin);
            GP_CUDA_TRY(c, cudaMemcpy(hcur.data(), A + off_cur, (size_t)nwin * 16, cudaMemcpyDeviceToHost));
            auto from_u4 = [](uint4 v) {
                return ((gp::u128)v.w << 96) | ((gp::u128)v.z << 64) | ((gp::u128)v.y << 32) | v.x;
            };
            for (auto& j : jobs) j.remaining.clear();
            for (int64_t w = 0; w < nwin; ++w) {
                const gp::u128 cw = from_u4(hcur[w]), ew = from_u4(end[w]);
                if (cw == ew) continue;
                JobRun& j = jobs[wjob[w]];
                const gp::u128 lo = gp::word_to_rank(cw, j.p.k, j.p.b, j.p.L);
                const gp::u128 hi = gp::word_to_rank(ew, j.p.k, j.p.b, j.p.L);
                if (lo < hi) j.remaining.emplace_back(lo, hi);
            }
            stop->stopped = true;
            break;
        }
    }
    GP_CUDA_TRY(c, cudaStreamSynchronize(s));
    for (int ji = 0; ji < nj; ++ji) {
        JobRun& j = jobs[ji];
        const int rc = drain_records(c, j, A, (int64_t)hctr[kCumBase + ji * kCumSlots + 1]);
        if (rc) return rc;
        j.st.necklaces += (int64_t)hctr[kCumBase + ji * kCumSlots + 0];
        j.st.psd_pass += (int64_t)hctr[kCumBase + ji * kCumSlots + 2];
    }
    t_iter = since(tb) - t_win - t_setup - t_capture;
    if (iterations) *iterations = iters;
    if (timing)
        fprintf(stderr, "[gen] windows %.4f s, setup %.4f s, capture %.4f s, %d iterations + drains %.4f s\n", t_win,
                t_setup, t_capture, iters, t_iter);
    return GP_OK;
}

// One order per call (gp_generate, gp_generate_window): larger iterations.
BatchCfg single_job_cfg() {
    BatchCfg b;
    b.cand_cap = int64_t(1) << 24;
    return b;
}

std::string batch_key(const std::vector<JobRun>& jobs) {
    std::string k;
    for (auto& j : jobs) {
        const double w = (double)range_words(j);
        char buf[96];
        snprintf(buf, sizeof buf, "%d/%d/%d/%d;", j.p.order, j.p.compress, j.p.paf, w > 0 ? (int)std::log2(w) : -1);
        k += buf;
    }
    return k;
}

// The tuner: times a few settings of the engine on a sample of every job
// (the first 1/32 of its words, at least 2^24 or all of them) and keeps the
// fastest.  Results are cached in the context by the batch's shape.
int tune_batch(gp_ctx* c, const std::vector<JobRun>& jobs, BatchCfg& best, double* seconds) {
    const auto t0 = std::chrono::steady_clock::now();
    const std::string key = "batch:" + batch_key(jobs);
    auto hit = c->tuned.find(key);
    if (hit != c->tuned.end() && hit->second.size() == 6) {
        const auto& v = hit->second;
        best.enum_variant = (int)v[0];
        best.windows_per_thread = (int)v[1];
        best.cand_cap = v[2];
        best.tc_ctas_per_sm = (int)v[3];
        best.use_graph = (int)v[4];
        best.multi_launch = (int)v[5];
        *seconds = 0;
        return GP_OK;
    }
    std::vector<JobRun> sample;
    for (auto& j : jobs) {
        JobRun s;
        s.p = j.p;
        const gp::u128 words = range_words(j);
        gp::u128 want = words / 32;
        if (want < ((gp::u128)1 << 24)) want = words < ((gp::u128)1 << 24) ? words : ((gp::u128)1 << 24);
        for (auto& r : j.ranges) {
            if (want == 0) break;
            const gp::u128 n = r.second - r.first;
            const gp::u128 t = n < want ? n : want;
            s.ranges.emplace_back(r.first, r.first + t);
            want -= t;
        }
        sample.push_back(std::move(s));
    }
    std::vector<BatchCfg> cands;
    BatchCfg base;
    cands.push_back(base);
    BatchCfg v1 = base;
    v1.enum_variant = 1;
    cands.push_back(v1);
    BatchCfg v2 = base;
    v2.enum_variant = 2;
    cands.push_back(v2);
    BatchCfg w4 = base;
    w4.windows_per_thread = 4;
    cands.push_back(w4);
    BatchCfg big = base;
    big.cand_cap = int64_t(1) << 24;
    cands.push_back(big);
    BatchCfg one = base;
    one.tc_ctas_per_sm = 1;
    cands.push_back(one);
    if (multi_launch_ok(jobs)) {
        // one launch per kernel over every job
        BatchCfg ml = base;
        ml.multi_launch = 1;
        cands.push_back(ml);
        BatchCfg ml1 = ml;
        ml1.tc_ctas_per_sm = 1;
        cands.push_back(ml1);
    }
    double best_t = 1e300;
    for (size_t ci = 0; ci <= cands.size(); ++ci) {
        // candidate 0 runs twice; its first run (module loading) is not scored
        const BatchCfg& cfg = cands[ci == 0 ? 0 : ci - 1];
        std::vector<JobRun> run = sample;
        const auto a = std::chrono::steady_clock::now();
        const int rc = run_batch(c, run, cfg, nullptr);
        if (rc) return rc;
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
        if (ci > 0 && el < best_t) {
            best_t = el;
            best = cfg;
        }
    }
    c->tuned[key] = {best.enum_variant, best.windows_per_thread, best.cand_cap, best.tc_ctas_per_sm, best.use_graph,
                     best.multi_launch};
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
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

int finish(gp_ctx* c, const GenPlan& p, const RecordSet& ra, const RecordSet& rb, const char* path_a,
           const char* path_b, gp_gen_stats* st) {
    int rc_a = GP_OK;
    std::thread ta([&] { rc_a = write_records(c, p, ra, 0, path_a); });  // A and B files side by side
    const int rc_b = write_records(c, p, rb, 1, path_b);
    ta.join();
    if (rc_a) return rc_a;
    if (rc_b) return rc_b;
    st->written_a = (int64_t)ra.size();
    st->written_b = (int64_t)rb.size();
    return GP_OK;
}

// Job split of src/utils/lyndon.cpp:93-106: prenecklace prefixes of the
// first length i with at least proc_num * 10000 necklaces, dealt out round
// robin (1-based count), each covering the words that extend it.
std::vector<std::pair<gp::u128, gp::u128>> shard_ranges(const GenPlan& p, int proc_id, int proc_num) {
    const int L = p.L, k = p.k;
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
    return ranges;
}

// ------------------------------------------------------------ checkpoints
//
// A checkpoint holds a generation stopped part way: the job, its counts so
// far, the word-rank ranges still to search and the survivor records found
// so far.  Binary, host byte order:
//   "GPCK0001"
//   int32 order, compress, paf, L; uint32 n; n bytes: the job ("shard i n"
//   or "window lo hi")
//   int64 necklaces, candidates, psd_pass, unsure
//   uint64 ranges; per range: lo, hi as (low, high) uint64 pairs
//   A then B: uint64 records; the words as (low, high) uint64 pairs; then
//   (L - 1) uint16 signature values per record
// It is written to "<path>.tmp" and renamed over <path>, so a crash leaves
// the previous checkpoint intact.
const char kCkptMagic[8] = {'G', 'P', 'C', 'K', '0', '0', '0', '1'};

std::string u128_dec(gp::u128 v) {
    std::string s;
    do {
        s.push_back((char)('0' + (int)(v % 10)));
        v /= 10;
    } while (v);
    return std::string(s.rbegin(), s.rend());
}

template <typename T>
bool put(FILE* f, const T& v) { return fwrite(&v, sizeof v, 1, f) == 1; }
template <typename T>
bool get(FILE* f, T& v) { return fread(&v, sizeof v, 1, f) == 1; }

bool put_u128(FILE* f, gp::u128 v) { return put(f, (uint64_t)v) && put(f, (uint64_t)(v >> 64)); }
bool get_u128(FILE* f, gp::u128& v) {
    uint64_t lo = 0, hi = 0;
    if (!get(f, lo) || !get(f, hi)) return false;
    v = ((gp::u128)hi << 64) | lo;
    return true;
}

int save_checkpoint(gp_ctx* c, const char* path, const GenPlan& p, const std::string& spec, const JobRun& j) {
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = fopen(tmp.c_str(), "wb");
    if (!f) return c->fail(GP_ERR_IO, "cannot write checkpoint %s", tmp.c_str());
    bool ok = fwrite(kCkptMagic, 1, 8, f) == 8;
    ok = ok && put(f, (int32_t)p.order) && put(f, (int32_t)p.compress) && put(f, (int32_t)p.paf) &&
         put(f, (int32_t)p.L) && put(f, (uint32_t)spec.size()) && fwrite(spec.data(), 1, spec.size(), f) == spec.size();
    ok = ok && put(f, j.st.necklaces) && put(f, j.st.candidates) && put(f, j.st.psd_pass) && put(f, j.st.unsure);
    ok = ok && put(f, (uint64_t)j.remaining.size());
    for (auto& r : j.remaining) ok = ok && put_u128(f, r.first) && put_u128(f, r.second);
    for (const RecordSet* rs : {&j.ra, &j.rb}) {
        ok = ok && put(f, (uint64_t)rs->size());
        for (gp::u128 w : rs->words) ok = ok && put_u128(f, w);
        ok = ok && fwrite(rs->sigs.data(), 2, rs->sigs.size(), f) == rs->sigs.size();
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok || rename(tmp.c_str(), path) != 0) return c->fail(GP_ERR_IO, "cannot write checkpoint %s", path);
    return GP_OK;
}

// Loads a checkpoint into j (ranges, records, counts).  GP_ERR_FORMAT when
// the file is damaged or belongs to another job.
int load_checkpoint(gp_ctx* c, const char* path, const GenPlan& p, const std::string& spec, JobRun& j) {
    FILE* f = fopen(path, "rb");
    if (!f) return c->fail(GP_ERR_IO, "cannot read checkpoint %s", path);
    // counts read from the file are checked against the bytes left before
    // anything is sized by them: a damaged file is GP_ERR_FORMAT
    fseek(f, 0, SEEK_END);
    const long fsize = ftell(f);
    fseek(f, 0, SEEK_SET);
    auto left = [&]() -> uint64_t {
        const long pos = ftell(f);
        return pos < 0 || fsize < pos ? 0 : (uint64_t)(fsize - pos);
    };
    char magic[8];
    int32_t order = 0, compress = 0, paf = 0, L = 0;
    uint32_t n = 0;
    bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, kCkptMagic, 8) == 0;
    ok = ok && get(f, order) && get(f, compress) && get(f, paf) && get(f, L) && get(f, n) && n < 4096;
    std::string got(ok ? n : 0, '\0');
    ok = ok && fread(&got[0], 1, n, f) == n;
    if (ok && (order != p.order || compress != p.compress || paf != p.paf || L != p.L || got != spec)) {
        fclose(f);
        return c->fail(GP_ERR_FORMAT, "checkpoint %s belongs to another job (%s)", path, got.c_str());
    }
    ok = ok && get(f, j.st.necklaces) && get(f, j.st.candidates) && get(f, j.st.psd_pass) && get(f, j.st.unsure);
    uint64_t nr = 0;
    ok = ok && get(f, nr) && nr <= left() / 32;
    j.ranges.clear();
    for (uint64_t i = 0; ok && i < nr; ++i) {
        gp::u128 lo = 0, hi = 0;
        ok = get_u128(f, lo) && get_u128(f, hi) && lo < hi;
        if (ok) j.ranges.emplace_back(lo, hi);
    }
    for (RecordSet* rs : {&j.ra, &j.rb}) {
        uint64_t m = 0;
        ok = ok && get(f, m) && m <= left() / (16 + 2 * (uint64_t)(p.L - 1));
        if (!ok) break;
        rs->words.resize(m);
        for (uint64_t i = 0; ok && i < m; ++i) ok = get_u128(f, rs->words[i]);
        rs->sigs.resize((size_t)m * (p.L - 1));
        ok = ok && fread(rs->sigs.data(), 2, rs->sigs.size(), f) == rs->sigs.size();
    }
    fclose(f);
    return ok ? GP_OK : c->fail(GP_ERR_FORMAT, "checkpoint %s is damaged", path);
}

// Generation that can stop after max_iterations pipeline iterations or
// max_seconds (either <= 0: no limit) and resume from a checkpoint file.
int generate_resumable(gp_ctx* c, const GenPlan& p, const std::string& spec,
                       std::vector<std::pair<gp::u128, gp::u128>> ranges, const char* path_a, const char* path_b,
                       const char* ckpt, int max_iterations, double max_seconds, int* done, gp_gen_stats* stats) {
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<JobRun> jobs(1);
    JobRun& j = jobs[0];
    j.p = p;
    FILE* probe = fopen(ckpt, "rb");
    if (probe) {
        fclose(probe);
        const int rc = load_checkpoint(c, ckpt, p, spec, j);
        if (rc) return rc;
    } else {
        j.ranges = std::move(ranges);
    }
    StopCtl stop;
    stop.max_iterations = max_iterations;
    stop.max_seconds = max_seconds;
    int rc = GP_OK;
    if (!j.ranges.empty()) {
        BatchCfg cfg;  // 2^22 candidates per iteration: iterations stay short
        rc = run_batch(c, jobs, cfg, nullptr, &stop);
        if (rc) return rc;
    }
    gp_gen_stats st = j.st;
    if (stop.stopped) {
        rc = save_checkpoint(c, ckpt, p, spec, j);
        if (rc) return rc;
        if (done) *done = 0;
    } else {
        rc = finish(c, p, j.ra, j.rb, path_a, path_b, &st);
        if (rc) return rc;
        remove(ckpt);
        if (done) *done = 1;
    }
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = st;
    return GP_OK;
}

}  // namespace

extern "C" {

int64_t gp_job_ranges(int order, int compress, int paf, int proc_id, int proc_num, uint64_t* out, int64_t cap) {
    (void)paf;
    if (compress < 1 || order < 1 || order % compress || proc_num < 1 || proc_id < 0 || proc_id >= proc_num)
        return GP_ERR_ARG;
    GenPlan p;
    p.order = order;
    p.compress = compress;
    p.paf = paf;
    p.L = order / compress;
    p.alpha = gp::alphabet(compress);
    p.k = (int)p.alpha.size();
    p.b = gp::bits_for(p.k);
    if (p.b * p.L > 126) return GP_ERR_UNSUPPORTED;
    const auto ranges = shard_ranges(p, proc_id, proc_num);
    for (size_t i = 0; i < ranges.size() && (int64_t)i < cap && out; ++i) {
        out[4 * i + 0] = (uint64_t)(ranges[i].first >> 64);
        out[4 * i + 1] = (uint64_t)ranges[i].first;
        out[4 * i + 2] = (uint64_t)(ranges[i].second >> 64);
        out[4 * i + 3] = (uint64_t)ranges[i].second;
    }
    return (int64_t)ranges.size();
}

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
    std::vector<std::pair<gp::u128, gp::u128>> ranges = shard_ranges(p, proc_id, proc_num);
    std::vector<JobRun> jobs(1);
    jobs[0].p = p;
    jobs[0].ranges = std::move(ranges);
    rc = run_batch(c, jobs, single_job_cfg(), nullptr);
    if (rc) return rc;
    st = jobs[0].st;
    const auto tf = std::chrono::steady_clock::now();
    rc = finish(c, p, jobs[0].ra, jobs[0].rb, path_a, path_b, &st);
    if (rc) return rc;
    if (getenv("GP_GEN_TIMING")) fprintf(stderr, "[gen] files %.4f s\n", since(tf));
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
    std::vector<JobRun> jobs(1);
    jobs[0].p = p;
    if (lo < hi) jobs[0].ranges.emplace_back(lo, hi);
    rc = run_batch(c, jobs, single_job_cfg(), nullptr);
    if (rc) return rc;
    st = jobs[0].st;
    rc = finish(c, p, jobs[0].ra, jobs[0].rb, path_a, path_b, &st);
    if (rc) return rc;
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = st;
    return GP_OK;
}

}  // extern "C"

extern "C" int gp_generate_batch(gp_ctx* c, const gp_gen_job* jobs, int njobs, int autotune, gp_batch_config* cfg,
                                 gp_gen_stats* stats) {
    if (!c || !jobs) return GP_ERR_ARG;
    if (njobs < 1 || njobs > gp::kMaxEnumJobs)
        return c->fail(GP_ERR_ARG, "batch of %d jobs (1..%d)", njobs, gp::kMaxEnumJobs);
    const auto t0 = std::chrono::steady_clock::now();
    cudaSetDevice(c->device);
    std::vector<JobRun> run(njobs);
    for (int i = 0; i < njobs; ++i) {
        const gp_gen_job& q = jobs[i];
        if (!q.path_a || !q.path_b) return c->fail(GP_ERR_ARG, "job %d: missing output path", i);
        int rc = plan_for(c, q.order, q.compress, q.paf, run[i].p);
        if (rc) return rc;
        if (run[i].p.dec.empty())
            return c->fail(GP_NO_DECOMPOSITION, "job %d: order %d cannot be decomposed", i, q.order);
        gp::u128 lo = ((gp::u128)q.begin_hi << 64) | q.begin_lo;
        gp::u128 hi = ((gp::u128)q.end_hi << 64) | q.end_lo;
        const gp::u128 space = gp::upow(run[i].p.k, run[i].p.L);
        if (hi > space) hi = space;
        if (lo < hi) run[i].ranges.emplace_back(lo, hi);
    }
    BatchCfg bc;
    double tune_s = 0;
    if (autotune) {
        int rc = tune_batch(c, run, bc, &tune_s);
        if (rc) return rc;
    } else if (cfg) {
        if (cfg->enum_variant == 1 || cfg->enum_variant == 2) bc.enum_variant = cfg->enum_variant;
        if (cfg->windows_per_thread > 0) bc.windows_per_thread = cfg->windows_per_thread;
        if (cfg->cand_cap > 0) bc.cand_cap = cfg->cand_cap;
        if (cfg->tc_ctas_per_sm > 0) bc.tc_ctas_per_sm = cfg->tc_ctas_per_sm;
        bc.use_graph = cfg->no_graph ? 0 : 1;
        if (cfg->multi_launch == 1) {
            if (!multi_launch_ok(run))
                return c->fail(GP_ERR_UNSUPPORTED, "batch generation: these jobs do not fit one filter launch");
            bc.multi_launch = 1;
        }
    }
    int iters = 0;
    int rc = run_batch(c, run, bc, &iters);
    if (rc) return rc;
    const auto tf = std::chrono::steady_clock::now();
    {
        // the jobs' files in parallel (each file is formatted by host threads too)
        std::vector<int> rcs(njobs, GP_OK);
        std::vector<std::thread> th;
        for (int i = 0; i < njobs; ++i)
            th.emplace_back([&, i] {
                rcs[i] = finish(c, run[i].p, run[i].ra, run[i].rb, jobs[i].path_a, jobs[i].path_b, &run[i].st);
            });
        for (auto& t : th) t.join();
        for (int i = 0; i < njobs; ++i)
            if (rcs[i]) return rcs[i];
    }
    if (getenv("GP_GEN_TIMING")) fprintf(stderr, "[gen] files %.4f s\n", since(tf));
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats)
        for (int i = 0; i < njobs; ++i) {
            stats[i] = run[i].st;
            stats[i].seconds = el;
        }
    if (cfg) {
        cfg->enum_variant = bc.enum_variant;
        cfg->windows_per_thread = bc.windows_per_thread;
        cfg->cand_cap = bc.cand_cap;
        cfg->tc_ctas_per_sm = bc.tc_ctas_per_sm;
        cfg->no_graph = bc.use_graph ? 0 : 1;
        cfg->multi_launch = bc.multi_launch;
        cfg->iterations = iters;
        cfg->tune_seconds = tune_s;
    }
    return GP_OK;
}

extern "C" int gp_generate_resumable(gp_ctx* c, int order, int compress, int paf, int proc_id, int proc_num,
                                     const char* path_a, const char* path_b, const char* checkpoint_path,
                                     int max_iterations, double max_seconds, int* done, gp_gen_stats* stats) {
    if (!c || !path_a || !path_b || !checkpoint_path) return GP_ERR_ARG;
    if (proc_num < 1 || proc_id < 0 || proc_id >= proc_num)
        return c->fail(GP_ERR_ARG, "bad job split %d of %d", proc_id, proc_num);
    cudaSetDevice(c->device);
    GenPlan p;
    int rc = plan_for(c, order, compress, paf, p);
    if (rc) return rc;
    if (p.dec.empty()) return c->fail(GP_NO_DECOMPOSITION, "Order %d cannot be decomposed", order);
    const std::string spec = "shard " + std::to_string(proc_id) + " " + std::to_string(proc_num);
    try {  // no C++ exception crosses the C ABI
        return generate_resumable(c, p, spec, shard_ranges(p, proc_id, proc_num), path_a, path_b, checkpoint_path,
                                  max_iterations, max_seconds, done, stats);
    } catch (const std::exception& e) {
        return c->fail(GP_ERR_NOMEM, "checkpointed generation: %s", e.what());
    }
}

extern "C" int gp_generate_window_resumable(gp_ctx* c, int order, int compress, int paf, uint64_t begin_hi,
                                            uint64_t begin_lo, uint64_t end_hi, uint64_t end_lo, const char* path_a,
                                            const char* path_b, const char* checkpoint_path, int max_iterations,
                                            double max_seconds, int* done, gp_gen_stats* stats) {
    if (!c || !path_a || !path_b || !checkpoint_path) return GP_ERR_ARG;
    cudaSetDevice(c->device);
    GenPlan p;
    int rc = plan_for(c, order, compress, paf, p);
    if (rc) return rc;
    if (p.dec.empty()) return c->fail(GP_NO_DECOMPOSITION, "Order %d cannot be decomposed", order);
    gp::u128 lo = ((gp::u128)begin_hi << 64) | begin_lo;
    gp::u128 hi = ((gp::u128)end_hi << 64) | end_lo;
    const gp::u128 space = gp::upow(p.k, p.L);
    if (hi > space) hi = space;
    std::vector<std::pair<gp::u128, gp::u128>> ranges;
    if (lo < hi) ranges.emplace_back(lo, hi);
    const std::string spec = "window " + u128_dec(lo) + " " + u128_dec(hi);
    try {  // no C++ exception crosses the C ABI
        return generate_resumable(c, p, spec, ranges, path_a, path_b, checkpoint_path, max_iterations, max_seconds,
                                  done, stats);
    } catch (const std::exception& e) {
        return c->fail(GP_ERR_NOMEM, "checkpointed generation: %s", e.what());
    }
}
