// golay -- command line driver with the reference's interface (src/main.cpp):
//
//   golay [OPTIONS] order SUBCOMMAND...
//     order                 required positional
//     -c,--compress INT...  compression list (default 1)
//     --paf INT             PAF constant (default 0)
//     -j,--jobid INT        job id (default 0)
//     -n,--numjob INT       number of jobs (default 1)
//     -d,--dir PATH         work directory (default "results")
//   subcommands (any number, run in pipeline order): all gen sort match
//   uncompress filter, with the reference's per-subcommand options; gen
//   also takes --checkpoint FILE [--max-seconds S] [--max-iterations N]
//   (not in the reference) for searches that stop and resume, and --binary
//   (binary survivor files, which sort reads and the export subcommand turns
//   into the reference's text; export runs on the host without a GPU).
//
// Files and their names are the reference's (src/main.cpp:32-44,62-67,
// 88-90,147-149).  Every stage runs on the GPU through the C ABI in
// include/golaypair_gb300.h; there is no CPU path.
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "golaypair_gb300.h"

namespace {

struct Options {
    int order = -1;
    int paf_constant = 0;
    int job_id = 0;
    int job_count = 1;
    std::vector<int> compress = {1};
    std::string temp_dir = "results";
    std::string work_dir() const { return temp_dir + "/order-" + std::to_string(order); }
};

struct GenOpts {
    std::string file_prefix = "filtered";
    std::string checkpoint;  // not in the reference: resumable generation
    double max_seconds = 0;
    int max_iterations = 0;
    bool binary = false;     // not in the reference: binary survivor files
    bool prune = false;      // not in the reference: spectral pruning of candidates
};
// not in the reference: binary survivor files -> the reference's text
struct ExportOpts { std::string input_prefix = "filtered", output_prefix = "filtered"; };
struct SortOpts { std::string input_prefix = "filtered", output_prefix = "filtered_sorted"; };
struct MatchOpts {
    std::string input_prefix = "filtered_sorted", output_prefix = "pairs";
    bool file_append = false;
};
struct UncompressOpts {
    std::string input_prefix = "pairs", internal_prefix = "filtered", sorted_prefix = "filtered_sorted";
    std::string output_prefix = "pairs", temp_prefix;
    // the reference parses these but does not use them; here they select the
    // input lines of the first level: --line N (1-based) or lines
    // range_begin, range_begin + range_step, ... < range_end (0-based)
    long long line = -1, range_begin = 0, range_end = -1, range_step = 1;
};
struct FilterOpts { std::string input_prefix = "pairs", output_prefix = "unique"; };

gp_ctx* g_ctx = nullptr;
// gen with --checkpoint stopped early: the checkpoint is written, run again
constexpr int kExitCheckpointed = 75;

int die(const char* what, int rc) {
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, g_ctx ? gp_last_error(g_ctx) : "");
    return 1;
}

std::string cand_file(const Options& o, const std::string& prefix, char ab, int job) {
    return o.work_dir() + "/" + std::to_string(o.order) + "-" + prefix + "-" + ab + "#" + std::to_string(job);
}
std::string sorted_file(const Options& o, const std::string& prefix, char ab) {
    return o.work_dir() + "/" + std::to_string(o.order) + "-" + prefix + "-" + ab;
}
std::string match_file(const Options& o, const std::string& prefix, int ci) {
    return o.work_dir() + "/" + std::to_string(o.order) + "-" + prefix + "-" + std::to_string(o.compress[ci]);
}

// src/main.cpp:47-54
int stage_generate(const Options& o, const GenOpts& g) {
    gp_gen_stats st;
    if (g.binary) {
        const int frc = gp_set_output_format(g_ctx, GP_FORMAT_BINARY);
        if (frc) return die("gen", frc);
    }
    if (g.prune) {
        const int prc = gp_set_spectral_prune(g_ctx, 1);
        if (prc) return die("gen", prc);
    }
    const std::string fa = cand_file(o, g.file_prefix, 'a', o.job_id);
    const std::string fb = cand_file(o, g.file_prefix, 'b', o.job_id);
    int done = 1;
    const int rc = g.checkpoint.empty()
                       ? gp_generate(g_ctx, o.order, o.compress[0], o.paf_constant, o.job_id, o.job_count, fa.c_str(),
                                     fb.c_str(), &st)
                       : gp_generate_resumable(g_ctx, o.order, o.compress[0], o.paf_constant, o.job_id, o.job_count,
                                               fa.c_str(), fb.c_str(), g.checkpoint.c_str(), g.max_iterations,
                                               g.max_seconds, &done, &st);
    if (rc == GP_NO_DECOMPOSITION) {
        fprintf(stderr, "Order %d cannot be decomposed into a sum of squares\n%d*2\nHence there are no solutions.\n",
                o.order, o.order);
        return 1;
    }
    if (rc) return die("gen", rc);
    if (!done) {
        printf("[gpu] stopped after %.3f s: %lld necklaces so far; checkpoint %s; run gen again to continue\n",
               st.seconds, (long long)st.necklaces, g.checkpoint.c_str());
        return kExitCheckpointed;
    }
    printf("Orderly Count: %lld\nPassed PSD filter: %lld\n", (long long)st.necklaces,
           (long long)(st.written_a + st.written_b));
    printf("[gpu] candidates %lld, exact PSD passes %lld, tensor-core unsure %lld, %.3f s\n",
           (long long)st.candidates, (long long)st.psd_pass, (long long)st.unsure, st.seconds);
    return 0;
}

// Text files of this job's binary survivor files (in place by default:
// written to a temporary file, then renamed over the binary one).  Text
// inputs are left as they are, or copied when the output is elsewhere.
int stage_export(const Options& o, const ExportOpts& e) {
    for (char ab : {'a', 'b'}) {
        const std::string in = cand_file(o, e.input_prefix, ab, o.job_id);
        const std::string out = cand_file(o, e.output_prefix, ab, o.job_id);
        const std::string tmp = out + ".tmp";
        int rc = gp_export_text(nullptr, in.c_str(), tmp.c_str());
        if (rc == GP_ERR_FORMAT) {  // a text file already
            std::remove(tmp.c_str());
            if (in == out) continue;
            FILE* fi = fopen(in.c_str(), "rb");
            FILE* fo = fi ? fopen(tmp.c_str(), "wb") : nullptr;
            bool ok = fi && fo;
            char buf[1 << 16];
            size_t got;
            while (ok && (got = fread(buf, 1, sizeof buf, fi)) > 0) ok = fwrite(buf, 1, got, fo) == got;
            if (fi) fclose(fi);
            if (fo) ok = (fclose(fo) == 0) && ok;
            rc = ok ? GP_OK : GP_ERR_IO;
        }
        if (rc) {
            std::remove(tmp.c_str());
            fprintf(stderr, "export: %s -> %s failed (%d)\n", in.c_str(), out.c_str(), rc);
            return 1;
        }
        if (std::rename(tmp.c_str(), out.c_str()) != 0) {
            fprintf(stderr, "export: cannot rename %s: %s\n", tmp.c_str(), strerror(errno));
            return 1;
        }
    }
    return 0;
}

// src/main.cpp:69-79
int stage_sort(const Options& o, const SortOpts& s) {
    printf("Sorting Candidates\n");
    for (char ab : {'a', 'b'}) {
        std::vector<std::string> files;
        for (int j = 0; j < o.job_count; ++j) files.push_back(cand_file(o, s.input_prefix, ab, j));
        std::vector<const char*> ptrs;
        for (auto& f : files) ptrs.push_back(f.c_str());
        const std::string out = sorted_file(o, s.output_prefix, ab);
        const int rc = gp_sort(g_ctx, ptrs.data(), (int)ptrs.size(), out.c_str());
        if (rc) {
            fprintf(stderr, "Sort failed\n");
            return die("sort", rc);
        }
    }
    return 0;
}

// src/main.cpp:92-102
int stage_match(const Options& o, const MatchOpts& m) {
    printf("Matching Candidates\n");
    const std::string a = sorted_file(o, m.input_prefix, 'a'), b = sorted_file(o, m.input_prefix, 'b');
    const std::string out = match_file(o, m.output_prefix, 0);
    int64_t np = 0;
    const int rc = gp_match(g_ctx, o.order, o.compress[0], o.paf_constant, a.c_str(), b.c_str(), out.c_str(),
                            m.file_append ? 1 : 0, &np);
    if (rc == GP_EMPTY_INPUT) return 1;
    if (rc) return die("match", rc);
    return 0;
}

// src/main.cpp:117-139: every level of the chain in one call; level i
// reads the pairs of level i - 1 from memory and writes its own file
int stage_uncompress(const Options& o, const UncompressOpts& u) {
    const int nlev = (int)o.compress.size() - 1;
    if (nlev < 1) return 0;
    const std::string in = match_file(o, u.input_prefix, 0);
    std::vector<std::string> outs;
    for (int i = 0; i < nlev; ++i) outs.push_back(match_file(o, u.output_prefix, i + 1));
    std::vector<const char*> out_ptrs;
    for (auto& s : outs) out_ptrs.push_back(s.c_str());
    int64_t first = 0, end = INT64_MAX, step = 1;
    if (u.line >= 1) {
        first = u.line - 1;
        end = u.line;
    } else {
        first = u.range_begin;
        end = u.range_end >= 0 ? u.range_end : INT64_MAX;
        step = u.range_step;
    }
    const int rc = gp_uncompress_chain(g_ctx, o.order, o.compress.data(), (int)o.compress.size(), o.paf_constant,
                                       in.c_str(), out_ptrs.data(), first, end, step);
    if (rc < 0) return die("uncompress", rc);
    return 0;
}

// src/main.cpp:151-159
int stage_filter(const Options& o, const FilterOpts& f) {
    printf("Filtering pairs of compression size %d\n", o.compress.back());
    const std::string in = match_file(o, f.input_prefix, (int)o.compress.size() - 1);
    const std::string out = o.work_dir() + "/" + std::to_string(o.order) + "-" + f.output_prefix;
    const int rc = gp_equiv_filter(g_ctx, o.order, o.compress.back(), in.c_str(), out.c_str());
    if (rc) return die("filter", rc);
    return 0;
}

bool is_int(const char* s) {
    if (*s == '-' || *s == '+') ++s;
    if (!*s) return false;
    for (; *s; ++s)
        if (*s < '0' || *s > '9') return false;
    return true;
}

bool mkdirs(const std::string& path) {
    std::string cur;
    for (size_t i = 0; i <= path.size(); ++i) {
        if (i == path.size() || path[i] == '/') {
            if (!cur.empty() && mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return false;
        }
        if (i < path.size()) cur.push_back(path[i]);
    }
    return true;
}

void usage() {
    printf(
        "Complementary Pairs Pipeline (GB300)\n"
        "Usage: golay [OPTIONS] order SUBCOMMAND...\n\n"
        "Positionals:\n  order INT REQUIRED          Order\n\n"
        "Options:\n"
        "  -h,--help                   Print this help message and exit\n"
        "  -c,--compress INT ...       Set compression level (default=1)\n"
        "  --paf INT                   Set PAF constant (default=0)\n"
        "  -j,--jobid INT              Set job id (default=0)\n"
        "  -n,--numjob INT             Set number of jobs (default=1)\n"
        "  -d,--dir TEXT               Set directory for populating temporary files (default=results)\n\n"
        "Subcommands:\n"
        "  all                         Run all steps in the pipeline\n"
        "  gen                         Candidate generation step (-o,--output)\n"
        "                              --checkpoint FILE [--max-seconds S] [--max-iterations N]:\n"
        "                              stop early and resume from FILE (exit code 75 = stopped)\n"
        "                              --binary: write binary survivor files (see export)\n"
        "                              --spectral-prune: leave out candidates that cannot have a\n"
        "                              partner (p(L/2), p(L/3) tests); pair files are unchanged\n"
        "  export                      Binary survivor files of this job -> the reference's text\n"
        "                              (-i,--input -o,--output; default in place); sort reads both\n"
        "  sort                        File sorting step (-i,--input -o,--output)\n"
        "  match                       Candidate matching step (-i,--input -o,--output -a,--append BOOL)\n"
        "  uncompress                  Pair uncompression step (-i -o --internal --sorted -l -b -e -s -p,--prefix\n"
        "                              -l N: only input line N (1-based); -b B -e E -s S: input lines\n"
        "                              B, B+S, ... below E (0-based), for splitting one uncompression\n"
        "                              -d,--device [cpu,gpu]; both devices run on the GPU here)\n"
        "  filter                      Pair equivalence filter step\n");
}

}  // namespace

int main(int argc, char** argv) {
    Options opts;
    GenOpts gen;
    SortOpts srt;
    MatchOpts mat;
    UncompressOpts unc;
    FilterOpts fil;
    ExportOpts exp;
    bool s_all = false, s_gen = false, s_sort = false, s_match = false, s_unc = false, s_filter = false;
    bool s_export = false;
    std::string ctx;  // current subcommand ("" = global)
    bool compress_given = false;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&](const char* what) -> std::string {
            if (i + 1 >= argc) {
                fprintf(stderr, "%s: 1 required argument missing\n", what);
                exit(108);
            }
            return argv[++i];
        };
        if (a == "-h" || a == "--help") {
            usage();
            return 0;
        }
        if (a == "all" || a == "gen" || a == "sort" || a == "match" || a == "uncompress" || a == "filter" ||
            a == "export") {
            ctx = a;
            s_export |= a == "export";
            s_all |= a == "all";
            s_gen |= a == "gen";
            s_sort |= a == "sort";
            s_match |= a == "match";
            s_unc |= a == "uncompress";
            s_filter |= a == "filter";
            continue;
        }
        if (ctx.empty()) {
            if (a == "-c" || a == "--compress") {
                opts.compress.clear();
                while (i + 1 < argc && is_int(argv[i + 1])) opts.compress.push_back(atoi(argv[++i]));
                if (opts.compress.empty()) {
                    fprintf(stderr, "--compress: argument missing\n");
                    return 108;
                }
                compress_given = true;
                continue;
            }
            if (a == "--paf") { opts.paf_constant = atoi(next("--paf").c_str()); continue; }
            if (a == "-j" || a == "--jobid") { opts.job_id = atoi(next("--jobid").c_str()); continue; }
            if (a == "-n" || a == "--numjob") { opts.job_count = atoi(next("--numjob").c_str()); continue; }
            if (a == "-d" || a == "--dir") { opts.temp_dir = next("--dir"); continue; }
            if (is_int(a.c_str()) && opts.order < 0) { opts.order = atoi(a.c_str()); continue; }
        } else if (ctx == "gen") {
            if (a == "-o" || a == "--output") { gen.file_prefix = next("--output"); continue; }
            if (a == "--checkpoint") { gen.checkpoint = next("--checkpoint"); continue; }
            if (a == "--max-seconds") { gen.max_seconds = atof(next("--max-seconds").c_str()); continue; }
            if (a == "--max-iterations") { gen.max_iterations = atoi(next("--max-iterations").c_str()); continue; }
            if (a == "--binary") { gen.binary = true; continue; }
            if (a == "--spectral-prune") { gen.prune = true; continue; }
        } else if (ctx == "export") {
            if (a == "-i" || a == "--input") { exp.input_prefix = next("--input"); continue; }
            if (a == "-o" || a == "--output") { exp.output_prefix = next("--output"); continue; }
        } else if (ctx == "sort") {
            if (a == "-i" || a == "--input") { srt.input_prefix = next("--input"); continue; }
            if (a == "-o" || a == "--output") { srt.output_prefix = next("--output"); continue; }
        } else if (ctx == "match") {
            if (a == "-i" || a == "--input") { mat.input_prefix = next("--input"); continue; }
            if (a == "-o" || a == "--output") { mat.output_prefix = next("--output"); continue; }
            if (a == "-a" || a == "--append") {
                const std::string v = next("--append");
                mat.file_append = v == "1" || v == "true" || v == "TRUE" || v == "on" || v == "yes";
                continue;
            }
        } else if (ctx == "uncompress") {
            if (a == "-i" || a == "--input") { unc.input_prefix = next("--input"); continue; }
            if (a == "-o" || a == "--output") { unc.output_prefix = next("--output"); continue; }
            if (a == "--internal") { unc.internal_prefix = next("--internal"); continue; }
            if (a == "--sorted") { unc.sorted_prefix = next("--sorted"); continue; }
            if (a == "-p" || a == "--prefix") { unc.temp_prefix = next("--prefix"); continue; }
            // parsed but unused by the reference (src/main.cpp:110-113,192-195): a line split here
            if (a == "-l" || a == "--line") { unc.line = atoll(next("--line").c_str()); continue; }
            if (a == "-b" || a == "--range_begin") { unc.range_begin = atoll(next("--range_begin").c_str()); continue; }
            if (a == "-e" || a == "--range_end") { unc.range_end = atoll(next("--range_end").c_str()); continue; }
            if (a == "-s" || a == "--range_step") { unc.range_step = atoll(next("--range_step").c_str()); continue; }
            if (a == "-d" || a == "--device") {
                std::string v = next("--device");
                for (auto& ch : v) ch = (char)tolower(ch);
                if (v != "cpu" && v != "gpu") {
                    fprintf(stderr, "--device: %s not in {cpu,gpu}\n", v.c_str());
                    return 105;
                }
                continue;
            }
        } else if (ctx == "filter") {
            // the reference binds these to the uncompress options (src/main.cpp:208-209): no effect
            if (a == "-i" || a == "--input" || a == "-o" || a == "--output") {
                (void)next(a.c_str());
                continue;
            }
        }
        fprintf(stderr, "The following argument was not expected: %s\nRun with --help for more information.\n",
                a.c_str());
        return 109;
    }
    (void)compress_given;
    if (opts.order < 0) {
        fprintf(stderr, "order is required\nRun with --help for more information.\n");
        return 106;
    }
    if (!(s_all || s_gen || s_sort || s_match || s_unc || s_filter || s_export)) {
        fprintf(stderr, "A subcommand is required\nRun with --help for more information.\n");
        return 106;
    }
    if (!mkdirs(opts.work_dir())) {
        fprintf(stderr, "Failed to create temp directories: %s\n", strerror(errno));
        return 1;
    }
    if (s_export && !(s_all || s_gen || s_sort || s_match || s_unc || s_filter))
        return stage_export(opts, exp);  // host only: no GPU needed
    const char* dev = getenv("GP_DEVICE");
    int rc = gp_ctx_create(&g_ctx, dev ? atoi(dev) : 0);
    if (rc) {
        fprintf(stderr, "golay: no usable sm_103a GPU (gp_ctx_create -> %d); this build has no CPU path\n", rc);
        return 1;
    }
    int status = 0;
    if (!status && (s_gen || s_all)) status = stage_generate(opts, gen);
    if (!status && s_export) status = stage_export(opts, exp);
    if (!status && (s_sort || s_all)) status = stage_sort(opts, srt);
    if (!status && (s_match || s_all)) status = stage_match(opts, mat);
    if (!status && (s_unc || s_all)) status = stage_uncompress(opts, unc);
    if (!status && (s_filter || s_all)) status = stage_filter(opts, fil);
    gp_ctx_destroy(g_ctx);
    return status ? 1 : 0;
}
