/*
 * golay_oracle -- command line driver of the CPU restatement, mirroring the
 * reference's src/main.cpp:14-251 (same positional order, options,
 * subcommands and file names).  TEST INFRASTRUCTURE ONLY: used to produce
 * the oracle's files for comparison and as the timed CPU baseline.
 */
#define _GNU_SOURCE
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "golay_oracle.h"

static int mkdirs(const char* path) {
    char buf[4096];
    snprintf(buf, sizeof buf, "%s", path);
    for (char* p = buf + 1; *p; ++p) {
        if (*p == '/') {
            *p = 0;
            if (mkdir(buf, 0755) && errno != EEXIST) return 1;
            *p = '/';
        }
    }
    if (mkdir(buf, 0755) && errno != EEXIST) return 1;
    return 0;
}

static int is_int(const char* s) {
    if (*s == '-' || *s == '+') ++s;
    if (!*s) return 0;
    for (; *s; ++s)
        if (*s < '0' || *s > '9') return 0;
    return 1;
}

int main(int argc, char** argv) {
    int order = -1, paf = 0, job_id = 0, job_count = 1;
    int compress[64] = {1};
    int ncompress = 1;
    const char* dir = "results";
    int s_all = 0, s_gen = 0, s_sort = 0, s_match = 0, s_unc = 0, s_filter = 0;
    const char* gen_out = "filtered";
    const char* sort_in = "filtered";
    const char* sort_out = "filtered_sorted";
    const char* match_in = "filtered_sorted";
    const char* match_out = "pairs";
    int match_append = 0;
    const char* unc_in = "pairs";
    const char* unc_out = "pairs";
    const char* unc_prefix = "";
    const char* ctx = "";
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        if (!strcmp(a, "all")) { s_all = 1; ctx = a; continue; }
        if (!strcmp(a, "gen")) { s_gen = 1; ctx = a; continue; }
        if (!strcmp(a, "sort")) { s_sort = 1; ctx = a; continue; }
        if (!strcmp(a, "match")) { s_match = 1; ctx = a; continue; }
        if (!strcmp(a, "uncompress")) { s_unc = 1; ctx = a; continue; }
        if (!strcmp(a, "filter")) { s_filter = 1; ctx = a; continue; }
#define NEXT() ((i + 1 < argc) ? argv[++i] : (fprintf(stderr, "%s needs a value\n", a), exit(109), ""))
        if (!strcmp(a, "-c") || !strcmp(a, "--compress")) {
            ncompress = 0;
            while (i + 1 < argc && is_int(argv[i + 1]) && ncompress < 64) compress[ncompress++] = atoi(argv[++i]);
            if (!ncompress) { fprintf(stderr, "--compress needs values\n"); return 109; }
            continue;
        }
        if (!strcmp(a, "--paf")) { paf = atoi(NEXT()); continue; }
        if (!strcmp(a, "-j") || !strcmp(a, "--jobid")) { job_id = atoi(NEXT()); continue; }
        if (!strcmp(a, "-n") || !strcmp(a, "--numjob")) { job_count = atoi(NEXT()); continue; }
        if (!strcmp(ctx, "uncompress") && (!strcmp(a, "-d") || !strcmp(a, "--device"))) { (void)NEXT(); continue; }
        if (!strcmp(a, "-d") || !strcmp(a, "--dir")) { dir = NEXT(); continue; }
        if (!strcmp(a, "-o") || !strcmp(a, "--output")) {
            const char* v = NEXT();
            if (!strcmp(ctx, "gen")) gen_out = v;
            else if (!strcmp(ctx, "sort")) sort_out = v;
            else if (!strcmp(ctx, "match")) match_out = v;
            else if (!strcmp(ctx, "uncompress")) unc_out = v;
            continue;
        }
        if (!strcmp(a, "-i") || !strcmp(a, "--input")) {
            const char* v = NEXT();
            if (!strcmp(ctx, "sort")) sort_in = v;
            else if (!strcmp(ctx, "match")) match_in = v;
            else if (!strcmp(ctx, "uncompress")) unc_in = v;
            continue;
        }
        if (!strcmp(a, "-a") || !strcmp(a, "--append")) {
            const char* v = NEXT();
            match_append = !strcmp(v, "1") || !strcmp(v, "true");
            continue;
        }
        if (!strcmp(a, "-p") || !strcmp(a, "--prefix")) { unc_prefix = NEXT(); continue; }
        if (!strcmp(a, "--internal") || !strcmp(a, "--sorted") || !strcmp(a, "-l") || !strcmp(a, "--line") ||
            !strcmp(a, "-b") || !strcmp(a, "--range_begin") || !strcmp(a, "-e") || !strcmp(a, "--range_end") ||
            !strcmp(a, "-s") || !strcmp(a, "--range_step")) {
            (void)NEXT();
            continue;
        }
        if (is_int(a) && order < 0) { order = atoi(a); continue; }
        fprintf(stderr, "unknown argument: %s\n", a);
        return 109;
    }
    if (order < 0) { fprintf(stderr, "order is required\n"); return 106; }
    if (!(s_all | s_gen | s_sort | s_match | s_unc | s_filter)) {
        fprintf(stderr, "A subcommand is required\n");
        return 106;
    }
    char wd[4096];
    snprintf(wd, sizeof wd, "%s/order-%d", dir, order);
    if (mkdirs(wd)) { fprintf(stderr, "Failed to create temp directories\n"); return 1; }

    if (s_gen || s_all) {
        char fa[4200], fb[4200];
        snprintf(fa, sizeof fa, "%s/%d-%s-a#%d", wd, order, gen_out, job_id);
        snprintf(fb, sizeof fb, "%s/%d-%s-b#%d", wd, order, gen_out, job_id);
        gpo_gen_stats st;
        int rc = gpo_generate(order, compress[0], paf, fa, fb, job_id, job_count, &st);
        if (rc) return 1;
        printf("Orderly Count: %lld\nPassed PSD filter: %lld\n", (long long)st.necklaces,
               (long long)(st.written_a + st.written_b));
    }
    if (s_sort || s_all) {
        const char** ia = (const char**)calloc((size_t)job_count, sizeof(char*));
        const char** ib = (const char**)calloc((size_t)job_count, sizeof(char*));
        for (int j = 0; j < job_count; ++j) {
            char* x = (char*)malloc(4200);
            char* y = (char*)malloc(4200);
            snprintf(x, 4200, "%s/%d-%s-a#%d", wd, order, sort_in, j);
            snprintf(y, 4200, "%s/%d-%s-b#%d", wd, order, sort_in, j);
            ia[j] = x;
            ib[j] = y;
        }
        char oa[4200], ob[4200];
        snprintf(oa, sizeof oa, "%s/%d-%s-a", wd, order, sort_out);
        snprintf(ob, sizeof ob, "%s/%d-%s-b", wd, order, sort_out);
        if (gpo_sort(ia, job_count, oa)) return 1;
        if (gpo_sort(ib, job_count, ob)) return 1;
    }
    if (s_match || s_all) {
        char ia[4200], ib[4200], o[4200];
        snprintf(ia, sizeof ia, "%s/%d-%s-a", wd, order, match_in);
        snprintf(ib, sizeof ib, "%s/%d-%s-b", wd, order, match_in);
        snprintf(o, sizeof o, "%s/%d-%s-%d", wd, order, match_out, compress[0]);
        int64_t np = 0;
        if (gpo_match(order, compress[0], paf, ia, ib, o, match_append, &np)) return 1;
    }
    if (s_unc || s_all) {
        for (int i = 0; i + 1 < ncompress; ++i) {
            const char* pre = i == 0 ? unc_in : unc_out;
            char in[4200], out[4200];
            snprintf(in, sizeof in, "%s/%d-%s-%d", wd, order, pre, compress[i]);
            snprintf(out, sizeof out, "%s/%d-%s-%d", wd, order, unc_out, compress[i + 1]);
            int rc = gpo_uncompress(order, compress[i], compress[i + 1], paf, in, out, wd, unc_prefix);
            if (rc == 2) return 1;
        }
    }
    if (s_filter || s_all) {
        char in[4200], out[4200];
        snprintf(in, sizeof in, "%s/%d-pairs-%d", wd, order, compress[ncompress - 1]);
        snprintf(out, sizeof out, "%s/%d-unique", wd, order);
        if (gpo_equiv_filter(order, compress[ncompress - 1], in, out)) return 1;
    }
    return 0;
}
