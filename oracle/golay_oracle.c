/*
 * golay_oracle.c -- CPU restatement of GolayPair's search path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline).  The
 * product never links or calls this file.  Each function names the
 * reference file:line it follows (paths inside the GolayPair project).
 *
 * Parity pin: the test suite checks this restatement against golden files
 * produced by the reference's own sources (compiled by oracle/build_ref.sh
 * against stand-in FFTW/Boost headers).  Real FFTW is not available, so the
 * last-ulp behaviour of FFTW's FFT itself is unpinned.
 */
#define _GNU_SOURCE
#include "golay_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------ */
/* small tables                                                        */
/* ------------------------------------------------------------------ */

/* src/utils/golay.cpp:60-75: even c -> {-c..c step 2}; odd c -> +-{1..c step 2} */
int gpo_alphabet(int compress, int* out) {
    int n = 0;
    if (compress % 2 == 0) {
        for (int v = -compress; v <= compress; v += 2) out[n++] = v;
    } else {
        for (int v = -compress; v <= -1; v += 2) out[n++] = v;
        for (int v = 1; v <= compress; v += 2) out[n++] = v;
    }
    return n;
}

/* src/utils/decomps.cpp:6-17 */
int gpo_decomps(int k, int* xs, int* ys, int max_out) {
    int n = 0;
    for (int x = 0; x <= k; ++x)
        for (int y = x; y <= k; ++y)
            if (x * x + y * y == k) {
                if (n < max_out) { xs[n] = x; ys[n] = y; }
                ++n;
            }
    return n;
}

/* src/core/generate/generate_hybrid.cpp:45-47 */
int gpo_sum_constant(int order, int paf) { return order * 2 + (order - 1) * paf; }

static int gcd_i(int a, int b) {
    while (b) { int t = a % b; a = b; b = t; }
    return a < 0 ? -a : a;
}

/* src/utils/lyndon.cpp:38-45: (1/L) sum_{i=1..L} k^gcd(i,L) */
int64_t gpo_necklace_count(int L, int k) {
    u128 sum = 0;
    for (int i = 1; i <= L; ++i) {
        int e = gcd_i(i, L);
        u128 p = 1;
        for (int t = 0; t < e; ++t) {
            p *= (u128)k;
            if (p > ((u128)1 << 100)) return INT64_MAX;
        }
        sum += p;
    }
    u128 r = sum / (u128)L;
    return r > (u128)INT64_MAX ? INT64_MAX : (int64_t)r;
}

/* ------------------------------------------------------------------ */
/* PSD                                                                 */
/* ------------------------------------------------------------------ */

typedef struct {
    int L;
    double* cs;
    double* sn;
} twiddles;

static twiddles g_tw[GPO_MAX_LEN + 1];
static pthread_mutex_t g_tw_mu = PTHREAD_MUTEX_INITIALIZER;

static const twiddles* get_twiddles(int L) {
    twiddles* t = &g_tw[L];
    pthread_mutex_lock(&g_tw_mu);
    if (!t->cs) {
        double* cs = (double*)malloc(sizeof(double) * (size_t)L);
        double* sn = (double*)malloc(sizeof(double) * (size_t)L);
        const double two_pi = 6.283185307179586476925286766559;
        for (int m = 0; m < L; ++m) {
            cs[m] = cos(two_pi * (double)m / (double)L);
            sn[m] = sin(two_pi * (double)m / (double)L);
        }
        t->sn = sn;
        t->L = L;
        __atomic_store_n(&t->cs, cs, __ATOMIC_RELEASE);
    }
    pthread_mutex_unlock(&g_tw_mu);
    return t;
}

/* src/utils/fourier.cpp:25-43: FFTW c2c forward of the real sequence,
 * psd[k] = re^2 + im^2.  Restated as a direct DFT whose twiddle for (j,k)
 * is exp(-2 pi i ((j k) mod L) / L). */
static void psd_tw(const int* seq, int L, const twiddles* tw, double* psd) {
    for (int k = 0; k < L; ++k) {
        double re = 0.0, im = 0.0;
        int m = 0;
        for (int j = 0; j < L; ++j) {
            re += (double)seq[j] * tw->cs[m];
            im -= (double)seq[j] * tw->sn[m];
            m += k;
            if (m >= L) m -= L;
        }
        psd[k] = re * re + im * im;
    }
}

void gpo_psd(const int* seq, int L, double* psd) { psd_tw(seq, L, get_twiddles(L), psd); }

/* src/utils/fourier.cpp:45-52: reject if psd[k] > 2n - paf + 0.001 for any
 * k = 1..L/2 */
int gpo_psd_filter(const double* psd, int L, int order, int paf) {
    for (int i = 1; i <= L / 2; ++i)
        if (psd[i] > 2 * order - paf + 0.001) return 0;
    return 1;
}

/* ------------------------------------------------------------------ */
/* hash set of int16 vectors (used for generator closures)             */
/* ------------------------------------------------------------------ */

typedef struct {
    int width;        /* int16 entries per item */
    int64_t cap;      /* slots (power of two) */
    int64_t count;
    int16_t* items;   /* count x width, insertion order */
    int64_t items_cap;
    int64_t* slots;   /* index into items, -1 = empty */
} vecset;

static uint64_t hash_vec(const int16_t* v, int w) {
    uint64_t h = 1469598103934665603ULL;
    for (int i = 0; i < w; ++i) {
        h ^= (uint16_t)v[i];
        h *= 1099511628211ULL;
    }
    return h ^ (h >> 29);
}

static void vecset_init(vecset* s, int width, int64_t cap_hint) {
    s->width = width;
    s->cap = 64;
    while (s->cap < 2 * cap_hint) s->cap <<= 1;
    s->count = 0;
    s->items_cap = cap_hint > 16 ? cap_hint : 16;
    s->items = (int16_t*)malloc(sizeof(int16_t) * (size_t)s->items_cap * (size_t)width);
    s->slots = (int64_t*)malloc(sizeof(int64_t) * (size_t)s->cap);
    memset(s->slots, 0xff, sizeof(int64_t) * (size_t)s->cap);
}

static void vecset_free(vecset* s) {
    free(s->items);
    free(s->slots);
    memset(s, 0, sizeof(*s));
}

static void vecset_clear(vecset* s) {
    s->count = 0;
    memset(s->slots, 0xff, sizeof(int64_t) * (size_t)s->cap);
}

static int64_t vecset_find(const vecset* s, const int16_t* v) {
    uint64_t h = hash_vec(v, s->width);
    int64_t mask = s->cap - 1;
    for (int64_t p = (int64_t)(h & (uint64_t)mask);; p = (p + 1) & mask) {
        int64_t idx = s->slots[p];
        if (idx < 0) return -1;
        if (memcmp(s->items + idx * s->width, v, sizeof(int16_t) * (size_t)s->width) == 0) return idx;
    }
}

static void vecset_grow(vecset* s) {
    s->cap <<= 1;
    free(s->slots);
    s->slots = (int64_t*)malloc(sizeof(int64_t) * (size_t)s->cap);
    memset(s->slots, 0xff, sizeof(int64_t) * (size_t)s->cap);
    int64_t mask = s->cap - 1;
    for (int64_t i = 0; i < s->count; ++i) {
        uint64_t h = hash_vec(s->items + i * s->width, s->width);
        int64_t p = (int64_t)(h & (uint64_t)mask);
        while (s->slots[p] >= 0) p = (p + 1) & mask;
        s->slots[p] = i;
    }
}

/* returns 1 if inserted, 0 if present */
static int vecset_insert(vecset* s, const int16_t* v) {
    if (vecset_find(s, v) >= 0) return 0;
    if (2 * (s->count + 1) > s->cap) vecset_grow(s);
    if (s->count == s->items_cap) {
        s->items_cap *= 2;
        s->items = (int16_t*)realloc(s->items, sizeof(int16_t) * (size_t)s->items_cap * (size_t)s->width);
    }
    memcpy(s->items + s->count * s->width, v, sizeof(int16_t) * (size_t)s->width);
    uint64_t h = hash_vec(v, s->width);
    int64_t mask = s->cap - 1;
    int64_t p = (int64_t)(h & (uint64_t)mask);
    while (s->slots[p] >= 0) p = (p + 1) & mask;
    s->slots[p] = s->count++;
    return 1;
}

/* ------------------------------------------------------------------ */
/* orderly canonical check                                             */
/* ------------------------------------------------------------------ */

/* src/utils/coprimes.cpp:12-33: 1 <= i < k with gcd(i,k) == 1 */
static int coprimes(int k, int* out) {
    int n = 0;
    for (int i = 1; i < k; ++i)
        if (gcd_i(i, k) == 1) out[n++] = i;
    return n;
}

/* src/utils/orderly_equivalence.cpp:17-51: closure of the identity
 * permutation under decimation (flag 0 only), rotation and reversal. */
static void build_orderly_generators(int L, int flag, vecset* out) {
    vecset_init(out, L, (int64_t)L * L);
    int16_t* cur = (int16_t*)malloc(sizeof(int16_t) * (size_t)L);
    int16_t* nxt = (int16_t*)malloc(sizeof(int16_t) * (size_t)L);
    int* cp = (int*)malloc(sizeof(int) * (size_t)(L + 1));
    int ncp = coprimes(L, cp);
    for (int i = 0; i < L; ++i) cur[i] = (int16_t)i;
    vecset_insert(out, cur);
    /* breadth-first: every item is expanded by every operation once */
    for (int64_t at = 0; at < out->count; ++at) {
        memcpy(cur, out->items + at * L, sizeof(int16_t) * (size_t)L);
        if (flag == 0) {
            for (int c = 0; c < ncp; ++c) {
                for (int i = 0; i < L; ++i) nxt[i] = cur[(int)(((long long)i * cp[c]) % L)];
                vecset_insert(out, nxt);
                memcpy(cur, out->items + at * L, sizeof(int16_t) * (size_t)L);
            }
        }
        for (int r = 1; r <= L; ++r) {
            for (int i = 0; i < L; ++i) nxt[i] = cur[(i + r) % L];
            vecset_insert(out, nxt);
            memcpy(cur, out->items + at * L, sizeof(int16_t) * (size_t)L);
        }
        for (int i = 0; i < L; ++i) nxt[i] = cur[L - 1 - i];
        vecset_insert(out, nxt);
    }
    free(cur);
    free(nxt);
    free(cp);
}

static vecset g_orderly[2][GPO_MAX_LEN + 1];

static const vecset* orderly_generators(int L, int flag) {
    vecset* s = &g_orderly[flag ? 1 : 0][L];
    if (!s->items) build_orderly_generators(L, flag ? 1 : 0, s);
    return s;
}

int gpo_orderly_generators(int L, int flag, int* out, int max_count) {
    const vecset* s = orderly_generators(L, flag);
    if (out) {
        int64_t n = s->count < max_count ? s->count : max_count;
        for (int64_t i = 0; i < n * L; ++i) out[i] = s->items[i];
    }
    return (int)s->count;
}

/* src/utils/orderly_equivalence.cpp:53-68: canonical iff seq <= seq o g for
 * every generator g (lexicographic). */
int gpo_is_canonical(const int* seq, int L, int flag) {
    const vecset* s = orderly_generators(L, flag);
    for (int64_t g = 0; g < s->count; ++g) {
        const int16_t* p = s->items + g * L;
        for (int i = 0; i < L; ++i) {
            int v = seq[p[i]];
            if (v < seq[i]) return 0;
            if (v > seq[i]) break;
        }
    }
    return 1;
}

/* ------------------------------------------------------------------ */
/* PAF check                                                           */
/* ------------------------------------------------------------------ */

static int paf(const int* s, int L, int shift) {
    int r = 0;
    for (int i = 0; i < L; ++i) r += s[i] * s[(i + shift) % L];
    return r;
}

/* src/utils/golay.cpp:27-44 */
int gpo_check_if_pair(const int* a, const int* b, int L, int pafc, int compress) {
    for (int s = 1; s <= L / 2; ++s)
        if (paf(a, L, s) + paf(b, L, s) != pafc * compress) return 0;
    return 1;
}

/* ------------------------------------------------------------------ */
/* text formatting                                                     */
/* ------------------------------------------------------------------ */

static int put_int(char* p, int v) {
    char tmp[16];
    int n = 0, neg = v < 0;
    unsigned u = neg ? (unsigned)(-(long long)v) : (unsigned)v;
    do { tmp[n++] = (char)('0' + u % 10); u /= 10; } while (u);
    int k = 0;
    if (neg) p[k++] = '-';
    while (n) p[k++] = tmp[--n];
    return k;
}

/* src/utils/io.cpp:14-36: "PSD" + rint(psd[1..L-1]) (or bound - rint) +
 * " " + each entry followed by " " + "\n" */
int gpo_format_candidate(char* buf, const int* seq, const double* psd, int L, int invert, int bound) {
    int n = 0;
    buf[n++] = 'P'; buf[n++] = 'S'; buf[n++] = 'D';
    for (int i = 1; i < L; ++i) {
        int r = (int)rint(psd[i]);
        n += put_int(buf + n, invert ? bound - r : r);
    }
    buf[n++] = ' ';
    for (int i = 0; i < L; ++i) {
        n += put_int(buf + n, seq[i]);
        buf[n++] = ' ';
    }
    buf[n++] = '\n';
    return n;
}

/* ------------------------------------------------------------------ */
/* generation                                                          */
/* ------------------------------------------------------------------ */

typedef struct {
    int order, L, paf, bound;
    int ndec;
    int dx[64], dy[64];
    FILE* fa;
    FILE* fb;
    int* seq;
    double* psd;
    char* line;
    const twiddles* tw;
    gpo_gen_stats st;
    /* rank window (window mode) */
    int windowed;
    u128 lo, hi;
    int k;          /* alphabet size */
    int alpha[64];
} gen_ctx;

static int rowsum(const int* s, int L) {
    int r = 0;
    for (int i = 0; i < L; ++i) r += s[i];
    return r;
}

/* generate_hybrid.cpp:136-156: per-necklace callback */
static void gen_callback(gen_ctx* g) {
    const int L = g->L;
    g->st.necklaces++;
    int rs = rowsum(g->seq, L);
    for (int d = 0; d < g->ndec; ++d) {
        if (rs == g->dx[d]) {
            gpo_psd(g->seq, L, g->psd);
            g->st.psd_evals++;
            if (gpo_psd_filter(g->psd, L, g->order, g->paf)) {
                g->st.psd_pass++;
                if (gpo_is_canonical(g->seq, L, 0)) {
                    int n = gpo_format_candidate(g->line, g->seq, g->psd, L, 0, g->bound);
                    fwrite(g->line, 1, (size_t)n, g->fa);
                    g->st.written_a++;
                }
            }
        }
        if (rs == g->dy[d]) {
            gpo_psd(g->seq, L, g->psd);
            g->st.psd_evals++;
            if (gpo_psd_filter(g->psd, L, g->order, g->paf)) {
                g->st.psd_pass++;
                if (gpo_is_canonical(g->seq, L, 1)) {
                    int n = gpo_format_candidate(g->line, g->seq, g->psd, L, 1, g->bound);
                    fwrite(g->line, 1, (size_t)n, g->fb);
                    g->st.written_b++;
                }
            }
        }
    }
}

static u128 rank_prefix(const gen_ctx* g, int upto) {
    u128 r = 0;
    for (int i = 0; i < upto; ++i) {
        int c = 0;
        while (g->alpha[c] != g->seq[i]) ++c;
        r = r * (u128)g->k + (u128)c;
    }
    return r;
}

/* In window mode, a subtree whose words all lie outside [lo, hi) is skipped */
static int subtree_outside(const gen_ctx* g, int depth) {
    if (!g->windowed) return 0;
    u128 span = 1;
    for (int i = depth; i < g->L; ++i) span *= (u128)g->k;
    u128 first = rank_prefix(g, depth) * span;
    u128 last = first + span; /* exclusive */
    return last <= g->lo || first >= g->hi;
}

/* src/utils/lyndon.cpp:47-85: recursive FKM over the sorted alphabet; the
 * callback sees every prenecklace of full length with its period. */
static void fkm(gen_ctx* g, int index, int period, int full_len, void (*cb)(gen_ctx*, int)) {
    if (subtree_outside(g, index)) return;
    if (index == full_len) {
        cb(g, period);
        return;
    }
    g->seq[index] = g->seq[index - period];
    fkm(g, index + 1, period, full_len, cb);
    int c = 0;
    while (g->alpha[c] != g->seq[index - period]) ++c;
    for (++c; c < g->k; ++c) {
        g->seq[index] = g->alpha[c];
        fkm(g, index + 1, index + 1, full_len, cb);
    }
}

static void necklace_cb(gen_ctx* g, int period) {
    if (g->L % period == 0) gen_callback(g);
}

/* prefix collection for the job split (lyndon.cpp:93-106) */
typedef struct {
    int len;
    int64_t count;
    int proc_id, proc_num;
    int* items;   /* prefixes (len ints each) */
    int* periods;
    int64_t n, cap;
} prefix_list;

static prefix_list* g_plist;

static void prefix_cb(gen_ctx* g, int period) {
    prefix_list* pl = g_plist;
    pl->count++;
    if (pl->count % pl->proc_num == pl->proc_id) {
        if (pl->n == pl->cap) {
            pl->cap = pl->cap ? pl->cap * 2 : 1024;
            pl->items = (int*)realloc(pl->items, sizeof(int) * (size_t)pl->cap * (size_t)pl->len);
            pl->periods = (int*)realloc(pl->periods, sizeof(int) * (size_t)pl->cap);
        }
        memcpy(pl->items + pl->n * pl->len, g->seq, sizeof(int) * (size_t)pl->len);
        pl->periods[pl->n] = period;
        pl->n++;
    }
}

static int gen_setup(gen_ctx* g, int order, int compress, int pafc, const char* path_a, const char* path_b) {
    memset(g, 0, sizeof(*g));
    g->order = order;
    g->L = order / compress;
    g->paf = pafc;
    g->bound = order * 2 - pafc;
    g->ndec = gpo_decomps(gpo_sum_constant(order, pafc), g->dx, g->dy, 64);
    if (g->ndec == 0) return 1;
    g->k = gpo_alphabet(compress, g->alpha);
    g->fa = fopen(path_a, "w");
    g->fb = fopen(path_b, "w");
    if (!g->fa || !g->fb) {
        if (g->fa) fclose(g->fa);
        if (g->fb) fclose(g->fb);
        return 2;
    }
    g->seq = (int*)calloc((size_t)g->L + 1, sizeof(int));
    g->psd = (double*)calloc((size_t)g->L + 1, sizeof(double));
    g->line = (char*)malloc((size_t)g->L * 32 + 64);
    g->tw = get_twiddles(g->L);
    return 0;
}

static void gen_teardown(gen_ctx* g, gpo_gen_stats* stats) {
    fclose(g->fa);
    fclose(g->fb);
    free(g->seq);
    free(g->psd);
    free(g->line);
    if (stats) *stats = g->st;
}

/* src/core/generate/generate_hybrid.cpp:107-163 and
 * src/utils/lyndon.cpp:87-121 */
int gpo_generate(int order, int compress, int pafc, const char* path_a, const char* path_b,
                 int proc_id, int proc_num, gpo_gen_stats* stats) {
    gen_ctx g;
    int rc = gen_setup(&g, order, compress, pafc, path_a, path_b);
    if (rc) return rc;
    const int L = g.L;
    int i = 1;
    for (; i <= L; ++i)
        if (gpo_necklace_count(i, g.k) >= (int64_t)proc_num * 10000) break;
    if (proc_num > 1 && i < L) {
        prefix_list pl;
        memset(&pl, 0, sizeof(pl));
        pl.len = i;
        pl.proc_id = proc_id;
        pl.proc_num = proc_num;
        g_plist = &pl;
        for (int c = 0; c < g.k; ++c) {
            g.seq[0] = g.alpha[c];
            fkm(&g, 1, 1, i, prefix_cb);
        }
        g_plist = NULL;
        for (int64_t w = 0; w < pl.n; ++w) {
            memcpy(g.seq, pl.items + w * i, sizeof(int) * (size_t)i);
            fkm(&g, i, pl.periods[w], L, necklace_cb);
        }
        free(pl.items);
        free(pl.periods);
    } else {
        for (int c = 0; c < g.k; ++c) {
            g.seq[0] = g.alpha[c];
            fkm(&g, 1, 1, L, necklace_cb);
        }
    }
    gen_teardown(&g, stats);
    return 0;
}

int gpo_generate_window(int order, int compress, int pafc, const char* path_a, const char* path_b,
                        uint64_t lo_hi, uint64_t lo_lo, uint64_t hi_hi, uint64_t hi_lo, gpo_gen_stats* stats) {
    gen_ctx g;
    int rc = gen_setup(&g, order, compress, pafc, path_a, path_b);
    if (rc) return rc;
    g.windowed = 1;
    g.lo = ((u128)lo_hi << 64) | lo_lo;
    g.hi = ((u128)hi_hi << 64) | hi_lo;
    for (int c = 0; c < g.k; ++c) {
        g.seq[0] = g.alpha[c];
        fkm(&g, 1, 1, g.L, necklace_cb);
    }
    gen_teardown(&g, stats);
    return 0;
}

/* ------------------------------------------------------------------ */
/* sort | uniq                                                         */
/* ------------------------------------------------------------------ */

typedef struct {
    char* p;
    size_t n; /* without newline */
} line_ref;

static int cmp_lines(const void* x, const void* y) {
    const line_ref* a = (const line_ref*)x;
    const line_ref* b = (const line_ref*)y;
    size_t m = a->n < b->n ? a->n : b->n;
    int c = memcmp(a->p, b->p, m);
    if (c) return c;
    return (a->n > b->n) - (a->n < b->n);
}

static char* slurp(const char* path, size_t* len) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    char* buf = (char*)malloc((size_t)sz + 2);
    size_t got = fread(buf, 1, (size_t)sz, f);
    fclose(f);
    buf[got] = 0;
    *len = got;
    return buf;
}

/* src/core/sort/sort.cpp:7-22: `sort -S 2G -T dir files | uniq > out`,
 * byte order (LC_ALL=C) */
int gpo_sort(const char** in_paths, int n_in, const char* out_path) {
    char** bufs = (char**)calloc((size_t)n_in, sizeof(char*));
    line_ref* lines = NULL;
    size_t nl = 0, cap = 0;
    for (int f = 0; f < n_in; ++f) {
        size_t len = 0;
        bufs[f] = slurp(in_paths[f], &len);
        if (!bufs[f]) {
            for (int g = 0; g < f; ++g) free(bufs[g]);
            free(bufs);
            free(lines);
            return 1; /* sort fails on a missing file */
        }
        char* p = bufs[f];
        char* end = p + len;
        while (p < end) {
            char* nlp = (char*)memchr(p, '\n', (size_t)(end - p));
            size_t n = nlp ? (size_t)(nlp - p) : (size_t)(end - p);
            if (nl == cap) {
                cap = cap ? cap * 2 : 4096;
                lines = (line_ref*)realloc(lines, sizeof(line_ref) * cap);
            }
            lines[nl].p = p;
            lines[nl].n = n;
            nl++;
            p += n + 1;
        }
    }
    qsort(lines, nl, sizeof(line_ref), cmp_lines);
    FILE* out = fopen(out_path, "w");
    if (!out) return 1;
    for (size_t i = 0; i < nl; ++i) {
        if (i > 0 && cmp_lines(&lines[i], &lines[i - 1]) == 0) continue;
        fwrite(lines[i].p, 1, lines[i].n, out);
        fputc('\n', out);
    }
    fclose(out);
    for (int f = 0; f < n_in; ++f) free(bufs[f]);
    free(bufs);
    free(lines);
    return 0;
}

/* ------------------------------------------------------------------ */
/* match                                                               */
/* ------------------------------------------------------------------ */

typedef struct {
    char* tok;  /* NUL-terminated first token */
    int* seq;   /* L ints */
} cand_line;

static cand_line* parse_candidates(char* buf, size_t len, int L, size_t* count) {
    cand_line* out = NULL;
    size_t n = 0, cap = 0;
    char* p = buf;
    char* end = buf + len;
    while (p < end) {
        char* nlp = (char*)memchr(p, '\n', (size_t)(end - p));
        if (!nlp) nlp = end;
        *nlp = 0;
        while (*p == ' ') ++p;
        if (*p) {
            if (n == cap) {
                cap = cap ? cap * 2 : 1024;
                out = (cand_line*)realloc(out, sizeof(cand_line) * cap);
            }
            char* sp = strchr(p, ' ');
            if (sp) *sp = 0;
            out[n].tok = p;
            out[n].seq = (int*)malloc(sizeof(int) * (size_t)L);
            char* q = sp ? sp + 1 : nlp;
            for (int i = 0; i < L; ++i) {
                char* e;
                out[n].seq[i] = (int)strtol(q, &e, 10);
                q = e;
            }
            n++;
        }
        p = nlp + 1;
    }
    *count = n;
    return out;
}

static void write_pair(FILE* f, const int* a, const int* b, int L) {
    for (int i = 0; i < L; ++i) fprintf(f, "%d ", a[i]);
    fputc(' ', f);
    for (int i = 0; i < L; ++i) fprintf(f, "%d ", b[i]);
    fputc('\n', f);
}

/* src/core/match/match_pairs.cpp:15-121: merge-join on the first token,
 * cross product of equal-token groups, exact PAF check (golay.cpp:35-44) */
static int match_to(FILE* out, int order, int compress, int pafc, const char* path_a, const char* path_b,
                    int64_t* n_pairs) {
    const int L = order / compress;
    size_t la = 0, lb = 0;
    char* ba = slurp(path_a, &la);
    char* bb = slurp(path_b, &lb);
    if (!ba || !bb || la == 0 || lb == 0) {
        free(ba);
        free(bb);
        return 1;
    }
    size_t na = 0, nb = 0;
    cand_line* A = parse_candidates(ba, la, L, &na);
    cand_line* B = parse_candidates(bb, lb, L, &nb);
    size_t i = 0, j = 0;
    int64_t np = 0;
    while (i < na && j < nb) {
        int c = strcmp(A[i].tok, B[j].tok);
        if (c == 0) {
            size_t i2 = i, j2 = j;
            while (i2 < na && strcmp(A[i2].tok, A[i].tok) == 0) ++i2;
            while (j2 < nb && strcmp(B[j2].tok, B[j].tok) == 0) ++j2;
            for (size_t x = i; x < i2; ++x)
                for (size_t y = j; y < j2; ++y)
                    if (gpo_check_if_pair(A[x].seq, B[y].seq, L, pafc, compress)) {
                        write_pair(out, A[x].seq, B[y].seq, L);
                        ++np;
                    }
            i = i2;
            j = j2;
        } else if (c < 0) {
            ++i;
        } else {
            ++j;
        }
    }
    for (size_t x = 0; x < na; ++x) free(A[x].seq);
    for (size_t y = 0; y < nb; ++y) free(B[y].seq);
    free(A);
    free(B);
    free(ba);
    free(bb);
    if (n_pairs) *n_pairs += np;
    return 0;
}

int gpo_match(int order, int compress, int pafc, const char* path_a, const char* path_b,
              const char* out_path, int append, int64_t* n_pairs) {
    FILE* out = fopen(out_path, append ? "a" : "w");
    if (!out) return 1;
    if (n_pairs) *n_pairs = 0;
    int rc = match_to(out, order, compress, pafc, path_a, path_b, n_pairs);
    fclose(out);
    return rc;
}

/* ------------------------------------------------------------------ */
/* uncompression                                                       */
/* ------------------------------------------------------------------ */

/* src/utils/array.cpp:131-160: non-decreasing sequences of length len over
 * the sorted alphabet, in lexicographic order.  Returns count. */
static int combinations(int len, const int* alpha, int k, int* out) {
    int n = 0;
    int idx[64];
    for (int i = 0; i < len; ++i) idx[i] = 0;
    for (;;) {
        for (int i = 0; i < len; ++i) out[n * len + i] = alpha[idx[i]];
        ++n;
        int p = len - 1;
        while (p >= 0 && idx[p] == k - 1) --p;
        if (p < 0) break;
        idx[p]++;
        for (int q = p + 1; q < len; ++q) idx[q] = idx[p];
    }
    return n;
}

static int next_permutation_i(int* a, int n) {
    int i = n - 2;
    while (i >= 0 && a[i] >= a[i + 1]) --i;
    if (i < 0) {
        for (int l = 0, r = n - 1; l < r; ++l, --r) { int t = a[l]; a[l] = a[r]; a[r] = t; }
        return 0;
    }
    int j = n - 1;
    while (a[j] <= a[i]) --j;
    int t = a[i]; a[i] = a[j]; a[j] = t;
    for (int l = i + 1, r = n - 1; l < r; ++l, --r) { t = a[l]; a[l] = a[r]; a[r] = t; }
    return 1;
}

static int lex_less(const int* a, const int* b, int n) {
    for (int i = 0; i < n; ++i) {
        if (a[i] != b[i]) return a[i] < b[i];
    }
    return 0;
}

typedef struct {
    int r;          /* parts per entry (compress / new_compress) */
    int nletters;
    int letters[64];
    int count[64];  /* partitions per letter */
    int* parts[64]; /* count x r ints, in reference order */
} partition_table;

/* uncompression.cpp:88-111 */
static void build_partitions(int compress, int new_compress, partition_table* t) {
    int alpha[64], nalpha[64];
    int k = gpo_alphabet(compress, alpha);
    int nk = gpo_alphabet(new_compress, nalpha);
    int r = compress / new_compress;
    t->r = r;
    t->nletters = k;
    int maxc = 1;
    for (int i = 0; i < r; ++i) maxc *= nk;
    int* combos = (int*)malloc(sizeof(int) * (size_t)maxc * (size_t)r);
    int nc = combinations(r, nalpha, nk, combos);
    int* perm = (int*)malloc(sizeof(int) * (size_t)r);
    for (int li = 0; li < k; ++li) {
        int letter = alpha[li];
        t->letters[li] = letter;
        t->count[li] = 0;
        t->parts[li] = (int*)malloc(sizeof(int) * (size_t)maxc * (size_t)r);
        for (int c = 0; c < nc; ++c) {
            int s = 0;
            for (int i = 0; i < r; ++i) s += combos[c * r + i];
            if (s != letter) continue;
            memcpy(perm, combos + c * r, sizeof(int) * (size_t)r);
            do {
                memcpy(t->parts[li] + t->count[li] * r, perm, sizeof(int) * (size_t)r);
                t->count[li]++;
            } while (next_permutation_i(perm, r));
        }
    }
    free(combos);
    free(perm);
}

static void free_partitions(partition_table* t) {
    for (int i = 0; i < t->nletters; ++i) free(t->parts[i]);
}

static int letter_index(const partition_table* t, int v) {
    for (int i = 0; i < t->nletters; ++i)
        if (t->letters[i] == v) return i;
    return -1;
}

/* src/utils/equivalence.cpp:26-44 then *set.begin(): lexicographic minimum
 * of the part under rotations and reversal */
static void min_rot_rev(const int* p, int r, int* out) {
    int cand[64];
    memcpy(out, p, sizeof(int) * (size_t)r);
    for (int rev = 0; rev < 2; ++rev) {
        for (int s = 0; s < r; ++s) {
            for (int i = 0; i < r; ++i) {
                int src = (i + s) % r;
                cand[i] = rev ? p[r - 1 - src] : p[src];
            }
            if (lex_less(cand, out, r)) memcpy(out, cand, sizeof(int) * (size_t)r);
        }
    }
}

typedef struct {
    int L, Lnew, r, order, paf, bound, seqflag;
    int* choice_count; /* per position */
    int** choices;     /* per position: count x r */
    int* seq;
    double* psd;
    char* line;
    FILE* out;
    int64_t leaves, written;
} unc_ctx;

static void unc_dfs(unc_ctx* u, int pos) {
    if (pos == u->L) {
        u->leaves++;
        gpo_psd(u->seq, u->Lnew, u->psd);
        if (gpo_psd_filter(u->psd, u->Lnew, u->order, u->paf)) {
            int n = gpo_format_candidate(u->line, u->seq, u->psd, u->Lnew, u->seqflag ? 0 : 1, u->bound);
            fwrite(u->line, 1, (size_t)n, u->out);
            u->written++;
        }
        return;
    }
    for (int c = 0; c < u->choice_count[pos]; ++c) {
        const int* p = u->choices[pos] + c * u->r;
        for (int i = 0; i < u->r; ++i) u->seq[pos + u->L * i] = p[i];
        unc_dfs(u, pos + 1);
    }
}

/* src/core/uncompression/uncompression.cpp:81-210 with PROC_ID=0,
 * PROC_NUM=1 (the only values uncompress_pipeline passes, :62-66) */
int gpo_uncompress_one(int* orig, int L, int compress, int new_compress, int pafc, int seqflag,
                       const char* path, int64_t* n_leaves, int64_t* n_written) {
    const int order = L * compress;
    partition_table t;
    build_partitions(compress, new_compress, &t);
    const int r = t.r;
    /* uncompression.cpp:113-126: first distinct element (ascending) with the
     * most partitions */
    size_t best_n = 0;
    int best = orig[0];
    for (int li = 0; li < t.nletters; ++li) {
        int present = 0;
        for (int i = 0; i < L; ++i) present |= orig[i] == t.letters[li];
        if (!present) continue;
        if ((size_t)t.count[li] > best_n) {
            best_n = (size_t)t.count[li];
            best = t.letters[li];
        }
    }
    /* uncompression.cpp:127-131: rotate left by i whenever orig[i] == best,
     * checking the already-rotated sequence each time */
    int* tmp = (int*)malloc(sizeof(int) * (size_t)L);
    for (int i = 0; i < L; ++i) {
        if (orig[i] == best) {
            for (int j = 0; j < L; ++j) tmp[j] = orig[(j + i) % L];
            memcpy(orig, tmp, sizeof(int) * (size_t)L);
        }
    }
    free(tmp);
    /* uncompression.cpp:133-142: reduced choices for position 0 (sorted set) */
    int li0 = letter_index(&t, orig[0]);
    int n0 = t.count[li0];
    int* first = (int*)malloc(sizeof(int) * (size_t)(n0 > 0 ? n0 : 1) * (size_t)r);
    int nfirst = 0;
    int mn[64];
    for (int c = 0; c < n0; ++c) {
        min_rot_rev(t.parts[li0] + c * r, r, mn);
        /* insert into sorted unique list */
        int pos = 0;
        while (pos < nfirst && lex_less(first + pos * r, mn, r)) ++pos;
        if (pos < nfirst && memcmp(first + pos * r, mn, sizeof(int) * (size_t)r) == 0) continue;
        memmove(first + (pos + 1) * r, first + pos * r, sizeof(int) * (size_t)(nfirst - pos) * (size_t)r);
        memcpy(first + pos * r, mn, sizeof(int) * (size_t)r);
        nfirst++;
    }
    unc_ctx u;
    memset(&u, 0, sizeof(u));
    u.L = L;
    u.r = r;
    u.Lnew = L * r;
    u.order = order;
    u.paf = pafc;
    u.bound = order * 2 - pafc;
    u.seqflag = seqflag;
    u.choice_count = (int*)malloc(sizeof(int) * (size_t)L);
    u.choices = (int**)malloc(sizeof(int*) * (size_t)L);
    u.choice_count[0] = nfirst;
    u.choices[0] = first;
    for (int i = 1; i < L; ++i) {
        int li = letter_index(&t, orig[i]);
        u.choice_count[i] = li >= 0 ? t.count[li] : 0;
        u.choices[i] = li >= 0 ? t.parts[li] : NULL;
    }
    u.seq = (int*)calloc((size_t)u.Lnew, sizeof(int));
    u.psd = (double*)calloc((size_t)u.Lnew, sizeof(double));
    u.line = (char*)malloc((size_t)u.Lnew * 32 + 64);
    u.out = fopen(path, "w");
    if (!u.out) return 1;
    unc_dfs(&u, 0);
    fclose(u.out);
    if (n_leaves) *n_leaves = u.leaves;
    if (n_written) *n_written = u.written;
    free(u.seq);
    free(u.psd);
    free(u.line);
    free(u.choice_count);
    free(u.choices);
    free(first);
    free_partitions(&t);
    return 0;
}

/* src/core/uncompression/uncompression.cpp:32-79 (CPU device) */
int gpo_uncompress(int order, int compress, int new_compress, int pafc, const char* in_pairs,
                   const char* out_pairs, const char* work_dir, const char* prefix) {
    if (compress <= 1) return 0;
    const int L = order / compress;
    char fa[4096], fb[4096], fas[4200], fbs[4200];
    snprintf(fa, sizeof fa, "%s/%suncompress_tmp_a", work_dir, prefix ? prefix : "");
    snprintf(fb, sizeof fb, "%s/%suncompress_tmp_b", work_dir, prefix ? prefix : "");
    snprintf(fas, sizeof fas, "%s.sorted", fa);
    snprintf(fbs, sizeof fbs, "%s.sorted", fb);
    size_t len = 0;
    char* buf = slurp(in_pairs, &len);
    FILE* out = fopen(out_pairs, "w");
    if (!out) { free(buf); return 1; }
    if (!buf) { fclose(out); return 0; }
    int* vals = (int*)malloc(sizeof(int) * (size_t)(4 * L + 8));
    char* p = buf;
    char* end = buf + len;
    long line_no = 0;
    while (p < end) {
        char* nlp = (char*)memchr(p, '\n', (size_t)(end - p));
        if (!nlp) nlp = end;
        *nlp = 0;
        int n = 0;
        char* q = p;
        for (;;) {
            while (*q == ' ' || *q == '\t' || *q == '\r') ++q;
            if (!*q) break;
            char* e;
            long v = strtol(q, &e, 10);
            if (e == q) break;
            if (n < 4 * L + 8) vals[n] = (int)v;
            n++;
            q = e;
        }
        /* io.cpp:52-55: a line with the wrong number of values throws */
        if (n != 2 * L) {
            fprintf(stderr, "PairReader: input line %ld: length is %d. Expected %d\n", line_no, n, 2 * L);
            fclose(out);
            free(vals);
            free(buf);
            return 2;
        }
        line_no++;
        int* a = vals;
        int* b = vals + L;
        int64_t lv, wr;
        gpo_uncompress_one(a, L, compress, new_compress, pafc, 0, fa, &lv, &wr);
        gpo_uncompress_one(b, L, compress, new_compress, pafc, 1, fb, &lv, &wr);
        const char* ia[1] = {fa};
        const char* ib[1] = {fb};
        gpo_sort(ia, 1, fas);
        gpo_sort(ib, 1, fbs);
        fflush(out);
        match_to(out, order, new_compress, pafc, fas, fbs, NULL);
        p = nlp + 1;
    }
    fclose(out);
    free(vals);
    free(buf);
    return 0;
}

/* ------------------------------------------------------------------ */
/* equivalence filter                                                  */
/* ------------------------------------------------------------------ */

/* Items are index pairs (a-part, b-part) of signed 1-based indices, stored
 * as 2L int16 values.  Operations restate src/utils/equivalence.cpp:146-277. */
static void pair_generators(int L, int compress, vecset* out) {
    const int W = 2 * L;
    int use_alt = !(compress > 1 || L % 2 == 1); /* filter.cpp:83-87 */
    vecset_init(out, W, 1 << 16);
    int16_t* cur = (int16_t*)malloc(sizeof(int16_t) * (size_t)W);
    int16_t* nxt = (int16_t*)malloc(sizeof(int16_t) * (size_t)W);
    int* cp = (int*)malloc(sizeof(int) * (size_t)(L + 1));
    int ncp = coprimes(L, cp);
    for (int i = 0; i < L; ++i) {
        cur[i] = (int16_t)(i + 1);
        cur[L + i] = (int16_t)(L + i + 1);
    }
    vecset_insert(out, cur);
    for (int64_t at = 0; at < out->count; ++at) {
#define RELOAD() memcpy(cur, out->items + at * W, sizeof(int16_t) * (size_t)W)
        RELOAD();
        /* shift_pair: rotate b left by 1..L-1 (equivalence.cpp:59-69) */
        for (int s = 1; s <= L - 1; ++s) {
            memcpy(nxt, cur, sizeof(int16_t) * (size_t)L);
            for (int i = 0; i < L; ++i) nxt[L + i] = cur[L + (i + s) % L];
            vecset_insert(out, nxt);
            RELOAD();
        }
        /* swap_pair (equivalence.cpp:46-56) */
        memcpy(nxt, cur + L, sizeof(int16_t) * (size_t)L);
        memcpy(nxt + L, cur, sizeof(int16_t) * (size_t)L);
        vecset_insert(out, nxt);
        RELOAD();
        /* reverse_pair: reverse b (equivalence.cpp:80-89) */
        memcpy(nxt, cur, sizeof(int16_t) * (size_t)L);
        for (int i = 0; i < L; ++i) nxt[L + i] = cur[L + L - 1 - i];
        vecset_insert(out, nxt);
        RELOAD();
        /* decimate_pair: both parts by every coprime (equivalence.cpp:154-167) */
        for (int c = 0; c < ncp; ++c) {
            for (int i = 0; i < L; ++i) {
                int src = (int)(((long long)i * cp[c]) % L);
                nxt[i] = cur[src];
                nxt[L + i] = cur[L + src];
            }
            vecset_insert(out, nxt);
            RELOAD();
        }
        if (use_alt) {
            /* altnegative_pair: negate odd positions of both (equivalence.cpp:119-131) */
            memcpy(nxt, cur, sizeof(int16_t) * (size_t)W);
            for (int i = 1; i < L; i += 2) {
                nxt[i] = (int16_t)-nxt[i];
                nxt[L + i] = (int16_t)-nxt[L + i];
            }
            vecset_insert(out, nxt);
        }
#undef RELOAD
    }
    free(cur);
    free(nxt);
    free(cp);
}

int64_t gpo_pair_generator_count(int L, int compress) {
    vecset s;
    pair_generators(L, compress, &s);
    int64_t n = s.count;
    vecset_free(&s);
    return n;
}

/* src/utils/equivalence.cpp:97-144: apply one generator item to a pair */
static void apply_pair_item(const int16_t* item, const int16_t* x, int L, int16_t* y) {
    const int16_t* ia = item;
    const int16_t* ib = item + L;
    const int16_t* xa = x;
    const int16_t* xb = x + L;
    int swapped = (ia[0] < 0 && -ia[0] > L) || (ia[0] > 0 && ia[0] > L);
    int16_t* ya = y;
    int16_t* yb = y + L;
    for (int i = 0; i < L; ++i) {
        int pa = ia[i] < 0 ? -ia[i] : ia[i];
        int pb = ib[i] < 0 ? -ib[i] : ib[i];
        if (swapped) {
            int16_t va = xa[(pa - 1) % L];
            int16_t vb = xb[(pb - 1) % L];
            yb[i] = ia[i] < 0 ? (int16_t)-va : va;
            ya[i] = ib[i] < 0 ? (int16_t)-vb : vb;
        } else {
            int16_t va = xa[(pa - 1) % L];
            int16_t vb = xb[(pb - 1) % L];
            ya[i] = ia[i] < 0 ? (int16_t)-va : va;
            yb[i] = ib[i] < 0 ? (int16_t)-vb : vb;
        }
    }
}

static int g_cmp_w;
static int cmp_vec16(const void* x, const void* y) {
    const int16_t* a = (const int16_t*)x;
    const int16_t* b = (const int16_t*)y;
    for (int i = 0; i < g_cmp_w; ++i)
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
}

/* src/core/filter/filter.cpp:18-163 */
int gpo_equiv_filter(int order, int compress, const char* in_path, const char* out_path) {
    const int L = order / compress;
    const int W = 2 * L;
    FILE* out = fopen(out_path, "w");
    size_t len = 0;
    char* buf = slurp(in_path, &len);
    if (!buf) {
        if (out) fclose(out);
        return 0; /* filter.cpp:33-37: "Bad File." and return 0 */
    }
    /* filter.cpp:45-62: read pairs of L + L integers into a sorted set */
    int16_t* P = NULL;
    int64_t np = 0, cap = 0;
    char* q = buf;
    int16_t* tmp = (int16_t*)malloc(sizeof(int16_t) * (size_t)W);
    for (;;) {
        int got = 0;
        for (int i = 0; i < W; ++i) {
            while (*q == ' ' || *q == '\n' || *q == '\t' || *q == '\r') ++q;
            if (!*q) break;
            char* e;
            long v = strtol(q, &e, 10);
            if (e == q) break;
            tmp[i] = (int16_t)v;
            q = e;
            got++;
        }
        if (got < W) break;
        if (np == cap) {
            cap = cap ? cap * 2 : 1024;
            P = (int16_t*)realloc(P, sizeof(int16_t) * (size_t)cap * (size_t)W);
        }
        memcpy(P + np * W, tmp, sizeof(int16_t) * (size_t)W);
        np++;
    }
    free(tmp);
    free(buf);
    g_cmp_w = W;
    if (np > 0) qsort(P, (size_t)np, sizeof(int16_t) * (size_t)W, cmp_vec16);
    /* unique */
    int64_t nu = 0;
    for (int64_t i = 0; i < np; ++i) {
        if (nu > 0 && cmp_vec16(P + (nu - 1) * W, P + i * W) == 0) continue;
        if (nu != i) memcpy(P + nu * W, P + i * W, sizeof(int16_t) * (size_t)W);
        nu++;
    }
    np = nu;
    char* alive = (char*)malloc((size_t)(np > 0 ? np : 1));
    memset(alive, 1, (size_t)(np > 0 ? np : 1));
    int64_t n_alive = np;

    vecset gens;
    pair_generators(L, compress, &gens);
    vecset cls;
    vecset_init(&cls, W, gens.count);
    int16_t* y = (int16_t*)malloc(sizeof(int16_t) * (size_t)W);

    int64_t it = 0;
    while (it < np && !alive[it]) ++it;
    while (it < np) {
        vecset_clear(&cls);
        for (int64_t g = 0; g < gens.count; ++g) {
            apply_pair_item(gens.items + g * W, P + it * W, L, y);
            vecset_insert(&cls, y);
        }
        /* filter.cpp:117-144 */
        if (cls.count > n_alive) {
            for (int64_t c = 0; c < cls.count; ++c) {
                const int16_t* m = cls.items + c * W;
                int16_t* hit = (int16_t*)bsearch(m, P, (size_t)np, sizeof(int16_t) * (size_t)W, cmp_vec16);
                if (!hit) continue;
                int64_t idx = (hit - P) / W;
                if (idx > it && alive[idx]) {
                    alive[idx] = 0;
                    n_alive--;
                }
            }
        } else {
            for (int64_t c = 0; c < cls.count; ++c) {
                const int16_t* m = cls.items + c * W;
                int16_t* hit = (int16_t*)bsearch(m, P, (size_t)np, sizeof(int16_t) * (size_t)W, cmp_vec16);
                if (!hit) continue;
                int64_t idx = (hit - P) / W;
                if (alive[idx]) {
                    alive[idx] = 0;
                    n_alive--;
                }
            }
            if (!alive[it]) {
                alive[it] = 1;
                n_alive++;
            }
        }
        ++it;
        while (it < np && !alive[it]) ++it;
    }
    if (out) {
        for (int64_t i = 0; i < np; ++i) {
            if (!alive[i]) continue;
            const int16_t* x = P + i * W;
            for (int k = 0; k < L; ++k) fprintf(out, "%d ", x[k]);
            fprintf(out, " ");
            for (int k = 0; k < L; ++k) fprintf(out, "%d ", x[L + k]);
            fprintf(out, "\n");
        }
        fclose(out);
    }
    free(y);
    free(alive);
    free(P);
    vecset_free(&gens);
    vecset_free(&cls);
    return 0;
}

/* ------------------------------------------------------------------ */
/* batched PSD filter (CPU baseline / checker)                          */
/* ------------------------------------------------------------------ */

typedef struct {
    const int8_t* seqs;
    int64_t begin, end;
    int L, order, paf;
    uint8_t* verdict;
    double* maxout;
    int64_t pass;
    const twiddles* tw;
} batch_job;

static void* batch_worker(void* arg) {
    batch_job* j = (batch_job*)arg;
    const int L = j->L;
    const int H = L / 2;
    const double thr = 2 * j->order - j->paf + 0.001;
    int seq[GPO_MAX_LEN];
    int64_t pass = 0;
    for (int64_t r = j->begin; r < j->end; ++r) {
        const int8_t* s = j->seqs + r * (int64_t)L;
        for (int i = 0; i < L; ++i) seq[i] = s[i];
        /* fourier.cpp:45-52 only looks at k = 1..L/2 */
        double mx = 0.0;
        int ok = 1;
        for (int k = 1; k <= H; ++k) {
            double re = 0.0, im = 0.0;
            int m = 0;
            for (int t = 0; t < L; ++t) {
                re += (double)seq[t] * j->tw->cs[m];
                im -= (double)seq[t] * j->tw->sn[m];
                m += k;
                if (m >= L) m -= L;
            }
            double p = re * re + im * im;
            if (p > mx) mx = p;
            if (p > thr) {
                ok = 0;
                if (!j->maxout) break;
            }
        }
        if (j->verdict) j->verdict[r] = (uint8_t)ok;
        if (j->maxout) j->maxout[r] = mx;
        pass += ok;
    }
    j->pass = pass;
    return NULL;
}

static int64_t run_batch(const int8_t* seqs, int64_t n, int L, int order, int pafc, uint8_t* verdict,
                         double* maxout, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    const twiddles* tw = get_twiddles(L);
    batch_job jobs[256];
    pthread_t th[256];
    int64_t per = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].seqs = seqs;
        jobs[t].begin = (int64_t)t * per < n ? (int64_t)t * per : n;
        jobs[t].end = (int64_t)(t + 1) * per < n ? (int64_t)(t + 1) * per : n;
        jobs[t].L = L;
        jobs[t].order = order;
        jobs[t].paf = pafc;
        jobs[t].verdict = verdict;
        jobs[t].maxout = maxout;
        jobs[t].pass = 0;
        jobs[t].tw = tw;
        if (nthreads > 1)
            pthread_create(&th[t], NULL, batch_worker, &jobs[t]);
        else
            batch_worker(&jobs[t]);
    }
    int64_t pass = 0;
    for (int t = 0; t < nthreads; ++t) {
        if (nthreads > 1) pthread_join(th[t], NULL);
        pass += jobs[t].pass;
    }
    return pass;
}

int64_t gpo_psd_filter_batch(const int8_t* seqs, int64_t n, int L, int order, int pafc, uint8_t* verdict,
                             int nthreads) {
    return run_batch(seqs, n, L, order, pafc, verdict, NULL, nthreads);
}

void gpo_psd_max_batch(const int8_t* seqs, int64_t n, int L, double* out, int nthreads) {
    run_batch(seqs, n, L, 1 << 20, 0, NULL, out, nthreads);
}
