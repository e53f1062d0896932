/*
 * golay_oracle.h -- CPU restatement of GolayPair's candidate-generation ->
 * PSD-filter -> sorted-PSD-matching path, plus uncompression and the
 * equivalence filter.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load this library, and only as the checker
 * or the timed CPU baseline.  The product (golaypair_gb300) never links it.
 *
 * Every function cites the reference file:line it restates.  The DFT is a
 * direct double-precision DFT (the reference calls FFTW 3.3.10, which is not
 * installed here); the two agree to last-ulp rounding.
 */
#ifndef GOLAY_ORACLE_H
#define GOLAY_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPO_MAX_LEN 512

/* src/utils/golay.cpp:60-75 -- sorted ascending, returns count */
int gpo_alphabet(int compress, int* out);
/* src/utils/decomps.cpp:6-17 -- (x,y) with x<=y, x^2+y^2=k, returns count */
int gpo_decomps(int k, int* xs, int* ys, int max_out);
/* src/core/generate/generate_hybrid.cpp:45-47 */
int gpo_sum_constant(int order, int paf);
/* src/utils/fourier.cpp:25-43 -- psd[k] = |DFT_k|^2, k = 0..L-1 */
void gpo_psd(const int* seq, int L, double* psd);
/* src/utils/fourier.cpp:45-52 */
int gpo_psd_filter(const double* psd, int L, int order, int paf);
/* src/utils/orderly_equivalence.cpp:17-68; flag 0 = shift+reverse+decimation
 * (A candidates), flag 1 = shift+reverse (B candidates) */
int gpo_is_canonical(const int* seq, int L, int flag);
/* Number of permutations in constructGenerators(flag, L), built by closure
 * exactly as src/utils/orderly_equivalence.cpp:28-51 does; writes them
 * (0-based, row-major, count x L) to out when out != NULL. */
int gpo_orderly_generators(int L, int flag, int* out, int max_count);
/* src/utils/golay.cpp:27-44 */
int gpo_check_if_pair(const int* a, const int* b, int L, int paf, int compress);
/* src/utils/io.cpp:14-36: formats one candidate line into buf (no NUL),
 * returns its length.  invert != 0 writes bound - rint(psd). */
int gpo_format_candidate(char* buf, const int* seq, const double* psd, int L, int invert, int bound);
/* src/utils/lyndon.cpp:38-45 (saturates at INT64_MAX) */
int64_t gpo_necklace_count(int L, int k);

typedef struct {
    int64_t necklaces;      /* callbacks (necklaces enumerated by this job) */
    int64_t psd_evals;      /* PSD evaluations (row-sum gate passed) */
    int64_t psd_pass;       /* passed the PSD filter (before canonical check) */
    int64_t written_a;      /* lines written to the A file */
    int64_t written_b;      /* lines written to the B file */
} gpo_gen_stats;

/* src/core/generate/generate_hybrid.cpp:107-163 with the job split of
 * src/utils/lyndon.cpp:87-121.  Returns 0, or 1 when 2n+(n-1)paf has no
 * two-square decomposition. */
int gpo_generate(int order, int compress, int paf, const char* path_a, const char* path_b,
                 int proc_id, int proc_num, gpo_gen_stats* stats);
/* Same enumeration restricted to words whose lexicographic rank over the
 * sorted alphabet lies in [rank_begin, rank_end) (the window convention of
 * the GPU enumerator). */
int gpo_generate_window(int order, int compress, int paf, const char* path_a, const char* path_b,
                        uint64_t rank_begin_hi, uint64_t rank_begin_lo,
                        uint64_t rank_end_hi, uint64_t rank_end_lo, gpo_gen_stats* stats);
/* src/core/sort/sort.cpp:7-22: `sort | uniq` in the C locale */
int gpo_sort(const char** in_paths, int n_in, const char* out_path);
/* src/core/match/match_pairs.cpp:15-121; returns 1 when an input is empty */
int gpo_match(int order, int compress, int paf, const char* path_a, const char* path_b,
              const char* out_path, int append, int64_t* n_pairs);
/* src/core/uncompression/uncompression.cpp:32-210 (CPU device) */
int gpo_uncompress(int order, int compress, int new_compress, int paf, const char* in_pairs,
                   const char* out_pairs, const char* work_dir, const char* prefix);
/* One sequence of uncompress_recursive (uncompression.cpp:81-210): writes the
 * candidate lines of every PSD-passing expansion of orig into path.  orig is
 * rotated in place exactly as the reference does. */
int gpo_uncompress_one(int* orig, int L, int compress, int new_compress, int paf, int seqflag,
                       const char* path, int64_t* n_leaves, int64_t* n_written);
/* src/core/filter/filter.cpp:18-163 */
int gpo_equiv_filter(int order, int compress, const char* in_path, const char* out_path);
/* Size of the pair-equivalence generator set of filter.cpp:70-87 */
int64_t gpo_pair_generator_count(int L, int compress);

/* Batched PSD filter of int8 sequences (row-major n x L) in FP64, split over
 * nthreads threads: verdict[i] = 1 iff the sequence passes
 * src/utils/fourier.cpp:45-52.  Used as the timed CPU baseline and the
 * parity checker of the batched GPU filter.  Returns the pass count. */
int64_t gpo_psd_filter_batch(const int8_t* seqs, int64_t n, int L, int order, int paf,
                             uint8_t* verdict, int nthreads);
/* max over k=1..L/2 of psd, per sequence (double) */
void gpo_psd_max_batch(const int8_t* seqs, int64_t n, int L, double* out, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
