/*
 * golaypair_gb300.h -- C ABI of the GB300 (sm_103a) implementation of
 * GolayPair's candidate-generation -> PSD-filter -> sorted-PSD-matching path.
 *
 * Plain C types only.  Every entry point returns GP_OK (0) or a negative
 * GP_ERR_* code; gp_last_error() describes the last failure on a context.
 * A context is bound to one GPU and is not thread-safe.
 *
 * The stage entry points (gp_generate ... gp_equiv_filter) replace the
 * reference's stage functions one for one and keep their file formats; the
 * comment above each names the reference function it replaces.
 */
#ifndef GOLAYPAIR_GB300_H
#define GOLAYPAIR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GP_OK 0
#define GP_ERR_ARG (-1)          /* invalid argument */
#define GP_ERR_CUDA (-2)         /* CUDA runtime error (no GPU, launch failure) */
#define GP_ERR_TIMEOUT (-3)      /* a bounded device wait gave up */
#define GP_ERR_NOMEM (-4)        /* device allocation failed */
#define GP_ERR_UNSUPPORTED (-5)  /* sequence length outside the supported range */
#define GP_ERR_IO (-6)           /* file could not be opened / written */
#define GP_ERR_FORMAT (-7)       /* malformed input line */
#define GP_ERR_OVERFLOW (-8)     /* a device output list ran out of room */
#define GP_NO_DECOMPOSITION 1    /* 2n+(n-1)paf has no two-square decomposition */
#define GP_EMPTY_INPUT 1         /* match: an input file is empty */

/* PSD filter arithmetic */
#define GP_PSD_FP64 0        /* plain FP64 CUDA-core direct DFT */
#define GP_PSD_TC_GUARDED 1  /* fp16 hi/lo twiddles on tcgen05, fp32 accumulate,
                                guard band + FP64 recheck; verdicts exact */

typedef struct gp_ctx gp_ctx;

typedef struct {
    int64_t n;           /* candidates filtered */
    int64_t n_pass;      /* final passes */
    int64_t n_unsure;    /* candidates sent to the FP64 recheck (TC mode) */
    float guard;         /* configured guard band (TC mode) */
    float err_coef;      /* per-candidate |DFT error| bound / sum|x| (TC mode) */
} gp_psd_stats;

/* Creates a context on CUDA device `device`. */
int gp_ctx_create(gp_ctx** out, int device);
int gp_ctx_destroy(gp_ctx* ctx);
const char* gp_last_error(const gp_ctx* ctx);
/* Number of SMs of the context's device. */
int gp_device_sm_count(const gp_ctx* ctx);

/*
 * Batched PSD filter.  Replaces Fourier::calculate_psd + Fourier::psd_filter
 * (src/utils/fourier.cpp:25-52) applied to every row:
 *   pass iff psd[k] <= 2*order - paf + 0.001 for k = 1..L/2.
 * seqs: n x L int8, row-major, HOST memory.  pass_mask: (n+31)/32 uint32
 * words, bit (i % 32) of word i/32 = row i passes, HOST memory.
 * The host buffers are copied in chunks with copies overlapped with compute.
 */
int gp_psd_filter(gp_ctx* ctx, const int8_t* seqs, int64_t n, int L, int order, int paf, int mode,
                  uint32_t* pass_mask, gp_psd_stats* stats);

/* Same on DEVICE buffers (seqs, pass_mask), enqueued on `stream`
 * (a cudaStream_t; NULL = the context's stream).  n < 2^31.  With stats !=
 * NULL the call synchronises and returns any device-side error.  With
 * stats == NULL it only enqueues: the mask is valid once gp_check(ctx,
 * stream) has returned GP_OK, which reports a bounded device wait that gave
 * up (GP_ERR_TIMEOUT) or an overflow (GP_ERR_OVERFLOW) of this call; until
 * then the error stays pending in the context.  The unsure list and counters
 * of the FP64 recheck belong to the context: calls on one context must not
 * overlap on the GPU (enqueue them on one stream, or wait in between).
 * d_seqs may start at any byte; the tensor-core filter streams whole tiles
 * through the bulk-copy engine only when it is 16-byte aligned, and reads
 * the rows with plain loads otherwise (same verdicts, slower). */
int gp_psd_filter_device(gp_ctx* ctx, const int8_t* d_seqs, int64_t n, int L, int order, int paf, int mode,
                         uint32_t* d_pass_mask, void* stream, gp_psd_stats* stats);

/* Waits for `stream` (NULL = the context's stream) and returns the status
 * the context's kernels recorded: GP_OK, GP_ERR_TIMEOUT (a bounded device
 * wait gave up) or GP_ERR_OVERFLOW (a device list ran out of room); the
 * status is cleared.  Asynchronous callers of gp_psd_filter_device call it
 * before reading the mask.  No counterpart in the reference, whose filter is
 * a synchronous host function. */
int gp_check(gp_ctx* ctx, void* stream);

/* Profiling: when enabled, CUDA events bracket every launch of the main
 * filter kernel (tensor-core or FP64) on its stream.  gp_kernel_time waits
 * for them, returns the summed device time and launch count, and clears. */
int gp_kernel_timing(gp_ctx* ctx, int enable);
int gp_kernel_time(gp_ctx* ctx, double* total_ms, int64_t* launches);
/* Diagnostics: per-role cycle counters of the tensor-core filter (converter,
 * epilogue, MMA and producer waits / work, tiles), summed over CTAs since the
 * previous call.  Copies up to nout counters, resets them, and turns the
 * counting on (enable != 0) or off for later launches. */
int gp_debug_tc_trace(gp_ctx* ctx, int enable, uint64_t* out, int nout);
/* Diagnostics: runs the bounded device wait of the pipeline kernels on a
 * barrier that nothing completes, with a limit of limit_ns (at most 2 s).
 * Returns GP_ERR_TIMEOUT (the kernel gave up and reported it); the context
 * stays usable.  Tests failure detection without faulting the GPU. */
int gp_debug_wait_timeout(gp_ctx* ctx, int64_t limit_ns);

/*
 * The batched tensor-core PSD filter for callers that cannot allocate device
 * memory (code running under another framework's allocator or memory pool,
 * allocation-free real-time loops, devices whose memory is reserved by their
 * owner).  No counterpart in the reference.  Same verdicts as
 * gp_psd_filter_device in GP_PSD_TC_GUARDED mode, on DEVICE buffers, on
 * `stream` (a cudaStream_t; NULL = legacy default stream), without a context.
 * Allocates nothing: its working buffers live in one fixed static device
 * array (about 4.3 MB, held by every GPU that loads the library until the
 * process exits).  Limits and rules:
 *   - n <= 2^20 rows (GP_ERR_ARG beyond, with a message on stderr);
 *     2 <= L <= 127 (GP_ERR_UNSUPPORTED otherwise);
 *   - the first call on a device looks up the array's device address there
 *     (with that device current) and keeps it; make it before any stream
 *     capture; after a cudaDeviceReset of that device the kept address is
 *     stale: do not call the entry point there again in the same process;
 *   - all calls share the array: calls that overlap on the GPU race;
 *   - synchronous: returns after `stream` has finished the work (it waits on
 *     that stream only).
 */
int gp_psd_filter_noalloc(const int8_t* d_seqs, int64_t n, int L, int order, int paf, uint32_t* d_pass_mask,
                          void* stream);

/* Tensor-core PSD values (fp32, bins 1..L/2) of n rows, for error analysis.
 * out: n x (L/2) floats, HOST memory. */
int gp_psd_tc_values(gp_ctx* ctx, const int8_t* seqs, int64_t n, int L, float* out);
/* FP64 PSD values (all bins 0..L-1) of n rows.  out: n x L doubles, HOST. */
int gp_psd_fp64_values(gp_ctx* ctx, const int8_t* seqs, int64_t n, int L, double* out);

/* ---------------------------------------------------------------- stages */

typedef struct {
    int64_t necklaces;   /* necklaces visited ("Orderly Count") */
    int64_t candidates;  /* necklaces that passed the row-sum gate */
    int64_t psd_pass;    /* candidates that passed the exact PSD filter */
    int64_t written_a;   /* lines written to the A file */
    int64_t written_b;   /* lines written to the B file */
    int64_t unsure;      /* candidates the tensor-core filter sent to FP64 */
    double seconds;
} gp_gen_stats;

/*
 * Candidate generation for job proc_id of proc_num.  Replaces
 *   int generate_hybrid(int ORDER, int COMPRESS, int PAF_CONSTANT,
 *                       std::ofstream& out_a, std::ofstream& out_b,
 *                       int PROC_ID, int PROC_NUM)
 * (src/core/generate/generate_hybrid.h; generate_hybrid.cpp:107-163) with the
 * job split of src/utils/lyndon.cpp:87-121.  Writes the A and B candidate
 * files (src/utils/io.cpp:14-36 format) in the reference's line order.
 * Returns GP_NO_DECOMPOSITION (1) when 2n+(n-1)paf is not a sum of two
 * squares, as the reference does.
 */
int gp_generate(gp_ctx* ctx, int order, int compress, int paf, int proc_id, int proc_num, const char* path_a,
                const char* path_b, gp_gen_stats* stats);

/* The word-rank ranges [begin, end) job proc_id of proc_num searches
 * (src/utils/lyndon.cpp:93-106: prenecklace prefixes of the first length
 * with at least proc_num * 10000 necklaces, dealt out round robin; one job
 * takes the whole space).  Writes up to cap ranges to out as (begin_hi,
 * begin_lo, end_hi, end_lo) and returns how many there are, or a negative
 * error.  Host only: replicas on several GPUs take disjoint jobs. */
int64_t gp_job_ranges(int order, int compress, int paf, int proc_id, int proc_num, uint64_t* out, int64_t cap);

/* Same over the words whose lexicographic rank (base-|alphabet| number,
 * first entry most significant) lies in [begin, end), 128-bit bounds as
 * (hi, lo) pairs.  No counterpart in the reference, which only splits by
 * prefix; used for windowed searches of orders too large to enumerate. */
int gp_generate_window(gp_ctx* ctx, int order, int compress, int paf, uint64_t begin_hi, uint64_t begin_lo,
                       uint64_t end_hi, uint64_t end_lo, const char* path_a, const char* path_b,
                       gp_gen_stats* stats);

/*
 * Checkpointed generation for searches that run for days: the same job as
 * gp_generate (job split proc_id of proc_num) or gp_generate_window (word
 * ranks [begin, end)), but the call stops after max_iterations pipeline
 * iterations or max_seconds of searching (either <= 0: no limit).  When it
 * stops early it writes checkpoint_path (the counts so far, the word ranges
 * still to search and the records found so far; written to a temporary file
 * and renamed, so an interrupted write keeps the previous checkpoint) and
 * sets *done = 0; the output files are not written yet.  The next call with
 * the same job and checkpoint_path resumes from it.  When the search
 * finishes, the call writes the A and B files -- identical to those of the
 * uninterrupted call -- removes the checkpoint and sets *done = 1.  stats
 * counts the whole search so far; its seconds field is this call's time.
 * A checkpoint of another job gives GP_ERR_FORMAT.  No counterpart in the
 * reference, whose only restart unit is a whole stage output file.
 */
int gp_generate_resumable(gp_ctx* ctx, int order, int compress, int paf, int proc_id, int proc_num,
                          const char* path_a, const char* path_b, const char* checkpoint_path, int max_iterations,
                          double max_seconds, int* done, gp_gen_stats* stats);
int gp_generate_window_resumable(gp_ctx* ctx, int order, int compress, int paf, uint64_t begin_hi, uint64_t begin_lo,
                                 uint64_t end_hi, uint64_t end_lo, const char* path_a, const char* path_b,
                                 const char* checkpoint_path, int max_iterations, double max_seconds, int* done,
                                 gp_gen_stats* stats);

/*
 * Format of the A and B files the generation entry points write (all of
 * them, this context, from the next call on):
 *   GP_FORMAT_TEXT   the reference's lines (src/utils/io.cpp:14-36), default;
 *   GP_FORMAT_BINARY a binary survivor file: an 80-byte header (magic
 *                    "GPSURV01", order, compress, paf, length, alphabet,
 *                    bits per digit, role, field widths, record count) and
 *                    one fixed-size record per line, in line order: the
 *                    packed word, then the line's L-1 signature values in 1
 *                    or 2 bytes each.  About a quarter of the text's size
 *                    (3.9x smaller at order 57, compression 3).
 * gp_sort reads either format.  No counterpart in the reference, whose
 * binary sketch (src/utils/binary.cpp:74-117) is never called.
 */
#define GP_FORMAT_TEXT 0
#define GP_FORMAT_BINARY 1
int gp_set_output_format(gp_ctx* ctx, int format);

/*
 * Spectral pruning of the generation files (off by default; this context,
 * from the next call on).  Every complementary pair (A, B) has
 * p_A(k) + p_B(k) = 2n - paf exactly for k != 0 (Parseval with the PAF
 * condition and the row sums), and p(L/2) is the square of an integer (even
 * L) and p(L/3) a norm a^2 - ab + b^2 of an Eisenstein integer (L divisible
 * by 3).  With pruning on, a candidate whose 2n - paf - p(L/2) is not a
 * square, or whose 2n - paf - p(L/3) is not such a norm, is not written: it
 * has no partner.  The pair files that match writes are unchanged; the
 * candidate files are smaller.  No counterpart in the reference, whose
 * sketches of these checks (src/utils/fourier.cpp:75-195) are never called.
 */
int gp_set_spectral_prune(gp_ctx* ctx, int on);

/* The text lines of a binary survivor file, byte for byte what the
 * generation call that wrote it writes as text.  Host only: ctx may be NULL
 * (then errors are only returned).  GP_ERR_FORMAT if in_path is not a valid
 * survivor file. */
int gp_export_text(gp_ctx* ctx, const char* in_path, const char* out_path);

/* One job of a batched generation: the words of one order / compression
 * whose rank lies in [begin, end) (end clipped to the word space), written
 * to its own A and B files. */
typedef struct gp_gen_job {
    int order, compress, paf;
    uint64_t begin_hi, begin_lo, end_hi, end_lo;
    const char* path_a;
    const char* path_b;
} gp_gen_job;

/* Settings of the batched generation engine; zero fields take defaults. */
typedef struct gp_batch_config {
    int enum_variant;        /* enumerator kernel: 0 = 64 registers (4 CTAs per SM), 1 = full
                                occupancy (32 registers), 2 = 72 registers, no spills (3 CTAs) */
    int windows_per_thread;  /* rank windows per enumerator thread (0: 1) */
    int64_t cand_cap;        /* candidates per job per pipeline iteration (0: 2^22) */
    int tc_ctas_per_sm;      /* tensor-core filter CTAs per SM (0: as many as fit) */
    int no_graph;            /* 1: launch each iteration's kernels directly instead of replaying a CUDA graph */
    int iterations;          /* out: pipeline iterations run */
    double tune_seconds;     /* out: time spent by the tuner (0 when its result was cached) */
    int multi_launch;        /* 1: one launch per kernel and iteration over every job (lengths
                                order / compression up to 63); 0: per-job launches on the jobs'
                                own streams */
} gp_batch_config;

/* Generation of up to 8 jobs of different orders / compressions at once:
 * one enumerator launch covers every job's rank windows, and the jobs'
 * filter / finalize kernels run either on one branch per job or (multi_launch)
 * as one launch each over every job, in a per-iteration CUDA graph that is
 * captured once and replayed until all windows are done.
 * With autotune != 0 the engine first times its settings on a sample of
 * the jobs and uses (and writes to *cfg) the fastest; otherwise it uses
 * *cfg (or defaults when cfg is NULL).  stats, when not NULL, receives one
 * entry per job.  Per job the files equal those of gp_generate_window over
 * the same window.  No counterpart in the reference, which runs one order
 * per process. */
int gp_generate_batch(gp_ctx* ctx, const gp_gen_job* jobs, int njobs, int autotune, gp_batch_config* cfg,
                      gp_gen_stats* stats);

/* The settings the tuners chose so far on this context, one line per tuned
 * workload: "batch:<jobs> enum_variant windows_per_thread cand_cap
 * tc_ctas_per_sm use_graph multi_launch" for gp_generate_batch, "sort:W<words> radix_bits
 * microseconds" for gp_sort (which tunes its radix width per key width on
 * first use).  Writes at most cap bytes (NUL-terminated) to buf; returns the
 * length needed including the NUL.  No counterpart in the reference. */
int gp_tuned_settings(const gp_ctx* ctx, char* buf, int cap);

/*
 * Replaces GNU_sort(const std::vector<std::string>& in, const std::string& out,
 * const std::string& tmpdir) (src/core/sort/sort.cpp:7-22), which runs
 * `sort | uniq` over the files: lines of all inputs, byte order (C locale),
 * adjacent duplicates removed, written to out_path.  An input that is a
 * binary survivor file (gp_set_output_format) contributes its text lines.
 */
int gp_sort(gp_ctx* ctx, const char** in_paths, int n_in, const char* out_path);

/*
 * Replaces int match_pairs(int ORDER, int COMPRESS, int PAF, std::ifstream& a,
 * std::ifstream& b, IO::PairWriter&) (src/core/match/match_pairs.h:5,
 * match_pairs.cpp:15-121): merge-join of two sorted candidate files on their
 * first token, each equal-token cross product checked by exact PAF
 * (src/utils/golay.cpp:27-44), pairs appended (append != 0) or written to
 * out_path (src/utils/io.cpp:75-95 format).  Returns GP_EMPTY_INPUT (1) when
 * an input is empty, after creating/truncating out_path like the reference.
 */
int gp_match(gp_ctx* ctx, int order, int compress, int paf, const char* path_a, const char* path_b,
             const char* out_path, int append, int64_t* n_pairs);

/*
 * Replaces uncompress_pipeline(int order, int c, int c_new, int paf,
 * IO::PairReader&, IO::PairWriter&, const std::string& work_dir,
 * const std::string& prefix, DeviceType) (src/core/uncompression/
 * uncompression.h:19-29, uncompression.cpp:32-79) for both of its devices:
 * every pair of in_pairs (compression c) is expanded to compression c_new,
 * PSD-filtered and matched; the pairs are written to out_pairs in input
 * order, in the order the reference's sorted scratch files give them.
 * Many pairs are processed per batch on the device; the candidates never
 * leave it (the reference's uncompress_tmp_* scratch files are not written;
 * work_dir and prefix are accepted for interface parity).  A line with the
 * wrong number of values is GP_ERR_FORMAT (the reference throws,
 * io.cpp:52-55); the pairs of the lines before it are still written.
 */
int gp_uncompress(gp_ctx* ctx, int order, int compress, int new_compress, int paf, const char* in_pairs,
                  const char* out_pairs, const char* work_dir, const char* prefix);

/* Same over the input lines first, first + step, ... below end_line
 * (0-based; end_line = INT64_MAX: to the end), so that several processes
 * or GPUs can split one uncompression: contiguous ranges whose outputs are
 * concatenated in range order give the file of one call over all lines.
 * This wires the reference's parsed-but-unused uncompress options --line,
 * --range_begin, --range_end, --range_step (src/main.cpp:110-113,192-195),
 * whose meaning the reference leaves undefined. */
int gp_uncompress_lines(gp_ctx* ctx, int order, int compress, int new_compress, int paf, const char* in_pairs,
                        const char* out_pairs, const char* work_dir, const char* prefix, int64_t first,
                        int64_t end_line, int64_t step);

/* A whole chain compress[0] -> compress[1] -> ... -> compress[ncomp-1]
 * (ncomp >= 2), as src/main.cpp:117-139 runs uncompress_pipeline once per
 * level: level i writes out_pairs[i] (ncomp - 1 paths).  Level 0 reads the
 * selected lines of in_pairs (first, end_line, step as gp_uncompress_lines);
 * each later level takes the previous level's pairs from memory, in the
 * order they were written, instead of reading the file back.  The files
 * equal those of one gp_uncompress_lines call per level.  A malformed line
 * of in_pairs stops the chain after level 0 with GP_ERR_FORMAT. */
int gp_uncompress_chain(gp_ctx* ctx, int order, const int* compress, int ncomp, int paf, const char* in_pairs,
                        const char* const* out_pairs, int64_t first, int64_t end_line, int64_t step);

/*
 * Replaces int cache_filter(int ORDER, int COMPRESS, const std::string& in,
 * const std::string& out) (src/core/filter/filter.h, filter.cpp:18-163):
 * keeps the first pair of every equivalence class (in the reference's set
 * order and erase rules) and writes them in sorted order.  The generator
 * group has 4 phi(L) L^2 elements (8 times more at compression 1 with even
 * L); classes are found from each pair's least image over the group, so no
 * table of the group is built for L >= 3 and every length up to 128 runs
 * (at L = 128, compression 1, the reference's table of 33.5 million
 * elements would run it out of memory).
 */
int gp_equiv_filter(gp_ctx* ctx, int order, int compress, const char* in_path, const char* out_path);

/* Diagnostics: size of the pair-equivalence generator set gp_equiv_filter
 * builds for length L (the closure of src/core/filter/filter.cpp:70-87), or
 * -1 for an unsupported length.  Host only. */
int64_t gp_debug_pair_generator_count(int L, int compress);

/* Diagnostics: 1 when the affine description of that group gp_equiv_filter
 * uses for L >= 3 (swap, multiplier +-u, shifts of each half, the
 * alternating signs) gives exactly the closure's elements, 0 when not, -1
 * when not applicable (L < 3 or an unsupported length).  Host only. */
int gp_debug_pair_group_check(int L, int compress);

#ifdef __cplusplus
}
#endif
#endif
