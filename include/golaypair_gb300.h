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
 * (a cudaStream_t; NULL = the context's stream).  With stats == NULL the call
 * does not synchronise.  n < 2^31. */
int gp_psd_filter_device(gp_ctx* ctx, const int8_t* d_seqs, int64_t n, int L, int order, int paf, int mode,
                         uint32_t* d_pass_mask, void* stream, gp_psd_stats* stats);

/* Profiling: when enabled, CUDA events bracket every launch of the main
 * filter kernel (tensor-core or FP64) on its stream.  gp_kernel_time waits
 * for them, returns the summed device time and launch count, and clears. */
int gp_kernel_timing(gp_ctx* ctx, int enable);
int gp_kernel_time(gp_ctx* ctx, double* total_ms, int64_t* launches);

/* Tensor-core PSD values (fp32, bins 1..L/2) of n rows, for error analysis.
 * out: n x (L/2) floats, HOST memory. */
int gp_psd_tc_values(gp_ctx* ctx, const int8_t* seqs, int64_t n, int L, float* out);
/* FP64 PSD values (all bins 0..L-1) of n rows.  out: n x L doubles, HOST. */
int gp_psd_fp64_values(gp_ctx* ctx, const int8_t* seqs, int64_t n, int L, double* out);

#ifdef __cplusplus
}
#endif
#endif
