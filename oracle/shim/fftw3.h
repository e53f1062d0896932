/*
 * Stand-in for the FFTW 3 API, used ONLY to compile the reference's own
 * sources for cross-checking the oracle (test infrastructure; never shipped).
 *
 * FFTW 3.3.10 is not installed on this machine.  This header provides the
 * handful of symbols the reference calls (src/utils/fourier.cpp:11-43):
 * fftw_complex, fftw_alloc_complex, fftw_free, fftw_plan_dft_1d,
 * fftw_execute, fftw_destroy_plan, FFTW_FORWARD, FFTW_MEASURE.
 *
 * The transform is a direct O(L^2) double-precision DFT,
 *   out[k] = sum_j in[j] * exp(-2*pi*i * ((j*k) mod L) / L),
 * with the twiddle table precomputed per plan.  It agrees with FFTW's FFT up
 * to last-ulp rounding; the consequence for parity is stated where the
 * oracle is described.
 */
#pragma once
#include <math.h>
#include <stdlib.h>

typedef double fftw_complex[2];

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

struct gp_shim_fftw_plan {
    int n;
    fftw_complex* in;
    fftw_complex* out;
    double* cs; /* cos table, n entries, index (j*k) mod n */
    double* sn; /* sin table */
    int sign;
};
typedef struct gp_shim_fftw_plan* fftw_plan;

static inline fftw_complex* fftw_alloc_complex(size_t n) {
    return (fftw_complex*)malloc(sizeof(fftw_complex) * (n ? n : 1));
}

static inline void fftw_free(void* p) { free(p); }

static inline fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags) {
    (void)flags;
    fftw_plan p = (fftw_plan)malloc(sizeof(struct gp_shim_fftw_plan));
    p->n = n;
    p->in = in;
    p->out = out;
    p->sign = sign;
    p->cs = (double*)malloc(sizeof(double) * (n ? n : 1));
    p->sn = (double*)malloc(sizeof(double) * (n ? n : 1));
    const double two_pi = 6.283185307179586476925286766559;
    for (int m = 0; m < n; ++m) {
        double ang = two_pi * (double)m / (double)n;
        p->cs[m] = cos(ang);
        p->sn[m] = sin(ang);
    }
    return p;
}

static inline void fftw_execute(const fftw_plan p) {
    const int n = p->n;
    const double s = (p->sign == FFTW_FORWARD) ? -1.0 : 1.0;
    for (int k = 0; k < n; ++k) {
        double re = 0.0, im = 0.0;
        int m = 0; /* (j*k) mod n, stepped by k: the same index, no division */
        for (int j = 0; j < n; ++j, m += k, m -= (m >= n) ? n : 0) {
            double c = p->cs[m], sv = s * p->sn[m];
            re += p->in[j][0] * c - p->in[j][1] * sv;
            im += p->in[j][0] * sv + p->in[j][1] * c;
        }
        p->out[k][0] = re;
        p->out[k][1] = im;
    }
}

static inline void fftw_destroy_plan(fftw_plan p) {
    if (!p) return;
    free(p->cs);
    free(p->sn);
    free(p);
}
