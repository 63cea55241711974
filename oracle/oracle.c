/*
 * oracle.c -- CPU oracle for the tridiagonal TPR / PTPR path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA solver.  Only tests,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * Contents
 *   - orc_{ptpr,tpr,cr,pcr,normalize}_{f32,f64}: restatement of the
 *     reference CPU solvers (oracle_impl.h; file:line there).
 *   - orc_thomas_*: FP64 Thomas algorithm (no pivoting), the accuracy truth
 *     for refined solves.  Own code.
 *   - orc_batch_*: OpenMP over independent systems, one private workspace
 *     per thread -- the pattern of the reference's multi-thread test
 *     (test/examples.cpp:130-154) -- used as the timed CPU baseline.
 *   - orc_time_plain_*: the reference's timed single-system loop
 *     (src/pm.cpp:160-194) with its solver-internal OpenMP.
 *   - orc_rel_l2: ||x - xt||_2 / ||xt||_2 accumulated in FP64, the
 *     reference's stability metric (src/numerical_stability.cpp:100-115).
 *
 * Build: see oracle/Makefile (-O2 -ffp-contract=off -fopenmp).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Monotonic wall clock in seconds. */
static double orc_now(void) {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
#endif
}

/* floor(log2(v)) for v >= 1 (src/lib.hpp:69-91). */
static int orc_ilog2(int v) {
    int r = 0;
    while (v > 1) {
        v >>= 1;
        ++r;
    }
    return r;
}

#define REAL float
#define SFX f32
#define ONE 1.0f
#define EPS FLT_EPSILON
#include "oracle_impl.h"
#undef REAL
#undef SFX
#undef ONE
#undef EPS

#define REAL double
#define SFX f64
#define ONE 1.0
#define EPS DBL_EPSILON
#include "oracle_impl.h"
#undef REAL
#undef SFX
#undef ONE
#undef EPS

/* Thomas algorithm in FP64 for a general (not diag-normalised) system:
 * a[i] x[i-1] + b[i] x[i] + c[i] x[i+1] = d[i]; a[0] and c[n-1] ignored. */
void orc_thomas_f64(int n, const double *a, const double *b, const double *c,
                    const double *d, double *x) {
    double *cp = (double *)malloc(sizeof(double) * (size_t)n);
    double den = b[0];
    cp[0] = (n > 1 ? c[0] : 0.0) / den;
    x[0] = d[0] / den;
    for (int i = 1; i < n; i++) {
        den = b[i] - a[i] * cp[i - 1];
        cp[i] = (i < n - 1 ? c[i] : 0.0) / den;
        x[i] = (d[i] - a[i] * x[i - 1]) / den;
    }
    for (int i = n - 2; i >= 0; i--) x[i] -= cp[i] * x[i + 1];
    free(cp);
}

/* Same, from FP32-stored coefficients (each widened exactly to FP64). */
static void thomas_from_f32(int n, const float *a, const float *b,
                            const float *c, const float *d, double *x,
                            double *cp) {
    double den = (double)b[0];
    cp[0] = (n > 1 ? (double)c[0] : 0.0) / den;
    x[0] = (double)d[0] / den;
    for (int i = 1; i < n; i++) {
        den = (double)b[i] - (double)a[i] * cp[i - 1];
        cp[i] = (i < n - 1 ? (double)c[i] : 0.0) / den;
        x[i] = ((double)d[i] - (double)a[i] * x[i - 1]) / den;
    }
    for (int i = n - 2; i >= 0; i--) x[i] -= cp[i] * x[i + 1];
}

/* FP64 Thomas truth for a batch of FP32-stored systems.  System k occupies
 * [off[k], off[k] + ns[k]) of every array. */
void orc_batch_thomas_f32in(int nsys, const int64_t *off, const int *ns,
                            const float *a, const float *b, const float *c,
                            const float *d, double *x, int nthreads) {
    int nmax = 1;
    for (int k = 0; k < nsys; k++)
        if (ns[k] > nmax) nmax = ns[k];
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        double *cp = (double *)malloc(sizeof(double) * (size_t)nmax);
#pragma omp for schedule(dynamic, 4)
        for (int k = 0; k < nsys; k++) {
            int64_t o = off[k];
            thomas_from_f32(ns[k], a + o, b + o, c + o, d + o, x + o, cp);
        }
        free(cp);
    }
}

/* FP64 Thomas truth for a batch of FP64 systems (plain FP64 path). */
void orc_batch_thomas_f64(int nsys, const int64_t *off, const int *ns,
                          const double *a, const double *b, const double *c,
                          const double *d, double *x, int nthreads) {
#pragma omp parallel for schedule(dynamic, 4) \
    num_threads(nthreads > 0 ? nthreads : 1)
    for (int k = 0; k < nsys; k++) {
        int64_t o = off[k];
        orc_thomas_f64(ns[k], a + o, b + o, c + o, d + o, x + o);
    }
}

/* Relative L2 error in FP64. */
double orc_rel_l2_f64(int64_t n, const double *x, const double *xt) {
    double s1 = 0.0, s2 = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double e = x[i] - xt[i];
        s1 += e * e;
        s2 += xt[i] * xt[i];
    }
    return sqrt(s1) / sqrt(s2);
}

/* Per-system relative L2 errors of a batch; returns the maximum. */
double orc_batch_rel_l2(int nsys, const int64_t *off, const int *ns,
                        const double *x, const double *xt, double *out,
                        int nthreads) {
    double worst = 0.0;
#pragma omp parallel for schedule(static) reduction(max : worst) \
    num_threads(nthreads > 0 ? nthreads : 1)
    for (int k = 0; k < nsys; k++) {
        double e = orc_rel_l2_f64(ns[k], x + off[k], xt + off[k]);
        if (out) out[k] = e;
        if (!(e <= worst)) worst = e; /* NaN propagates as the maximum */
    }
    return worst;
}

/* Batched PTPR / TPR baseline: OpenMP over systems, one workspace per
 * thread, diag normalisation on private copies inside the timed region
 * (the 4-argument setter, src/ptpr.hpp:80-89).  kind: 0 = PTPR, 1 = TPR.
 * Uniform batch: system k at k*n. */
void orc_batch_tpr_f32(int kind, int nsys, int n, int s, const float *a,
                       const float *b, const float *c, const float *d,
                       float *x, int nthreads) {
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        /* one solver object per thread: its workspace is allocated once,
         * as the reference's init does (src/ptpr.cpp:54-96) */
        size_t wsz = kind == 0 ? orc_ptpr_ws_size_f32(n, s) : orc_tpr_ws_size_f32(n, s);
        float *wa = (float *)malloc(sizeof(float) * ((size_t)n * 3 + wsz));
        float *wc = wa + n, *wr = wa + 2 * n, *ws = wa + 3 * n;
#pragma omp for schedule(static)
        for (int k = 0; k < nsys; k++) {
            size_t o = (size_t)k * (size_t)n;
            memcpy(wa, a + o, sizeof(float) * (size_t)n);
            memcpy(wc, c + o, sizeof(float) * (size_t)n);
            memcpy(wr, d + o, sizeof(float) * (size_t)n);
            orc_normalize_f32(n, wa, b + o, wc, wr);
            if (kind == 0)
                orc_ptpr_ws_f32(n, s, wa, wc, wr, x + o, ws);
            else
                orc_tpr_ws_f32(n, s, wa, wc, wr, x + o, ws);
        }
        free(wa);
    }
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
