/*
 * sbo_maxcut.c -- FP64 CPU oracle, MaxCut side.  TEST INFRASTRUCTURE ONLY
 * (see sbo.h): the checker for the CUDA engine, never part of the product.
 *
 * Each function cites the reference file:line it restates.  Arithmetic is
 * written in the reference's evaluation order; the file is compiled with
 * -ffp-contract=off so that no multiply-add is fused.
 */
#include "sbo.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* (signbit(val) * -2) + 1, src/kernels.cu:40 and every other sign site. */
static inline int sgn(double v) { return signbit(v) ? -1 : 1; }

void sbo_rand_stream(uint32_t seed, int64_t count, int32_t *out)
{
    srand(seed);
    for (int64_t i = 0; i < count; i++) out[i] = rand();
}

/* src/ising.cu:103-125.  The reference multiplies nrows*nrows in int, which
 * overflows for n >= 46341; here the product is formed in double, which is
 * identical below that size. */
double sbo_xi0(const sbo_csr *J)
{
    double nn = (double)J->n * (double)J->n;
    double sum = 0.0;
    for (int64_t i = 0; i < J->nnz; i++) sum += J->val[i];
    double mean = sum / nn;
    double nonzero = 0.0;
    for (int64_t i = 0; i < J->nnz; i++) nonzero += pow(J->val[i] - mean, 2);
    double zero = (nn - (double)J->nnz) * mean * mean;
    sum = nonzero + zero;
    double sigma = pow(sum / (nn - 1.0), 0.5);
    return 0.7 / (sigma * pow((double)J->n, 0.5));
}

/* src/ising.cu:91-95: X then Y from one rand() stream, interleaved. */
void sbo_init_maxcut(int64_t n, int64_t A, uint32_t seed, double *x, double *y)
{
    srand(seed);
    for (int64_t i = 0; i < n * A; i++) {
        x[i] = (((double)rand() / RAND_MAX) * 2 - 1) / 10;
        y[i] = (((double)rand() / RAND_MAX) * 2 - 1) / 10;
    }
}

/* src/kernels.cu:8-22 (pressure not clamped). */
void sbo_update_xy(double *x, double *y, int64_t count, int32_t step,
                   int32_t max_steps, double dt)
{
    double p = 1.025 * (double)step / max_steps;
    for (int64_t i = 0; i < count; i++) {
        y[i] += dt * (p - 1) * x[i];
        x[i] += dt * (p + 1) * y[i];
    }
}

static double clamp_pressure(int32_t step, int32_t max_steps)
{
    double p = 1.025 * (double)step / max_steps;   /* kernels.cu:225-226 */
    return p < 1.0 ? p : 1.0;
}

/* One thread of symplectic_kernel_maxcut (src/kernels.cu:228-262) for
 * (row r, agent c), gathering signs through `sign_of(j)`. */
#define FUSED_THREAD(SIGN_OF_J)                                               \
    do {                                                                      \
        double *xr = &x[r * A + c], *yr = &y[r * A + c];                      \
        double val = *xr;                                                     \
        if (fabs(val) > 1) {                                                  \
            *xr = (double)sgn(val);                                           \
            *yr = 0;                                                          \
        } else {                                                              \
            double total = 0;                                                 \
            for (int32_t e = J->rowptr[r]; e < J->rowptr[r + 1]; e++) {       \
                int32_t j = J->col[e];                                        \
                total -= J->val[e] * (double)(SIGN_OF_J);                     \
            }                                                                 \
            *yr += dt * xi0 * total;                                          \
        }                                                                     \
        *xr += dt * (p + 1) * *yr;                                            \
        *yr += dt * (p - 1) * *xr;                                            \
    } while (0)

void sbo_fused_step(const sbo_csr *J, double *x, double *y, int64_t A,
                    int32_t step, int32_t max_steps, double dt, double xi0,
                    int schedule, int nthreads)
{
    const int64_t n = J->n;
    if (schedule == SBO_SERIAL) {
        /* CUDA linear order: thread (0,0) reads `step` and increments it
         * before any other thread reads it (kernels.cu:225,232). */
        for (int64_t r = 0; r < n; r++)
            for (int64_t c = 0; c < A; c++) {
                double p = clamp_pressure(r == 0 && c == 0 ? step : step + 1,
                                          max_steps);
                FUSED_THREAD(sgn(x[(int64_t)j * A + c]));
            }
        return;
    }
    /* Jacobi: all gathers see the signs at the start of the launch. */
    int8_t *s = (int8_t *)malloc((size_t)(n * A));
    for (int64_t i = 0; i < n * A; i++) s[i] = (int8_t)sgn(x[i]);
    const double p = clamp_pressure(step, max_steps);
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
    {
        double *total = (double *)malloc((size_t)A * sizeof(double));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t r = 0; r < n; r++) {
            /* Vectorised over agents; per agent the subtraction order over
             * the row's entries is the reference's (e ascending). */
            for (int64_t c = 0; c < A; c++) total[c] = 0;
            for (int32_t e = J->rowptr[r]; e < J->rowptr[r + 1]; e++) {
                const int8_t *sj = &s[(int64_t)J->col[e] * A];
                const double w = J->val[e];
                for (int64_t c = 0; c < A; c++) total[c] -= w * (double)sj[c];
            }
            for (int64_t c = 0; c < A; c++) {
                double *xr = &x[r * A + c], *yr = &y[r * A + c];
                double val = *xr;
                if (fabs(val) > 1) {
                    *xr = (double)sgn(val);
                    *yr = 0;
                } else {
                    *yr += dt * xi0 * total[c];
                }
                *xr += dt * (p + 1) * *yr;
                *yr += dt * (p - 1) * *xr;
            }
        }
        free(total);
    }
    free(s);
    (void)nthreads;
}

/* Unfused trio, one step (src/ising.cu:168-171): Update_XY (kernels.cu:8-22),
 * mat_mult (:178-209), confine (:150-167); the caller advances the step. */
void sbo_unfused_step(const sbo_csr *J, double *x, double *y, int64_t A,
                      int32_t step, int32_t max_steps, double dt, double xi0)
{
    const int64_t n = J->n;
    sbo_update_xy(x, y, n * A, step, max_steps, dt);
    int8_t *s = (int8_t *)malloc((size_t)(n * A));
    for (int64_t i = 0; i < n * A; i++) s[i] = (int8_t)sgn(x[i]);
    for (int64_t r = 0; r < n; r++)
        for (int64_t c = 0; c < A; c++) {
            double total = 0;
            for (int32_t e = J->rowptr[r]; e < J->rowptr[r + 1]; e++)
                total -= J->val[e] * (double)s[(int64_t)J->col[e] * A + c];
            y[r * A + c] += dt * xi0 * total;
        }
    for (int64_t i = 0; i < n * A; i++)
        if (fabs(x[i]) > 1) {
            x[i] = (double)sgn(x[i]);
            y[i] = 0;
        }
    free(s);
}

/* src/kernels.cu:24-91 with every read of current_spins taking the value of
 * the previous window.  (In the reference, rows >= 1 overwrite
 * current_spins (:84-90) while the row-0 thread may still be reading them
 * (:37-44); reading first is the order the kernel's comments describe.) */
void sbo_window(const double *x, int64_t n, int64_t A, int32_t *cur,
                int32_t *fin, uint8_t *bif, uint8_t *prev, int32_t *stab,
                int32_t threshold)
{
    for (int64_t c = 0; c < A; c++) {
        int64_t sum = 0;
        for (int64_t i = 0; i < n; i++) sum += sgn(x[i * A + c]) * cur[i * A + c];
        int equal = (sum == n);
        int not_equal = !equal;
        int not_bif = !bif[c];
        stab[c] += equal && not_bif;
        stab[c] = not_equal && not_bif ? 0 : stab[c];
        bif[c] = stab[c] == threshold - 1;
        int newb = bif[c] ^ prev[c];
        prev[c] = bif[c];
        if (newb)
            for (int64_t i = 0; i < n; i++) fin[i * A + c] = sgn(x[i * A + c]);
    }
    for (int64_t i = 0; i < n * A; i++) cur[i] = sgn(x[i]);
}

/* compute_max_cut + sum_max_cut, src/kernels.cu:360-400. */
void sbo_cut(const sbo_csr *J, const int32_t *spins, int64_t A, double *cut)
{
    const int64_t n = J->n;
    for (int64_t c = 0; c < A; c++) {
        double tmp = 0;
        for (int64_t r = 0; r < n; r++) {
            double rs = 0;
            for (int32_t e = J->rowptr[r]; e < J->rowptr[r + 1]; e++)
                rs += J->val[e] * spins[(int64_t)J->col[e] * A + c];
            tmp += rs * spins[r * A + c] * (0.5);
        }
        cut[c] = (-0.5) * (tmp - J->wsum);
    }
}

/* src/ising.cu:238-265. */
void sbo_stats(const double *v, int64_t A, sbo_result *r)
{
    double mx = -DBL_MAX, mn = DBL_MAX, total = 0, sd = 0;
    for (int64_t i = 0; i < A; i++) {
        if (v[i] > mx) mx = v[i];
        if (v[i] < mn) mn = v[i];
        total += v[i];
    }
    double avg = total / A;
    int64_t nmax = 0;
    for (int64_t i = 0; i < A; i++) {
        sd += pow(v[i] - avg, 2);
        if (v[i] == mx) nmax++;
    }
    r->min = mn;
    r->max = mx;
    r->mean = avg;
    r->std = pow(sd / (A - 1), 0.5);
    r->ps = (double)nmax / A;
}

/* src/ising.cu:85-271: reset, pre-step, graph launches of `period` steps plus
 * one window, optional early exit, final cut and statistics. */
int sbo_maxcut_solve(const sbo_csr *J, const sbo_params *p, sbo_result *r,
                     double *cut, double *xo, double *yo, int32_t *spins)
{
    const int64_t n = J->n, A = p->agents;
    if (n <= 0 || A <= 0 || p->steps < 0 || p->period <= 0) return -1;
    double *x = (double *)malloc((size_t)(n * A) * sizeof(double));
    double *y = (double *)malloc((size_t)(n * A) * sizeof(double));
    int32_t *cur = (int32_t *)malloc((size_t)(n * A) * sizeof(int32_t));
    int32_t *fin = (int32_t *)malloc((size_t)(n * A) * sizeof(int32_t));
    uint8_t *bif = (uint8_t *)calloc((size_t)A, 1);
    uint8_t *prev = (uint8_t *)calloc((size_t)A, 1);
    int32_t *stab = (int32_t *)calloc((size_t)A, sizeof(int32_t));
    double *cutv = (double *)malloc((size_t)A * sizeof(double));

    sbo_init_maxcut(n, A, p->seed, x, y);
    double xi0 = sbo_xi0(J);
    for (int64_t i = 0; i < n * A; i++) cur[i] = fin[i] = -1;

    int32_t dstep = 0;       /* the device step counter (step_gpu) */
    int64_t hstep = 0;       /* the host step counter (Ising::step) */
    int64_t windows = 0;
    sbo_update_xy(x, y, n * A, dstep, p->steps, p->dt);   /* ising.cu:188 */
    const int64_t limit = p->run_steps > 0 && p->run_steps < p->steps ? p->run_steps : p->steps;
    int run = hstep < limit;
    while (run) {
        for (int32_t i = 0; i < p->period; i++) {
            if (p->fused)
                sbo_fused_step(J, x, y, A, dstep, p->steps, p->dt, xi0,
                               p->schedule, p->nthreads);
            else
                sbo_unfused_step(J, x, y, A, dstep, p->steps, p->dt, xi0);
            dstep++;
        }
        sbo_window(x, n, A, cur, fin, bif, prev, stab, p->threshold);
        windows++;
        hstep += p->period;
        run = hstep < limit;
        if (p->uw) {
            int64_t nb = 0;
            for (int64_t c = 0; c < A; c++) nb += bif[c];
            if (nb == A) run = 0;
        }
    }
    sbo_cut(J, cur, A, cutv);
    sbo_stats(cutv, A, r);
    r->xi0 = xi0;
    r->steps_run = dstep;
    r->windows_run = windows;
    r->valid = 0;
    r->bifurcated = 0;
    for (int64_t c = 0; c < A; c++) r->bifurcated += bif[c];
    if (cut) memcpy(cut, cutv, (size_t)A * sizeof(double));
    if (xo) memcpy(xo, x, (size_t)(n * A) * sizeof(double));
    if (yo) memcpy(yo, y, (size_t)(n * A) * sizeof(double));
    if (spins) memcpy(spins, cur, (size_t)(n * A) * sizeof(int32_t));
    free(x); free(y); free(cur); free(fin); free(bif); free(prev); free(stab);
    free(cutv);
    return 0;
}
