/*
 * sbo_lp.c -- CPU oracle of the engine's lower-precision MaxCut modes.
 * TEST INFRASTRUCTURE ONLY (see sbo.h): the checker for the CUDA engine,
 * never part of the product.
 *
 * The reference computes in FP64 only.  Its FP32, BF16 and FP16 state modes
 * are the engine's, so this file states the arithmetic those modes are
 * defined to perform, on the reference's algorithm:
 *   - src/ising.cu:91-95     init: the double value of the rand() stream,
 *                            rounded to float, then to the storage type;
 *   - src/kernels.cu:8-22    Update_XY: y = fmaf(c_w, x, y); x = fmaf(c_z, y, x)
 *                            with c_z = (float)(dt (p+1)), c_w = (float)(dt (p-1));
 *   - src/kernels.cu:211-269 fused step: force F = -sum_j J_ij s_j (float,
 *                            the row's entries in order), K = fmaf(c0, F, y)
 *                            with c0 = (float)(dt xi0); if |x| > 1 then
 *                            x = +-1, y = 0 else y = K; x = fmaf(c_x, y, x);
 *                            y = fmaf(c_y, x, y) with c_x, c_y of the clamped
 *                            pressure;
 *   - src/kernels.cu:150-209 unfused trio: Update_XY(k), force, clamp;
 *   - src/kernels.cu:24-91   window, src/kernels.cu:360-400 cut (exact).
 * x and y are rounded to the storage type (round to nearest even) each time
 * the engine stores them: after the pre-step, after every fused step, and in
 * the unfused mode after each window's opening Update_XY and after each
 * force + clamp (merged with the next step's Update_XY inside a window).
 * Every sign is read from the stored value.  fmaf is the correctly rounded
 * fused multiply-add of C99; the file is compiled with -ffp-contract=off, so
 * nothing else is fused.
 */
#include "sbo.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline uint32_t f2u(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static inline float u2f(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}

/* float -> bfloat16 (round to nearest even), returned as the float it
 * denotes.  bfloat16 keeps float's exponent, so the rounding is an integer
 * rounding of the low 16 bits, subnormals included.  No NaN reaches it. */
static inline float round_bf16(float f)
{
    uint32_t u = f2u(f);
    u += 0x7fffu + ((u >> 16) & 1u);
    return u2f(u & 0xffff0000u);
}

/* float -> binary16 (round to nearest even) -> float. */
static inline float round_f16(float f)
{
    const uint32_t u = f2u(f);
    const uint32_t sign = u & 0x80000000u;
    const uint32_t a = u & 0x7fffffffu;
    if (a >= 0x7f800000u) return f;                       /* inf (no NaN here) */
    if (a >= 0x477ff000u) return u2f(sign | 0x7f800000u); /* >= 65520: inf */
    if (a < 0x38800000u) {
        /* below 2^-14: multiples of 2^-24, ties to even (rint) */
        const double q = rint((double)u2f(a) * 16777216.0);
        const float v = (float)(q / 16777216.0);
        return u2f(sign | f2u(v));
    }
    /* normal: keep 10 mantissa bits, ties to even */
    uint32_t r = a + 0xfffu + ((a >> 13) & 1u);
    r &= 0xffffe000u;
    return u2f(sign | r);
}

float sbo_round_storage(int prec, float v)
{
    if (prec == SBO_BF16) return round_bf16(v);
    if (prec == SBO_F16) return round_f16(v);
    return v;
}

static inline int sgnf(float v) { return signbit(v) ? -1 : 1; }
static inline float spinf(float v) { return signbit(v) ? -1.0f : 1.0f; }

/* src/ising.cu:91-95, each value rounded as the engine stores it. */
void sbo_init_maxcut_lp(int64_t n, int64_t A, uint32_t seed, int prec, float *x,
                        float *y)
{
    srand(seed);
    for (int64_t i = 0; i < n * A; i++) {
        const double xv = (((double)rand() / RAND_MAX) * 2 - 1) / 10;
        const double yv = (((double)rand() / RAND_MAX) * 2 - 1) / 10;
        x[i] = sbo_round_storage(prec, (float)xv);
        y[i] = sbo_round_storage(prec, (float)yv);
    }
}

/* dt (p+1), dt (p-1) of step k in float; p = 1.025 k / max_steps
 * (src/kernels.cu:15), clamped at 1 when `clamp` (src/kernels.cu:225-226). */
static void coef(int32_t k, int32_t max_steps, double dt, int clamp, float *cp,
                 float *cm)
{
    double p = 1.025 * (double)k / max_steps;
    if (clamp) p = p < 1.0 ? p : 1.0;
    *cp = (float)(dt * (p + 1));
    *cm = (float)(dt * (p - 1));
}

/* Update_XY of step k over count values, rounded (src/kernels.cu:8-22). */
void sbo_update_xy_lp(float *x, float *y, int64_t count, int32_t step,
                      int32_t max_steps, double dt, int prec)
{
    float cz, cw;
    coef(step, max_steps, dt, 0, &cz, &cw);
    for (int64_t i = 0; i < count; i++) {
        const float yv = fmaf(cw, x[i], y[i]);
        const float xv = fmaf(cz, yv, x[i]);
        y[i] = sbo_round_storage(prec, yv);
        x[i] = sbo_round_storage(prec, xv);
    }
}

/* The force of every (row, agent) from the signs s (Jacobi), then the
 * fused step (mode 0) or the unfused force + clamp with, when xy_next, the
 * next step's Update_XY (mode 1); one rounding per value at the end. */
static void step_lp(const sbo_csr *J, float *x, float *y, int64_t A,
                    const int8_t *s, int32_t step, int32_t max_steps, double dt,
                    double xi0, int prec, int fused, int xy_next, int nthreads)
{
    const int64_t n = J->n;
    const float c0 = (float)(dt * xi0);
    float cx, cy, nz = 0, nw = 0;
    coef(step, max_steps, dt, 1, &cx, &cy);
    if (!fused && xy_next) coef(step + 1, max_steps, dt, 0, &nz, &nw);
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
    {
        float *tot = (float *)malloc((size_t)A * sizeof(float));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t r = 0; r < n; r++) {
            for (int64_t c = 0; c < A; c++) tot[c] = 0.0f;
            for (int32_t e = J->rowptr[r]; e < J->rowptr[r + 1]; e++) {
                const int8_t *sj = &s[(int64_t)J->col[e] * A];
                const float w = (float)J->val[e];
                for (int64_t c = 0; c < A; c++) tot[c] = tot[c] - w * (float)sj[c];
            }
            for (int64_t c = 0; c < A; c++) {
                float xv = x[r * A + c], yv = y[r * A + c];
                const float k = fmaf(c0, tot[c], yv);
                const int clamp = fabsf(xv) > 1.0f;
                yv = clamp ? 0.0f : k;
                xv = clamp ? spinf(xv) : xv;
                if (fused) {
                    xv = fmaf(cx, yv, xv);
                    yv = fmaf(cy, xv, yv);
                } else if (xy_next) {
                    yv = fmaf(nw, xv, yv);
                    xv = fmaf(nz, yv, xv);
                }
                x[r * A + c] = sbo_round_storage(prec, xv);
                y[r * A + c] = sbo_round_storage(prec, yv);
            }
        }
        free(tot);
    }
    (void)nthreads;
}

static void signs_of(const float *x, int64_t count, int8_t *s)
{
    for (int64_t i = 0; i < count; i++) s[i] = (int8_t)sgnf(x[i]);
}

/* src/kernels.cu:24-91 on stored values, every read of current_spins taking
 * the previous window's value (as sbo_window). */
static void window_lp(const float *x, int64_t n, int64_t A, int32_t *cur, int32_t *fin,
                      uint8_t *bif, uint8_t *prev, int32_t *stab, int32_t threshold)
{
    for (int64_t c = 0; c < A; c++) {
        int64_t sum = 0;
        for (int64_t i = 0; i < n; i++) sum += sgnf(x[i * A + c]) * cur[i * A + c];
        const int equal = (sum == n);
        const int not_bif = !bif[c];
        stab[c] += equal && not_bif;
        stab[c] = !equal && not_bif ? 0 : stab[c];
        bif[c] = stab[c] == threshold - 1;
        const int newb = bif[c] ^ prev[c];
        prev[c] = bif[c];
        if (newb)
            for (int64_t i = 0; i < n; i++) fin[i * A + c] = sgnf(x[i * A + c]);
    }
    for (int64_t i = 0; i < n * A; i++) cur[i] = sgnf(x[i]);
}

/* src/ising.cu:85-271 in the engine's storage precision `prec`: the same
 * orchestration as sbo_maxcut_solve (pre-step, windows of `period` steps,
 * optional early exit, cut of current_spins, statistics). */
int sbo_maxcut_solve_lp(const sbo_csr *J, const sbo_params *p, int prec,
                        sbo_result *r, double *cut, float *xo, float *yo,
                        int32_t *spins)
{
    const int64_t n = J->n, A = p->agents;
    if (n <= 0 || A <= 0 || p->steps < 0 || p->period <= 0) return -1;
    if (prec != SBO_F32 && prec != SBO_BF16 && prec != SBO_F16) return -1;
    float *x = (float *)malloc((size_t)(n * A) * sizeof(float));
    float *y = (float *)malloc((size_t)(n * A) * sizeof(float));
    int8_t *s = (int8_t *)malloc((size_t)(n * A));
    int32_t *cur = (int32_t *)malloc((size_t)(n * A) * sizeof(int32_t));
    int32_t *fin = (int32_t *)malloc((size_t)(n * A) * sizeof(int32_t));
    uint8_t *bif = (uint8_t *)calloc((size_t)A, 1);
    uint8_t *prev = (uint8_t *)calloc((size_t)A, 1);
    int32_t *stab = (int32_t *)calloc((size_t)A, sizeof(int32_t));
    double *cutv = (double *)malloc((size_t)A * sizeof(double));

    sbo_init_maxcut_lp(n, A, p->seed, prec, x, y);
    const double xi0 = sbo_xi0(J);
    for (int64_t i = 0; i < n * A; i++) cur[i] = fin[i] = -1;

    int32_t dstep = 0;
    int64_t hstep = 0, windows = 0;
    const int64_t limit = p->run_steps > 0 && p->run_steps < p->steps ? p->run_steps : p->steps;
    sbo_update_xy_lp(x, y, n * A, dstep, p->steps, p->dt, prec);   /* ising.cu:188 */
    int run = hstep < limit;
    while (run) {
        /* unfused: each window opens with Update_XY of its first step, stored */
        if (!p->fused) sbo_update_xy_lp(x, y, n * A, dstep, p->steps, p->dt, prec);
        for (int32_t i = 0; i < p->period; i++) {
            signs_of(x, n * A, s);
            step_lp(J, x, y, A, s, dstep, p->steps, p->dt, xi0, prec, p->fused,
                    i < p->period - 1, p->nthreads);
            dstep++;
        }
        window_lp(x, n, A, cur, fin, bif, prev, stab, p->threshold);
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
    if (xo) memcpy(xo, x, (size_t)(n * A) * sizeof(float));
    if (yo) memcpy(yo, y, (size_t)(n * A) * sizeof(float));
    if (spins) memcpy(spins, cur, (size_t)(n * A) * sizeof(int32_t));
    free(x); free(y); free(s); free(cur); free(fin); free(bif); free(prev); free(stab);
    free(cutv);
    return 0;
}
