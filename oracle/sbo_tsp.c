/*
 * sbo_tsp.c -- FP64 CPU oracle, TSP side.  TEST INFRASTRUCTURE ONLY (see
 * sbo.h): the checker for the CUDA engine, never part of the product.
 */
#include "sbo.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

static inline int sgn(double v) { return signbit(v) ? -1 : 1; }

/* Packed upper-triangular index of (c1 < c2), src/kernels.cu:420,439 and
 * src/ising_tsp.cu:283 (the same value as tsp_gpu.cu:80's formula). */
static inline int64_t packed_index(int64_t c1, int64_t c2, int64_t N)
{
    return c2 + (c1 * N) - ((c1 + 2) * (c1 + 1) / 2);
}

/* TSP_distances_EUC_2D / TSP_distances_GEO, src/kernels.cu:404-442, with the
 * reference's (int) truncation; SBO_DIST_EUC_2D_FLOAT keeps the double. */
int sbo_tsp_distances(int32_t N, const double *xc, const double *yc, int kind,
                      double *packed)
{
    if (N < 2) return -1;
    for (int32_t c1 = 0; c1 < N; c1++)
        for (int32_t c2 = c1 + 1; c2 < N; c2++) {
            double d;
            if (kind == SBO_DIST_GEO) {
                double R = 6378.388;
                double q1 = cos(yc[c1] - yc[c2]);
                double q2 = cos(xc[c1] - xc[c2]);
                double q3 = cos(xc[c1] + xc[c2]);
                d = (R * acos(0.5 * ((1.0 + q1) * q2 - (1.0 - q1) * q3)) + 1.0);
                d = (double)(int)d;
            } else {
                double xd = xc[c1] - xc[c2];
                double yd = yc[c1] - yc[c2];
                d = pow(xd * xd + yd * yd, 0.5);
                if (kind == SBO_DIST_EUC_2D) d = (double)(int)d;
            }
            packed[packed_index(c1, c2, N)] = d;
        }
    return 0;
}

/* src/tsp_gpu.cu:51-68: per-city distance sums, the maximum and the total,
 * walking the packed array in its storage order. */
void sbo_tsp_rowsums(int32_t N, const double *packed, double *rowsum,
                     double *maxd, double *sumd)
{
    int64_t nd = (int64_t)N * (N - 1) / 2;
    int32_t i = 0, j = 0;
    double mx = 0, sm = 0;
    for (int32_t k = 0; k < N; k++) rowsum[k] = 0;
    for (int64_t k = 0; k < nd; k++) {
        if (j == N - 1) {
            i++;
            j = i;
        }
        j++;
        double d = packed[k];
        rowsum[i] += d;
        rowsum[j] += d;
        sm += d;
        if (d > mx) mx = d;
    }
    *maxd = mx;
    *sumd = sm;
}

/* TSP_GPU::construct_matrix, src/tsp_gpu.cu:76-112: dense N^2 x N^2 QUBO,
 * row (position i, city k), column (position j, city l). */
int sbo_tsp_qubo_dense(int32_t N, const double *packed, double A, double B,
                       double C, double *dense)
{
    if (N < 2) return -1;
    int64_t m = (int64_t)N * N, idx = 0;
    for (int32_t i = 0; i < N; i++)
        for (int32_t k = 0; k < N; k++)
            for (int32_t j = 0; j < N; j++)
                for (int32_t l = 0; l < N; l++) {
                    double v;
                    int adj = (i == j + 1 || j == i + 1 || (i == 0 && j == N - 1) ||
                               (i == N - 1 && j == 0));
                    if (i != j && k == l) {
                        v = C / 4;
                    } else if (adj && k != l) {
                        int32_t c1 = k < l ? k : l, c2 = k < l ? l : k;
                        int64_t pos = ((2 * (int64_t)N - c1 - 3) * c1) / 2 + c2 - 1;
                        v = A * packed[pos] / 8;
                    } else if (i == j && k != l) {
                        v = B / 4;
                    } else if (i == j && k == l) {
                        v = (B + C) / 4;
                    } else {
                        v = 0;
                    }
                    dense[idx++] = v;
                }
    (void)m;
    return 0;
}

/* src/ising_tsp.cu:55-59: X = 0, Y from rand(). */
void sbo_init_tsp(int64_t n, int64_t A, uint32_t seed, double *x, double *y)
{
    srand(seed);
    for (int64_t i = 0; i < n * A; i++) {
        x[i] = 0;
        y[i] = (((double)rand() / RAND_MAX) * 2 - 1) / 10;
    }
}

/* One thread of symplectic_kernel_tsp, src/kernels.cu:553-597. */
static void tsp_thread(const sbo_csr *J, const double *rowsum, double *x,
                       double *y, const double *xg, int64_t A, int64_t r,
                       int64_t c, int32_t step, int32_t max_steps, double dt,
                       double xi0, int32_t N, double qa, double qb, double qc)
{
    const int n = 2;   /* ising_tsp.cu:134 */
    double a_t = n * 1.04 * (double)step / max_steps;
    double b_t = 0.5 + ((double)0.5 * pow((double)step / (double)max_steps, 1.9));
    a_t = a_t < n ? a_t : n;
    b_t = b_t < 1 ? b_t : 1;
    double *xr = &x[r * A + c], *yr = &y[r * A + c];
    double val = *xr;
    if (fabs(val) > 1) {
        *xr = (double)sgn(val);
        *yr = 0;
        return;
    }
    double i1 = 0;
    for (int32_t e = J->rowptr[r]; e < J->rowptr[r + 1]; e++) {
        double xv = xg[(int64_t)J->col[e] * A + c];
        double act = xv * 1.005;
        i1 -= J->val[e] * act;
    }
    int32_t city = (int32_t)(r % N);
    double i2 = -1 * (qa * rowsum[city] + (N - 2) * (qb + qc)) / 2;
    *yr += dt * (xi0 * (2 * i1 + b_t * i2));
    *xr += dt * 1 * *yr;
    *yr += dt * -(1 - a_t) * *xr;
}

void sbo_tsp_step(const sbo_csr *J, const double *rowsum, double *x, double *y,
                  int64_t A, int32_t step, int32_t max_steps, double dt,
                  double xi0, int32_t N, double qa, double qb, double qc,
                  int schedule)
{
    const int64_t n = J->n;
    if (schedule == SBO_SERIAL) {
        for (int64_t r = 0; r < n; r++)
            for (int64_t c = 0; c < A; c++)
                tsp_thread(J, rowsum, x, y, x, A, r, c,
                           r == 0 && c == 0 ? step : step + 1, max_steps, dt,
                           xi0, N, qa, qb, qc);
        return;
    }
    double *x0 = (double *)malloc((size_t)(n * A) * sizeof(double));
    memcpy(x0, x, (size_t)(n * A) * sizeof(double));
    /* Jacobi: every (row, agent) reads x0 only, so rows run in parallel */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 8)
#endif
    for (int64_t r = 0; r < n; r++)
        for (int64_t c = 0; c < A; c++)
            tsp_thread(J, rowsum, x, y, x0, A, r, c, step, max_steps, dt, xi0,
                       N, qa, qb, qc);
    free(x0);
}

/* update_window_tsp, src/kernels.cu:461-541 (current_spins read before they
 * are rewritten, as in sbo_window). */
void sbo_tsp_window(const double *x, int64_t A, int32_t N, int32_t *cur,
                    int32_t *fin, uint8_t *bif, uint8_t *prev, int32_t *stab,
                    int32_t *valid_list, int32_t step, int32_t threshold)
{
    const int64_t n = (int64_t)N * N;
    int32_t *cv = (int32_t *)calloc((size_t)N, sizeof(int32_t));
    int32_t *ov = (int32_t *)calloc((size_t)N, sizeof(int32_t));
    for (int64_t c = 0; c < A; c++) {
        int valid = 1;
        int64_t sum = 0;
        for (int64_t i = 0; i < n; i++) {
            int s = sgn(x[i * A + c]);
            sum += s * cur[i * A + c];
            if (s == 1) {
                int64_t cc = i % N;
                int64_t rr = (i - cc) / N;
                cv[cc] += 1;
                ov[rr] += 1;
            }
        }
        for (int32_t i = 0; i < N; i++)
            if (cv[i] != 1 || ov[i] != 1) {
                valid = 0;
                break;
            }
        for (int32_t i = 0; i < N; i++) cv[i] = ov[i] = 0;
        int equal = (sum == n);
        int not_equal = !equal;
        int not_bif = !bif[c];
        stab[c] += equal && not_bif;
        stab[c] = not_equal && not_bif ? 0 : stab[c];
        bif[c] = stab[c] == threshold - 1;
        prev[c] = bif[c];
        if (valid) {
            valid_list[c] = step;
            for (int64_t i = 0; i < n; i++) fin[i * A + c] = sgn(x[i * A + c]);
        }
    }
    for (int64_t i = 0; i < n * A; i++) cur[i] = sgn(x[i]);
    free(cv);
    free(ov);
}

/* Ising_TSP::calculate_distance_of_tour, src/ising_tsp.cu:272-287. */
double sbo_tsp_tour_length(int32_t N, const double *packed, const int32_t *tour)
{
    double sum = 0.0;
    for (int32_t i = 0; i < N; i++) {
        int32_t a = tour[i], b = tour[i == N - 1 ? 0 : i + 1];
        int32_t c1 = a < b ? a : b, c2 = a < b ? b : a;
        sum += packed[packed_index(c1, c2, N)];
    }
    return sum;
}

/* Ising_TSP::reset_initialization + symplectic_update,
 * src/ising_tsp.cu:50-253. */
int sbo_tsp_solve(const sbo_csr *J, int32_t N, const double *packed,
                  const double *rowsum, double qa, double qb, double qc,
                  const sbo_params *p, sbo_result *r, double *lengths,
                  int32_t *tours, double *xo, double *yo, int32_t *valid_out)
{
    const int64_t n = (int64_t)N * N, A = p->agents;
    if (N < 2 || J->n != n || A <= 0 || p->steps < 0) return -1;
    /* period = max_steps / 10 (ising_tsp.cu:132); 1..9 steps never end in
     * the reference (the host loop adds 0 each launch) and are refused. */
    const int32_t period = p->steps / 10;
    if (p->steps > 0 && period == 0) return -1;
    double *x = (double *)malloc((size_t)(n * A) * sizeof(double));
    double *y = (double *)malloc((size_t)(n * A) * sizeof(double));
    int32_t *cur = (int32_t *)malloc((size_t)(n * A) * sizeof(int32_t));
    int32_t *fin = (int32_t *)malloc((size_t)(n * A) * sizeof(int32_t));
    uint8_t *bif = (uint8_t *)calloc((size_t)A, 1);
    uint8_t *prev = (uint8_t *)calloc((size_t)A, 1);
    int32_t *stab = (int32_t *)calloc((size_t)A, sizeof(int32_t));
    int32_t *vl = (int32_t *)calloc((size_t)A, sizeof(int32_t));

    sbo_init_tsp(n, A, p->seed, x, y);
    const double xi0 = 0.002;   /* ising_tsp.cu:61 */
    for (int64_t i = 0; i < n * A; i++) cur[i] = fin[i] = -1;

    int32_t dstep = 0;
    int64_t hstep = 0, windows = 0;
    sbo_update_xy(x, y, n * A, dstep, p->steps, p->dt);   /* ising_tsp.cu:155 */
    int run = 1;
    while (run) {
        for (int32_t i = 0; i < period; i++) {
            sbo_tsp_step(J, rowsum, x, y, A, dstep, p->steps, p->dt, xi0, N,
                         qa, qb, qc, p->schedule);
            dstep++;
        }
        sbo_tsp_window(x, A, N, cur, fin, bif, prev, stab, vl, dstep,
                       p->threshold);
        windows++;
        hstep += period;
        run = hstep < p->steps;
    }

    /* Decode (ising_tsp.cu:188-239). */
    int64_t nvalid = 0;
    double total = 0, mn = DBL_MAX, mx = -DBL_MAX;
    double *all = (double *)malloc((size_t)A * sizeof(double));
    int32_t *tour = (int32_t *)malloc((size_t)N * sizeof(int32_t));
    for (int64_t c = 0; c < A; c++) {
        if (lengths) lengths[c] = NAN;
        if (vl[c] <= 0) continue;
        int32_t k = 0;
        for (int32_t order = 0; order < N; order++)
            for (int32_t city = 0; city < N; city++)
                if (fin[((int64_t)order * N + city) * A + c] == 1) tour[k++] = city;
        double d = sbo_tsp_tour_length(N, packed, tour);
        all[nvalid++] = d;
        total += d;
        if (d < mn) mn = d;
        if (d > mx) mx = d;
        if (lengths) lengths[c] = d;
        if (tours) memcpy(&tours[c * N], tour, (size_t)N * sizeof(int32_t));
    }
    double avg = total / nvalid, sd = 0;
    for (int64_t i = 0; i < nvalid; i++) sd += pow(all[i] - avg, 2);
    sd = pow(sd / (nvalid - 1), 0.5);
    r->min = mn;
    r->max = mx;
    r->mean = avg;
    r->std = sd;
    r->ps = 0;
    r->xi0 = xi0;
    r->steps_run = dstep;
    r->windows_run = windows;
    r->valid = nvalid;
    r->bifurcated = 0;
    for (int64_t c = 0; c < A; c++) r->bifurcated += bif[c];
    if (xo) memcpy(xo, x, (size_t)(n * A) * sizeof(double));
    if (yo) memcpy(yo, y, (size_t)(n * A) * sizeof(double));
    if (valid_out) memcpy(valid_out, vl, (size_t)A * sizeof(int32_t));
    free(all); free(tour);
    free(x); free(y); free(cur); free(fin); free(bif); free(prev); free(stab);
    free(vl);
    return 0;
}
