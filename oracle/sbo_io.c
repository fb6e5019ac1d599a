/*
 * sbo_io.c -- oracle restatement of the reference's file loaders.  TEST
 * INFRASTRUCTURE ONLY (see sbo.h): the product's own loaders live in the
 * package; these are what they are checked against.
 *
 * The readers follow the reference's std::ifstream token logic (csr.cpp:15-109,
 * tsp_cpu.cpp:9-45), except that they return an error where the reference
 * loops forever on a missing file or a malformed header, and that rows without
 * entries keep their (empty) row pointer (csr.cpp:168-186 drops them).
 */
#define _GNU_SOURCE
#include "sbo.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    FILE *f;
} rd;

/* operator>>(std::string): skip whitespace, read up to the next whitespace. */
static int rd_word(rd *r, char *buf, size_t cap)
{
    int ch;
    do {
        ch = fgetc(r->f);
    } while (ch != EOF && isspace(ch));
    if (ch == EOF) return 0;
    size_t k = 0;
    while (ch != EOF && !isspace(ch)) {
        if (k + 1 < cap) buf[k++] = (char)ch;
        ch = fgetc(r->f);
    }
    if (ch != EOF) ungetc(ch, r->f);
    buf[k] = 0;
    return 1;
}

/* istream::ignore(2048, '\n'). */
static void rd_ignore_line(rd *r)
{
    int ch, k = 0;
    while (k < 2048 && (ch = fgetc(r->f)) != EOF) {
        k++;
        if (ch == '\n') break;
    }
}

static int rd_peek(rd *r)
{
    int ch = fgetc(r->f);
    if (ch != EOF) ungetc(ch, r->f);
    return ch;
}

static int rd_long(rd *r, long *v)
{
    char buf[128];
    if (!rd_word(r, buf, sizeof buf)) return 0;
    char *end;
    *v = strtol(buf, &end, 10);
    return end != buf;
}

static int rd_double(rd *r, double *v)
{
    char buf[128];
    if (!rd_word(r, buf, sizeof buf)) return 0;
    char *end;
    *v = strtod(buf, &end);
    return end != buf;
}

typedef struct {
    int32_t r, c;
    double v;
} trip;

static int trip_cmp(const void *a, const void *b)
{
    const trip *x = (const trip *)a, *y = (const trip *)b;
    if (x->r != y->r) return x->r < y->r ? -1 : 1;
    if (x->c != y->c) return x->c < y->c ? -1 : 1;
    if (x->v != y->v) return x->v < y->v ? -1 : 1;
    return 0;
}

/* construct_csr (csr.cpp:157-192): sort (row, col, value) tuples, then row
 * pointers; every row, including empty ones, gets its pointer. */
static void build_csr(int64_t n, trip *t, int64_t m, int32_t *rowptr,
                      int32_t *col, double *val)
{
    qsort(t, (size_t)m, sizeof(trip), trip_cmp);
    for (int64_t i = 0; i <= n; i++) rowptr[i] = 0;
    for (int64_t k = 0; k < m; k++) rowptr[t[k].r + 1]++;
    for (int64_t i = 0; i < n; i++) rowptr[i + 1] += rowptr[i];
    for (int64_t k = 0; k < m; k++) {
        col[k] = t[k].c;
        val[k] = t[k].v;
    }
}

int sbo_mtx_load(const char *path, int64_t *n_out, int64_t *nnz_out,
                 int32_t *rowptr, int32_t *col, double *val, double *wsum)
{
    rd r;
    r.f = fopen(path, "r");
    if (!r.f) return -1;
    int symmetric = 1, pattern = 0, found = 0;
    char w[4096];
    while (!found) {
        if (!rd_word(&r, w, sizeof w)) {
            fclose(r.f);
            return -2;
        }
        if (!strcmp(w, "symmetric")) { symmetric = 1; found = 1; }
        else if (!strcmp(w, "pattern")) pattern = 1;
        else if (!strcmp(w, "integer")) pattern = 0;
        else if (!strcmp(w, "general")) { symmetric = 0; found = 1; }
    }
    rd_ignore_line(&r);
    while (rd_peek(&r) == '%') rd_ignore_line(&r);
    long M, N, L;
    if (!rd_long(&r, &M) || !rd_long(&r, &N) || !rd_long(&r, &L) || M < 0 ||
        L < 0) {
        fclose(r.f);
        return -3;
    }
    (void)N;
    trip *t = (trip *)malloc(sizeof(trip) * (size_t)(2 * L + 1));
    int64_t m = 0;
    double sum = 0;
    for (long l = 0; l < L; l++) {
        long row, cl;
        double d = 1;
        if (!rd_long(&r, &row) || !rd_long(&r, &cl) ||
            (!pattern && !rd_double(&r, &d))) {
            free(t);
            fclose(r.f);
            return -4;
        }
        if (row < 1 || row > M || cl < 1 || cl > M) {
            free(t);
            fclose(r.f);
            return -5;
        }
        if (row != cl) {   /* diagonal dropped, csr.cpp:65,80 */
            t[m].r = (int32_t)(row - 1);
            t[m].c = (int32_t)(cl - 1);
            t[m].v = d;
            m++;
            sum += d;
        }
    }
    fclose(r.f);
    if (symmetric) {   /* mirror, csr.cpp:91-104 */
        int64_t m0 = m;
        for (int64_t i = 0; i < m0; i++)
            if (t[i].c != t[i].r) {
                t[m].r = t[i].c;
                t[m].c = t[i].r;
                t[m].v = t[i].v;
                m++;
            }
    }
    *n_out = M;
    *nnz_out = m;
    if (wsum) *wsum = sum;
    if (rowptr && col && val) build_csr(M, t, m, rowptr, col, val);
    free(t);
    return 0;
}

/* CSR::from_matrix (csr.cpp:137-155): every nonzero of a dense matrix. */
int64_t sbo_dense_to_csr(int64_t dim, const double *dense, int32_t *rowptr,
                         int32_t *col, double *val)
{
    int64_t m = 0;
    for (int64_t i = 0; i < dim * dim; i++)
        if (dense[i] != 0) m++;
    if (!rowptr) return m;
    trip *t = (trip *)malloc(sizeof(trip) * (size_t)(m + 1));
    int64_t k = 0;
    for (int64_t r = 0; r < dim; r++)
        for (int64_t c = 0; c < dim; c++) {
            double v = dense[r * dim + c];
            if (v != 0) {
                t[k].r = (int32_t)r;
                t[k].c = (int32_t)c;
                t[k].v = v;
                k++;
            }
        }
    build_csr(dim, t, m, rowptr, col, val);
    free(t);
    return m;
}

/* TSP_CPU::read_file, src/tsp_cpu.cpp:9-45. */
int sbo_tsplib_load(const char *path, int32_t *N_out, double *xc, double *yc,
                    int *kind)
{
    rd r;
    r.f = fopen(path, "r");
    if (!r.f) return -1;
    char w[4096];
    long N = 0;
    while (rd_peek(&r) != 'D') {
        if (rd_peek(&r) == EOF) goto bad;
        rd_ignore_line(&r);
    }
    /* "DIMENSION: 14" (the reference's only form) or "DIMENSION : 14". */
    if (!rd_word(&r, w, sizeof w)) goto bad;
    if (!strcmp(w, "DIMENSION") && !rd_word(&r, w, sizeof w)) goto bad;
    if (!rd_long(&r, &N) || N < 2) goto bad;
    while (rd_peek(&r) != 'E') {
        if (rd_peek(&r) == EOF) goto bad;
        rd_ignore_line(&r);
    }
    char dtype[64];
    if (!rd_word(&r, w, sizeof w)) goto bad;
    if (!strcmp(w, "EDGE_WEIGHT_TYPE") && !rd_word(&r, w, sizeof w)) goto bad;
    if (!rd_word(&r, dtype, sizeof dtype)) goto bad;
    if (!strcmp(dtype, "GEO")) *kind = SBO_DIST_GEO;
    else if (!strcmp(dtype, "EUC_2D")) *kind = SBO_DIST_EUC_2D;
    else goto bad;
    *N_out = (int32_t)N;
    if (!xc || !yc) {
        fclose(r.f);
        return 0;
    }
    while (rd_peek(&r) != '1') {
        if (rd_peek(&r) == EOF) goto bad;
        rd_ignore_line(&r);
    }
    const double PI = 3.14159265358979323846;
    for (long i = 0; i < N; i++) {
        double id, la, lo;
        if (!rd_double(&r, &id) || !rd_double(&r, &la) || !rd_double(&r, &lo))
            goto bad;
        if (*kind == SBO_DIST_GEO) {
            int lat_deg = (int)la, long_deg = (int)lo;
            double lat_min = la - lat_deg, long_min = lo - long_deg;
            la = PI * (lat_deg + 5.0 * lat_min / 3.0) / 180.0;
            lo = PI * (long_deg + 5.0 * long_min / 3.0) / 180.0;
        }
        xc[i] = la;
        yc[i] = lo;
    }
    fclose(r.f);
    return 0;
bad:
    fclose(r.f);
    return -2;
}
