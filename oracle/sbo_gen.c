/*
 * sbo_gen.c -- the seeded synthetic instances, restated for the oracle side.
 * TEST INFRASTRUCTURE ONLY (see sbo.h): it lets the CPU legs of the benchmark
 * and the tests build the same instances as the engine's generators
 * (sbx_gen_* in libsbx.so) without loading the engine.  The reference ships
 * no instances for its benchmarks (Gset, TSPLIB); these seeded graphs with
 * the benchmark configurations' shapes stand in for them.  A CPU test checks
 * that both sides produce identical CSR arrays, weight sums and cities.
 *
 * Every generator draws from splitmix64 (Steele, Lea, Flood 2014) seeded with
 * `seed`; uniform doubles are the top 53 bits.  Graphs are undirected edge
 * lists turned into a symmetric CSR sorted by (row, column); W is the sum of
 * the edge weights in generation order (the reference's csr.sum, one triangle).
 */
#include "sbo.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    uint64_t s;
} rng_t;

static uint64_t rng_next(rng_t *g)
{
    uint64_t z = (g->s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static double rng_uniform(rng_t *g) { return (double)(rng_next(g) >> 11) * (1.0 / 9007199254740992.0); }

typedef struct {
    int32_t r, c;
    double v;
} edge_t;

typedef struct {
    edge_t *e;
    int64_t n, cap;
} edges_t;

static int push(edges_t *E, int32_t r, int32_t c, double v)
{
    if (E->n == E->cap) {
        int64_t nc = E->cap ? E->cap * 2 : 1024;
        edge_t *ne = (edge_t *)realloc(E->e, (size_t)nc * sizeof(edge_t));
        if (!ne) return -1;
        E->e = ne;
        E->cap = nc;
    }
    E->e[E->n].r = r;
    E->e[E->n].c = c;
    E->e[E->n].v = v;
    E->n++;
    return 0;
}

/* Undirected edges (u != v, no duplicates) -> symmetric CSR sorted by (row,
 * column): a counting sort by column, then a stable one by row. */
static int finish(int64_t n, edges_t *E, sbo_graph *out)
{
    const int64_t m = E->n, nnz = 2 * m;
    double W = 0;
    for (int64_t i = 0; i < m; i++) W += E->e[i].v;
    int32_t *rp = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
    int32_t *col = (int32_t *)malloc((size_t)(nnz ? nnz : 1) * sizeof(int32_t));
    double *val = (double *)malloc((size_t)(nnz ? nnz : 1) * sizeof(double));
    edge_t *t = (edge_t *)malloc((size_t)(nnz ? nnz : 1) * sizeof(edge_t));
    edge_t *u = (edge_t *)malloc((size_t)(nnz ? nnz : 1) * sizeof(edge_t));
    int64_t *cnt = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
    if (!rp || !col || !val || !t || !u || !cnt) {
        free(rp); free(col); free(val); free(t); free(u); free(cnt);
        return -1;
    }
    for (int64_t i = 0; i < m; i++) {
        t[2 * i] = E->e[i];
        t[2 * i + 1].r = E->e[i].c;
        t[2 * i + 1].c = E->e[i].r;
        t[2 * i + 1].v = E->e[i].v;
    }
    /* by column */
    for (int64_t i = 0; i < nnz; i++) cnt[t[i].c + 1]++;
    for (int64_t i = 0; i < n; i++) cnt[i + 1] += cnt[i];
    for (int64_t i = 0; i < nnz; i++) u[cnt[t[i].c]++] = t[i];
    /* stable by row */
    memset(cnt, 0, ((size_t)n + 1) * sizeof(int64_t));
    for (int64_t i = 0; i < nnz; i++) cnt[u[i].r + 1]++;
    for (int64_t i = 0; i < n; i++) cnt[i + 1] += cnt[i];
    for (int64_t i = 0; i <= n; i++) rp[i] = (int32_t)cnt[i];
    for (int64_t i = 0; i < nnz; i++) {
        const int64_t k = cnt[u[i].r]++;
        col[k] = u[i].c;
        val[k] = u[i].v;
    }
    free(t); free(u); free(cnt);
    free(E->e);
    E->e = NULL;
    out->n = n;
    out->nnz = nnz;
    out->rowptr = rp;
    out->col = col;
    out->val = val;
    out->wsum = W;
    return 0;
}

void sbo_graph_free(sbo_graph *g)
{
    free(g->rowptr);
    free(g->col);
    free(g->val);
    g->rowptr = NULL;
    g->col = NULL;
    g->val = NULL;
}

/* Erdos-Renyi G(n, p): geometric skips over the pairs (i < j) in row-major
 * order; weight +1, or +-1 from the top bit of a draw when pm1. */
int sbo_gen_er(int64_t n, double p, int pm1, uint64_t seed, sbo_graph *out)
{
    if (n < 1 || !(p >= 0 && p <= 1)) return -1;
    rng_t g = {seed};
    edges_t E = {0};
    if (p > 0) {
        const double lq = log(1.0 - (p < 1.0 - 1e-15 ? p : 1.0 - 1e-15));
        int64_t i = 0, j = 0;
        for (;;) {
            const double u = rng_uniform(&g);
            const int64_t skip = p >= 1.0 ? 0 : (int64_t)floor(log(1.0 - u) / lq);
            j += skip + 1;
            while (i < n && j >= n) {
                j = j - n + i + 2;
                i++;
            }
            if (i >= n - 1) break;
            const double w = pm1 ? ((rng_next(&g) >> 63) ? 1.0 : -1.0) : 1.0;
            if (push(&E, (int32_t)i, (int32_t)j, w)) return -1;
        }
    }
    return finish(n, &E, out);
}

/* rows x cols torus: right and down neighbours, +-1 per edge. */
int sbo_gen_torus(int32_t rows, int32_t cols, uint64_t seed, sbo_graph *out)
{
    if (rows < 3 || cols < 3) return -1;
    rng_t g = {seed};
    edges_t E = {0};
    for (int32_t r = 0; r < rows; r++)
        for (int32_t c = 0; c < cols; c++) {
            const int32_t v = r * cols + c;
            const int32_t right = r * cols + (c + 1) % cols, down = ((r + 1) % rows) * cols + c;
            if (push(&E, v, right, (rng_next(&g) >> 63) ? 1.0 : -1.0)) return -1;
            if (push(&E, v, down, (rng_next(&g) >> 63) ? 1.0 : -1.0)) return -1;
        }
    return finish((int64_t)rows * cols, &E, out);
}

static int cmp_u64(const void *a, const void *b)
{
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : x > y;
}

/* R-MAT (Chakrabarti, Zhan, Faloutsos 2004): edge_factor * 2^scale draws of
 * `scale` quadrant choices (a, b, c, rest); self loops and duplicates
 * dropped; weights +1; isolated vertices kept as empty rows. */
int sbo_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c,
                 uint64_t seed, sbo_graph *out)
{
    if (scale < 1 || scale > 30 || edge_factor < 1) return -1;
    const int64_t n = (int64_t)1 << scale, m = (int64_t)edge_factor << scale;
    rng_t g = {seed};
    uint64_t *keys = (uint64_t *)malloc((size_t)m * sizeof(uint64_t));
    if (!keys) return -1;
    int64_t k = 0;
    for (int64_t e = 0; e < m; e++) {
        uint64_t u = 0, v = 0;
        for (int l = 0; l < scale; l++) {
            const double x = rng_uniform(&g);
            const int q = x < a ? 0 : x < a + b ? 1 : x < a + b + c ? 2 : 3;
            u = (u << 1) | (uint64_t)(q >> 1);
            v = (v << 1) | (uint64_t)(q & 1);
        }
        if (u == v) continue;
        const uint64_t lo = u < v ? u : v, hi = u < v ? v : u;
        keys[k++] = (lo << 32) | hi;
    }
    qsort(keys, (size_t)k, sizeof(uint64_t), cmp_u64);
    edges_t E = {0};
    for (int64_t i = 0; i < k; i++) {
        if (i > 0 && keys[i] == keys[i - 1]) continue;
        if (push(&E, (int32_t)(keys[i] >> 32), (int32_t)(keys[i] & 0xffffffffu), 1.0)) {
            free(keys);
            return -1;
        }
    }
    free(keys);
    return finish(n, &E, out);
}

static int cmp_edge(const void *a, const void *b)
{
    const edge_t *x = (const edge_t *)a, *y = (const edge_t *)b;
    if (x->r != y->r) return x->r < y->r ? -1 : 1;
    return x->c < y->c ? -1 : x->c > y->c;
}

/* Random geometric graph: n points uniform in the unit square, an edge when
 * two lie within the radius that gives avg_degree; the edges sorted by
 * (i, j) then given +-1 weights. */
int sbo_gen_rgg(int64_t n, double avg_degree, uint64_t seed, sbo_graph *out)
{
    if (n < 2 || !(avg_degree > 0)) return -1;
    rng_t g = {seed};
    double *px = (double *)malloc((size_t)n * sizeof(double));
    double *py = (double *)malloc((size_t)n * sizeof(double));
    if (!px || !py) {
        free(px); free(py);
        return -1;
    }
    for (int64_t i = 0; i < n; i++) {
        px[i] = rng_uniform(&g);
        py[i] = rng_uniform(&g);
    }
    const double rad = sqrt(avg_degree / ((double)n * 3.14159265358979323846));
    int cells = (int)floor(1.0 / rad);
    if (cells < 1) cells = 1;
    /* points bucketed by cell, in index order within a cell */
    int64_t *head = (int64_t *)calloc((size_t)cells * cells + 1, sizeof(int64_t));
    int32_t *pts = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *cell = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    for (int64_t i = 0; i < n; i++) {
        int cx = (int)(px[i] * cells), cy = (int)(py[i] * cells);
        if (cx > cells - 1) cx = cells - 1;
        if (cy > cells - 1) cy = cells - 1;
        cell[i] = cy * cells + cx;
        head[cell[i] + 1]++;
    }
    for (int64_t q = 0; q < (int64_t)cells * cells; q++) head[q + 1] += head[q];
    {
        int64_t *at = (int64_t *)malloc((size_t)cells * cells * sizeof(int64_t));
        memcpy(at, head, (size_t)cells * cells * sizeof(int64_t));
        for (int64_t i = 0; i < n; i++) pts[at[cell[i]]++] = (int32_t)i;
        free(at);
    }
    edges_t E = {0};
    const double r2 = rad * rad;
    for (int cy = 0; cy < cells; cy++)
        for (int cx = 0; cx < cells; cx++)
            for (int64_t a = head[cy * cells + cx]; a < head[cy * cells + cx + 1]; a++) {
                const int32_t i = pts[a];
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        const int nx = cx + dx, ny = cy + dy;
                        if (nx < 0 || ny < 0 || nx >= cells || ny >= cells) continue;
                        for (int64_t b = head[ny * cells + nx]; b < head[ny * cells + nx + 1]; b++) {
                            const int32_t j = pts[b];
                            if (j <= i) continue;
                            const double ddx = px[i] - px[j], ddy = py[i] - py[j];
                            if (ddx * ddx + ddy * ddy <= r2) push(&E, i, j, 0.0);
                        }
                    }
            }
    free(px); free(py); free(head); free(pts); free(cell);
    qsort(E.e, (size_t)E.n, sizeof(edge_t), cmp_edge);
    for (int64_t i = 0; i < E.n; i++) E.e[i].v = (rng_next(&g) >> 63) ? 1.0 : -1.0;
    return finish(n, &E, out);
}

/* N cities uniform in [0, scale)^2. */
int sbo_gen_cities(int32_t N, double scale, uint64_t seed, double *xc, double *yc)
{
    if (N < 2 || !(scale > 0)) return -1;
    rng_t g = {seed};
    for (int32_t i = 0; i < N; i++) {
        xc[i] = rng_uniform(&g) * scale;
        yc[i] = rng_uniform(&g) * scale;
    }
    return 0;
}
