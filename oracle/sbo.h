/*
 * sbo.h -- FP64 CPU oracle for the simulated-bifurcation (SB) hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py call it to
 * produce the expected results.  Nothing in the product (libsbx.so, the
 * `program` CLI) links or calls it.
 *
 * It restates, in plain C and FP64, the reference Sparse-Ising-Solver path:
 *   - src/kernels.cu:8-22      Update_XY            -> sbo_update_xy
 *   - src/kernels.cu:211-269   fused MaxCut step    -> sbo_fused_step
 *   - src/kernels.cu:150-209   unfused step trio    -> sbo_unfused_step
 *   - src/kernels.cu:24-91     bifurcation window   -> sbo_window
 *   - src/kernels.cu:360-400   cut evaluation       -> sbo_cut
 *   - src/ising.cu:85-138      init + xi0           -> sbo_init_maxcut, sbo_xi0
 *   - src/ising.cu:140-271     orchestration/stats  -> sbo_maxcut_solve
 *   - src/kernels.cu:543-599   TSP bSB step         -> sbo_tsp_step
 *   - src/kernels.cu:461-541   TSP validity window  -> sbo_tsp_window
 *   - src/kernels.cu:404-442   TSP distances        -> sbo_tsp_distances
 *   - src/tsp_gpu.cu:51-112    row sums + QUBO      -> sbo_tsp_rowsums, sbo_tsp_qubo_dense
 *   - src/ising_tsp.cu:50-287  TSP orchestration    -> sbo_tsp_solve
 *   - src/csr.cpp:15-192       MTX loader, CSR      -> sbo_mtx_load, sbo_dense_to_csr
 *   - src/tsp_cpu.cpp:9-45     TSPLIB loader        -> sbo_tsplib_load
 * and, in sbo_lp.c, the same MaxCut path in the engine's FP32 / BF16 / FP16
 * state modes (float arithmetic, rounded to the storage type on each store).
 *
 * Floating-point semantics: every operation is a separately rounded IEEE
 * double operation in the order the reference source writes it (the library
 * is compiled with -ffp-contract=off).  Parity is pinned by running the
 * reference's own kernels.cu (compiled for the CPU through a CUDA-emulation
 * header) and its own csr.cpp / tsp_cpu.cpp against this file, bit for bit.
 *
 * Execution schedule of the racy reference kernels: the reference updates X
 * in place while other threads gather it, and thread (0,0) increments the
 * step counter that the other threads read (src/kernels.cu:225-262).  The
 * oracle offers two legal schedules of that kernel:
 *   SBO_JACOBI  every thread reads the state as it was when the launch began
 *               (the semantics of the CUDA engine);
 *   SBO_SERIAL  threads run one after another in CUDA's linear order
 *               (rows ascending), so later rows see earlier rows' updates and
 *               every thread but (0,0) sees the incremented step counter.
 */
#ifndef SBO_H
#define SBO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { SBO_JACOBI = 0, SBO_SERIAL = 1 };

/* TSP distance kinds (src/kernels.cu:404-442, src/tsp_cpu.cpp:33-38). */
enum { SBO_DIST_EUC_2D = 0,       /* (int) truncation, as the reference */
       SBO_DIST_GEO = 1,          /* (int) truncation, as the reference */
       SBO_DIST_EUC_2D_FLOAT = 2  /* no truncation (unit-square instances) */ };

typedef struct {
    int64_t n;             /* rows (spins) */
    int64_t nnz;           /* stored entries, both triangles */
    const int32_t *rowptr; /* n+1 */
    const int32_t *col;    /* nnz */
    const double *val;     /* nnz */
    double wsum;           /* W: sum of file weights (one triangle), csr.cpp:69,84 */
} sbo_csr;

typedef struct {
    double dt;             /* time step */
    int32_t steps;         /* max_steps */
    int32_t agents;        /* columns of X */
    int32_t fused;         /* 1: symplectic_kernel_maxcut, 0: unfused trio */
    int32_t uw;            /* update-window early exit (MaxCut) */
    int32_t period;        /* steps per window (MaxCut reference: 100) */
    int32_t threshold;     /* convergence threshold (MaxCut 25, TSP 50) */
    uint32_t seed;         /* srand() seed */
    int32_t schedule;      /* SBO_JACOBI or SBO_SERIAL */
    int32_t nthreads;      /* OpenMP threads for SBO_JACOBI (<=0: all) */
    int32_t run_steps;     /* run only the windows covering the first
                              run_steps steps of the `steps` schedule
                              (0: all of them) */
} sbo_params;

typedef struct {
    double min, max, mean, std, ps;   /* ising.cu:238-265 */
    double xi0;
    int64_t steps_run;                /* SB steps executed after the pre-step */
    int64_t windows_run;
    int64_t bifurcated;               /* agents with bifurcated flag set */
    int64_t valid;                    /* TSP: agents with a valid tour */
} sbo_result;

/* ---- random numbers: glibc srand()/rand(), as the reference uses ---- */
void sbo_rand_stream(uint32_t seed, int64_t count, int32_t *out);

/* ---- MaxCut ---- */
double sbo_xi0(const sbo_csr *J);
void sbo_init_maxcut(int64_t n, int64_t A, uint32_t seed, double *x, double *y);
void sbo_update_xy(double *x, double *y, int64_t count, int32_t step,
                   int32_t max_steps, double dt);
void sbo_fused_step(const sbo_csr *J, double *x, double *y, int64_t A,
                    int32_t step, int32_t max_steps, double dt, double xi0,
                    int schedule, int nthreads);
void sbo_unfused_step(const sbo_csr *J, double *x, double *y, int64_t A,
                      int32_t step, int32_t max_steps, double dt, double xi0);
void sbo_window(const double *x, int64_t n, int64_t A, int32_t *cur,
                int32_t *fin, uint8_t *bif, uint8_t *prev, int32_t *stab,
                int32_t threshold);
void sbo_cut(const sbo_csr *J, const int32_t *spins, int64_t A, double *cut);
void sbo_stats(const double *v, int64_t A, sbo_result *r);
/* Full MaxCut run (ising.cu:85-271).  x, y, spins may be NULL; when given
 * they receive the final state (n*A each) and current_spins. */
int sbo_maxcut_solve(const sbo_csr *J, const sbo_params *p, sbo_result *r,
                     double *cut, double *x, double *y, int32_t *spins);

/* ---- MaxCut in the engine's lower-precision state modes (sbo_lp.c) ---- */
/* Storage precisions (the engine's SBX_F32, SBX_BF16, SBX_F16 values). */
enum { SBO_F32 = 0, SBO_BF16 = 1, SBO_F16 = 2 };
float sbo_round_storage(int prec, float v);
void sbo_init_maxcut_lp(int64_t n, int64_t A, uint32_t seed, int prec, float *x,
                        float *y);
void sbo_update_xy_lp(float *x, float *y, int64_t count, int32_t step,
                      int32_t max_steps, double dt, int prec);
/* As sbo_maxcut_solve, with float state rounded to `prec` on every store;
 * x, y (n*A floats) and spins may be NULL. */
int sbo_maxcut_solve_lp(const sbo_csr *J, const sbo_params *p, int prec,
                        sbo_result *r, double *cut, float *x, float *y,
                        int32_t *spins);

/* ---- TSP ---- */
int sbo_tsp_distances(int32_t N, const double *xc, const double *yc, int kind,
                      double *packed);
void sbo_tsp_rowsums(int32_t N, const double *packed, double *rowsum,
                     double *maxd, double *sumd);
int sbo_tsp_qubo_dense(int32_t N, const double *packed, double A, double B,
                       double C, double *dense);
void sbo_init_tsp(int64_t n, int64_t A, uint32_t seed, double *x, double *y);
void sbo_tsp_step(const sbo_csr *J, const double *rowsum, double *x, double *y,
                  int64_t A, int32_t step, int32_t max_steps, double dt,
                  double xi0, int32_t N, double qa, double qb, double qc,
                  int schedule);
void sbo_tsp_window(const double *x, int64_t A, int32_t N, int32_t *cur,
                    int32_t *fin, uint8_t *bif, uint8_t *prev, int32_t *stab,
                    int32_t *valid_list, int32_t step, int32_t threshold);
double sbo_tsp_tour_length(int32_t N, const double *packed, const int32_t *tour);
/* Full TSP run (ising_tsp.cu:50-253).  lengths[A] receives each agent's tour
 * length (NaN for agents without a valid tour); tours[A*N] the city order. */
int sbo_tsp_solve(const sbo_csr *J, int32_t N, const double *packed,
                  const double *rowsum, double qa, double qb, double qc,
                  const sbo_params *p, sbo_result *r, double *lengths,
                  int32_t *tours, double *x, double *y, int32_t *valid_list);

/* ---- seeded synthetic instances (sbo_gen.c) ---- */
/* A generated graph: arrays malloc'ed by the generator, freed by
 * sbo_graph_free. */
typedef struct {
    int64_t n, nnz;
    int32_t *rowptr, *col;
    double *val;
    double wsum;
} sbo_graph;
void sbo_graph_free(sbo_graph *g);
int sbo_gen_er(int64_t n, double p, int pm1, uint64_t seed, sbo_graph *out);
int sbo_gen_torus(int32_t rows, int32_t cols, uint64_t seed, sbo_graph *out);
int sbo_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c,
                 uint64_t seed, sbo_graph *out);
int sbo_gen_rgg(int64_t n, double avg_degree, uint64_t seed, sbo_graph *out);
int sbo_gen_cities(int32_t N, double scale, uint64_t seed, double *xc, double *yc);

/* ---- loaders ---- */
/* csr.cpp:15-109 + construct_csr (:157-192) with empty rows kept.
 * Two-call protocol: call with NULL arrays to get n and nnz, then again. */
int sbo_mtx_load(const char *path, int64_t *n, int64_t *nnz, int32_t *rowptr,
                 int32_t *col, double *val, double *wsum);
/* csr.cpp:137-155 + construct_csr: dense dim x dim -> CSR of nonzeros. */
int64_t sbo_dense_to_csr(int64_t dim, const double *dense, int32_t *rowptr,
                         int32_t *col, double *val);
/* tsp_cpu.cpp:9-45.  kind receives SBO_DIST_EUC_2D or SBO_DIST_GEO.
 * Two-call protocol on xc/yc as above. */
int sbo_tsplib_load(const char *path, int32_t *N, double *xc, double *yc,
                    int *kind);

#ifdef __cplusplus
}
#endif
#endif
