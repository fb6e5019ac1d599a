/*
 * sbx.h -- C ABI of the GB300 simulated-bifurcation (SB) engine.
 *
 * Plain C: pointers, sizes and POD structs; no CUDA or C++ types cross this
 * boundary.  Every call returns SBX_OK (0) or a negative status (sbx_strerror
 * names it); nothing calls exit().  Host buffers belong to the caller and are
 * copied; device buffers belong to the context.  One context per host thread.
 *
 * It replaces the reference's class interface (Sparse-Ising-Solver):
 *   sbx_problem_csr   <- CSR(string) + CSR_GPU(CSR&)          src/csr.cuh:26-47,89-95
 *   sbx_problem_tsp   <- TSP_GPU(TSP_CPU&) + construct_matrix  src/csr.cuh:65-87
 *   sbx_problem_tsp_cities <- the same, distances on the device
 *                                       src/kernels.cu:404-442, tsp_gpu.cu:51-112
 *   sbx_solve (MaxCut)<- Ising::Ising + Ising::symplectic_update
 *                                                             src/csr.cuh:97-104
 *   sbx_solve (TSP)   <- Ising_TSP::Ising_TSP + symplectic_update
 *                                                             src/csr.cuh:156-163
 *   sbx_load_mtx      <- CSR::from_file                       src/csr.cpp:15-109
 *   sbx_load_tsplib   <- TSP_CPU::read_file                   src/tsp_cpu.cpp:9-45
 *   sbx_tsp_distances <- TSP_distances_EUC_2D / _GEO          src/kernels.cu:404-442
 * The `program` CLI built beside libsbx.so keeps src/main.cu:255-312's
 * arguments and the output-file line of src/ising.cu:267 + src/main.cu:223.
 */
#ifndef SBX_H
#define SBX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SBX_OK 0
#define SBX_ERR_ARG (-1)         /* invalid argument */
#define SBX_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define SBX_ERR_NOMEM (-3)       /* host or device allocation failed */
#define SBX_ERR_IO (-4)          /* file cannot be opened or read */
#define SBX_ERR_FORMAT (-5)      /* malformed .mtx / .tsp file */
#define SBX_ERR_UNSUPPORTED (-6) /* valid request this build cannot serve */
#define SBX_ERR_NODEVICE (-7)    /* no usable CUDA device */
#define SBX_ERR_STATE (-8)       /* call out of order (e.g. no solve yet) */

/* agent-state storage precision (arithmetic of the force is exact) */
enum { SBX_F32 = 0, SBX_BF16 = 1, SBX_F16 = 2, SBX_F64 = 3 };
/* kernel family: chosen by shape (AUTO) or forced.  RESIDENT keeps a CTA's
 * agents in shared memory; RESIDENT_SPLIT (MaxCut, fused, 16-bit state) keeps
 * 8 agents per CTA split between registers and shared memory, for graphs too
 * large for the former.  TENSOR (TSP, 16-bit state, 3 <= N <= 32) is the
 * resident TSP kernel with the distance product on the tensor cores
 * (tcgen05): AUTO's choice for BF16 and FP16 TSP states that fit it. */
enum { SBX_KERNEL_AUTO = 0, SBX_KERNEL_STREAM = 1, SBX_KERNEL_RESIDENT = 2, SBX_KERNEL_RESIDENT_SPLIT = 3,
       SBX_KERNEL_TENSOR = 4 };
/* TSP distance kinds, src/kernels.cu:404-442 */
enum { SBX_DIST_EUC_2D = 0, SBX_DIST_GEO = 1, SBX_DIST_EUC_2D_FLOAT = 2 };
/* sbx_params.flags */
#define SBX_FLAG_NO_PDL 1u      /* launch without programmatic dependent launch */
#define SBX_FLAG_NO_GRAPH 2u    /* launch kernels directly, not through a graph */
#define SBX_FLAG_PROFILE 4u     /* time every hot-kernel launch with events */
#define SBX_FLAG_NO_TUNE 8u     /* streaming tile from the fixed heuristic, not timed */
/* Test only: every bounded device wait of the solve (the co-resident window
 * barrier, the staged-row copy waits, the TSP tensor-core kernel's wait for
 * its MMAs) gives up at its first check, as a wait
 * that never completes would after its limit.  The kernels flag the error,
 * let their copies in flight land and return; the solve returns SBX_ERR_CUDA
 * and the context stays usable for the next solve. */
#define SBX_FLAG_TEST_GIVEUP 16u

typedef struct sbx_ctx sbx_ctx;
typedef struct sbx_problem sbx_problem;

typedef struct sbx_params {
    double dt;              /* time_step; reference default 0.1 (main.cu:272) */
    int32_t steps;          /* max_steps; reference default 10000 */
    int32_t agents;         /* columns of X; reference default 1024 */
    int32_t fused;          /* 1: fused step kernel (default); 0: unfused trio */
    int32_t update_window;  /* MaxCut early exit once every agent bifurcated */
    int32_t period;         /* steps per window; 0: reference (100 / steps/10) */
    int32_t threshold;      /* window convergence threshold; 0: reference (25 / 50) */
    int32_t precision;      /* SBX_F32 (default), SBX_BF16, SBX_F16, SBX_F64 */
    uint32_t seed;          /* srand() seed of the reference's init stream */
    int32_t kernel;         /* SBX_KERNEL_* */
    int32_t agents_per_block; /* resident kernel tile; 0: autotuned */
    int32_t trace;          /* 1: record the best cut at every window */
    uint32_t flags;         /* SBX_FLAG_* */
    int32_t run_steps;      /* run only the first run_steps steps of the
                               schedule set by `steps` (0: all of them) */
    /* Streaming step tile; 0 leaves the field to the autotuner, which times
     * the candidate tiles on the problem once and caches the fastest.  Every
     * tile computes identical results. */
    int32_t lane_agents;    /* agents per lane: 1, 2, 4 or 8 (16-bit states) */
    int32_t row_lanes;      /* lanes per row: 32, or 16/8/4 (several rows per
                               warp; then lane_agents * row_lanes = padded agents) */
    int32_t block_threads;  /* threads per CTA: 128 or 256 */
    int32_t count_mode;     /* +-1 weights: 1 byte counters per lane, 2 bit
                               planes per sign word (neighbours split across
                               the word's lanes), 3 mixed (rows with more than
                               127 neighbours present: bit planes for rows of
                               12 or more neighbours, byte counters below),
                               4 (batched, 16-bit state, 32/64/128 agents,
                               degree <= 127) each instance's sign plane in
                               shared memory, a lane per 32-agent word --
                               block_threads 512, 640 (default) or 1024
                               sets its CTA size;
                               0: autotuned (batches that fit take 4) */
    int32_t staging;        /* state larger than L2, whole-warp rows: 1 direct
                               loads, 2 rows copied ahead into shared memory
                               (bulk asynchronous copies); 0: autotuned */
    double target;          /* MaxCut: a cut; > 0 records the per-window best
                               cut (as trace = 1) and times its first reach */
} sbx_params;

typedef struct sbx_result {
    double time_us;         /* SB loop wall time: pre-step .. last window done */
    double min, max, mean, std, ps; /* MaxCut: cuts (ising.cu:238-265);
                                       TSP: tour lengths of valid agents */
    double xi0;
    int64_t steps_run;      /* SB steps after the pre-step */
    int64_t windows_run;
    int64_t bifurcated;     /* agents whose bifurcated flag is set */
    int64_t valid;          /* TSP: agents holding a valid tour */
    int32_t best_agent;     /* first agent reaching max (MaxCut) / min (TSP) */
    int32_t kernel_used;    /* SBX_KERNEL_STREAM or SBX_KERNEL_RESIDENT */
    int32_t agents_per_block;
    int32_t lane_agents;    /* streaming tile used (0 for other kernels) */
    int32_t row_lanes;
    int32_t block_threads;
    int32_t count_mode;
    int32_t staging;
    double kernel_ms;       /* SBX_FLAG_PROFILE: summed hot-kernel time */
    int64_t kernel_launches;/* hot-kernel launches issued by the solve */
    int64_t gpu_launches;   /* all kernel launches issued by the solve */
    double time_to_target_us; /* params.target: first window whose best cut
                                 reaches it, microseconds after the SB loop
                                 began (device clock); -1 if never */
    int64_t steps_to_target;  /* SB steps run at that window; -1 if never */
} sbx_result;

const char *sbx_strerror(int status);
/* Text of the last failure on this thread (empty when none). */
const char *sbx_last_error(void);
const char *sbx_version(void);
/* Reference defaults (main.cu:269-274 with dt 0.1). */
void sbx_params_default(sbx_params *p);

int sbx_create(sbx_ctx **ctx, int device);
/* Problems outlive their context only as handles to destroy. */
int sbx_destroy(sbx_ctx *ctx);
/* Run on a caller's cudaStream_t (passed as void*); NULL selects the
 * context's own stream. */
int sbx_set_stream(sbx_ctx *ctx, void *cuda_stream);

/* MaxCut / Ising problem from host CSR arrays (copied).  weight_sum is the
 * reference's csr.sum (one triangle of the file's weights). */
int sbx_problem_csr(sbx_ctx *ctx, int64_t n, int64_t nnz, const int32_t *rowptr,
                    const int32_t *col, const double *val, double weight_sum,
                    sbx_problem **out);
/* TSP-QUBO problem from packed upper-triangular distances (N(N-1)/2), the
 * distance weight A and the row/column penalties B, C (tsp_gpu.cu:76-112). */
int sbx_problem_tsp(sbx_ctx *ctx, int32_t ncities, const double *packed_dist,
                    double A, double B, double C, sbx_problem **out);
/* The same problem from city coordinates, set up on the device: the packed
 * distances of src/kernels.cu:404-442 (kind SBX_DIST_*), the per-city sums
 * and the largest distance of src/tsp_gpu.cu:51-68, and the QUBO of
 * src/tsp_gpu.cu:76-112 with distance weight A and B = C = penalty_scale *
 * the largest distance (the reference: A = 1, penalty_scale = 1).
 * Replaces TSP_GPU(TSP_CPU&) with its distance kernels, src/csr.cuh:65-87. */
int sbx_problem_tsp_cities(sbx_ctx *ctx, int32_t ncities, const double *xc,
                           const double *yc, int32_t kind, double A,
                           double penalty_scale, sbx_problem **out);
int sbx_problem_destroy(sbx_problem *p);
int sbx_problem_info(const sbx_problem *p, int64_t *n, int64_t *nnz,
                     int32_t *is_tsp);

/* One SB run.  agent_values (optional, [agents]) receives each agent's cut
 * (MaxCut) or tour length (TSP, NaN when the agent holds no valid tour). */
int sbx_solve(sbx_ctx *ctx, const sbx_problem *p, const sbx_params *params,
              sbx_result *res, double *agent_values);
/* State of the last solve, [n*agents] each, row-major (row*agents+agent);
 * spins are the window spins (current_spins) as +1/-1.  NULL skips. */
int sbx_get_state(sbx_ctx *ctx, double *x, double *y, int32_t *spins);
/* TSP tours of the last solve: tours[agents*N] (city order, -1 when the agent
 * has no valid tour) and valid_step[agents] (ising_tsp.cu valid_list). */
int sbx_get_tours(sbx_ctx *ctx, int32_t *tours, int32_t *valid_step);
/* Per-window record of the last MaxCut solve run with params.trace = 1 or
 * params.target > 0: SB steps run, best cut over agents of the window spins,
 * and microseconds since the SB loop began (device clock).  Up to cap entries
 * are written; *count receives the number recorded.  NULL arrays skip. */
int sbx_get_trace(sbx_ctx *ctx, int64_t cap, int64_t *steps, double *best,
                  double *t_us, int64_t *count);

/* ---- batched MaxCut: many independent instances, one launch per step ---- */
/* Each instance keeps its own xi0, weight sum and agent count; all share
 * dt/steps/precision from params.  Per-instance results go to res[count]
 * and agent_values (concatenated, sum of agents) when given.  targets
 * (optional, [count]): per-instance cuts; each instance's first window whose
 * best cut reaches its target sets its time_to_target_us (from the start of
 * the run of its agent class) and steps_to_target. */
int sbx_solve_batch(sbx_ctx *ctx, int32_t count, sbx_problem *const *problems,
                    const int32_t *agents, const sbx_params *params,
                    const double *targets, sbx_result *res, double *agent_values,
                    double *batch_time_us);

/* State of instance `index` (its position in the last sbx_solve_batch
 * call), as sbx_get_state: x, y, spins [n_i * agents_i] each, row-major in
 * the instance's own row order (the batch renumbers rows internally).
 * No counterpart in the reference (it has no batched solve).  Instances are
 * solved one agent class (padded agent count) after another in the same
 * buffers, so only the last class's instances are available; others give
 * SBX_ERR_STATE, as does any call after a later sbx_solve. */
int sbx_get_batch_state(sbx_ctx *ctx, int32_t index, double *x, double *y,
                        int32_t *spins);

/* ---- fused steps without device allocation ---- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory (a process whose device memory is all held by its own arena, or a
 * loop that cannot take cudaMalloc's synchronisation): runs fused SB steps
 * step0 .. step0+nsteps-1 of a max_steps schedule (FP32 state, any float
 * weights, src/kernels.cu:211-269 in Jacobi order) on caller-owned device
 * buffers -- CSR d_rowptr[n+1], d_col[nnz], d_val[nnz]; d_x, d_y [n][agents],
 * updated in place -- on cuda_stream (NULL: the legacy default stream).  Its
 * only scratch, two sign planes, lives in a static device array of
 * 2 * SBX_NOALLOC_MAX_WORDS words (16 MiB, held by every GPU that loads the
 * library); n * agents / 32 must not exceed SBX_NOALLOC_MAX_WORDS and agents
 * must be a multiple of 32, else SBX_ERR_ARG.  Every pointer must be valid,
 * d_col and d_val too when the matrix has no entries (NULL: SBX_ERR_ARG).
 * The first call on a device looks up the array's device address (make it
 * before any stream capture) and keeps it for the process: after a device
 * reset the entry point must not be called again.  Calls share the array,
 * so calls that overlap on the GPU race.  Nothing is allocated or freed. */
#define SBX_NOALLOC_MAX_WORDS (1 << 21)
int sbx_fused_steps_noalloc(const int32_t *d_rowptr, const int32_t *d_col,
                            const float *d_val, int64_t n, int32_t agents,
                            float *d_x, float *d_y, double dt, double xi0,
                            int32_t step0, int32_t nsteps, int32_t max_steps,
                            void *cuda_stream);

/* ---- host-side loaders (no device needed) ---- */
/* csr.cpp:15-109: two-call protocol, first with NULL arrays for the sizes. */
int sbx_load_mtx(const char *path, int64_t *n, int64_t *nnz, int32_t *rowptr,
                 int32_t *col, double *val, double *weight_sum);
/* tsp_cpu.cpp:9-45: two-call protocol on xc / yc. */
int sbx_load_tsplib(const char *path, int32_t *ncities, double *xc, double *yc,
                    int32_t *kind);
/* kernels.cu:404-442 on the host: packed distances of N cities. */
int sbx_tsp_distances(int32_t ncities, const double *xc, const double *yc,
                      int32_t kind, double *packed);

/* ---- seeded synthetic instances (host; two-call like sbx_load_mtx) ---- */
/* Erdos-Renyi G(n, p), weights +1, or +-1 uniform when pm1 != 0. */
int sbx_gen_er(int64_t n, double p, int32_t pm1, uint64_t seed, int64_t *nnz,
               int32_t *rowptr, int32_t *col, double *val, double *weight_sum);
/* rows x cols 2-D torus, degree 4, weights +-1 uniform per edge. */
int sbx_gen_torus(int32_t rows, int32_t cols, uint64_t seed, int64_t *nnz,
                  int32_t *rowptr, int32_t *col, double *val, double *weight_sum);
/* R-MAT, 2^scale vertices, edge_factor*2^scale edge draws, (a, b, c),
 * self loops and duplicates removed, weights +1, empty rows kept. */
int sbx_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b,
                 double c, uint64_t seed, int64_t *nnz, int32_t *rowptr,
                 int32_t *col, double *val, double *weight_sum);
/* Random geometric graph in the unit square with the radius that gives
 * avg_degree, weights +-1 uniform. */
int sbx_gen_rgg(int64_t n, double avg_degree, uint64_t seed, int64_t *nnz,
                int32_t *rowptr, int32_t *col, double *val, double *weight_sum);
/* ncities uniform in [0, scale)^2. */
int sbx_gen_cities(int32_t ncities, double scale, uint64_t seed, double *xc,
                   double *yc);

#ifdef __cplusplus
}
#endif
#endif
