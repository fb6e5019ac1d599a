// engine.h -- internal interface between the C-ABI host layer (api.cpp) and
// the CUDA launchers (k_*.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace sbx {

enum Prec { P_F32 = 0, P_BF16 = 1, P_F16 = 2, P_F64 = 3 };

// One instance of the reference's init stream (k_init.cu): rows
// [row_off, row_off + n) x agents [0, A) of x, y from srand(seed)'s window V0;
// its device threads are thread_base .. thread_base + ceil(outputs/L) - 1.
struct RandInst {
    int64_t row_off, n, thread_base;
    int32_t A, pad;
    uint32_t V0[31];
};

// Rows with more neighbours than this are "heavy" (+-1 weights): the step
// kernel counts them in chunks of kHeavy; byte counters (2 per neighbour)
// never overflow.
constexpr int kHeavy = 127;

// Mixed count mode (kernels with heavy rows): light rows of at least this
// many neighbours are counted in bit planes, shorter ones in byte counters
// (R-MAT scale 20 on GB300: 8, 12 and 20 timed within 1%).
constexpr int kBitsMin = 12;

inline size_t prec_bytes(int p) { return p == P_F64 ? 8 : p == P_F32 ? 4 : 2; }

// An attribute of the calling thread's current device (0 when the query
// fails); queried each time, so contexts on different devices see their own.
inline int dev_attr(cudaDeviceAttr a)
{
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, a, dev) != cudaSuccess) return 0;
    return v;
}

struct DevBsm;

// MaxCut / QUBO matrix on the device.  colw holds the column index; when every
// weight is +-1 ("unit"), bit 31 holds the weight's sign and no value array is
// read by the step kernels.
struct DevCsr {
    int64_t n = 0, nnz = 0;
    int32_t *rowptr = nullptr;
    uint32_t *colw = nullptr;
    double *vald = nullptr;
    float *valf = nullptr;
    int32_t *perm = nullptr; // rows in decreasing degree (resident kernel order)
    bool skewed = false;     // max degree > 8x mean: the step kernel visits rows in perm order
    int64_t nheavy = 0;      // heavy rows: the first nheavy entries of perm
    int64_t niso = 0;        // isolated rows (degree 0): the last niso entries of perm
    // Heavy rows (unit weights, degree > kHeavy) are split into chunks of
    // kHeavy neighbours, each counted by its own work item of the step kernel.
    int32_t *hchunk = nullptr;    // per row: first chunk of a heavy row, else -1
    int32_t *chunk_row = nullptr; // per chunk: its row
    int32_t nchunks = 0;
    // Batched (block-diagonal) matrices: dt*xi0 of each row's instance, and
    // the instance of each row; null for a single problem.
    float *c0r32 = nullptr;
    double *c0r64 = nullptr;
    int32_t *rinst = nullptr;
    // batched: instances, their agent counts and weight sums (per-window trace)
    int32_t ninst = 0;
    int32_t *iagents = nullptr;
    double *iwsum = nullptr;
    bool weights_always = false;  // the device copy holds the weights even when all are +-1
    bool unit = false;       // all |w| == 1
    bool allpos = false;     // all w == +1 (unit, no sign bits)
    bool integer = false;    // all integer-valued, small enough for int32 sums
    double wsum = 0;         // reference csr.sum
    int32_t max_deg = 0;
    std::vector<double> hval;   // host copy of values (xi0)
    std::vector<int32_t> hrowptr, hcol, hperm;
    // The matrix relabelled into perm order (row and column s = perm slot s),
    // built on first use by the register + shared resident kernel.
    // Batched: the plan of the shared-memory-plane step kernel, when the
    // solve uses it (k_batch_smem.cu)
    const DevBsm *bsm = nullptr;
    int32_t *rs_rowptr = nullptr;
    uint32_t *rs_colw = nullptr;
    float *rs_valf = nullptr;
};

// Control words shared by the kernels of one solve.
// CTL_ERR: a kernel gave up a bounded wait (set, never cleared by kernels).
enum Ctl { CTL_STEP = 0, CTL_STOP = 1, CTL_WINDOWS = 2, CTL_NBIF = 3, CTL_TRACED = 4, CTL_ERR = 5, CTL_N = 8 };

// One window of a traced solve: SB steps run, best cut over the agents of
// the window spins, nanoseconds since the loop began (device clock).
struct TraceRec {
    long long steps;
    double best;
    long long t_ns;
    long long pad;
};

// Device buffers of one solve (grown on demand, owned by the context).
struct Work {
    void *x = nullptr, *y = nullptr, *x2 = nullptr;
    uint32_t *S[2] = {nullptr, nullptr};
    uint32_t *Wp = nullptr, *fin = nullptr, *chg = nullptr, *newmask = nullptr;
    int32_t *stab = nullptr;
    uint8_t *bif = nullptr, *prev = nullptr;
    int32_t *ctl = nullptr;
    int32_t *wincount = nullptr;          // bifurcated agents after each window
    int32_t *visits = nullptr;            // TSP streaming window scratch
    double2 *ab = nullptr;                // TSP (a_t, b_t) per step, FP64
    float2 *sched = nullptr;              // TSP (b_t, dt*-(1-a_t)) per step
    uint32_t *part = nullptr;             // heavy-row partial counts
    int32_t *hcount = nullptr;            // heavy rows: finished chunks per (row, segment)
    int32_t *gbar = nullptr;              // window barrier of co-resident launches
    unsigned long long *eacc = nullptr;   // per-agent cut accumulators
    double *cut = nullptr;                // per-agent cuts
    double *stats = nullptr;              // k_stats output, 7 per problem
    TraceRec *trace = nullptr;            // per-window records; trace_t0: loop start
    long long *trace_t0 = nullptr;
    double *btrace = nullptr;             // batched: best cut [window][instance]
    int32_t *tours = nullptr, *valid = nullptr;
    uint32_t *rjump = nullptr;            // rand jump matrices (computed once)
    RandInst *rinst = nullptr;            // init instances of the current solve
    float *coef32 = nullptr;              // per-step coefficients (float4 / step)
    double *coef64 = nullptr;             // the same in FP64 (double4 / step)
    size_t cap_x = 0, cap_y = 0, cap_x2 = 0, cap_S0 = 0, cap_S1 = 0, cap_Wp = 0, cap_fin = 0,
           cap_chg = 0, cap_new = 0, cap_stab = 0, cap_bif = 0, cap_prev = 0, cap_ctl = 0,
           cap_win = 0, cap_visits = 0, cap_ab = 0, cap_sched = 0, cap_eacc = 0, cap_cut = 0,
           cap_trace = 0, cap_t0 = 0, cap_btrace = 0, cap_tours = 0, cap_valid = 0, cap_rj = 0, cap_c32 = 0, cap_c64 = 0, cap_part = 0, cap_rinst = 0, cap_hcount = 0, cap_gbar = 0, cap_stats = 0;
    bool rjump_ready = false;
};

// One solve's shape and scalars.
struct SolveDims {
    int64_t n = 0;
    int32_t A = 0, Ap = 0, W = 0;
    int prec = P_F32;
    int32_t steps = 0, period = 100, threshold = 25;
    int32_t nwin = 0;   // TSP: windows to run
    int fused = 1, uw = 0;
    double dt = 0.1, xi0 = 0, c0 = 0;
    bool pdl = true;
    // streaming step tile: agents per lane (0: widest vector that divides
    // Ap), lanes per row (32, 16, 8, 4), threads per CTA
    int32_t tv = 0, tlr = 32, tbt = 256;
    int32_t tcm = 0;         // +-1 rows: 0 byte counters per lane, 1 bit planes per word, 2 mixed
    int32_t tst = 0;         // 1: whole-warp rows staged through shared memory (bulk copies)
    int trace = 0;           // per-window best-cut records: 1 one problem, 2 batched
    int32_t steps_run = 0;   // resident batch: SB steps of the run
    int giveup = 0;          // SBX_FLAG_TEST_GIVEUP: bounded waits give up at once
    int tbsm = 0;            // batched: the shared-memory-plane step kernel (J.bsm),
                             // its CTA size (512 or 1024); 0: not used
};

// Plan of the batched step kernel with per-instance sign planes in shared
// memory (k_batch_smem.cu): the rows cut into one contiguous run per CTA,
// each run into segments at instance boundaries.
struct DevBsm {
    uint16_t *lcol = nullptr;     // per entry: local column | weight sign << 15; rows padded
                                  // to blocks of eight with the all-zero row (local row n_i)
    uint32_t *rinfo = nullptr;    // per row: first block of eight entries << 7 | degree
    int32_t *seg = nullptr;       // per segment: instance, first row, end row (global rows)
    int32_t *cta_seg = nullptr;   // per CTA: first segment; grid + 1 entries
    int32_t *ioff = nullptr;      // per instance: first row
    int32_t *in = nullptr;        // per instance: rows
    int32_t grid = 0;
    int64_t max_rows = 0;         // largest instance: the shared-memory plane's rows
};

// A batch class packed for the resident batch kernel (k_resident_batch.cu):
// whole instances in bins, rows of a bin by decreasing degree ("slots"), the
// matrix relabelled into slot order.
struct DevRb {
    int32_t *rowptr = nullptr;   // [slots + 1]
    uint32_t *colw = nullptr;    // columns as slots, bit 31 the weight sign
    float *valf = nullptr;
    float *c0 = nullptr;         // dt * xi0 per slot
    int32_t *perm = nullptr;     // slot -> row
    int32_t *bin_off = nullptr;  // [nbins + 1]
    int32_t *cta_bin = nullptr;  // bins, largest first
    int32_t nbins = 0;
    int64_t max_bin_rows = 0;
    bool unit = false;
    double dt = -1;              // dt of the uploaded c0
};

// ---- launchers (k_*.cu) ----

// glibc rand() on the device (k_init.cu).
void rand_seed_window(uint32_t seed, uint32_t *V0);
// out[b] = M^(L * 2^b), b < nbits (31x31 each): independent of the seed.
void rand_jump_matrices(int64_t L, int nbits, std::vector<uint32_t> &out);
int rand_threads_bits(int64_t outputs, int64_t L);
// slot: null, or (batched MaxCut) the state row of each instance row.
cudaError_t launch_rand_init(int prec, void *x, void *y, int32_t Ap, bool tsp, int64_t L,
                             const uint32_t *mats, const RandInst *inst, int count,
                             int64_t total_threads, const int32_t *slot, cudaStream_t s);

// Streaming MaxCut kernels (k_stream.cu).
cudaError_t launch_prestep(const SolveDims &d, const DevCsr &J, Work &w, cudaStream_t s,
                           int *launches);
// evs (optional): 2*period events recorded around each step kernel.
cudaError_t launch_chunk(const SolveDims &d, const DevCsr &J, Work &w, cudaStream_t s,
                         int *launches, cudaEvent_t *evs = nullptr);
cudaError_t launch_cut(const SolveDims &d, const DevCsr &J, Work &w, const uint32_t *plane,
                       cudaStream_t s, int *launches);
// count plain (non-window) steps of the solve's kind at step 0: the
// autotuner's timing runs.
cudaError_t launch_plain_steps(const SolveDims &d, const DevCsr &J, Work &w, int count, cudaStream_t s);
// Traced solves: stamp the loop start on the device clock.
cudaError_t launch_trace_start(Work &w, cudaStream_t s);
// The statistics of src/ising.cu:238-265 on the device (k_stats): out[7] =
// min, max, total and mean (agent order), sum of squared deviations (agent
// order), agents at the maximum, first agent at the maximum.
cudaError_t launch_stats(const double *v, int32_t A, double *out, cudaStream_t s);
// Batched: cut[agent_off[i] + a] from instance i's exact sums, and out[7 i..]
// its statistics.
cudaError_t launch_stats_batch(const unsigned long long *eacc, int32_t Ap, const int32_t *agents,
                               const int32_t *agent_off, const double *wsum, int32_t ninst, double *cut,
                               double *out, cudaStream_t s);
// Integer weights, block-diagonal J: eacc[instance][Ap] += s_r sum_j J_rj s_j.
cudaError_t launch_cut_batch(const SolveDims &d, const DevCsr &J, const uint32_t *plane,
                             unsigned long long *eacc, cudaStream_t s);

// Batched step with shared-memory sign planes (k_batch_smem.cu): bytes of
// dynamic shared memory for the largest instance; one launch of a fused or
// force + clamp step (kind K_FUSED / K_FC of k_step.cuh).
size_t bsm_smem_bytes(int64_t max_rows, int W);
struct StepP;
cudaError_t launch_batch_smem(const SolveDims &d, const DevBsm &M, const StepP &P, int kind, bool win,
                              int offset, cudaStream_t s);

// Resident MaxCut kernel (k_resident.cu): returns cudaErrorInvalidValue when the
// shape does not fit.
int resident_pick_ka(const SolveDims &d, const DevCsr &J, int requested);
size_t resident_smem_bytes(const SolveDims &d, int ka);
cudaError_t launch_resident(const SolveDims &d, const DevCsr &J, Work &w, int ka,
                            int32_t step0, int32_t nsteps, bool first, cudaStream_t s);
// Resident batch kernel (k_resident_batch.cu): bins hold at most this many
// rows; one launch runs d.steps_run fused steps of every instance.
int64_t resident_batch_max_rows();
cudaError_t launch_resident_batch(const SolveDims &d, const DevRb &B, Work &w, cudaStream_t s);

// Register + shared-memory resident kernel (k_resident_rs.cu), 8 agents per
// CTA, 16-bit fused state: a configuration number > 0 when the shape fits.
int resident_rs_pick(const SolveDims &d, const DevCsr &J, bool forced);
// coop: the update-window mode's windows in one co-resident launch (a
// bounded barrier per window); cudaErrorCooperativeLaunchTooLarge when the
// CTAs cannot all be resident.
cudaError_t launch_resident_rs(const SolveDims &d, const DevCsr &J, Work &w, int cfg, int32_t step0,
                               int32_t nsteps, bool first, bool coop, cudaStream_t s);

// TSP kernels (k_tsp.cu).
struct DevTsp {
    int32_t N = 0;
    double A = 1, B = 0, C = 0;
    std::vector<double> packed, rowsum, I2h;   // host
    float *D = nullptr;                   // device N x N distances (float)
    float *I2 = nullptr;                  // device per-city linear field (float)
    double *I2d = nullptr;                // the same in FP64
    double *Dd = nullptr;                 // device N x N distances (FP64, exact)
    DevCsr qubo;                          // the QUBO as CSR (streaming path)
};
int tsp_pick_ka(const SolveDims &d, const DevTsp &t, int requested);
cudaError_t launch_tsp_resident(const SolveDims &d, const DevTsp &t, Work &w, int ka,
                                cudaStream_t s);
cudaError_t launch_tsp_stream(const SolveDims &d, const DevTsp &t, Work &w, cudaStream_t s,
                              int *launches);
// Resident TSP kernel with the distance product on the tensor cores
// (k_tsp_tc.cu): 16-bit state, 3 <= N <= 32, 8 agents per CTA.
bool tsp_tensor_fits(const SolveDims &d, const DevTsp &t);
constexpr int kTspTensorAgents = 8;
// threads_per_row: 1, 2 or 4 threads share a (position, agent) row's
// cities; 0 picks the default.
int tsp_tensor_threads_per_row(int requested);
cudaError_t launch_tsp_tensor(const SolveDims &d, const DevTsp &t, Work &w, int threads_per_row, cudaStream_t s);
// TSP setup on the device from city coordinates (device xc, yc): packed
// distances (src/kernels.cu:404-442), the tables t.D / t.Dd, the largest
// distance *mx, per-city sums (src/tsp_gpu.cu:51-68) and the linear field
// t.I2d / t.I2 with B = C = scale * max distance.
cudaError_t launch_tsp_setup(const double *xc, const double *yc, int32_t N, int32_t kind, double A, double scale,
                             double *packed, double *mx, double *rowsum, DevTsp &t, cudaStream_t s);
// Tour length of every agent holding a valid tour (NaN otherwise) into len[A].
cudaError_t launch_tsp_lengths(const DevTsp &t, const int32_t *tours, const int32_t *valid, int32_t A,
                               double *len, cudaStream_t s);

}  // namespace sbx
