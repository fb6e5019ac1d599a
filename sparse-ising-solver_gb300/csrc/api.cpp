// api.cpp -- the C ABI (include/sbx.h): contexts, problems, solves.
//
// Host orchestration of one MaxCut solve follows Ising::symplectic_update
// (src/ising.cu:140-271): init from the seed, the pre-step Update_XY, windows
// of `period` steps, the optional all-bifurcated early exit, the cut of the
// window spins and the statistics line.  The TSP solve follows
// Ising_TSP::symplectic_update (src/ising_tsp.cu:111-253).  Every CUDA error
// becomes a negative status; nothing exits the process.
#include "../../include/sbx.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "engine.h"
#include "host_par.h"

using namespace sbx;

// Streaming step tile (agents per lane, lanes per row, threads per CTA).
struct Tile {
    int32_t v = 0, lr = 32, bt = 256, cm = 0, st = 0;
};

struct sbx_problem {
    sbx_ctx *ctx = nullptr;
    bool tsp = false;
    DevCsr J;
    DevTsp T;
};

// A class of batched instances sharing one padded agent count, packed into
// one block-diagonal matrix.
struct BatchClass {
    std::vector<const sbx_problem *> probs;
    std::vector<int> idx;                 // positions in the caller's batch
    std::vector<int32_t> agents;
    std::vector<int64_t> row_off;
    std::vector<double> xi0, wsum;
    int32_t Ap = 0;
    DevCsr J;
    double dt = -1;                       // dt of the uploaded per-row c0
    DevRb rb;                             // packed for the resident batch kernel (on first use)
    int64_t rb_max = 0;                   // bin capacity the packing was made for
    DevBsm bsm;                           // plan of the shared-memory-plane step (on first use)
    std::vector<int32_t> agent_off;       // instance i's cuts at [agent_off[i], agent_off[i + 1])
    int32_t *daoff = nullptr;             // the same on the device
    // Each instance's rows are renumbered by decreasing degree inside its
    // block: slot[row_off + r] is the class row of the instance's row r.
    std::vector<int32_t> slot;
    int32_t *dslot = nullptr;             // the same on the device (the init writes through it)
};

struct sbx_ctx {
    int device = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    Work w;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evp[4] = {};
    int32_t *pinned = nullptr;   // stop-flag ring for the update-window poll
    // graph cache for the streaming chunk
    cudaGraphExec_t gexec = nullptr;
    std::string gkey;
    int gper_chunk = 0;
    std::vector<cudaEvent_t> prof;   // SBX_FLAG_PROFILE: events around step kernels
    // last solve
    bool have = false, last_tsp = false;
    SolveDims d;
    int32_t N = 0;
    std::string err;
    std::set<sbx_problem *> problems;   // live problems; orphaned on destroy
    std::vector<BatchClass> batch;      // packed classes of the last batch
    std::string batch_key;
    int batch_last = -1;                // class whose state the work buffers hold
    std::vector<TraceRec> trace;        // per-window records of the last traced solve
    // autotuned tiles by matrix shape (rows, entries, degrees, weight kind),
    // precision, agents and mode: a problem uploaded again reuses its tile
    std::map<std::string, Tile> tiles;
};

namespace {

thread_local std::string g_err;
uint64_t g_alloc_gen = 0;   // bumped by every (re)allocation of a work buffer

int fail(sbx_ctx *c, int code, const std::string &m)
{
    if (c) c->err = m;
    g_err = m;
    return code;
}

// A failed call's error is also the thread's pending CUDA error; it is
// consumed here so that it is not reported again by a later call's check.
#define CK(call)                                                                   \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            (void)cudaGetLastError();                                              \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? SBX_ERR_NOMEM : SBX_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));       \
        }                                                                          \
    } while (0)

template <class T> cudaError_t grow(T *&p, size_t &cap, size_t count)
{
    size_t bytes = count * sizeof(T);
    if (bytes == 0) bytes = sizeof(T);
    if (cap >= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc((void **)&p, bytes);
    if (e == cudaSuccess) cap = bytes;
    g_alloc_gen++;
    return e;
}

cudaError_t growv(void *&p, size_t &cap, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    if (cap >= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) cap = bytes;
    g_alloc_gen++;
    return e;
}

void free_csr(DevCsr &J)
{
    cudaFree(J.rowptr);
    cudaFree(J.colw);
    cudaFree(J.vald);
    cudaFree(J.valf);
    cudaFree(J.perm);
    cudaFree(J.hchunk);
    cudaFree(J.chunk_row);
    cudaFree(J.c0r32);
    cudaFree(J.c0r64);
    cudaFree(J.rinst);
    cudaFree(J.iagents);
    cudaFree(J.iwsum);
    cudaFree(J.rs_rowptr);
    cudaFree(J.rs_colw);
    cudaFree(J.rs_valf);
    J.rs_rowptr = nullptr;
    J.rs_colw = nullptr;
    J.rs_valf = nullptr;
    J.iagents = nullptr;
    J.iwsum = nullptr;
    J.ninst = 0;
    J.c0r32 = nullptr;
    J.c0r64 = nullptr;
    J.rinst = nullptr;
    J.hchunk = J.chunk_row = nullptr;
    J.nchunks = 0;
    J.nheavy = 0;
    J.niso = 0;
    J.rowptr = nullptr;
    J.colw = nullptr;
    J.vald = nullptr;
    J.valf = nullptr;
    J.perm = nullptr;
}

int upload_device(sbx_ctx *ctx, DevCsr &J);

// Validate a CSR, classify its weights and keep it on the host; its device
// arrays are made by upload_device, at once or -- defer -- when a solve first
// needs them (a problem that only ever goes into batches never needs its own).
int upload_csr(sbx_ctx *ctx, DevCsr &J, int64_t n, int64_t nnz, const int32_t *rowptr,
               const int32_t *col, const double *val, double wsum, bool weights_always = false,
               bool keep_host = true, bool defer = false)
{
    if (n <= 0 || n > INT32_MAX - 1 || nnz < 0 || nnz > INT32_MAX || !rowptr || (nnz && (!col || !val)))
        return fail(ctx, SBX_ERR_ARG, "bad CSR sizes or pointers");
    if (rowptr[0] != 0 || rowptr[n] != nnz) return fail(ctx, SBX_ERR_ARG, "rowptr[0] != 0 or rowptr[n] != nnz");
    // Checks and classification on host threads over row ranges (large
    // matrices); each range keeps its own flags, merged after.
    const int T = nnz > (1 << 20) ? host_threads() : 1;
    struct Part {
        int err = 0;   // 1 rowptr, 2 column, 3 weight
        int32_t maxdeg = 0;
        int64_t niso = 0;
        bool unit = true, integer = true, neg = false;
        double rowabs = 0;
    };
    std::vector<Part> part((size_t)T);
    parallel(T, [&](int t, int TT) {
        Part &a = part[(size_t)t];
        const int64_t r0 = n * t / TT, r1 = n * (t + 1) / TT;
        for (int64_t r = r0; r < r1; r++) {
            const int32_t deg = rowptr[r + 1] - rowptr[r];
            if (deg < 0) {
                a.err = 1;
                return;
            }
            a.maxdeg = std::max(a.maxdeg, deg);
            a.niso += deg == 0;
        }
    });
    for (const Part &a : part)
        if (a.err) return fail(ctx, SBX_ERR_ARG, "rowptr not monotone");
    parallel(T, [&](int t, int TT) {
        Part &a = part[(size_t)t];
        const int64_t r0 = n * t / TT, r1 = n * (t + 1) / TT;
        for (int64_t r = r0; r < r1 && !a.err; r++) {
            double ra = 0;
            for (int32_t e = rowptr[r]; e < rowptr[r + 1]; e++) {
                if (col[e] < 0 || col[e] >= n) {
                    a.err = 2;
                    break;
                }
                const double v = val[e];
                if (!std::isfinite(v)) {
                    a.err = 3;
                    break;
                }
                if (std::fabs(v) != 1.0) a.unit = false;
                if (v != std::floor(v) || std::fabs(v) > 16777216.0) a.integer = false;
                a.neg |= v < 0;
                ra += std::fabs(v);
            }
            a.rowabs = std::max(a.rowabs, ra);
        }
    });
    int32_t maxdeg = 0;
    int64_t niso = 0;
    bool unit = true, integer = true, neg = false;
    double rowabs_max = 0;
    for (const Part &a : part) {
        if (a.err == 2) return fail(ctx, SBX_ERR_ARG, "column index out of range");
        if (a.err == 3) return fail(ctx, SBX_ERR_ARG, "non-finite weight");
        maxdeg = std::max(maxdeg, a.maxdeg);
        niso += a.niso;
        unit &= a.unit;
        integer &= a.integer;
        neg |= a.neg;
        rowabs_max = std::max(rowabs_max, a.rowabs);
    }
    if (rowabs_max >= 2147483647.0) integer = false;
    // rows by decreasing degree, ties in row order (a counting sort): a warp
    // of the resident kernel gets rows of similar length
    std::vector<int32_t> perm((size_t)n);
    {
        std::vector<int64_t> at((size_t)maxdeg + 2, 0);
        for (int64_t r = 0; r < n; r++) at[(size_t)(maxdeg - (rowptr[r + 1] - rowptr[r])) + 1]++;
        for (int32_t k = 0; k <= maxdeg; k++) at[(size_t)k + 1] += at[(size_t)k];
        for (int64_t r = 0; r < n; r++) perm[(size_t)at[(size_t)(maxdeg - (rowptr[r + 1] - rowptr[r]))]++] = (int32_t)r;
    }
    J.n = n;
    J.nnz = nnz;
    J.unit = unit;
    J.allpos = unit && !neg;
    J.integer = integer;
    J.wsum = wsum;
    J.max_deg = maxdeg;
    J.skewed = (double)maxdeg > 8.0 * std::max(1.0, (double)nnz / (double)n);
    J.niso = niso;
    J.weights_always = weights_always;
    if (keep_host) {   // else the caller moves its arrays in
        J.hval.assign(val, val + nnz);
        J.hrowptr.assign(rowptr, rowptr + n + 1);
        J.hcol.assign(col, col + nnz);
    }
    J.hperm = std::move(perm);
    // heavy rows (+-1, more than kHeavy neighbours) in chunks of kHeavy
    J.nheavy = 0;
    J.nchunks = 0;
    if (unit && maxdeg > kHeavy)
        for (int64_t r = 0; r < n; r++) {
            const int32_t deg = rowptr[r + 1] - rowptr[r];
            if (deg <= kHeavy) continue;
            J.nheavy++;
            J.nchunks += (deg + kHeavy - 1) / kHeavy;
        }
    return defer ? SBX_OK : upload_device(ctx, J);
}

// The device arrays of a CSR from its host copies: row pointers, column
// words (bit 31: a -1 weight), FP32/FP64 weights where the kernels read
// them, the degree order and the heavy rows' chunks.
int upload_device(sbx_ctx *ctx, DevCsr &J)
{
    if (J.rowptr) return SBX_OK;
    const int64_t n = J.n, nnz = J.nnz;
    const int32_t *rowptr = J.hrowptr.data(), *col = J.hcol.data();
    const double *val = J.hval.data();
    const int T = nnz > (1 << 20) ? host_threads() : 1;
    std::vector<uint32_t> colw((size_t)nnz);
    const bool dev_weights = !J.unit || J.weights_always;
    std::vector<float> valf(dev_weights ? (size_t)nnz : 0);
    parallel(T, [&](int t, int TT) {
        const int64_t e0 = nnz * t / TT, e1 = nnz * (t + 1) / TT;
        for (int64_t e = e0; e < e1; e++) {
            colw[e] = (uint32_t)col[e] | ((J.unit && val[e] < 0) ? 0x80000000u : 0u);
            if (dev_weights) valf[e] = (float)val[e];
        }
    });
    CK(cudaMalloc(&J.rowptr, sizeof(int32_t) * (n + 1)));
    CK(cudaMalloc(&J.colw, sizeof(uint32_t) * std::max<int64_t>(nnz, 1)));
    CK(cudaMalloc(&J.perm, sizeof(int32_t) * n));
    CK(cudaMemcpy(J.rowptr, rowptr, sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice));
    if (nnz) CK(cudaMemcpy(J.colw, colw.data(), sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice));
    // weights on the device only when they are not all +-1 (the MaxCut
    // kernels read the sign bit of colw for +-1 matrices), or when asked (the
    // TSP QUBO's kernels always read them)
    if (dev_weights) {
        CK(cudaMalloc(&J.vald, sizeof(double) * std::max<int64_t>(nnz, 1)));
        CK(cudaMalloc(&J.valf, sizeof(float) * std::max<int64_t>(nnz, 1)));
        if (nnz) {
            CK(cudaMemcpy(J.vald, val, sizeof(double) * nnz, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(J.valf, valf.data(), sizeof(float) * nnz, cudaMemcpyHostToDevice));
        }
    }
    CK(cudaMemcpy(J.perm, J.hperm.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
    if (J.nchunks) {
        std::vector<int32_t> hchunk((size_t)n, -1), crow;
        crow.reserve((size_t)J.nchunks);
        for (int64_t r = 0; r < n; r++) {
            const int32_t deg = rowptr[r + 1] - rowptr[r];
            if (deg <= kHeavy) continue;
            hchunk[r] = (int32_t)crow.size();
            for (int32_t c = 0; c < (deg + kHeavy - 1) / kHeavy; c++) crow.push_back((int32_t)r);
        }
        CK(cudaMalloc(&J.hchunk, sizeof(int32_t) * n));
        CK(cudaMalloc(&J.chunk_row, sizeof(int32_t) * crow.size()));
        CK(cudaMemcpy(J.hchunk, hchunk.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(J.chunk_row, crow.data(), sizeof(int32_t) * crow.size(), cudaMemcpyHostToDevice));
    }
    return SBX_OK;
}

// src/ising.cu:103-125 (with n*n formed in double).
double xi0_of(const DevCsr &J)
{
    const double nn = (double)J.n * (double)J.n;
    double sum = 0.0;
    for (double v : J.hval) sum += v;
    const double mean = sum / nn;
    double nonzero = 0.0;
    for (double v : J.hval) nonzero += std::pow(v - mean, 2);
    const double zero = (nn - (double)J.nnz) * mean * mean;
    sum = nonzero + zero;
    const double sigma = std::pow(sum / (nn - 1.0), 0.5);
    return 0.7 / (sigma * std::pow((double)J.n, 0.5));
}

// The statistics from the device's reduction (launch_stats): min, max and
// mean as reduced there, the standard deviation and ps finished here with
// the reference's expressions (src/ising.cu:258-265).
void finish_stats(const double *st, int64_t A, sbx_result *r)
{
    r->min = st[0];
    r->max = st[1];
    r->mean = st[3];
    r->std = std::pow(st[4] / (A - 1), 0.5);
    r->ps = st[5] / A;
    r->best_agent = (int32_t)st[6];
}

int ensure_common(sbx_ctx *ctx, const SolveDims &d, int64_t total_steps, int32_t J_nchunks = 0)
{
    Work &w = ctx->w;
    const size_t es = prec_bytes(d.prec);
    const size_t nst = (size_t)d.n * d.Ap;
    const size_t npl = (size_t)d.n * d.W;
    // sign planes: one extra row (n), always zero, that the step kernels
    // read for neighbours past a row's end
    const size_t nsp = npl + (size_t)d.W;
    CK(growv(w.x, w.cap_x, nst * es));
    CK(growv(w.y, w.cap_y, nst * es));
    CK(grow(w.S[0], w.cap_S0, nsp));
    CK(grow(w.S[1], w.cap_S1, nsp));
    CK(grow(w.Wp, w.cap_Wp, npl));
    CK(grow(w.fin, w.cap_fin, npl));
    CK(grow(w.chg, w.cap_chg, (size_t)d.W));
    CK(grow(w.newmask, w.cap_new, (size_t)d.W));
    CK(grow(w.stab, w.cap_stab, (size_t)d.Ap));
    CK(grow(w.bif, w.cap_bif, (size_t)d.Ap));
    CK(grow(w.prev, w.cap_prev, (size_t)d.Ap));
    CK(grow(w.ctl, w.cap_ctl, (size_t)CTL_N));
    CK(grow(w.eacc, w.cap_eacc, (size_t)d.Ap));
    if (J_nchunks) {
        CK(grow(w.part, w.cap_part, (size_t)J_nchunks * d.Ap * 2));
        CK(grow(w.hcount, w.cap_hcount, (size_t)J_nchunks * d.W));
    }
    CK(grow(w.cut, w.cap_cut, (size_t)d.Ap));
    const int64_t nwin = d.period > 0 ? total_steps / d.period + 2 : 2;
    CK(grow(w.wincount, w.cap_win, (size_t)nwin));
    CK(grow(w.coef32, w.cap_c32, (size_t)(total_steps + 2) * 4));
    CK(grow(w.coef64, w.cap_c64, (size_t)(total_steps + 2) * 4));
    if (d.trace) {
        CK(grow(w.trace, w.cap_trace, (size_t)nwin));
        CK(grow(w.trace_t0, w.cap_t0, (size_t)1));
    }
    cudaStream_t s = ctx->stream;
    CK(cudaMemsetAsync(w.Wp, 0xff, npl * 4, s));   // current_spins = -1 (ising.cu:128)
    CK(cudaMemsetAsync(w.fin, 0xff, npl * 4, s));  // final_spins = -1 (ising.cu:129)
    CK(cudaMemsetAsync(w.S[0], 0, nsp * 4, s));
    CK(cudaMemsetAsync(w.S[1], 0, nsp * 4, s));
    CK(cudaMemsetAsync(w.chg, 0, (size_t)d.W * 4, s));
    CK(cudaMemsetAsync(w.newmask, 0, (size_t)d.W * 4, s));
    CK(cudaMemsetAsync(w.stab, 0, (size_t)d.Ap * 4, s));
    CK(cudaMemsetAsync(w.bif, 0, (size_t)d.Ap, s));
    CK(cudaMemsetAsync(w.prev, 0, (size_t)d.Ap, s));
    CK(cudaMemsetAsync(w.ctl, 0, CTL_N * 4, s));
    CK(cudaMemsetAsync(w.wincount, 0, (size_t)nwin * 4, s));
    if (J_nchunks) CK(cudaMemsetAsync(w.hcount, 0, (size_t)J_nchunks * d.W * 4, s));
    return SBX_OK;
}

constexpr int64_t kRandChunk = 31 * 32;   // outputs per init thread
constexpr int kRandBits = 40;             // jump matrices kept: 2^40 threads

// x, y of one or more instances from their seeds' glibc rand() streams
// (src/ising.cu:91-95, src/ising_tsp.cu:55-59), one launch.  Padded agents
// and rows outside every instance are zero.  slot: null, or the state row of
// each instance row (a batch class's renumbering).
int init_instances(sbx_ctx *ctx, const SolveDims &d, std::vector<RandInst> &inst, bool tsp,
                   const int32_t *slot = nullptr)
{
    Work &w = ctx->w;
    cudaStream_t s = ctx->stream;
    if (!w.rjump_ready) {
        std::vector<uint32_t> mats;
        rand_jump_matrices(kRandChunk, kRandBits, mats);
        CK(grow(w.rjump, w.cap_rj, mats.size()));
        CK(cudaMemcpy(w.rjump, mats.data(), mats.size() * 4, cudaMemcpyHostToDevice));
        w.rjump_ready = true;
    }
    int64_t threads = 0;
    for (auto &I : inst) {
        I.thread_base = threads;
        const int64_t outputs = I.n * I.A * (tsp ? 1 : 2);
        threads += (outputs + kRandChunk - 1) / kRandChunk;
    }
    const size_t es = prec_bytes(d.prec), nst = (size_t)d.n * d.Ap;
    CK(cudaMemsetAsync(w.x, 0, nst * es, s));
    CK(cudaMemsetAsync(w.y, 0, nst * es, s));
    CK(grow(w.rinst, w.cap_rinst, inst.size()));
    CK(cudaMemcpyAsync(w.rinst, inst.data(), sizeof(RandInst) * inst.size(), cudaMemcpyHostToDevice, s));
    CK(launch_rand_init(d.prec, w.x, w.y, d.Ap, tsp, kRandChunk, w.rjump, w.rinst, (int)inst.size(),
                        threads, slot, s));
    // the instance table must outlive the async copy
    CK(cudaStreamSynchronize(s));
    return SBX_OK;
}

int init_state(sbx_ctx *ctx, const SolveDims &d, uint32_t seed, bool tsp)
{
    std::vector<RandInst> inst(1);
    inst[0].row_off = 0;
    inst[0].n = d.n;
    inst[0].A = d.A;
    rand_seed_window(seed, inst[0].V0);
    return init_instances(ctx, d, inst, tsp);
}

int upload_coef(sbx_ctx *ctx, const SolveDims &d, int64_t total_steps)
{
    std::vector<float> c32((size_t)(total_steps + 2) * 4);
    std::vector<double> c64((size_t)(total_steps + 2) * 4);
    for (int64_t k = 0; k < total_steps + 2; k++) {
        const double p = 1.025 * (double)k / d.steps;    // kernels.cu:15 / :225
        const double pc = p < 1.0 ? p : 1.0;
        const double v[4] = {d.dt * (pc + 1), d.dt * (pc - 1), d.dt * (p + 1), d.dt * (p - 1)};
        for (int j = 0; j < 4; j++) {
            c64[k * 4 + j] = v[j];
            c32[k * 4 + j] = (float)v[j];
        }
    }
    CK(cudaMemcpyAsync(ctx->w.coef32, c32.data(), c32.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->w.coef64, c64.data(), c64.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SBX_OK;
}

bool poll_stop(sbx_ctx *ctx, int64_t c, bool force_all)
{
    // Enqueue a read of the stop flag after chunk c; wait for the one issued
    // three chunks earlier.  At most three chunks run past the exit.
    const int slot = (int)(c & 3);
    cudaMemcpyAsync(&ctx->pinned[slot], ctx->w.ctl + CTL_STOP, 4, cudaMemcpyDeviceToHost, ctx->stream);
    cudaEventRecord(ctx->evp[slot], ctx->stream);
    const int64_t old = force_all ? c : c - 3;
    if (old < 0) return false;
    cudaEventSynchronize(ctx->evp[old & 3]);
    return ctx->pinned[old & 3] != 0;
}

// ---- streaming step tile

// The state (x and y) is more than half of L2: it streams from DRAM each step.
bool state_exceeds_half_l2(const SolveDims &d)
{
    return 2.0 * (double)d.n * d.Ap * prec_bytes(d.prec) > 0.5 * (double)dev_attr(cudaDevAttrL2CacheSize);
}

// A tile the step kernels are built for (k_step.cuh, step_kw): whole-warp
// rows take any vector width dividing the padded agents; 16, 8 or 4 lanes
// per row take the two widest vectors and exactly the padded agents, and
// rows with split heavy neighbour lists need whole-warp rows.
bool tile_ok(const SolveDims &d, bool big, int v, int lr, int bt)
{
    const int vm = 16 / (int)prec_bytes(d.prec);
    if ((v != 1 && v != 2 && v != 4 && v != 8) || v > vm) return false;
    if (bt != 128 && bt != 256) return false;
    if (lr == 32) return d.Ap % (32 * v) == 0;
    if (lr != 16 && lr != 8 && lr != 4) return false;
    return !big && (v == vm || v == vm / 2) && v * lr == d.Ap;
}

int default_v(const SolveDims &d)
{
    int v = 16 / (int)prec_bytes(d.prec);
    while (v > 1 && d.Ap % (32 * v)) v >>= 1;
    return v;
}

// The tile of a streaming solve.  Fields the caller set are kept; the rest
// come from the problem's cache or from timing every candidate tile over a
// few plain steps on the live state (*timed then asks the caller to set the
// initial state again).  Every tile computes the same results.
int pick_tile(sbx_ctx *ctx, SolveDims &d, const DevCsr &J, const sbx_params *pr, bool *timed)
{
    *timed = false;
    const bool big = J.unit && J.nchunks > 0;
    const int fv = pr->lane_agents, flr = pr->row_lanes, fbt = pr->block_threads;
    const int fcm = pr->count_mode;   // 1 byte counters, 2 bit planes, 3 mixed
    const int fst = pr->staging;      // 1 direct loads, 2 staged rows
    // staged rows pay off only when the state streams from DRAM
    const bool can_stage = J.unit && state_exceeds_half_l2(d);
    std::vector<Tile> cands;
    const int vs[4] = {8, 4, 2, 1}, lrs[4] = {32, 16, 8, 4}, bts[2] = {256, 128};
    const int st_forced = (fst == 2 && J.unit) ? 1 : 0;   // staging asked for: whole-warp rows only
    // mixed counting exists in the heavy-row kernels only
    for (int cm = 0; cm < (J.unit ? (big ? 3 : 2) : 1); cm++)
        for (int v : vs)
            for (int lr : lrs)
                for (int bt : bts) {
                    if ((fv && v != fv) || (flr && lr != flr) || (fbt && bt != fbt) || (fcm && cm != fcm - 1))
                        continue;
                    if (st_forced && lr != 32) continue;
                    if (tile_ok(d, big, v, lr, bt)) cands.push_back(Tile{v, lr, bt, cm, st_forced});
                }
    if (cands.empty())
        return fail(ctx, SBX_ERR_ARG, "no streaming tile fits lane_agents / row_lanes / block_threads / count_mode");
    auto apply = [&](const Tile &t) {
        d.tv = t.v;
        d.tlr = t.lr;
        d.tbt = t.bt;
        d.tcm = t.cm;
        d.tst = t.st;
    };
    apply(cands[0]);
    if (cands.size() == 1) return SBX_OK;
    if (pr->flags & SBX_FLAG_NO_TUNE) {
        // fixed heuristic: widest dividing vector, whole-warp rows, 256
        // threads, byte counters
        for (const Tile &t : cands)
            if (t.v == default_v(d) && t.lr == 32 && t.bt == 256 && t.cm == 0 && t.st == 0) apply(t);
        return SBX_OK;
    }
    char key[192];
    snprintf(key, sizeof key, "%lld/%lld/%d/%d/%lld/%d%d%d/%d/%d/%d/%d/%d/%d/%d/%d", (long long)J.n,
             (long long)J.nnz, J.max_deg, J.nchunks, (long long)J.nheavy, (int)J.unit, (int)J.skewed,
             (int)(J.c0r32 != nullptr), d.prec, d.Ap, d.fused, fv, flr, fbt, fcm, fst);
    auto &cache = ctx->tiles;
    auto it = cache.find(key);
    if (it != cache.end()) {
        apply(it->second);
        return SBX_OK;
    }
    cudaStream_t s = ctx->stream;
    Work &w = ctx->w;
    // about 2 ms of launches per measurement, best of two rounds
    CK(launch_plain_steps(d, J, w, 1, s));
    CK(cudaEventRecord(ctx->ev0, s));
    CK(launch_plain_steps(d, J, w, 1, s));
    CK(cudaEventRecord(ctx->ev1, s));
    CK(cudaEventSynchronize(ctx->ev1));
    float one = 0;
    CK(cudaEventElapsedTime(&one, ctx->ev0, ctx->ev1));
    const int reps = std::max(3, std::min(64, (int)(2.0 / std::max(one, 1e-3f))));
    std::vector<float> best(cands.size(), 1e30f);
    for (int round = 0; round < 2; round++)
        for (size_t i = 0; i < cands.size(); i++) {
            apply(cands[i]);
            CK(launch_plain_steps(d, J, w, 1, s));
            CK(cudaEventRecord(ctx->ev0, s));
            CK(launch_plain_steps(d, J, w, reps, s));
            CK(cudaEventRecord(ctx->ev1, s));
            CK(cudaEventSynchronize(ctx->ev1));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
            best[i] = std::min(best[i], ms / reps);
        }
    size_t bi = 0;
    for (size_t i = 1; i < cands.size(); i++)
        if (best[i] < best[bi]) bi = i;
    Tile win = cands[bi];
    // staged rows: tried on the winning tile only, when the state streams
    if (!fst && can_stage && win.lr == 32 && !win.st) {
        Tile t = win;
        t.st = 1;
        float bs = 1e30f;
        for (int round = 0; round < 2; round++) {
            apply(t);
            CK(launch_plain_steps(d, J, w, 1, s));
            CK(cudaEventRecord(ctx->ev0, s));
            CK(launch_plain_steps(d, J, w, reps, s));
            CK(cudaEventRecord(ctx->ev1, s));
            CK(cudaEventSynchronize(ctx->ev1));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
            bs = std::min(bs, ms / reps);
        }
        if (bs < best[bi]) win = t;
    }
    apply(win);
    cache[key] = win;
    *timed = true;
    return SBX_OK;
}

// Trace of the last solve: records to the context; the first window whose
// best cut reaches target gives the time and steps to target.
int read_trace(sbx_ctx *ctx, const SolveDims &d, int32_t traced, double target, sbx_result *res)
{
    res->time_to_target_us = -1;
    res->steps_to_target = -1;
    ctx->trace.clear();
    if (!d.trace) return SBX_OK;
    const size_t cnt = std::min((size_t)std::max(traced, 0), ctx->w.cap_trace);
    ctx->trace.resize(cnt);
    if (cnt)
        CK(cudaMemcpy(ctx->trace.data(), ctx->w.trace, sizeof(TraceRec) * cnt, cudaMemcpyDeviceToHost));
    if (target > 0)
        for (const TraceRec &r : ctx->trace)
            if (r.best >= target) {
                res->time_to_target_us = (double)r.t_ns / 1000.0;
                res->steps_to_target = r.steps;
                break;
            }
    return SBX_OK;
}

// The streaming loop of one solve: the pre-step Update_XY, then windows of
// d.period steps (a captured CUDA graph per window, replayed), with the
// all-bifurcated exit polled when d.uw.  Profile mode launches directly and
// times every step kernel with events.
int run_stream(sbx_ctx *ctx, const void *key_obj, const SolveDims &d, const DevCsr &J,
               int64_t nchunks, bool profile, bool use_graph, int *launches_out, double *kernel_ms_out)
{
    cudaStream_t s = ctx->stream;
    int launches = 0;
    double kernel_ms = 0;
    if (d.trace) {
        CK(launch_trace_start(ctx->w, s));
        launches++;
    }
    CK(launch_prestep(d, J, ctx->w, s, &launches));
    if (nchunks) {
        int per_chunk = 0;
        if (use_graph) {
            char key[256];
            snprintf(key, sizeof key, "%p/%lld/%d/%d/%d/%d/%d/%d/%d/%d/%.17g/%llu/%p/%d/%d/%d/%d/%d/%d/%d/%d",
                     key_obj, (long long)d.n, d.A, d.prec, d.period, d.fused, d.uw, d.threshold,
                     (int)d.pdl, d.steps, d.c0, (unsigned long long)g_alloc_gen, (void *)s, d.tv,
                     d.tlr, d.tbt, d.tcm, d.tst, d.trace, d.giveup, d.tbsm);
            if (!ctx->gexec || ctx->gkey != key) {
                if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
                ctx->gexec = nullptr;
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = launch_chunk(d, J, ctx->w, s, &per_chunk);
                cudaError_t e2 = cudaStreamEndCapture(s, &g);
                CK(e);
                CK(e2);
                CK(cudaGraphInstantiate(&ctx->gexec, g, 0));
                cudaGraphDestroy(g);
                ctx->gkey = key;
                ctx->gper_chunk = per_chunk;
            } else {
                per_chunk = ctx->gper_chunk;
            }
            for (int64_t c = 0; c < nchunks; c++) {
                CK(cudaGraphLaunch(ctx->gexec, s));
                launches += per_chunk;
                if (d.uw && poll_stop(ctx, c, false)) break;
            }
        } else {
            cudaEvent_t *evs = nullptr;
            if (profile) {
                while ((int)ctx->prof.size() < 2 * d.period + 2) {
                    cudaEvent_t e;
                    CK(cudaEventCreate(&e));
                    ctx->prof.push_back(e);
                }
                evs = ctx->prof.data();
            }
            for (int64_t c = 0; c < nchunks; c++) {
                CK(launch_chunk(d, J, ctx->w, s, &launches, evs));
                if (profile) {
                    CK(cudaStreamSynchronize(s));
                    // the step kernels, and the isolated rows' window kernel
                    for (int i = 0; i <= d.period; i++) {
                        if (i == d.period && !(d.fused && J.niso && !d.tbsm)) break;
                        float t = 0;
                        CK(cudaEventElapsedTime(&t, evs[2 * i], evs[2 * i + 1]));
                        kernel_ms += t;
                    }
                }
                if (d.uw && poll_stop(ctx, c, profile)) break;
            }
        }
    }
    *launches_out += launches;
    *kernel_ms_out += kernel_ms;
    return SBX_OK;
}

int ensure_rs_csr(sbx_ctx *ctx, DevCsr &J);

int solve_maxcut(sbx_ctx *ctx, const sbx_problem *p, const sbx_params *pr, sbx_result *res,
                 double *agent_values)
{
    // the problem's device arrays, made on its first single solve
    int urc = upload_device(ctx, const_cast<DevCsr &>(p->J));
    if (urc) return urc;
    SolveDims d;
    d.n = p->J.n;
    d.A = pr->agents;
    d.Ap = (pr->agents + 31) / 32 * 32;
    d.W = d.Ap / 32;
    d.prec = pr->precision;
    d.steps = pr->steps;
    d.period = pr->period > 0 ? pr->period : 100;       // csr.cuh:109
    d.threshold = pr->threshold > 0 ? pr->threshold : 25; // csr.cuh:108
    d.fused = pr->fused ? 1 : 0;
    d.uw = pr->update_window ? 1 : 0;
    d.dt = pr->dt;
    d.xi0 = xi0_of(p->J);
    d.c0 = d.dt * d.xi0;
    d.pdl = !(pr->flags & SBX_FLAG_NO_PDL);
    d.giveup = (pr->flags & SBX_FLAG_TEST_GIVEUP) ? 1 : 0;
    d.trace = (pr->trace || pr->target > 0) ? 1 : 0;
    const bool profile = (pr->flags & SBX_FLAG_PROFILE) != 0;
    const bool use_graph = !(pr->flags & SBX_FLAG_NO_GRAPH) && !profile;
    double kernel_ms = 0;
    const int32_t run = pr->run_steps > 0 ? std::min(pr->run_steps, pr->steps) : pr->steps;
    const int64_t nchunks = run > 0 ? (run + d.period - 1) / d.period : 0;
    const int64_t total = nchunks * d.period;
    cudaStream_t s = ctx->stream;
    if (d.trace && pr->kernel == SBX_KERNEL_RESIDENT)
        return fail(ctx, SBX_ERR_UNSUPPORTED, "trace / target: streaming kernel only");
    int rc = ensure_common(ctx, d, total, p->J.nchunks);
    if (rc) return rc;
    if ((rc = upload_coef(ctx, d, total))) return rc;
    if ((rc = init_state(ctx, d, pr->seed, false))) return rc;

    // on-chip kernels first: shared-memory resident, then register + shared
    int ka = 0, rs = 0;
    if ((pr->kernel == SBX_KERNEL_AUTO || pr->kernel == SBX_KERNEL_RESIDENT) && !d.trace)
        ka = resident_pick_ka(d, p->J, pr->agents_per_block);
    if ((pr->kernel == SBX_KERNEL_AUTO || pr->kernel == SBX_KERNEL_RESIDENT_SPLIT) && !d.trace && !ka &&
        !pr->agents_per_block)
        rs = resident_rs_pick(d, p->J, pr->kernel == SBX_KERNEL_RESIDENT_SPLIT);
    if (pr->kernel == SBX_KERNEL_RESIDENT && !ka)
        return fail(ctx, SBX_ERR_UNSUPPORTED, "resident kernel: shape does not fit on chip (or FP64)");
    if (pr->kernel == SBX_KERNEL_RESIDENT_SPLIT && !rs)
        return fail(ctx, SBX_ERR_UNSUPPORTED,
                    "split resident kernel: 16-bit fused state, degree <= 127 and fitting on chip only");
    if (rs && (rc = ensure_rs_csr(ctx, const_cast<DevCsr &>(p->J)))) return rc;
    if (!ka && !rs) {
        bool timed = false;
        if ((rc = pick_tile(ctx, d, p->J, pr, &timed))) return rc;
        if (timed && (rc = init_state(ctx, d, pr->seed, false))) return rc;
    }
    int launches = 0, hot = 0;
    CK(cudaEventRecord(ctx->ev0, s));
    auto resident = [&](int32_t step0, int32_t nsteps, bool first) {
        return ka ? launch_resident(d, p->J, ctx->w, ka, step0, nsteps, first, s)
                  : launch_resident_rs(d, p->J, ctx->w, rs, step0, nsteps, first, false, s);
    };
    bool coop_done = false;
    if (rs && d.uw && nchunks > 0) {
        // every window in one co-resident launch, the exit decided on the device
        CK(grow(ctx->w.gbar, ctx->w.cap_gbar, (size_t)1));
        CK(cudaMemsetAsync(ctx->w.gbar, 0, sizeof(int32_t), s));
        const cudaError_t e = launch_resident_rs(d, p->J, ctx->w, rs, 0, (int32_t)total, true, true, s);
        if (e == cudaSuccess) {
            coop_done = true;
            launches++;
            hot++;
        } else if (e != cudaErrorCooperativeLaunchTooLarge) {
            CK(e);
        } else {
            (void)cudaGetLastError();
        }
    }
    if (coop_done) {
    } else if (ka || rs) {
        if (d.uw) {
            for (int64_t c = 0; c < std::max<int64_t>(nchunks, 1); c++) {
                CK(resident((int32_t)(c * d.period), nchunks ? d.period : 0, c == 0));
                launches++;
                hot++;
                if (poll_stop(ctx, c, false)) break;
            }
        } else {
            CK(resident(0, (int32_t)total, true));
            launches++;
            hot++;
        }
    } else {
        if ((rc = run_stream(ctx, p, d, p->J, nchunks, profile, use_graph, &launches, &kernel_ms)))
            return rc;
        hot = launches;
    }
    CK(cudaEventRecord(ctx->ev1, s));
    const int loop_launches = launches;
    CK(launch_cut(d, p->J, ctx->w, ctx->w.Wp, s, &launches));
    // the statistics line on the device (src/ising.cu:238-265)
    CK(grow(ctx->w.stats, ctx->w.cap_stats, (size_t)7));
    CK(launch_stats(ctx->w.cut, d.A, ctx->w.stats, s));
    launches++;
    double st[7];
    int32_t ctl[CTL_N];
    std::vector<uint8_t> bif((size_t)d.A);
    CK(cudaMemcpyAsync(st, ctx->w.stats, sizeof st, cudaMemcpyDeviceToHost, s));
    if (agent_values)
        CK(cudaMemcpyAsync(agent_values, ctx->w.cut, sizeof(double) * d.A, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ctl, ctx->w.ctl, sizeof ctl, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(bif.data(), ctx->w.bif, d.A, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    if (ctl[CTL_ERR]) return fail(ctx, SBX_ERR_CUDA, "a bounded wait in the step kernel gave up");
    memset(res, 0, sizeof *res);
    finish_stats(st, d.A, res);
    res->time_us = ms * 1000.0;
    res->xi0 = d.xi0;
    res->steps_run = ctl[CTL_STEP];
    res->windows_run = ctl[CTL_WINDOWS];
    for (uint8_t b : bif) res->bifurcated += b;
    res->kernel_used = ka ? SBX_KERNEL_RESIDENT : rs ? SBX_KERNEL_RESIDENT_SPLIT : SBX_KERNEL_STREAM;
    res->agents_per_block = ka ? ka : rs ? 8 : 0;
    if (!ka && !rs) {
        res->lane_agents = d.tv ? d.tv : default_v(d);
        res->row_lanes = d.tlr;
        res->block_threads = d.tbt;
        res->count_mode = d.tcm + 1;
        res->staging = d.tst + 1;
    }
    if ((rc = read_trace(ctx, d, ctl[CTL_TRACED], pr->target, res))) return rc;
    if (ka || rs) {
        res->kernel_launches = hot;
        res->kernel_ms = profile ? ms : 0;
    } else {
        // the step kernels: one per SB step actually run
        res->kernel_launches = profile ? (int64_t)res->steps_run : loop_launches;
        res->kernel_ms = kernel_ms;
    }
    res->gpu_launches = launches + 1;   // + the init kernel
    ctx->have = true;
    ctx->last_tsp = false;
    ctx->d = d;
    return SBX_OK;
}

int solve_tsp(sbx_ctx *ctx, const sbx_problem *p, const sbx_params *pr, sbx_result *res,
              double *agent_values)
{
    const DevTsp &t = p->T;
    SolveDims d;
    d.n = (int64_t)t.N * t.N;
    d.A = pr->agents;
    d.Ap = (pr->agents + 31) / 32 * 32;
    d.W = d.Ap / 32;
    d.prec = pr->precision;
    d.steps = pr->steps;
    d.period = pr->period > 0 ? pr->period : pr->steps / 10;   // ising_tsp.cu:132
    if (d.steps > 0 && d.period <= 0)
        return fail(ctx, SBX_ERR_ARG, "TSP: 1..9 steps give a zero window period (the reference never ends)");
    d.threshold = pr->threshold > 0 ? pr->threshold : 50;        // csr.cuh:167
    d.dt = pr->dt;
    d.xi0 = 0.002;                                               // ising_tsp.cu:61
    d.c0 = d.dt * d.xi0;
    d.pdl = !(pr->flags & SBX_FLAG_NO_PDL);
    d.giveup = (pr->flags & SBX_FLAG_TEST_GIVEUP) ? 1 : 0;
    const int32_t run = pr->run_steps > 0 ? std::min(pr->run_steps, pr->steps) : pr->steps;
    const int64_t nwin = d.period > 0 ? (run + d.period - 1) / d.period : 1;
    const int64_t total = d.period > 0 ? nwin * d.period : 0;
    d.nwin = (int32_t)nwin;
    cudaStream_t s = ctx->stream;
    int rc = ensure_common(ctx, d, total);
    if (rc) return rc;
    Work &w = ctx->w;
    CK(grow(w.tours, w.cap_tours, (size_t)d.Ap * t.N));
    CK(grow(w.valid, w.cap_valid, (size_t)d.Ap));
    CK(cudaMemsetAsync(w.tours, 0xff, sizeof(int32_t) * d.Ap * t.N, s));
    CK(cudaMemsetAsync(w.valid, 0, sizeof(int32_t) * d.Ap, s));
    // schedules a(t), b(t) (kernels.cu:553-559), n = 2 (ising_tsp.cu:134)
    std::vector<float> sch((size_t)(total + 1) * 2);
    std::vector<double> ab((size_t)(total + 1) * 2);
    for (int64_t k = 0; k <= total; k++) {
        const int n2 = 2;
        double a_t = n2 * 1.04 * (double)k / d.steps;
        double b_t = 0.5 + ((double)0.5 * std::pow((double)k / (double)d.steps, 1.9));
        a_t = a_t < n2 ? a_t : n2;
        b_t = b_t < 1 ? b_t : 1;
        ab[k * 2] = a_t;
        ab[k * 2 + 1] = b_t;
        sch[k * 2] = (float)b_t;
        sch[k * 2 + 1] = (float)(d.dt * -(1 - a_t));
    }
    CK(grow(w.sched, w.cap_sched, (size_t)(total + 1)));
    CK(grow(w.ab, w.cap_ab, (size_t)(total + 1)));
    CK(cudaMemcpyAsync(w.sched, sch.data(), sch.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(w.ab, ab.data(), ab.size() * 8, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    if ((rc = init_state(ctx, d, pr->seed, true))) return rc;
    // the tensor-core kernel for 16-bit states that fit it (AUTO or forced),
    // else the CUDA-core resident kernel, else streaming
    const bool tc = (pr->kernel == SBX_KERNEL_AUTO || pr->kernel == SBX_KERNEL_TENSOR) && tsp_tensor_fits(d, t) &&
                    (pr->agents_per_block <= 0 || pr->agents_per_block == kTspTensorAgents);
    if (pr->kernel == SBX_KERNEL_TENSOR && !tc)
        return fail(ctx, SBX_ERR_UNSUPPORTED, "TSP tensor-core kernel: BF16/FP16 state and 3 <= N <= 32 only");
    int ka = tc ? kTspTensorAgents : 0;
    if (!tc && pr->kernel != SBX_KERNEL_STREAM) ka = tsp_pick_ka(d, t, pr->agents_per_block);
    if (pr->kernel == SBX_KERNEL_RESIDENT && !ka)
        return fail(ctx, SBX_ERR_UNSUPPORTED, "TSP resident kernel: N > 32, FP64 or tile too wide");
    if (!ka) {
        CK(growv(w.x2, w.cap_x2, (size_t)d.n * d.Ap * prec_bytes(d.prec)));
        CK(grow(w.visits, w.cap_visits, (size_t)2 * t.N * d.Ap));
        CK(cudaMemsetAsync(w.visits, 0, sizeof(int32_t) * 2 * t.N * d.Ap, s));
    }
    int launches = 0, hot = 0;
    CK(cudaEventRecord(ctx->ev0, s));
    if (tc) {
        CK(launch_tsp_tensor(d, t, w, pr->row_lanes, s));
        launches = hot = 1;
    } else if (ka) {
        CK(launch_tsp_resident(d, t, w, ka, s));
        launches = hot = 1;
    } else {
        CK(launch_tsp_stream(d, t, w, s, &launches));
        hot = launches;
        int32_t c2[2] = {(int32_t)total, (int32_t)nwin};
        CK(cudaMemcpyAsync(w.ctl, c2, sizeof c2, cudaMemcpyHostToDevice, s));
    }
    CK(cudaEventRecord(ctx->ev1, s));
    // tour lengths on the device (src/ising_tsp.cu:272-287, FP64 in tour order)
    CK(launch_tsp_lengths(t, w.tours, w.valid, d.A, w.cut, s));
    launches++;
    std::vector<int32_t> valid((size_t)d.A);
    std::vector<double> lens((size_t)d.A);
    std::vector<uint8_t> bif((size_t)d.A);
    int32_t ctl[CTL_N];
    CK(cudaMemcpyAsync(lens.data(), w.cut, lens.size() * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(valid.data(), w.valid, valid.size() * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(bif.data(), w.bif, d.A, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(ctl, w.ctl, sizeof ctl, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (ctl[CTL_ERR]) return fail(ctx, SBX_ERR_CUDA, "a bounded wait in the step kernel gave up");
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    // Decode and statistics, src/ising_tsp.cu:188-239 and :272-287.
    memset(res, 0, sizeof *res);
    res->time_to_target_us = -1;
    res->steps_to_target = -1;
    std::vector<double> all;
    double total_len = 0, mn = DBL_MAX, mx = -DBL_MAX;
    int32_t best = -1;
    const int N = t.N;
    for (int32_t a = 0; a < d.A; a++) {
        double len = NAN;
        if (valid[a] > 0) {
            len = lens[(size_t)a];
            all.push_back(len);
            total_len += len;
            if (len < mn) {
                mn = len;
                best = a;
            }
            if (len > mx) mx = len;
        }
        if (agent_values) agent_values[a] = len;
    }
    const int64_t nv = (int64_t)all.size();
    const double avg = total_len / nv;
    double sd = 0;
    for (double v : all) sd += std::pow(v - avg, 2);
    sd = std::pow(sd / (nv - 1), 0.5);
    res->min = mn;
    res->max = mx;
    res->mean = avg;
    res->std = sd;
    res->valid = nv;
    res->best_agent = best;
    res->time_us = ms * 1000.0;
    res->xi0 = d.xi0;
    res->steps_run = ctl[CTL_STEP];
    res->windows_run = ctl[CTL_WINDOWS];
    for (uint8_t b : bif) res->bifurcated += b;
    res->kernel_used = tc ? SBX_KERNEL_TENSOR : ka ? SBX_KERNEL_RESIDENT : SBX_KERNEL_STREAM;
    res->agents_per_block = ka;
    if (tc) res->row_lanes = tsp_tensor_threads_per_row(pr->row_lanes);
    res->kernel_launches = hot;
    // SBX_FLAG_PROFILE: the SB loop's kernels (the whole solve is one
    // resident launch, or the streaming steps and windows)
    res->kernel_ms = (pr->flags & SBX_FLAG_PROFILE) ? ms : 0.0;
    res->gpu_launches = launches + 1;
    ctx->have = true;
    ctx->last_tsp = true;
    ctx->d = d;
    ctx->N = N;
    return SBX_OK;
}


// Pack the instances of one agent class into a block-diagonal matrix.
int build_class(sbx_ctx *ctx, BatchClass &c)
{
    const size_t ni = c.probs.size();
    int64_t n = 0, nnz = 0;
    std::vector<int64_t> e_off(ni + 1, 0);
    for (size_t i = 0; i < ni; i++) {
        const sbx_problem *p = c.probs[i];
        c.row_off.push_back(n);
        n += p->J.n;
        nnz += p->J.nnz;
        e_off[i + 1] = nnz;
        c.wsum.push_back(p->J.wsum);
    }
    if (n > INT32_MAX - 1 || nnz > INT32_MAX) return fail(ctx, SBX_ERR_UNSUPPORTED, "batch too large for int32 indices");
    std::vector<int32_t> rp((size_t)n + 1), col((size_t)nnz), rinst((size_t)n);
    std::vector<double> val((size_t)nnz);
    c.xi0.assign(ni, 0.0);
    c.slot.assign((size_t)n, 0);
    // instances on host threads: each one's xi0 (its sums in the reference's
    // order) and its block of the block-diagonal matrix, rows renumbered by
    // decreasing degree (ties in row order) so that the rows a warp takes
    // together have about the same number of neighbours; each row keeps its
    // entries in their order, columns renamed.  Cuts, windows and integer
    // neighbour sums do not depend on the numbering; the init and the state
    // readback go through slot.
    const int T = nnz > (1 << 20) ? host_threads() : 1;
    parallel(T, [&](int t, int TT) {
        std::vector<int32_t> ord, inv;
        for (size_t i = (size_t)t; i < ni; i += (size_t)TT) {
            const DevCsr &J = c.probs[i]->J;
            c.xi0[i] = xi0_of(J);
            const int64_t r0 = c.row_off[i];
            const std::vector<int32_t> &hr = J.hrowptr;
            ord.resize((size_t)J.n);
            inv.resize((size_t)J.n);
            std::iota(ord.begin(), ord.end(), 0);
            std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) {
                return hr[(size_t)a + 1] - hr[(size_t)a] > hr[(size_t)b + 1] - hr[(size_t)b];
            });
            for (int64_t k = 0; k < J.n; k++) inv[(size_t)ord[(size_t)k]] = (int32_t)k;
            int64_t e = e_off[i];
            for (int64_t k = 0; k < J.n; k++) {
                const int32_t o = ord[(size_t)k];
                rp[r0 + k] = (int32_t)e;
                rinst[r0 + k] = (int32_t)i;
                c.slot[(size_t)(r0 + o)] = (int32_t)(r0 + k);
                for (int32_t j = hr[(size_t)o]; j < hr[(size_t)o + 1]; j++, e++) {
                    col[e] = inv[(size_t)J.hcol[(size_t)j]] + (int32_t)r0;
                    val[e] = J.hval[(size_t)j];
                }
            }
        }
    });
    rp[n] = (int32_t)nnz;
    int rc = upload_csr(ctx, c.J, n, nnz, rp.data(), col.data(), val.data(), 0.0, false, false, true);
    if (rc) return rc;
    c.J.hrowptr = std::move(rp);
    c.J.hcol = std::move(col);
    c.J.hval = std::move(val);
    if ((rc = upload_device(ctx, c.J))) return rc;
    CK(cudaMalloc(&c.J.rinst, sizeof(int32_t) * n));
    CK(cudaMalloc(&c.J.c0r32, sizeof(float) * n));
    CK(cudaMalloc(&c.J.c0r64, sizeof(double) * n));
    CK(cudaMemcpy(c.J.rinst, rinst.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&c.dslot, sizeof(int32_t) * n));
    CK(cudaMemcpy(c.dslot, c.slot.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
    c.J.ninst = (int32_t)c.probs.size();
    CK(cudaMalloc(&c.J.iagents, sizeof(int32_t) * c.J.ninst));
    CK(cudaMalloc(&c.J.iwsum, sizeof(double) * c.J.ninst));
    CK(cudaMemcpy(c.J.iagents, c.agents.data(), sizeof(int32_t) * c.J.ninst, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c.J.iwsum, c.wsum.data(), sizeof(double) * c.J.ninst, cudaMemcpyHostToDevice));
    c.agent_off.assign(ni + 1, 0);
    for (size_t i = 0; i < ni; i++) c.agent_off[i + 1] = c.agent_off[i] + c.agents[i];
    CK(cudaMalloc(&c.daoff, sizeof(int32_t) * (ni + 1)));
    CK(cudaMemcpy(c.daoff, c.agent_off.data(), sizeof(int32_t) * (ni + 1), cudaMemcpyHostToDevice));
    return SBX_OK;
}

// The matrix in perm order for the register + shared resident kernel: row s
// is row perm[s], its columns renamed to their slots, entries in the original
// order within the row (the FP32 sums of real weights keep their order).
int ensure_rs_csr(sbx_ctx *ctx, DevCsr &J)
{
    if (J.rs_rowptr) return SBX_OK;
    const int64_t n = J.n;
    std::vector<int32_t> inv((size_t)n), rp((size_t)n + 1, 0);
    for (int64_t s = 0; s < n; s++) inv[(size_t)J.hperm[(size_t)s]] = (int32_t)s;
    std::vector<uint32_t> cw((size_t)std::max<int64_t>(J.nnz, 1));
    std::vector<float> vf((size_t)std::max<int64_t>(J.nnz, 1));
    int64_t e = 0;
    for (int64_t s = 0; s < n; s++) {
        const int32_t r = J.hperm[(size_t)s];
        for (int32_t k = J.hrowptr[(size_t)r]; k < J.hrowptr[(size_t)r + 1]; k++, e++) {
            const double v = J.hval[(size_t)k];
            cw[(size_t)e] = (uint32_t)inv[(size_t)J.hcol[(size_t)k]] | ((J.unit && v < 0) ? 0x80000000u : 0u);
            vf[(size_t)e] = (float)v;
        }
        rp[(size_t)s + 1] = (int32_t)e;
    }
    CK(cudaMalloc(&J.rs_rowptr, sizeof(int32_t) * (n + 1)));
    CK(cudaMalloc(&J.rs_colw, sizeof(uint32_t) * cw.size()));
    CK(cudaMalloc(&J.rs_valf, sizeof(float) * vf.size()));
    CK(cudaMemcpy(J.rs_rowptr, rp.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(J.rs_colw, cw.data(), sizeof(uint32_t) * cw.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(J.rs_valf, vf.data(), sizeof(float) * vf.size(), cudaMemcpyHostToDevice));
    return SBX_OK;
}

// dt * xi0 of each row's instance (src/ising.cu:258 with the instance's xi0).
int upload_c0(sbx_ctx *ctx, BatchClass &c, double dt)
{
    if (c.dt == dt) return SBX_OK;
    std::vector<float> f((size_t)c.J.n);
    std::vector<double> d((size_t)c.J.n);
    for (size_t i = 0; i < c.probs.size(); i++) {
        const double c0 = dt * c.xi0[i];
        for (int64_t r = 0; r < c.probs[i]->J.n; r++) {
            d[c.row_off[i] + r] = c0;
            f[c.row_off[i] + r] = (float)c0;
        }
    }
    CK(cudaMemcpy(c.J.c0r32, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c.J.c0r64, d.data(), sizeof(double) * d.size(), cudaMemcpyHostToDevice));
    c.dt = dt;
    return SBX_OK;
}

void free_rb(DevRb &B)
{
    cudaFree(B.rowptr);
    cudaFree(B.colw);
    cudaFree(B.valf);
    cudaFree(B.c0);
    cudaFree(B.perm);
    cudaFree(B.bin_off);
    cudaFree(B.cta_bin);
    B = DevRb();
}

void free_bsm(DevBsm &M)
{
    cudaFree(M.lcol);
    cudaFree(M.rinfo);
    cudaFree(M.seg);
    cudaFree(M.cta_seg);
    cudaFree(M.ioff);
    cudaFree(M.in);
    M = DevBsm();
}

// Can the class run the shared-memory-plane step kernel: 16-bit state, +-1
// weights, at most 127 neighbours per row (seven count planes), 32, 64 or 128
// padded agents, instances of at most 32,767 rows (15-bit local columns), and
// the largest instance's plane fits in shared memory.
bool bsm_ok(const BatchClass &c, const SolveDims &d)
{
    if (d.prec != P_BF16 && d.prec != P_F16) return false;
    if (!c.J.unit || c.J.max_deg > kHeavy) return false;
    if (d.W != 1 && d.W != 2 && d.W != 4) return false;
    int64_t maxn = 0;
    for (const sbx_problem *q : c.probs) maxn = std::max<int64_t>(maxn, q->J.n);
    if (maxn > 32767) return false;
    const int optin = dev_attr(cudaDevAttrMaxSharedMemoryPerBlockOptin);
    return (int64_t)bsm_smem_bytes(maxn, d.W) + 1024 <= (int64_t)optin;
}

// The plan: columns as byte offsets into the instance's plane, and the rows
// (in instance order) cut into one contiguous run per CTA of about equal
// cost, each run split at instance boundaries.  A row costs its neighbours
// plus the update of its agents, 20 (W + 1) neighbours' worth (timed on
// GB300 for batch512 at 64 agents: 240.7 us a step, against 243.0 with
// 16 (W + 1), 242.4 with 24 (W + 1) and 263.1 with 8 (W + 1)).
int build_bsm(sbx_ctx *ctx, BatchClass &c, int W)
{
    DevBsm &M = c.bsm;
    const int64_t n = c.J.n;
    const size_t ni = c.probs.size();
    // each row's entries padded to whole blocks of eight (the padding reads
    // the instance's all-zero row); rinfo = first block << 7 | degree
    std::vector<uint32_t> rinfo((size_t)n);
    int64_t blocks = 0;
    for (int64_t r = 0; r < n; r++) {
        const int64_t deg = c.J.hrowptr[(size_t)r + 1] - c.J.hrowptr[(size_t)r];
        if (deg > 127 || blocks >= ((int64_t)1 << 25))
            return fail(ctx, SBX_ERR_UNSUPPORTED, "batch: shared-plane kernel row index out of range");
        rinfo[(size_t)r] = (uint32_t)(blocks << 7) | (uint32_t)deg;
        blocks += (deg + 7) / 8;
    }
    const int64_t nnz_p = blocks * 8;
    std::vector<uint16_t> lcol((size_t)nnz_p);
    std::vector<int32_t> ioff(ni), in(ni);
    int64_t maxn = 0;
    for (size_t i = 0; i < ni; i++) {
        ioff[i] = (int32_t)c.row_off[i];
        in[i] = (int32_t)c.probs[i]->J.n;
        maxn = std::max<int64_t>(maxn, in[i]);
        if (in[i] > 32767) return fail(ctx, SBX_ERR_UNSUPPORTED, "batch: shared-plane kernel instance too large");
    }
    // the instances' blocks on host threads (disjoint ranges of lcol)
    std::atomic<int> outside(0);
    parallel(c.J.nnz > (1 << 20) ? host_threads() : 1, [&](int t, int TT) {
        for (size_t i = (size_t)t; i < ni; i += (size_t)TT) {
            const int64_t r0 = ioff[i], rn = in[i];
            const uint16_t zrow = (uint16_t)rn;
            for (int64_t r = r0; r < r0 + rn; r++) {
                int64_t o = (int64_t)(rinfo[(size_t)r] >> 7) * 8;
                const int64_t e1 = c.J.hrowptr[(size_t)r + 1];
                for (int64_t e = c.J.hrowptr[(size_t)r]; e < e1; e++) {
                    const int64_t lc = (int64_t)c.J.hcol[(size_t)e] - r0;
                    // the kernel reads the plane at this offset: it must be
                    // a row of the instance (a block-diagonal matrix
                    // guarantees it)
                    if (lc < 0 || lc >= rn) {
                        outside = 1;
                        return;
                    }
                    lcol[(size_t)o++] = (uint16_t)((uint32_t)lc | (c.J.hval[(size_t)e] < 0 ? 0x8000u : 0u));
                }
                while (o & 7) lcol[(size_t)o++] = zrow;
            }
        }
    });
    if (outside) return fail(ctx, SBX_ERR_ARG, "batch: a column outside its instance");
    const int grid = std::max(1, dev_attr(cudaDevAttrMultiProcessorCount));
    const double row_cost = 20.0 * W + 20.0;
    double total = 0;
    for (int64_t r = 0; r < n; r++) total += row_cost + (c.J.hrowptr[(size_t)r + 1] - c.J.hrowptr[(size_t)r]);
    std::vector<int32_t> seg, cta((size_t)grid + 1, 0);
    int64_t r = 0;
    size_t inst = 0;
    double acc = 0;
    for (int k = 0; k < grid; k++) {
        cta[(size_t)k] = (int32_t)(seg.size() / 3);
        const double goal = total * (double)(k + 1) / grid;
        const int64_t a = r;
        while (r < n && (k == grid - 1 || acc < goal)) {
            acc += row_cost + (c.J.hrowptr[(size_t)r + 1] - c.J.hrowptr[(size_t)r]);
            r++;
        }
        // [a, r) split at instance boundaries
        int64_t x = a;
        while (x < r) {
            while (inst + 1 < ni && ioff[inst + 1] <= x) inst++;
            const int64_t end = std::min<int64_t>(r, (int64_t)ioff[inst] + in[inst]);
            seg.push_back((int32_t)inst);
            seg.push_back((int32_t)x);
            seg.push_back((int32_t)end);
            x = end;
        }
    }
    cta[(size_t)grid] = (int32_t)(seg.size() / 3);
    free_bsm(M);
    CK(cudaMalloc(&M.lcol, sizeof(uint16_t) * std::max<int64_t>(nnz_p, 8)));
    CK(cudaMalloc(&M.rinfo, sizeof(uint32_t) * std::max<int64_t>(n, 1)));
    CK(cudaMalloc(&M.seg, sizeof(int32_t) * std::max<size_t>(seg.size(), 3)));
    CK(cudaMalloc(&M.cta_seg, sizeof(int32_t) * cta.size()));
    CK(cudaMalloc(&M.ioff, sizeof(int32_t) * ni));
    CK(cudaMalloc(&M.in, sizeof(int32_t) * ni));
    if (nnz_p) CK(cudaMemcpy(M.lcol, lcol.data(), sizeof(uint16_t) * nnz_p, cudaMemcpyHostToDevice));
    if (n) CK(cudaMemcpy(M.rinfo, rinfo.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    if (!seg.empty()) CK(cudaMemcpy(M.seg, seg.data(), sizeof(int32_t) * seg.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(M.cta_seg, cta.data(), sizeof(int32_t) * cta.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(M.ioff, ioff.data(), sizeof(int32_t) * ni, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(M.in, in.data(), sizeof(int32_t) * ni, cudaMemcpyHostToDevice));
    M.grid = grid;
    M.max_rows = maxn;
    return SBX_OK;
}

// Pack a class for the resident batch kernel: whole instances into bins of
// at most max_rows rows (first-fit decreasing), the rows of a bin by
// decreasing degree, the matrix relabelled into that slot order.
int build_rb(sbx_ctx *ctx, BatchClass &c, int64_t max_rows)
{
    free_rb(c.rb);
    const DevCsr &J = c.J;
    const size_t ni = c.probs.size();
    std::vector<size_t> ord(ni);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return c.probs[a]->J.n > c.probs[b]->J.n; });
    std::vector<std::vector<size_t>> bins;
    std::vector<int64_t> fill;
    for (size_t i : ord) {
        const int64_t n = c.probs[i]->J.n;
        size_t b = 0;
        while (b < bins.size() && fill[b] + n > max_rows) b++;
        if (b == bins.size()) {
            bins.emplace_back();
            fill.push_back(0);
        }
        bins[b].push_back(i);
        fill[b] += n;
    }
    const int64_t rows = J.n;
    std::vector<int32_t> perm;
    perm.reserve((size_t)rows);
    std::vector<int32_t> bin_off(1, 0);
    for (auto &bi : bins) {
        const size_t first = perm.size();
        for (size_t i : bi)
            for (int64_t r = 0; r < c.probs[i]->J.n; r++) perm.push_back((int32_t)(c.row_off[i] + r));
        std::stable_sort(perm.begin() + (long)first, perm.end(), [&](int32_t a, int32_t b) {
            return J.hrowptr[(size_t)a + 1] - J.hrowptr[(size_t)a] > J.hrowptr[(size_t)b + 1] - J.hrowptr[(size_t)b];
        });
        bin_off.push_back((int32_t)perm.size());
    }
    std::vector<int32_t> inv((size_t)rows), rp((size_t)rows + 1, 0);
    for (size_t s = 0; s < perm.size(); s++) inv[(size_t)perm[s]] = (int32_t)s;
    std::vector<uint32_t> cw((size_t)std::max<int64_t>(J.nnz, 1));
    std::vector<float> vf((size_t)std::max<int64_t>(J.nnz, 1));
    int64_t e = 0;
    for (size_t s = 0; s < perm.size(); s++) {
        const int32_t r = perm[s];
        for (int32_t k = J.hrowptr[(size_t)r]; k < J.hrowptr[(size_t)r + 1]; k++, e++) {
            const double v = J.hval[(size_t)k];
            cw[(size_t)e] = (uint32_t)inv[(size_t)J.hcol[(size_t)k]] | ((J.unit && v < 0) ? 0x80000000u : 0u);
            vf[(size_t)e] = (float)v;
        }
        rp[s + 1] = (int32_t)e;
    }
    std::vector<int32_t> cta_bin(bins.size());
    std::iota(cta_bin.begin(), cta_bin.end(), 0);
    std::stable_sort(cta_bin.begin(), cta_bin.end(), [&](int32_t a, int32_t b) { return fill[(size_t)a] > fill[(size_t)b]; });
    DevRb &B = c.rb;
    B.nbins = (int32_t)bins.size();
    B.max_bin_rows = fill.empty() ? 0 : *std::max_element(fill.begin(), fill.end());
    B.unit = J.unit;
    CK(cudaMalloc(&B.rowptr, sizeof(int32_t) * (rows + 1)));
    CK(cudaMalloc(&B.colw, sizeof(uint32_t) * cw.size()));
    CK(cudaMalloc(&B.valf, sizeof(float) * vf.size()));
    CK(cudaMalloc(&B.c0, sizeof(float) * std::max<int64_t>(rows, 1)));
    CK(cudaMalloc(&B.perm, sizeof(int32_t) * std::max<int64_t>(rows, 1)));
    CK(cudaMalloc(&B.bin_off, sizeof(int32_t) * bin_off.size()));
    CK(cudaMalloc(&B.cta_bin, sizeof(int32_t) * std::max<size_t>(cta_bin.size(), 1)));
    CK(cudaMemcpy(B.rowptr, rp.data(), sizeof(int32_t) * (rows + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.colw, cw.data(), sizeof(uint32_t) * cw.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.valf, vf.data(), sizeof(float) * vf.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.perm, perm.data(), sizeof(int32_t) * rows, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.bin_off, bin_off.data(), sizeof(int32_t) * bin_off.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.cta_bin, cta_bin.data(), sizeof(int32_t) * cta_bin.size(), cudaMemcpyHostToDevice));
    c.rb_max = max_rows;
    return SBX_OK;
}

// dt * xi0 of each slot's instance for the resident batch kernel.
int upload_rb_c0(sbx_ctx *ctx, BatchClass &c, double dt)
{
    if (c.rb.dt == dt) return SBX_OK;
    std::vector<int32_t> perm((size_t)c.J.n);
    CK(cudaMemcpy(perm.data(), c.rb.perm, sizeof(int32_t) * perm.size(), cudaMemcpyDeviceToHost));
    std::vector<float> rowc0((size_t)c.J.n), f((size_t)c.J.n);
    for (size_t i = 0; i < c.probs.size(); i++)
        for (int64_t r = 0; r < c.probs[i]->J.n; r++) rowc0[(size_t)(c.row_off[i] + r)] = (float)(dt * c.xi0[i]);
    for (size_t s = 0; s < perm.size(); s++) f[s] = rowc0[(size_t)perm[s]];
    CK(cudaMemcpy(c.rb.c0, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
    c.rb.dt = dt;
    return SBX_OK;
}

void free_batch(sbx_ctx *ctx)
{
    if (!ctx->batch.empty() && ctx->gexec) {   // a cached graph may point at a packed matrix
        cudaGraphExecDestroy(ctx->gexec);
        ctx->gexec = nullptr;
        ctx->gkey.clear();
    }
    for (auto &c : ctx->batch) {
        free_csr(c.J);
        free_rb(c.rb);
        free_bsm(c.bsm);
        cudaFree(c.daoff);
        cudaFree(c.dslot);
    }
    ctx->batch.clear();
    ctx->batch_key.clear();
    ctx->batch_last = -1;
}

// Many MaxCut instances in one run per agent class: one block-diagonal
// matrix, one init launch (each instance from its own seed, params.seed + its
// position), the shared step kernels (the grid-stride row scheduler balances
// instances of any size), and per-instance exact cuts and statistics.
int solve_batch(sbx_ctx *ctx, int32_t count, sbx_problem *const *problems, const int32_t *agents,
                const sbx_params *pr, const double *targets, sbx_result *res, double *agent_values,
                double *batch_time_us)
{
    if (count < 1 || !problems || !agents || !pr || !res) return fail(ctx, SBX_ERR_ARG, "null argument");
    if (pr->update_window)
        return fail(ctx, SBX_ERR_UNSUPPORTED, "batched solve: update_window (per-instance exit) is not supported");
    if (pr->target > 0)
        return fail(ctx, SBX_ERR_ARG, "batched solve: per-instance targets go in the targets array");
    if (pr->steps < 0 || pr->precision < 0 || pr->precision > 3 || pr->run_steps < 0 || pr->period < 0 ||
        pr->count_mode < 0 || pr->count_mode > 4)
        return fail(ctx, SBX_ERR_ARG, "bad params");
    ctx->batch_last = -1;
    std::string key;
    for (int32_t i = 0; i < count; i++) {
        const sbx_problem *p = problems[i];
        if (!p || p->tsp || p->ctx != ctx) return fail(ctx, SBX_ERR_ARG, "batch: MaxCut problems of this context only");
        if (agents[i] < 1) return fail(ctx, SBX_ERR_ARG, "batch: agents must be >= 1");
        char b[64];
        snprintf(b, sizeof b, "%p:%d;", (const void *)p, agents[i]);
        key += b;
    }
    if (key != ctx->batch_key) {
        free_batch(ctx);
        std::vector<int32_t> aps;
        for (int32_t i = 0; i < count; i++) {
            const int32_t ap = (agents[i] + 31) / 32 * 32;
            size_t k = 0;
            while (k < aps.size() && aps[k] != ap) k++;
            if (k == aps.size()) {
                aps.push_back(ap);
                ctx->batch.emplace_back();
                ctx->batch.back().Ap = ap;
            }
            ctx->batch[k].probs.push_back(problems[i]);
            ctx->batch[k].idx.push_back(i);
            ctx->batch[k].agents.push_back(agents[i]);
        }
        for (auto &c : ctx->batch) {
            int rc = build_class(ctx, c);
            if (rc) {
                free_batch(ctx);
                return rc;
            }
        }
        ctx->batch_key = key;
    }
    std::vector<int64_t> val_off((size_t)count + 1, 0);
    for (int32_t i = 0; i < count; i++) val_off[i + 1] = val_off[i] + agents[i];
    const bool profile = (pr->flags & SBX_FLAG_PROFILE) != 0;
    const bool use_graph = !(pr->flags & SBX_FLAG_NO_GRAPH) && !profile;
    cudaStream_t s = ctx->stream;
    double total_us = 0;
    for (auto &c : ctx->batch) {
        if (!c.J.integer) return fail(ctx, SBX_ERR_UNSUPPORTED, "batched solve needs integer weights");
        int rc = upload_c0(ctx, c, pr->dt);
        if (rc) return rc;
        SolveDims d;
        d.n = c.J.n;
        d.A = c.Ap;
        d.Ap = c.Ap;
        d.W = c.Ap / 32;
        d.prec = pr->precision;
        d.steps = pr->steps;
        d.period = pr->period > 0 ? pr->period : 100;
        d.threshold = pr->threshold > 0 ? pr->threshold : 25;
        d.fused = pr->fused ? 1 : 0;
        d.uw = 0;
        d.dt = pr->dt;
        d.pdl = !(pr->flags & SBX_FLAG_NO_PDL);
        d.giveup = (pr->flags & SBX_FLAG_TEST_GIVEUP) ? 1 : 0;
        d.trace = (pr->trace || targets) ? 2 : 0;
        const int32_t run = pr->run_steps > 0 ? std::min(pr->run_steps, pr->steps) : pr->steps;
        const int64_t nchunks = run > 0 ? (run + d.period - 1) / d.period : 0;
        const int64_t total = nchunks * d.period;
        if ((rc = ensure_common(ctx, d, total, c.J.nchunks))) return rc;
        const size_t ne = c.probs.size() * (size_t)c.Ap;
        CK(grow(ctx->w.eacc, ctx->w.cap_eacc, ne));
        if (d.trace) CK(grow(ctx->w.btrace, ctx->w.cap_btrace, ctx->w.cap_trace * c.probs.size()));
        if ((rc = upload_coef(ctx, d, total))) return rc;
        std::vector<RandInst> inst(c.probs.size());
        for (size_t i = 0; i < c.probs.size(); i++) {
            inst[i].row_off = c.row_off[i];
            inst[i].n = c.probs[i]->J.n;
            inst[i].A = c.agents[i];
            rand_seed_window(pr->seed + (uint32_t)c.idx[i], inst[i].V0);
        }
        if ((rc = init_instances(ctx, d, inst, false, c.dslot))) return rc;
        // the resident batch kernel when every instance fits a bin on chip
        int64_t maxn = 0;
        for (const sbx_problem *q : c.probs) maxn = std::max<int64_t>(maxn, q->J.n);
        const int64_t rb_rows = (d.prec == P_BF16 || d.prec == P_F16) ? resident_batch_max_rows() : 0;
        const bool rb_ok = !d.trace && d.fused && rb_rows > 0 && maxn <= rb_rows &&
                           (!c.J.unit || c.J.max_deg <= kHeavy) && c.J.n < (int64_t)1 << 30 && nchunks > 0;
        // Each 4-agent CTA re-reads its bin's rows every step and gathers
        // neighbour signs from shared memory, so by itself the resident batch
        // is taken only for low-degree classes (mean degree <= 8); measured on
        // GB300 it trails the streaming kernel at degree ~20.
        const bool low_degree = c.J.nnz <= 8 * c.J.n;
        const bool want_rb = (pr->kernel == SBX_KERNEL_AUTO && low_degree) || pr->kernel == SBX_KERNEL_RESIDENT ||
                             pr->kernel == SBX_KERNEL_RESIDENT_SPLIT;
        if (pr->kernel != SBX_KERNEL_AUTO && pr->kernel != SBX_KERNEL_STREAM && !rb_ok)
            return fail(ctx, SBX_ERR_UNSUPPORTED,
                        "batched resident kernel: fused 16-bit state, degree <= 127, instances that fit on chip");
        const bool use_rb = want_rb && rb_ok;
        // the shared-memory-plane step kernel, unless a streaming tile or
        // another count mode is asked for (count_mode 4 insists on it)
        const bool bsm_threads = pr->block_threads == 512 || pr->block_threads == 640 || pr->block_threads == 1024;
        const bool tile_pinned = pr->lane_agents || pr->row_lanes || (pr->block_threads && !bsm_threads) ||
                                 pr->staging || (pr->count_mode && pr->count_mode != 4);
        const bool bsm_fit = !use_rb && bsm_ok(c, d);
        if (pr->count_mode == 4 && !bsm_fit)
            return fail(ctx, SBX_ERR_UNSUPPORTED,
                        "count_mode 4 (shared-memory planes): 16-bit state, +-1 weights, degree <= 127, "
                        "32/64/128 agents and instances whose plane fits in shared memory");
        const bool use_bsm = bsm_fit && !tile_pinned && pr->kernel != SBX_KERNEL_RESIDENT &&
                             pr->kernel != SBX_KERNEL_RESIDENT_SPLIT;
        c.J.bsm = nullptr;
        if (use_rb) {
            if (!c.rb.rowptr || c.rb_max != rb_rows) {
                if ((rc = build_rb(ctx, c, rb_rows))) return rc;
            }
            if ((rc = upload_rb_c0(ctx, c, pr->dt))) return rc;
        } else if (use_bsm) {
            if (!c.bsm.lcol && (rc = build_bsm(ctx, c, d.W))) return rc;
            c.J.bsm = &c.bsm;
            // 640 threads (96 registers each) measured fastest on GB300
            // (batch512: 257 us a step against 271 with 512 and 277 with 1024)
            d.tbsm = bsm_threads ? pr->block_threads : 640;
        } else if (nchunks) {
            bool timed = false;
            if ((rc = pick_tile(ctx, d, c.J, pr, &timed))) return rc;
            if (timed && (rc = init_instances(ctx, d, inst, false, c.dslot))) return rc;
        }
        int launches = 0;
        double kms = 0;
        CK(cudaEventRecord(ctx->ev0, s));
        if (use_rb) {
            d.steps_run = (int32_t)total;
            CK(launch_resident_batch(d, c.rb, ctx->w, s));
            launches = 1;
        } else {
            if ((rc = run_stream(ctx, &c.J, d, c.J, nchunks, profile, use_graph, &launches, &kms))) return rc;
        }
        CK(cudaEventRecord(ctx->ev1, s));
        ctx->d = d;
        ctx->batch_last = (int)(&c - &ctx->batch[0]);
        // per-instance best cut of every window: the first reaching the target
        std::vector<double> bt;
        std::vector<TraceRec> recs;
        if (d.trace) {
            const size_t nw = std::min((size_t)nchunks, ctx->w.cap_trace);
            bt.resize(nw * c.probs.size());
            recs.resize(nw);
            if (nw) {
                CK(cudaMemcpyAsync(bt.data(), ctx->w.btrace, sizeof(double) * bt.size(), cudaMemcpyDeviceToHost, s));
                CK(cudaMemcpyAsync(recs.data(), ctx->w.trace, sizeof(TraceRec) * nw, cudaMemcpyDeviceToHost, s));
            }
        }
        CK(cudaMemsetAsync(ctx->w.eacc, 0, sizeof(unsigned long long) * ne, s));
        CK(launch_cut_batch(d, c.J, ctx->w.Wp, ctx->w.eacc, s));
        // every instance's cuts (src/kernels.cu:383-398) and its statistics
        // line (src/ising.cu:238-265) on the device
        const size_t ni = c.probs.size();
        const int64_t nvals = c.agent_off.back();
        CK(grow(ctx->w.cut, ctx->w.cap_cut, (size_t)nvals));
        CK(grow(ctx->w.stats, ctx->w.cap_stats, 7 * ni));
        CK(launch_stats_batch(ctx->w.eacc, c.Ap, c.J.iagents, c.daoff, c.J.iwsum, (int32_t)ni, ctx->w.cut,
                              ctx->w.stats, s));
        std::vector<double> st(7 * ni), cutv(agent_values ? (size_t)nvals : 0);
        int32_t ctl[CTL_N];
        CK(cudaMemcpyAsync(st.data(), ctx->w.stats, sizeof(double) * st.size(), cudaMemcpyDeviceToHost, s));
        if (agent_values)
            CK(cudaMemcpyAsync(cutv.data(), ctx->w.cut, sizeof(double) * nvals, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(ctl, ctx->w.ctl, sizeof ctl, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (ctl[CTL_ERR]) return fail(ctx, SBX_ERR_CUDA, "a bounded wait in the step kernel gave up");
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        total_us += ms * 1000.0;
        for (size_t i = 0; i < ni; i++) {
            const int gi = c.idx[i];
            sbx_result *r = &res[gi];
            memset(r, 0, sizeof *r);
            r->time_to_target_us = -1;
            r->steps_to_target = -1;
            if (d.tbsm) {
                r->lane_agents = 32;
                r->row_lanes = d.W;
                r->block_threads = d.tbsm;
                r->count_mode = 4;
                r->staging = 1;
            } else if (!use_rb) {
                r->lane_agents = d.tv ? d.tv : default_v(d);
                r->row_lanes = d.tlr;
                r->block_threads = d.tbt;
                r->count_mode = d.tcm + 1;
                r->staging = d.tst + 1;
            }
            if (targets)
                for (size_t k = 0; k < recs.size(); k++)
                    if (bt[k * c.probs.size() + i] >= targets[gi]) {
                        r->time_to_target_us = (double)recs[k].t_ns / 1000.0;
                        r->steps_to_target = recs[k].steps;
                        break;
                    }
            finish_stats(&st[7 * i], c.agents[i], r);
            r->time_us = ms * 1000.0;
            r->xi0 = c.xi0[i];
            r->steps_run = total;
            r->windows_run = nchunks;
            r->kernel_used = use_rb ? SBX_KERNEL_RESIDENT : SBX_KERNEL_STREAM;
            r->agents_per_block = use_rb ? 4 : 0;
            r->kernel_launches = launches;
            r->kernel_ms = use_rb ? (profile ? ms : 0.0) : kms;
            r->gpu_launches = launches + 4;
            if (agent_values)
                memcpy(agent_values + val_off[gi], &cutv[(size_t)c.agent_off[i]], sizeof(double) * c.agents[i]);
        }
    }
    if (batch_time_us) *batch_time_us = total_us;
    ctx->have = false;
    return SBX_OK;
}

float bf16_to_f(uint16_t h);
float f16_to_f(uint16_t h);

// x, y (storage values as double) and window spins of rows [row0, row0 + rows)
// and agents [0, A) of the state in the work buffers, laid out as dims d.
int read_state(sbx_ctx *ctx, const SolveDims &d, int64_t row0, int64_t rows, int32_t A, double *x,
               double *y, int32_t *spins, const int32_t *slot = nullptr)
{
    // row r of the output is state row row0 + slot[r] - row0 (slot: the
    // global state row of each row, or null for the identity)
    auto src_row = [&](int64_t r) { return slot ? (int64_t)slot[r] - row0 : r; };
    const size_t es = prec_bytes(d.prec), nst = (size_t)rows * d.Ap;
    std::vector<unsigned char> buf(nst * es);
    for (int which = 0; which < 2; which++) {
        double *out = which ? y : x;
        if (!out) continue;
        const unsigned char *src = (const unsigned char *)(which ? ctx->w.y : ctx->w.x) + (size_t)row0 * d.Ap * es;
        CK(cudaMemcpy(buf.data(), src, nst * es, cudaMemcpyDeviceToHost));
        for (int64_t r = 0; r < rows; r++)
            for (int a = 0; a < A; a++) {
                const size_t i = (size_t)src_row(r) * d.Ap + a;
                double v;
                if (d.prec == P_F64) memcpy(&v, &buf[i * 8], 8);
                else if (d.prec == P_F32) {
                    float f;
                    memcpy(&f, &buf[i * 4], 4);
                    v = f;
                } else {
                    uint16_t h;
                    memcpy(&h, &buf[i * 2], 2);
                    v = d.prec == P_BF16 ? bf16_to_f(h) : f16_to_f(h);
                }
                out[(size_t)r * A + a] = v;
            }
    }
    if (spins) {
        std::vector<uint32_t> pl((size_t)rows * d.W);
        CK(cudaMemcpy(pl.data(), ctx->w.Wp + (size_t)row0 * d.W, pl.size() * 4, cudaMemcpyDeviceToHost));
        for (int64_t r = 0; r < rows; r++)
            for (int a = 0; a < A; a++)
                spins[(size_t)r * A + a] = ((pl[(size_t)src_row(r) * d.W + a / 32] >> (a % 32)) & 1u) ? -1 : 1;
    }
    return SBX_OK;
}

// The QUBO as CSR, tsp_gpu.cu:76-112 then CSR::from_matrix (row-major
// nonzeros), for the streaming TSP kernel.
int tsp_qubo(sbx_ctx *ctx, DevTsp &t, const double *packed)
{
    const int N = t.N;
    const double A = t.A, B = t.B, C = t.C;
    int rc = SBX_OK;
    {
        const int64_t m = (int64_t)N * N;
        std::vector<int32_t> rp(m + 1, 0), col;
        std::vector<double> val;
        for (int i = 0; i < N; i++)
            for (int k = 0; k < N; k++) {
                for (int j = 0; j < N; j++)
                    for (int l = 0; l < N; l++) {
                        double v;
                        const bool adj = (i == j + 1 || j == i + 1 || (i == 0 && j == N - 1) ||
                                          (i == N - 1 && j == 0));
                        if (i != j && k == l) v = C / 4;
                        else if (adj && k != l) {
                            const int c1 = std::min(k, l), c2 = std::max(k, l);
                            v = A * packed[((2 * (int64_t)N - c1 - 3) * c1) / 2 + c2 - 1] / 8;
                        } else if (i == j && k != l) v = B / 4;
                        else if (i == j && k == l) v = (B + C) / 4;
                        else v = 0;
                        if (v != 0) {
                            col.push_back(j * N + l);
                            val.push_back(v);
                        }
                    }
                rp[(size_t)i * N + k + 1] = (int32_t)col.size();
            }
        rc = upload_csr(ctx, t.qubo, m, (int64_t)col.size(), rp.data(), col.data(), val.data(), 0.0, true);
    }
    return rc;
}

float bf16_to_f(uint16_t h)
{
    uint32_t u = (uint32_t)h << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

float f16_to_f(uint16_t h)
{
    const uint32_t sign = (uint32_t)(h >> 15) << 31;
    uint32_t ex = (h >> 10) & 0x1f, man = h & 0x3ff, u;
    if (ex == 0) {
        if (man == 0) u = sign;
        else {   // subnormal
            ex = 127 - 15 + 1;
            while (!(man & 0x400)) {
                man <<= 1;
                ex--;
            }
            man &= 0x3ff;
            u = sign | (ex << 23) | (man << 13);
        }
    } else if (ex == 31) {
        u = sign | 0x7f800000u | (man << 13);
    } else {
        u = sign | ((ex + 127 - 15) << 23) | (man << 13);
    }
    float f;
    memcpy(&f, &u, 4);
    return f;
}

}  // namespace

namespace sbx {
// Lets the other translation units of the library report through sbx_last_error.
void set_last_error(const std::string &m) { g_err = m; }
}  // namespace sbx

extern "C" {

const char *sbx_strerror(int status)
{
    switch (status) {
    case SBX_OK: return "ok";
    case SBX_ERR_ARG: return "invalid argument";
    case SBX_ERR_CUDA: return "CUDA runtime error";
    case SBX_ERR_NOMEM: return "out of memory";
    case SBX_ERR_IO: return "cannot open or read file";
    case SBX_ERR_FORMAT: return "malformed input file";
    case SBX_ERR_UNSUPPORTED: return "unsupported request";
    case SBX_ERR_NODEVICE: return "no usable CUDA device";
    case SBX_ERR_STATE: return "no solve to read back";
    default: return "unknown status";
    }
}

const char *sbx_version(void) { return "sbx 0.1 (sm_103a)"; }

const char *sbx_last_error(void) { return g_err.c_str(); }

void sbx_params_default(sbx_params *p)
{
    memset(p, 0, sizeof *p);
    p->dt = 0.1;
    p->steps = 10000;
    p->agents = 1024;
    p->fused = 1;
    p->precision = SBX_F32;
    p->seed = 1;
}

int sbx_create(sbx_ctx **out, int device)
{
    sbx_ctx *ctx = nullptr;
    if (!out) return fail(ctx, SBX_ERR_ARG, "null ctx pointer");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0 || device < 0 || device >= n)
        return fail(ctx, SBX_ERR_NODEVICE, "no CUDA device");
    ctx = new sbx_ctx;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    for (int i = 0; i < 4 && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&ctx->evp[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->pinned, 16);
    if (e != cudaSuccess) {
        sbx_destroy(ctx);
        return fail(nullptr, SBX_ERR_CUDA, std::string("sbx_create: ") + cudaGetErrorString(e));
    }
    ctx->stream = ctx->own;
    *out = ctx;
    return SBX_OK;
}

int sbx_destroy(sbx_ctx *ctx)
{
    if (!ctx) return SBX_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    Work &w = ctx->w;
    void *ptrs[] = {w.x, w.y, w.x2, w.S[0], w.S[1], w.Wp, w.fin, w.chg, w.newmask, w.stab, w.bif,
                    w.prev, w.ctl, w.wincount, w.visits, w.ab, w.sched, w.eacc, w.cut, w.trace,
                    w.tours, w.valid, w.rjump, w.coef32, w.coef64, w.part, w.rinst, w.trace_t0,
                    w.btrace, w.hcount, w.gbar, w.stats};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    free_batch(ctx);   // (destroys the cached graph when a batch was packed)
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (auto &e : ctx->evp)
        if (e) cudaEventDestroy(e);
    for (auto &e : ctx->prof) cudaEventDestroy(e);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    for (sbx_problem *p : ctx->problems) p->ctx = nullptr;   // they stay valid to destroy
    delete ctx;
    return SBX_OK;
}

int sbx_set_stream(sbx_ctx *ctx, void *stream)
{
    if (!ctx) return SBX_ERR_ARG;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
    ctx->gkey.clear();
    return SBX_OK;
}

int sbx_problem_csr(sbx_ctx *ctx, int64_t n, int64_t nnz, const int32_t *rowptr,
                    const int32_t *col, const double *val, double weight_sum, sbx_problem **out)
{
    if (!ctx || !out) return fail(ctx, SBX_ERR_ARG, "null argument");
    CK(cudaSetDevice(ctx->device));
    sbx_problem *p = new sbx_problem;
    p->ctx = ctx;
    int rc = upload_csr(ctx, p->J, n, nnz, rowptr, col, val, weight_sum, false, true, true);
    if (rc) {
        free_csr(p->J);
        delete p;
        return rc;
    }
    ctx->problems.insert(p);
    *out = p;
    return SBX_OK;
}

int sbx_problem_tsp(sbx_ctx *ctx, int32_t N, const double *packed, double A, double B, double C,
                    sbx_problem **out)
{
    if (!ctx || !out || !packed) return fail(ctx, SBX_ERR_ARG, "null argument");
    if (N < 2 || N > 4096) return fail(ctx, SBX_ERR_ARG, "TSP: need 2 <= N <= 4096 cities");
    CK(cudaSetDevice(ctx->device));
    sbx_problem *p = new sbx_problem;
    p->ctx = ctx;
    p->tsp = true;
    DevTsp &t = p->T;
    t.N = N;
    t.A = A;
    t.B = B;
    t.C = C;
    const int64_t nd = (int64_t)N * (N - 1) / 2;
    t.packed.assign(packed, packed + nd);
    // per-city sums in the reference's walk order (tsp_gpu.cu:51-68)
    t.rowsum.assign(N, 0.0);
    {
        int i = 0, j = 0;
        for (int64_t k = 0; k < nd; k++) {
            if (j == N - 1) {
                i++;
                j = i;
            }
            j++;
            t.rowsum[i] += packed[k];
            t.rowsum[j] += packed[k];
        }
    }
    auto pidx = [&](int c1, int c2) { return (int64_t)c2 + (int64_t)c1 * N - (int64_t)(c1 + 2) * (c1 + 1) / 2; };
    std::vector<float> D((size_t)N * N, 0.f);
    for (int k = 0; k < N; k++)
        for (int l = 0; l < N; l++)
            if (k != l) D[(size_t)k * N + l] = (float)packed[pidx(std::min(k, l), std::max(k, l))];
    t.I2h.resize(N);
    std::vector<float> I2f(N);
    for (int c = 0; c < N; c++) {   // kernels.cu:591-592
        t.I2h[c] = -1 * (A * t.rowsum[c] + (N - 2) * (B + C)) / 2;
        I2f[c] = (float)t.I2h[c];
    }
    int rc = SBX_OK;
    cudaError_t e = cudaMalloc(&t.D, sizeof(float) * N * N);
    if (e == cudaSuccess) e = cudaMalloc(&t.I2, sizeof(float) * N);
    if (e == cudaSuccess) e = cudaMalloc(&t.I2d, sizeof(double) * N);
    if (e == cudaSuccess) e = cudaMalloc(&t.Dd, sizeof(double) * N * N);
    if (e == cudaSuccess) {
        std::vector<double> Dd((size_t)N * N, 0.0);
        for (int k = 0; k < N; k++)
            for (int l = 0; l < N; l++)
                if (k != l) Dd[(size_t)k * N + l] = packed[pidx(std::min(k, l), std::max(k, l))];
        e = cudaMemcpy(t.Dd, Dd.data(), sizeof(double) * N * N, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemcpy(t.D, D.data(), sizeof(float) * N * N, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t.I2, I2f.data(), sizeof(float) * N, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t.I2d, t.I2h.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = fail(ctx, SBX_ERR_CUDA, cudaGetErrorString(e));
    if (!rc) rc = tsp_qubo(ctx, t, packed);
    if (rc) {
        cudaFree(t.D);
        cudaFree(t.I2);
        cudaFree(t.I2d);
        cudaFree(t.Dd);
        free_csr(t.qubo);
        delete p;
        return rc;
    }
    ctx->problems.insert(p);
    *out = p;
    return SBX_OK;
}

int sbx_problem_tsp_cities(sbx_ctx *ctx, int32_t N, const double *xc, const double *yc, int32_t kind, double A,
                           double penalty_scale, sbx_problem **out)
{
    if (!ctx || !out || !xc || !yc) return fail(ctx, SBX_ERR_ARG, "null argument");
    if (N < 2 || N > 4096) return fail(ctx, SBX_ERR_ARG, "TSP: need 2 <= N <= 4096 cities");
    if (kind < 0 || kind > 2 || !(penalty_scale > 0)) return fail(ctx, SBX_ERR_ARG, "TSP: bad distance kind or scale");
    CK(cudaSetDevice(ctx->device));
    sbx_problem *p = new sbx_problem;
    p->ctx = ctx;
    p->tsp = true;
    DevTsp &t = p->T;
    t.N = N;
    t.A = A;
    const int64_t nd = (int64_t)N * (N - 1) / 2;
    double *dx = nullptr, *dy = nullptr, *dp = nullptr, *dmx = nullptr, *drs = nullptr;
    std::vector<double> packed((size_t)nd), rowsum((size_t)N), I2d((size_t)N);
    double mx = 0;
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaMalloc(&t.D, sizeof(float) * N * N);
    if (e == cudaSuccess) e = cudaMalloc(&t.I2, sizeof(float) * N);
    if (e == cudaSuccess) e = cudaMalloc(&t.I2d, sizeof(double) * N);
    if (e == cudaSuccess) e = cudaMalloc(&t.Dd, sizeof(double) * N * N);
    if (e == cudaSuccess) e = cudaMalloc(&dx, sizeof(double) * N);
    if (e == cudaSuccess) e = cudaMalloc(&dy, sizeof(double) * N);
    if (e == cudaSuccess) e = cudaMalloc(&dp, sizeof(double) * nd);
    if (e == cudaSuccess) e = cudaMalloc(&dmx, sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&drs, sizeof(double) * N);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, xc, sizeof(double) * N, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dy, yc, sizeof(double) * N, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_tsp_setup(dx, dy, N, kind, A, penalty_scale, dp, dmx, drs, t, s);
    // the packed distances come back for the CSR form of the QUBO
    if (e == cudaSuccess) e = cudaMemcpyAsync(packed.data(), dp, sizeof(double) * nd, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&mx, dmx, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rowsum.data(), drs, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(I2d.data(), t.I2d, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dp);
    cudaFree(dmx);
    cudaFree(drs);
    int rc = e == cudaSuccess ? SBX_OK : fail(ctx, SBX_ERR_CUDA, cudaGetErrorString(e));
    if (!rc) {
        t.B = t.C = penalty_scale * mx;
        t.packed = packed;
        t.rowsum = rowsum;
        t.I2h = I2d;
        rc = tsp_qubo(ctx, t, packed.data());
    }
    if (rc) {
        cudaFree(t.D);
        cudaFree(t.I2);
        cudaFree(t.I2d);
        cudaFree(t.Dd);
        free_csr(t.qubo);
        delete p;
        return rc;
    }
    ctx->problems.insert(p);
    *out = p;
    return SBX_OK;
}



int sbx_problem_destroy(sbx_problem *p)
{
    if (!p) return SBX_ERR_ARG;
    if (p->ctx) {
        p->ctx->problems.erase(p);
        for (auto &c : p->ctx->batch)
            for (const sbx_problem *q : c.probs)
                if (q == p) {
                    free_batch(p->ctx);   // the packed copy is stale
                    goto freed;
                }
    freed:
        if (p->ctx->gexec) {   // a cached graph may point at this problem
            cudaGraphExecDestroy(p->ctx->gexec);
            p->ctx->gexec = nullptr;
            p->ctx->gkey.clear();
        }
    }
    free_csr(p->J);
    free_csr(p->T.qubo);
    cudaFree(p->T.D);
    cudaFree(p->T.I2);
    cudaFree(p->T.I2d);
    cudaFree(p->T.Dd);
    delete p;
    return SBX_OK;
}

int sbx_problem_info(const sbx_problem *p, int64_t *n, int64_t *nnz, int32_t *is_tsp)
{
    if (!p) return SBX_ERR_ARG;
    const DevCsr &J = p->tsp ? p->T.qubo : p->J;
    if (n) *n = J.n;
    if (nnz) *nnz = J.nnz;
    if (is_tsp) *is_tsp = p->tsp;
    return SBX_OK;
}

int sbx_solve(sbx_ctx *ctx, const sbx_problem *p, const sbx_params *pr, sbx_result *res,
              double *agent_values)
{
    if (!ctx || !p || !pr || !res) return fail(ctx, SBX_ERR_ARG, "null argument");
    if (p->ctx != ctx) return fail(ctx, SBX_ERR_ARG, "problem belongs to another (or a destroyed) context");
    if (pr->agents < 1 || pr->steps < 0 || !(pr->dt == pr->dt) || pr->precision < 0 ||
        pr->precision > 3 || pr->run_steps < 0 || pr->period < 0 || pr->threshold < 0 ||
        pr->lane_agents < 0 || pr->row_lanes < 0 || pr->block_threads < 0 || pr->count_mode < 0 ||
        pr->count_mode > 3 || pr->staging < 0 || pr->staging > 2 || !(pr->target == pr->target))
        return fail(ctx, SBX_ERR_ARG, "bad params (agents >= 1, steps >= 0, precision 0..3)");
    if (pr->agents < 2 && !p->tsp) {
        // the reference's std dev divides by agents-1; one agent is allowed
    }
    const int64_t n = p->tsp ? (int64_t)p->T.N * p->T.N : p->J.n;
    if ((double)n * ((pr->agents + 31) / 32 * 32) * 8.0 > 200e9)
        return fail(ctx, SBX_ERR_NOMEM, "state larger than the device");
    CK(cudaSetDevice(ctx->device));
    ctx->have = false;
    ctx->batch_last = -1;   // the work buffers are about to be reused
    if (p->tsp && pr->target > 0) return fail(ctx, SBX_ERR_UNSUPPORTED, "target: MaxCut only");
    if (pr->kernel < 0 || pr->kernel > SBX_KERNEL_TENSOR) return fail(ctx, SBX_ERR_ARG, "bad params: kernel");
    if (!p->tsp && pr->kernel == SBX_KERNEL_TENSOR)
        return fail(ctx, SBX_ERR_UNSUPPORTED, "the tensor-core kernel is the TSP distance product's");
    return p->tsp ? solve_tsp(ctx, p, pr, res, agent_values) : solve_maxcut(ctx, p, pr, res, agent_values);
}

int sbx_get_state(sbx_ctx *ctx, double *x, double *y, int32_t *spins)
{
    if (!ctx) return SBX_ERR_ARG;
    if (!ctx->have) return fail(ctx, SBX_ERR_STATE, "no solve yet");
    CK(cudaSetDevice(ctx->device));
    return read_state(ctx, ctx->d, 0, ctx->d.n, ctx->d.A, x, y, spins);
}

int sbx_get_batch_state(sbx_ctx *ctx, int32_t index, double *x, double *y, int32_t *spins)
{
    if (!ctx) return SBX_ERR_ARG;
    if (ctx->batch_last < 0 || ctx->batch_last >= (int)ctx->batch.size())
        return fail(ctx, SBX_ERR_STATE, "no batched solve yet");
    const BatchClass &c = ctx->batch[(size_t)ctx->batch_last];
    for (size_t i = 0; i < c.idx.size(); i++)
        if (c.idx[i] == index) {
            CK(cudaSetDevice(ctx->device));
            return read_state(ctx, ctx->d, c.row_off[i], c.probs[i]->J.n, c.agents[i], x, y, spins,
                              c.slot.data() + c.row_off[i]);
        }
    return fail(ctx, SBX_ERR_STATE, "instance not in the last agent class solved (its state was overwritten)");
}

int sbx_get_tours(sbx_ctx *ctx, int32_t *tours, int32_t *valid_step)
{
    if (!ctx) return SBX_ERR_ARG;
    if (!ctx->have || !ctx->last_tsp) return fail(ctx, SBX_ERR_STATE, "no TSP solve yet");
    const int A = ctx->d.A, N = ctx->N;
    std::vector<int32_t> v((size_t)A);
    CK(cudaMemcpy(v.data(), ctx->w.valid, sizeof(int32_t) * A, cudaMemcpyDeviceToHost));
    if (valid_step) memcpy(valid_step, v.data(), sizeof(int32_t) * A);
    if (tours) {
        CK(cudaMemcpy(tours, ctx->w.tours, sizeof(int32_t) * A * N, cudaMemcpyDeviceToHost));
        for (int a = 0; a < A; a++)
            if (v[a] <= 0)
                for (int i = 0; i < N; i++) tours[(size_t)a * N + i] = -1;
    }
    return SBX_OK;
}

int sbx_solve_batch(sbx_ctx *ctx, int32_t count, sbx_problem *const *problems, const int32_t *agents,
                    const sbx_params *params, const double *targets, sbx_result *res,
                    double *agent_values, double *batch_time_us)
{
    if (!ctx) return fail(ctx, SBX_ERR_ARG, "null context");
    CK(cudaSetDevice(ctx->device));
    return solve_batch(ctx, count, problems, agents, params, targets, res, agent_values, batch_time_us);
}

int sbx_get_trace(sbx_ctx *ctx, int64_t cap, int64_t *steps, double *best, double *t_us, int64_t *count)
{
    if (!ctx) return SBX_ERR_ARG;
    if (count) *count = 0;
    if (!ctx->have || ctx->last_tsp || ctx->trace.empty())
        return fail(ctx, SBX_ERR_STATE, "no traced MaxCut solve (params.trace or params.target)");
    const int64_t k = std::min<int64_t>(std::max<int64_t>(cap, 0), (int64_t)ctx->trace.size());
    for (int64_t i = 0; i < k; i++) {
        const TraceRec &r = ctx->trace[(size_t)i];
        if (steps) steps[i] = r.steps;
        if (best) best[i] = r.best;
        if (t_us) t_us[i] = (double)r.t_ns / 1000.0;
    }
    if (count) *count = (int64_t)ctx->trace.size();
    return SBX_OK;
}

}  // extern "C"
