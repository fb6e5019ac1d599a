// k_stream.cu -- the streaming solve around the step kernel (k_step.cuh):
// step dispatch by precision, the pre-step, one window of steps, the window
// bookkeeping kernels and the exact cut.
#include "k_step.cuh"

#include <cfloat>

namespace sbx {

namespace {

struct WinP {
    uint32_t *chg, *newmask, *Wp, *fin;
    int32_t *stab;
    uint8_t *bif, *prev;
    int32_t *ctl;
    int64_t n;
    int32_t A, W, threshold, period, uw;
};

// Per-agent window bookkeeping, src/kernels.cu:46-69.
__global__ void __launch_bounds__(256) k_win_agents(const WinP P)
{
    pdl_wait();
    if (P.ctl[CTL_STOP]) return;
    pdl_trigger();
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = a >> 5, lane = a & 31;
    if (w >= P.W) return;
    const uint32_t ch = P.chg[w];
    int newb = 0, isb = 0;
    if (a < P.A) {
        const bool equal = !((ch >> lane) & 1u);
        const bool nb = !P.bif[a];
        int s = P.stab[a];
        s += (equal && nb);
        s = (!equal && nb) ? 0 : s;
        const bool b = (s == P.threshold - 1);
        newb = b ^ (P.prev[a] != 0);
        P.prev[a] = b;
        P.bif[a] = b;
        P.stab[a] = s;
        isb = b;
    }
    const uint32_t nm = __ballot_sync(FULL, newb), bm = __ballot_sync(FULL, isb);
    if (lane == 0) {
        P.newmask[w] = nm;
        P.chg[w] = 0;
        if (bm) atomicAdd(&P.ctl[CTL_NBIF], __popc(bm));
    }
}

// Final-spins snapshot of newly bifurcated agents (:73-79), and the host-loop
// bookkeeping of src/ising.cu:196-213 (step += period, all-bifurcated exit).
__global__ void __launch_bounds__(256) k_win_snap(const WinP P)
{
    pdl_wait();
    pdl_trigger();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.n * P.W) {
        const uint32_t m = P.newmask[i % P.W];
        if (m) P.fin[i] = (P.fin[i] & ~m) | (P.Wp[i] & m);
    }
    if (i == 0 && !P.ctl[CTL_STOP]) {
        const int nb = P.ctl[CTL_NBIF];
        P.ctl[CTL_NBIF] = 0;
        P.ctl[CTL_STEP] += P.period;
        P.ctl[CTL_WINDOWS] += 1;
        if (P.uw && nb == P.A) P.ctl[CTL_STOP] = 1;
    }
}

__device__ __forceinline__ long long global_ns()
{
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void k_trace_start(long long *t0, int32_t *ctl)
{
    *t0 = global_ns();
    ctl[CTL_TRACED] = 0;
}

// Record of the window that just closed: the best of the A agents' cuts.
// Chunks that run past an early exit close no window and record nothing.
__global__ void __launch_bounds__(256) k_trace_window(const double *__restrict__ cut, int32_t A,
                                                      int32_t *ctl, TraceRec *rec,
                                                      const long long *t0, int64_t cap)
{
    const int traced = ctl[CTL_TRACED];
    if (traced >= ctl[CTL_WINDOWS]) return;   // block-uniform
    double best = -INFINITY;
    for (int a = threadIdx.x; a < A; a += blockDim.x) best = fmax(best, cut[a]);
    for (int o = 16; o; o >>= 1) best = fmax(best, __shfl_xor_sync(FULL, best, o));
    __shared__ double wb[8];
    if ((threadIdx.x & 31) == 0) wb[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) best = fmax(best, wb[k]);
        if (traced < cap) {
            TraceRec r;
            r.steps = ctl[CTL_STEP];
            r.best = best;
            r.t_ns = global_ns() - *t0;
            r.pad = 0;
            rec[traced] = r;
        }
        ctl[CTL_TRACED] = traced + 1;
    }
}

// Batched record of the window that just closed (every window closes: the
// batched solve has no early exit): block i writes instance i's best cut,
// -0.5 * (0.5 * E - W_i) exactly (src/kernels.cu:383-398); block 0 the
// window's steps and time.
__global__ void __launch_bounds__(64) k_trace_batch(const unsigned long long *__restrict__ eacc,
                                                    int32_t Ap, const int32_t *__restrict__ agents,
                                                    const double *__restrict__ wsum, int32_t ninst,
                                                    const int32_t *ctl, TraceRec *rec, double *best,
                                                    const long long *t0, int64_t cap)
{
    const int i = blockIdx.x;
    const int win = ctl[CTL_WINDOWS] - 1;
    if (win < 0 || win >= cap) return;   // block-uniform
    double b = -INFINITY;
    for (int a = threadIdx.x; a < agents[i]; a += blockDim.x) {
        const double tmp = 0.5 * (double)(long long)eacc[(int64_t)i * Ap + a];
        b = fmax(b, __dmul_rn(-0.5, __dsub_rn(tmp, wsum[i])));
    }
    for (int o = 16; o; o >>= 1) b = fmax(b, __shfl_xor_sync(FULL, b, o));
    __shared__ double wb[2];
    if ((threadIdx.x & 31) == 0) wb[threadIdx.x >> 5] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        best[(int64_t)win * ninst + i] = fmax(wb[0], wb[1]);
        if (i == 0) {
            TraceRec r;
            r.steps = ctl[CTL_STEP];
            r.best = 0;
            r.t_ns = global_ns() - *t0;
            r.pad = 0;
            rec[win] = r;
        }
    }
}

StepP make_step(const SolveDims &d, const DevCsr &J, Work &w)
{
    StepP P;
    P.rowptr = J.rowptr;
    P.colw = J.colw;
    P.valf = J.valf;
    P.vald = J.vald;
    P.x = w.x;
    P.y = w.y;
    P.S0 = w.S[0];
    P.S1 = w.S[1];
    P.Wp = w.Wp;
    P.chg = w.chg;
    P.ctl = w.ctl;
    P.coef32 = (const float4 *)w.coef32;
    P.coef64 = (const Coef4 *)w.coef64;
    P.hchunk = J.hchunk;
    P.chunk_row = J.chunk_row;
    P.part = (uint2 *)w.part;
    P.hcount = w.hcount;
    P.allpos = J.allpos ? 1 : 0;
    P.bits_min = d.tcm == 2 ? kBitsMin : INT32_MAX;
    P.niso = 0;
    P.nchunks = J.nchunks;
    P.order = nullptr;   // set per kernel (step_vl)
    P.row0 = 0;
    P.c0r32 = J.c0r32;
    P.c0r64 = J.c0r64;
    P.n = d.n;
    P.zrow = (uint32_t)d.n;
    P.W = d.W;
    {
        const double state = 2.0 * (double)d.n * d.Ap * prec_bytes(d.prec);
        P.stream_state = state > 0.5 * (double)dev_attr(cudaDevAttrL2CacheSize) ? 1 : 0;
    }
    P.Ap = d.Ap;
    P.c0 = d.c0;
    P.giveup = d.giveup;
    return P;
}

cudaError_t step(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win,
                 int offset, cudaStream_t s)
{
    if (d.tbsm && J.bsm && kind != K_XY) return launch_batch_smem(d, *J.bsm, P, kind, win, offset, s);
    switch (d.prec) {
    case P_F32: return step_f32(d, J, P, kind, win, offset, s);
    case P_BF16: return step_bf16(d, J, P, kind, win, offset, s);
    case P_F16: return step_f16(d, J, P, kind, win, offset, s);
    default: return step_f64(d, J, P, kind, win, offset, s);
    }
}

cudaError_t iso(const SolveDims &d, const DevCsr &J, const StepP &P, cudaStream_t s)
{
    switch (d.prec) {
    case P_F32: return iso_f32(d, J, P, s);
    case P_BF16: return iso_bf16(d, J, P, s);
    case P_F16: return iso_f16(d, J, P, s);
    default: return iso_f64(d, J, P, s);
    }
}

}  // namespace

cudaError_t launch_prestep(const SolveDims &d, const DevCsr &J, Work &w, cudaStream_t s,
                           int *launches)
{
    StepP P = make_step(d, J, w);
    (*launches)++;
    return step(d, J, P, K_XY, false, 0, s);
}

cudaError_t launch_chunk(const SolveDims &d, const DevCsr &J, Work &w, cudaStream_t s,
                         int *launches, cudaEvent_t *evs)
{
    StepP P = make_step(d, J, w);
    cudaError_t e = cudaSuccess;
    if (!d.fused) {
        e = step(d, J, P, K_XY, false, 0, s);
        *launches += 1;
    } else if (J.niso && !d.tbsm) {
        // isolated rows: the whole window in one launch, which the step
        // kernels skip (events evs[2 * period], [2 * period + 1] in profile
        // mode).  Run beside the step kernels on a second stream it was
        // slower: they take the SMs' issue slots and registers.
        P.niso = J.niso;
        P.order = J.perm;
        if (evs) cudaEventRecord(evs[2 * d.period], s);
        e = iso(d, J, P, s);
        if (evs) cudaEventRecord(evs[2 * d.period + 1], s);
        *launches += 1;
    }
    for (int i = 0; i < d.period && e == cudaSuccess; i++) {
        if (evs) cudaEventRecord(evs[2 * i], s);
        e = step(d, J, P, d.fused ? K_FUSED : K_FC, i == d.period - 1, i, s);
        if (evs) cudaEventRecord(evs[2 * i + 1], s);
    }
    *launches += d.period;
    if (e != cudaSuccess) return e;
    WinP Q;
    Q.chg = w.chg;
    Q.newmask = w.newmask;
    Q.Wp = w.Wp;
    Q.fin = w.fin;
    Q.stab = w.stab;
    Q.bif = w.bif;
    Q.prev = w.prev;
    Q.ctl = w.ctl;
    Q.n = d.n;
    Q.A = d.A;
    Q.W = d.W;
    Q.threshold = d.threshold;
    Q.period = d.period;
    Q.uw = d.uw;
    e = launch(k_win_agents, dim3((unsigned)((d.W * 32 + 255) / 256)), dim3(256), 0, s, d.pdl, Q);
    if (e != cudaSuccess) return e;
    e = launch(k_win_snap, dim3((unsigned)((d.n * d.W + 255) / 256)), dim3(256), 0, s, d.pdl, Q);
    *launches += 2;
    if (e != cudaSuccess || !d.trace) return e;
    if (d.trace == 2) {
        // batched: exact cuts per instance, best of each instance's agents
        e = cudaMemsetAsync(w.eacc, 0, sizeof(unsigned long long) * J.ninst * d.Ap, s);
        if (e == cudaSuccess) e = launch_cut_batch(d, J, w.Wp, w.eacc, s);
        if (e != cudaSuccess) return e;
        k_trace_batch<<<J.ninst, 64, 0, s>>>(w.eacc, d.Ap, J.iagents, J.iwsum, J.ninst, w.ctl, w.trace,
                                             w.btrace, w.trace_t0, (int64_t)w.cap_trace);
        *launches += 2;
        return cudaGetLastError();
    }
    // traced: exact cut of every agent's window spins, then the window's record
    e = launch_cut(d, J, w, w.Wp, s, launches);
    if (e != cudaSuccess) return e;
    k_trace_window<<<1, 256, 0, s>>>(w.cut, d.A, w.ctl, w.trace, w.trace_t0, (int64_t)w.cap_trace);
    *launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_plain_steps(const SolveDims &d, const DevCsr &J, Work &w, int count, cudaStream_t s)
{
    StepP P = make_step(d, J, w);
    for (int i = 0; i < count; i++) {
        const cudaError_t e = step(d, J, P, d.fused ? K_FUSED : K_FC, false, 0, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_trace_start(Work &w, cudaStream_t s)
{
    k_trace_start<<<1, 1, 0, s>>>(w.trace_t0, w.ctl);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- cut

namespace {

// Integer weights: E_a = sum_r s_r sum_j J_rj s_j exactly (int64); the
// reference's FP64 sum of halves (src/kernels.cu:360-400) equals 0.5*E_a
// exactly, so the cut below is bit-identical to it.
__global__ void __launch_bounds__(256) k_cut_int(const int32_t *__restrict__ rowptr,
                                                 const uint32_t *__restrict__ colw,
                                                 const float *__restrict__ valf, int unit,
                                                 const uint32_t *__restrict__ plane, int64_t n,
                                                 int32_t W, unsigned long long *eacc)
{
    pdl_wait();
    const int w = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    long long acc = 0;
    for (int64_t r = (int64_t)blockIdx.y * 8 + warp; r < n; r += (int64_t)gridDim.y * 8) {
        const int32_t e0 = rowptr[r], e1 = rowptr[r + 1];
        long long t = 0;
        for (int32_t e = e0; e < e1; e++) {
            const uint32_t cw = colw[e];
            const uint32_t word = plane[(int64_t)(cw & 0x7fffffffu) * W + w];
            const int neg = (word >> lane) & 1u;
            if (unit) t += (((uint32_t)neg ^ (cw >> 31)) & 1u) ? -1 : 1;
            else t += neg ? -(long long)valf[e] : (long long)valf[e];
        }
        const int sr = (plane[r * W + w] >> lane) & 1u;
        acc += sr ? -t : t;
    }
    __shared__ long long red[8][32];
    red[warp][lane] = acc;
    __syncthreads();
    if (warp == 0) {
        long long s = 0;
        for (int k = 0; k < 8; k++) s += red[k][lane];
        atomicAdd(&eacc[w * 32 + lane], (unsigned long long)s);
    }
}

// Block-diagonal (batched) matrices: as k_cut_int, but each row adds into its
// instance's accumulators; a warp flushes when its rows change instance.
__global__ void __launch_bounds__(256) k_cut_batch(const int32_t *__restrict__ rowptr,
                                                   const uint32_t *__restrict__ colw,
                                                   const float *__restrict__ valf, int unit,
                                                   const uint32_t *__restrict__ plane, int64_t n,
                                                   int32_t W, int32_t Ap,
                                                   const int32_t *__restrict__ rinst,
                                                   int64_t rows_per_block, unsigned long long *eacc)
{
    const int w = blockIdx.y, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
    const int64_t r1 = min(n, r0 + rows_per_block);
    long long acc = 0;
    int cur = -1;
    for (int64_t r = r0 + warp; r < r1; r += 8) {
        const int inst = rinst[r];
        if (inst != cur) {
            if (cur >= 0 && acc) atomicAdd(&eacc[(int64_t)cur * Ap + w * 32 + lane], (unsigned long long)acc);
            acc = 0;
            cur = inst;
        }
        long long t = 0;
        for (int32_t e = rowptr[r]; e < rowptr[r + 1]; e++) {
            const uint32_t cw = colw[e];
            const uint32_t word = plane[(int64_t)(cw & 0x7fffffffu) * W + w];
            const int neg = (word >> lane) & 1u;
            if (unit) t += (((uint32_t)neg ^ (cw >> 31)) & 1u) ? -1 : 1;
            else t += neg ? -(long long)valf[e] : (long long)valf[e];
        }
        const int sr = (plane[r * W + w] >> lane) & 1u;
        acc += sr ? -t : t;
    }
    if (cur >= 0 && acc) atomicAdd(&eacc[(int64_t)cur * Ap + w * 32 + lane], (unsigned long long)acc);
}

__global__ void k_cut_finish(const unsigned long long *eacc, int32_t A, double wsum, double *cut)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    const double tmp = 0.5 * (double)(long long)eacc[a];
    cut[a] = __dmul_rn(-0.5, __dsub_rn(tmp, wsum));
}

// Non-integer weights: the reference's FP64 order, one agent per thread:
// row sums in CSR order, halves summed over rows ascending.
__global__ void k_cut_ordered(const int32_t *__restrict__ rowptr, const uint32_t *__restrict__ colw,
                              const double *__restrict__ vald, const uint32_t *__restrict__ plane,
                              int64_t n, int32_t W, int32_t A, double wsum, double *cut)
{
    pdl_wait();
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    const int w = a >> 5, lane = a & 31;
    double tmp = 0;
    for (int64_t r = 0; r < n; r++) {
        double rs = 0;
        for (int32_t e = rowptr[r]; e < rowptr[r + 1]; e++) {
            const uint32_t word = plane[(int64_t)(colw[e] & 0x7fffffffu) * W + w];
            rs = __dadd_rn(rs, __dmul_rn(vald[e], ((word >> lane) & 1u) ? -1.0 : 1.0));
        }
        const double sr = ((plane[r * W + w] >> lane) & 1u) ? -1.0 : 1.0;
        tmp = __dadd_rn(tmp, __dmul_rn(__dmul_rn(rs, sr), 0.5));
    }
    cut[a] = __dmul_rn(-0.5, __dsub_rn(tmp, wsum));
}

// The statistics line of src/ising.cu:238-265 over the A values v[i] = val(i),
// one warp: min and max (exact in any order) across the lanes; the total and
// the sum of squared deviations from the mean in agent order by one lane, as
// the reference's loop adds them; the agents at the maximum and the first of
// them.  out: min, max, total, mean, sum of squared deviations, agents at max,
// first agent at max.  The host takes the standard deviation
// pow(sd / (A - 1), 0.5) and ps = n_max / A from these.
template <class F>
__device__ __forceinline__ void stats_warp(F val, int32_t A, double *out)
{
    const int lane = threadIdx.x & 31;
    double mn = DBL_MAX, mx = -DBL_MAX;
    for (int32_t i = lane; i < A; i += 32) {
        const double v = val(i);
        mn = fmin(mn, v);
        mx = fmax(mx, v);
    }
    for (int o = 16; o; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(FULL, mn, o));
        mx = fmax(mx, __shfl_xor_sync(FULL, mx, o));
    }
    int32_t nmax = 0, first = INT32_MAX;
    for (int32_t i = lane; i < A; i += 32)
        if (val(i) == mx) {
            nmax++;
            first = min(first, i);
        }
    nmax = __reduce_add_sync(FULL, nmax);
    first = __reduce_min_sync(FULL, first);
    if (lane == 0) {
        double total = 0;
#pragma unroll 8
        for (int32_t i = 0; i < A; i++) total = __dadd_rn(total, val(i));
        const double avg = __ddiv_rn(total, (double)A);
        double sd = 0;
#pragma unroll 8
        for (int32_t i = 0; i < A; i++) {
            const double dv = __dsub_rn(val(i), avg);
            sd = __dadd_rn(sd, __dmul_rn(dv, dv));
        }
        out[0] = mn;
        out[1] = mx;
        out[2] = total;
        out[3] = avg;
        out[4] = sd;
        out[5] = (double)nmax;
        out[6] = (double)(first == INT32_MAX ? -1 : first);
    }
}

__global__ void __launch_bounds__(32) k_stats(const double *__restrict__ v, int32_t A, double *out)
{
    stats_warp([&](int32_t i) { return v[i]; }, A, out);
}

// Batched: block i converts instance i's exact sums to cuts (src/kernels.cu:
// 383-398, as k_cut_finish), writes them to cut[off_i ...] and its statistics
// to out[7 i ...].
__global__ void __launch_bounds__(32) k_stats_batch(const unsigned long long *__restrict__ eacc, int32_t Ap,
                                                    const int32_t *__restrict__ agents,
                                                    const int32_t *__restrict__ agent_off,
                                                    const double *__restrict__ wsum, double *cut,
                                                    double *out)
{
    const int i = blockIdx.x;
    const int32_t A = agents[i];
    const double W = wsum[i];
    const unsigned long long *e = eacc + (int64_t)i * Ap;
    double *c = cut + agent_off[i];
    for (int32_t a = threadIdx.x; a < A; a += 32) {
        const double tmp = 0.5 * (double)(long long)e[a];
        c[a] = __dmul_rn(-0.5, __dsub_rn(tmp, W));
    }
    __syncwarp();
    stats_warp([&](int32_t a) { return c[a]; }, A, out + 7 * (int64_t)i);
}

}  // namespace

cudaError_t launch_stats(const double *v, int32_t A, double *out, cudaStream_t s)
{
    k_stats<<<1, 32, 0, s>>>(v, A, out);
    return cudaGetLastError();
}

cudaError_t launch_stats_batch(const unsigned long long *eacc, int32_t Ap, const int32_t *agents,
                               const int32_t *agent_off, const double *wsum, int32_t ninst, double *cut,
                               double *out, cudaStream_t s)
{
    k_stats_batch<<<ninst, 32, 0, s>>>(eacc, Ap, agents, agent_off, wsum, cut, out);
    return cudaGetLastError();
}

cudaError_t launch_cut_batch(const SolveDims &d, const DevCsr &J, const uint32_t *plane,
                             unsigned long long *eacc, cudaStream_t s)
{
    const int64_t rpb = 256;
    const dim3 grid((unsigned)((d.n + rpb - 1) / rpb), (unsigned)d.W);
    k_cut_batch<<<grid, 256, 0, s>>>(J.rowptr, J.colw, J.valf, J.unit ? 1 : 0, plane, d.n, d.W, d.Ap,
                                     J.rinst, rpb, eacc);
    return cudaGetLastError();
}

cudaError_t launch_cut(const SolveDims &d, const DevCsr &J, Work &w, const uint32_t *plane,
                       cudaStream_t s, int *launches)
{
    cudaError_t e;
    if (J.integer) {
        e = cudaMemsetAsync(w.eacc, 0, sizeof(unsigned long long) * d.Ap, s);
        if (e != cudaSuccess) return e;
        int gy = (int)((d.n + 7) / 8);
        int cap = (152 * 8 + d.W - 1) / d.W;
        if (gy > cap) gy = cap;
        k_cut_int<<<dim3(d.W, gy), 256, 0, s>>>(J.rowptr, J.colw, J.valf, J.unit ? 1 : 0, plane,
                                                d.n, d.W, w.eacc);
        k_cut_finish<<<(d.A + 255) / 256, 256, 0, s>>>(w.eacc, d.A, J.wsum, w.cut);
        *launches += 2;
    } else {
        k_cut_ordered<<<(d.A + 127) / 128, 128, 0, s>>>(J.rowptr, J.colw, J.vald, plane, d.n, d.W,
                                                        d.A, J.wsum, w.cut);
        *launches += 1;
    }
    return cudaGetLastError();
}

}  // namespace sbx
