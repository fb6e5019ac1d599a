// k_stream.cu -- streaming MaxCut SB step: one launch per SB step over the
// whole state, which lives in HBM (or L2 when it fits).
//
// Layout.  x, y: [n][Ap] in the storage precision (Ap = agents rounded up to
// 32).  Sign planes S[2], window plane Wp (the reference's current_spins),
// final plane fin: [n][Ap/32] uint32, bit a%32 of word (r, a/32) = signbit of
// x[r][a] (1 = spin -1).  A warp owns one (row, 32-agent word): lane = agent.
//
// Semantics (Jacobi): every gather of step k reads the sign plane written by
// step k-1, so each step is the reference kernel run with all threads reading
// the state the launch began with (src/kernels.cu:211-269 for the fused mode;
// src/ising.cu:168-171 for the unfused trio).  The force only needs signs, so
// a neighbour costs one 4-byte word per 32 agents instead of 32 FP64 loads.
#include "common.cuh"
#include "engine.h"

#include <type_traits>

namespace sbx {

namespace {

enum Kind { K_FUSED = 0, K_XY = 1, K_FC = 2 };
enum WMode { W_UNIT = 0, W_F32 = 1, W_F64 = 2 };

struct alignas(32) Coef4 {
    double x, y, z, w;
};

struct StepP {
    const int32_t *__restrict__ rowptr;
    const uint32_t *__restrict__ colw;
    const float *__restrict__ valf;
    const double *__restrict__ vald;
    void *x, *y;
    uint32_t *S0, *S1, *Wp, *chg;
    int32_t *ctl;
    const float4 *__restrict__ coef32;    // per step: k1, k2 (clamped p), k1, k2 (raw p)
    const Coef4 *__restrict__ coef64;
    int64_t n;
    int32_t W, Ap;
    double c0;
};

// Coefficients dt*(p+1), dt*(p-1) of step k: .x/.y with the pressure clamped
// at 1 (src/kernels.cu:225-226), .z/.w unclamped (src/kernels.cu:15).
template <class A> struct Coef;
template <> struct Coef<float> {
    static __device__ __forceinline__ float4 get(const StepP &P, int k) { return __ldg(&P.coef32[k]); }
};
template <> struct Coef<double> {
    static __device__ __forceinline__ Coef4 get(const StepP &P, int k) {
        const Coef4 *p = &P.coef64[k];
        return Coef4{__ldg(&p->x), __ldg(&p->y), __ldg(&p->z), __ldg(&p->w)};
    }
};

// -sum_j J_rj s_j for the 32 agents of word w (lane = agent), src/kernels.cu
// :247-255.  Unit weights: count the negative products (sign bit XOR weight
// sign) and return 2*count - degree, exact.  Other weights: the reference's
// subtraction order over the row.
template <int WM>
__device__ __forceinline__ typename std::conditional<WM == W_F64, double, float>::type
force(const StepP &P, int64_t r, int w, int lane, const uint32_t *__restrict__ Sin)
{
    using R = typename std::conditional<WM == W_F64, double, float>::type;
    const int32_t e0 = __ldg(&P.rowptr[r]), e1 = __ldg(&P.rowptr[r + 1]);
    int cnt = 0;
    R tot = 0;
    for (int32_t base = e0; base < e1; base += 32) {
        const int m = min(32, e1 - base);
        const uint32_t mycw = lane < m ? __ldg(&P.colw[base + lane]) : 0u;
        R myv = 0;
        if (WM == W_F32) myv = lane < m ? __ldg(&P.valf[base + lane]) : 0.f;
        if (WM == W_F64) myv = lane < m ? __ldg(&P.vald[base + lane]) : 0.0;
#pragma unroll 8
        for (int k = 0; k < m; k++) {
            const uint32_t cw = __shfl_sync(FULL, mycw, k);
            const uint32_t word = __ldg(&Sin[(int64_t)(cw & 0x7fffffffu) * P.W + w]);
            if (WM == W_UNIT) {
                cnt += ((word >> lane) ^ (cw >> 31)) & 1u;
            } else {
                const R v = __shfl_sync(FULL, myv, k);
                const R s = ((word >> lane) & 1u) ? R(-1) : R(1);
                if (WM == W_F64) tot = sub(tot, mul(v, s));
                else tot -= v * s;
            }
        }
    }
    if (WM == W_UNIT) return (R)(2 * cnt - (e1 - e0));
    return tot;
}

template <class T, int KIND, bool WIN, int WM>
__global__ void __launch_bounds__(256) k_step(const StepP P, const int offset)
{
    using A = typename St<T>::A;
    pdl_wait();
    if (P.ctl[CTL_STOP]) return;
    const int step = P.ctl[CTL_STEP] + offset;
    const int64_t gw = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    pdl_trigger();
    if (gw >= P.n * P.W) return;
    const int64_t r = gw / P.W;
    const int w = (int)(gw - r * P.W);
    const int64_t idx = r * P.Ap + (int64_t)w * 32 + lane;
    T *xp = (T *)P.x, *yp = (T *)P.y;
    A x = St<T>::ld(xp[idx]), y = St<T>::ld(yp[idx]);
    uint32_t *Sin = (step & 1) ? P.S1 : P.S0;
    uint32_t *Snext = (step & 1) ? P.S0 : P.S1;
    const int64_t wi = r * P.W + w;

    if (KIND == K_XY) {
        // Update_XY, src/kernels.cu:8-22 (pressure not clamped); writes the
        // plane that step `step` gathers from.
        const auto c = Coef<A>::get(P, step);
        y = add(y, mul((A)c.w, x));
        x = add(x, mul((A)c.z, y));
        xp[idx] = St<T>::st(x);
        yp[idx] = St<T>::st(y);
        const uint32_t b = __ballot_sync(FULL, sbit(x));
        if (lane == 0) Sin[wi] = b;
        return;
    }

    const A total = (A)force<WM>(P, r, w, lane, Sin);
    if (KIND == K_FUSED) {
        // src/kernels.cu:236-262: clamp or kick, then the drift/kick pair that
        // runs unconditionally (so a clamped oscillator leaves with
        // y = dt (p-1) sign(x)).
        const auto c = Coef<A>::get(P, step);
        if (fabs(x) > A(1)) {
            x = spin_of(x);
            y = A(0);
        } else {
            y = add(y, mul((A)P.c0, total));
        }
        x = add(x, mul((A)c.x, y));
        y = add(y, mul((A)c.y, x));
    } else {
        // K_FC: mat_mult (:207) then confine (:158-165) of step `step`; then,
        // unless the window closes here, Update_XY of step+1.
        y = add(y, mul((A)P.c0, total));
        if (fabs(x) > A(1)) {
            x = spin_of(x);
            y = A(0);
        }
        if (!WIN) {
            const auto c = Coef<A>::get(P, step + 1);
            y = add(y, mul((A)c.w, x));
            x = add(x, mul((A)c.z, y));
        }
    }
    xp[idx] = St<T>::st(x);
    yp[idx] = St<T>::st(y);
    const uint32_t b = __ballot_sync(FULL, sbit(x));
    if (lane == 0) {
        if (KIND == K_FUSED || !WIN) Snext[wi] = b;
        if (WIN) {
            // window compare, src/kernels.cu:37-46 + :84-90
            const uint32_t ch = b ^ P.Wp[wi];
            if (ch) atomicOr(&P.chg[w], ch);
            P.Wp[wi] = b;
        }
    }
}

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

template <class K, class... Args>
cudaError_t launch(K kern, dim3 grid, dim3 block, cudaStream_t s, bool pdl, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, args...);
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
    P.n = d.n;
    P.W = d.W;
    P.Ap = d.Ap;
    P.c0 = d.c0;
    return P;
}

template <class T, int KIND, bool WIN>
cudaError_t step_wm(const SolveDims &d, const DevCsr &J, const StepP &P, int offset,
                    cudaStream_t s)
{
    const dim3 grid((unsigned)((d.n * d.W + 7) / 8)), block(256);
    if (KIND == K_XY) return launch(k_step<T, KIND, WIN, W_UNIT>, grid, block, s, d.pdl, P, offset);
    if (J.unit) return launch(k_step<T, KIND, WIN, W_UNIT>, grid, block, s, d.pdl, P, offset);
    if (d.prec == P_F64) return launch(k_step<T, KIND, WIN, W_F64>, grid, block, s, d.pdl, P, offset);
    return launch(k_step<T, KIND, WIN, W_F32>, grid, block, s, d.pdl, P, offset);
}

template <class T>
cudaError_t step_t(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win,
                   int offset, cudaStream_t s)
{
    if (kind == K_XY) return step_wm<T, K_XY, false>(d, J, P, offset, s);
    if (kind == K_FUSED)
        return win ? step_wm<T, K_FUSED, true>(d, J, P, offset, s)
                   : step_wm<T, K_FUSED, false>(d, J, P, offset, s);
    return win ? step_wm<T, K_FC, true>(d, J, P, offset, s)
               : step_wm<T, K_FC, false>(d, J, P, offset, s);
}

cudaError_t step(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win,
                 int offset, cudaStream_t s)
{
    switch (d.prec) {
    case P_F32: return step_t<float>(d, J, P, kind, win, offset, s);
    case P_BF16: return step_t<__nv_bfloat16>(d, J, P, kind, win, offset, s);
    case P_F16: return step_t<__half>(d, J, P, kind, win, offset, s);
    default: return step_t<double>(d, J, P, kind, win, offset, s);
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
    e = launch(k_win_agents, dim3((unsigned)((d.W * 32 + 255) / 256)), dim3(256), s, d.pdl, Q);
    if (e != cudaSuccess) return e;
    e = launch(k_win_snap, dim3((unsigned)((d.n * d.W + 255) / 256)), dim3(256), s, d.pdl, Q);
    *launches += 2;
    return e;
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

}  // namespace

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
