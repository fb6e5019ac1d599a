// k_resident.cu -- resident MaxCut SB kernel: one CTA owns KA agents (8, 16 or
// 32) for every row and keeps their x, y and sign words in shared memory for
// all the steps of a launch.  Agents never interact (the product J.X couples
// rows of one agent only), so a CTA needs no other CTA between steps: one
// __syncthreads() per step separates the writes of the sign words of step k
// from their reads in step k+1 (double-buffered), which is the Jacobi order of
// the reference kernel (src/kernels.cu:211-269).
//
// Force for +-1 weights: the neighbour's sign word (KA bits) XOR the weight's
// sign gives the negative products; their per-agent counts are kept 8 agents
// at a time in byte lanes of two 32-bit registers (a 4-bit nibble times
// 0x00204081 spreads its bits to bit 0 of four bytes), so one neighbour costs a
// handful of integer operations for 8 agents.  Total = 2*count - degree,
// exact.  Rows are visited in degree order (perm) so a warp's rows have
// similar lengths.
#include "common.cuh"
#include "engine.h"

namespace sbx {

namespace {

struct ResP {
    const int32_t *__restrict__ rowptr;
    const uint32_t *__restrict__ colw;
    const float *__restrict__ valf;
    const int32_t *__restrict__ perm;
    const float4 *__restrict__ coef;    // per step: k1, k2 (clamped), k1, k2 (raw)
    void *x, *y;                        // global [n][Ap]
    uint32_t *Wp, *fin;                 // global planes [n][W]
    int32_t *stab;
    uint8_t *bif, *prev;
    int32_t *ctl;
    int32_t *wincount;                  // bifurcated agents after each window
    int64_t n;
    int32_t A, Ap, W, period, threshold, uw, fused;
    int32_t step0, nsteps, first, unit;
    float c0;
};

__device__ __forceinline__ uint32_t spread4(uint32_t nib) { return (nib * 0x00204081u) & 0x01010101u; }

// Merge `bits` (KA wide, at bit offset sh) into a shared global plane word.
template <int KA>
__device__ __forceinline__ void plane_put(uint32_t *p, uint32_t bits, int sh)
{
    if constexpr (KA == 32) {
        *p = bits;
    } else {
        const uint32_t m = ((1u << KA) - 1u) << sh;
        atomicAnd(p, ~m);
        atomicOr(p, (bits << sh) & m);
    }
}

template <class T, int KA>
__global__ void __launch_bounds__(1024) k_resident(const ResP P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int64_t n = P.n;
    T *xs = (T *)smem;
    T *ys = xs + n * KA;
    uint32_t *S0 = (uint32_t *)(ys + n * KA);
    uint32_t *S1 = S0 + n;
    uint32_t *Wps = S1 + n;
    __shared__ uint32_t s_chg, s_new, s_stop;
    __shared__ int32_t s_stab[KA];
    __shared__ uint8_t s_bif[KA], s_prev[KA];

    pdl_wait();
    const int tid = threadIdx.x, T_ = blockDim.x;
    const int a0 = blockIdx.x * KA;          // first agent of this CTA
    const int wg = a0 >> 5, sh = a0 & 31;    // its word and bit offset in planes
    T *xg = (T *)P.x, *yg = (T *)P.y;

    // Early exit of the update-window mode (src/ising.cu:200-211): the
    // previous window left every agent bifurcated.
    if (tid == 0) {
        s_stop = P.ctl[CTL_STOP];
        if (!s_stop && P.uw && P.step0 > 0) {
            const int widx = P.step0 / P.period - 1;
            if (P.wincount[widx] == P.A) s_stop = 1;
        }
        s_chg = 0;
    }
    if (tid < KA) {
        const int a = a0 + tid;
        s_stab[tid] = P.stab[a];
        s_bif[tid] = P.bif[a];
        s_prev[tid] = P.prev[a];
    }
    __syncthreads();
    if (s_stop) {
        if (blockIdx.x == 0 && tid == 0) P.ctl[CTL_STOP] = 1;
        return;
    }

    // Load the state; build the sign words of the step about to run.
    const int32_t k0 = P.step0;
    uint32_t *Scur = (k0 & 1) ? S1 : S0;
    for (int64_t r = tid; r < n; r += T_) {
        uint32_t bits = 0;
        const float4 cu = P.coef[k0];
#pragma unroll
        for (int q = 0; q < KA; q++) {
            float x = St<T>::ld(xg[r * P.Ap + a0 + q]);
            float y = St<T>::ld(yg[r * P.Ap + a0 + q]);
            if (P.first) {   // the pre-step Update_XY at step 0 (src/ising.cu:188)
                y = y + cu.w * x;
                x = x + cu.z * y;
            }
            if (!P.fused) {  // the unfused step begins with Update_XY(k0)
                y = y + cu.w * x;
                x = x + cu.z * y;
            }
            T xt = St<T>::st(x), yt = St<T>::st(y);
            xs[r * KA + q] = xt;
            ys[r * KA + q] = yt;
            bits |= sbit(St<T>::ld(xt)) << q;
        }
        Scur[r] = bits;
        Wps[r] = (P.Wp[r * P.W + wg] >> sh) & (KA == 32 ? 0xffffffffu : ((1u << KA) - 1u));
    }
    __syncthreads();

    for (int32_t it = 0; it < P.nsteps; it++) {
        const int32_t k = k0 + it;
        const uint32_t *Sin = (k & 1) ? S1 : S0;
        uint32_t *Snx = (k & 1) ? S0 : S1;
        const bool win = ((k + 1) % P.period) == 0;
        const bool last = it == P.nsteps - 1;
        const float4 ck = P.coef[k];
        const float4 cn = P.coef[k + 1];
        uint32_t chg = 0;
        for (int64_t i = tid; i < n; i += T_) {
            const int32_t r = P.perm[i];
            const int32_t e0 = P.rowptr[r], e1 = P.rowptr[r + 1];
            const int deg = e1 - e0;
            uint32_t nbits = 0, wbits = 0;
#pragma unroll
            for (int g = 0; g < KA / 8; g++) {
                int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                float ftot[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                if (P.unit) {
                    for (int32_t base = e0; base < e1; base += 255) {
                        const int32_t end = min(e1, base + 255);
                        uint32_t lo = 0, hi = 0;
#pragma unroll 4
                        for (int32_t e = base; e < end; e++) {
                            const uint32_t cw = __ldg(&P.colw[e]);
                            uint32_t wd = Sin[cw & 0x7fffffffu] >> (8 * g);
                            wd ^= 0u - (cw >> 31);
                            lo += spread4(wd & 0xfu);
                            hi += spread4((wd >> 4) & 0xfu);
                        }
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            cnt[q] += (lo >> (8 * q)) & 0xffu;
                            cnt[4 + q] += (hi >> (8 * q)) & 0xffu;
                        }
                    }
                } else {
                    for (int32_t e = e0; e < e1; e++) {
                        const uint32_t cw = __ldg(&P.colw[e]);
                        const float v = __ldg(&P.valf[e]);
                        const uint32_t wd = Sin[cw & 0x7fffffffu] >> (8 * g);
#pragma unroll
                        for (int q = 0; q < 8; q++) ftot[q] -= ((wd >> q) & 1u) ? -v : v;
                    }
                }
#pragma unroll
                for (int q8 = 0; q8 < 8; q8++) {
                    const int q = g * 8 + q8;
                    const float total = P.unit ? (float)(2 * cnt[q8] - deg) : ftot[q8];
                    float x = St<T>::ld(xs[(int64_t)r * KA + q]);
                    float y = St<T>::ld(ys[(int64_t)r * KA + q]);
                    if (P.fused) {
                        // src/kernels.cu:236-262
                        if (fabsf(x) > 1.f) {
                            x = spin_of(x);
                            y = 0.f;
                        } else {
                            y = y + P.c0 * total;
                        }
                        x = x + ck.x * y;
                        y = y + ck.y * x;
                        wbits |= sbit(x) << q;
                    } else {
                        // mat_mult + confine of step k (src/kernels.cu:150-209);
                        // the window sees x here; then Update_XY of step k+1
                        // unless the launch ends with this step.
                        y = y + P.c0 * total;
                        if (fabsf(x) > 1.f) {
                            x = spin_of(x);
                            y = 0.f;
                        }
                        wbits |= sbit(x) << q;
                        if (!last) {
                            y = y + cn.w * x;
                            x = x + cn.z * y;
                        }
                    }
                    nbits |= sbit(x) << q;
                    xs[(int64_t)r * KA + q] = St<T>::st(x);
                    ys[(int64_t)r * KA + q] = St<T>::st(y);
                }
            }
            if (win) {
                chg |= wbits ^ Wps[r];
                Wps[r] = wbits;
            }
            Snx[r] = nbits;
        }
        if (win) {
            // Per-agent window bookkeeping inside the CTA, src/kernels.cu:46-79.
            chg = __reduce_or_sync(FULL, chg);
            if ((tid & 31) == 0 && chg) atomicOr(&s_chg, chg);
            __syncthreads();
            if (tid < KA) {
                const int a = a0 + tid;
                const bool equal = !((s_chg >> tid) & 1u);
                const bool nb = !s_bif[tid];
                int s = s_stab[tid];
                s += (equal && nb);
                s = (!equal && nb) ? 0 : s;
                const bool b = (s == P.threshold - 1);
                const bool newb = b ^ (s_prev[tid] != 0);
                s_prev[tid] = b;
                s_bif[tid] = b;
                s_stab[tid] = s;
                const uint32_t nm = __ballot_sync((KA == 32) ? FULL : ((1u << KA) - 1u), newb && a < P.A);
                const uint32_t bm = __ballot_sync((KA == 32) ? FULL : ((1u << KA) - 1u), b && a < P.A);
                if (tid == 0) {
                    s_new = nm;
                    if (P.uw) atomicAdd(&P.wincount[(k + 1) / P.period - 1], __popc(bm));
                }
            }
            __syncthreads();
            if (s_new) {
                for (int64_t r = tid; r < n; r += T_) {
                    uint32_t *p = &P.fin[r * P.W + wg];
                    const uint32_t m = s_new << sh;
                    if (KA == 32) *p = (*p & ~m) | (Wps[r] & s_new);
                    else {
                        atomicAnd(p, ~m);
                        atomicOr(p, (Wps[r] & s_new) << sh);
                    }
                }
            }
            if (tid == 0) s_chg = 0;
        }
        __syncthreads();
    }

    // Write the state back (chunked runs continue from it; get_state reads it).
    for (int64_t r = tid; r < n; r += T_) {
#pragma unroll
        for (int q = 0; q < KA; q++) {
            xg[r * P.Ap + a0 + q] = xs[r * KA + q];
            yg[r * P.Ap + a0 + q] = ys[r * KA + q];
        }
        plane_put<KA>(&P.Wp[r * P.W + wg], Wps[r], sh);
    }
    if (tid < KA) {
        const int a = a0 + tid;
        P.stab[a] = s_stab[tid];
        P.bif[a] = s_bif[tid];
        P.prev[a] = s_prev[tid];
    }
    if (blockIdx.x == 0 && tid == 0) {
        P.ctl[CTL_STEP] = P.step0 + P.nsteps;
        P.ctl[CTL_WINDOWS] = (P.step0 + P.nsteps) / P.period;
    }
}

}  // namespace

size_t resident_smem_bytes(const SolveDims &d, int ka)
{
    return (size_t)d.n * ka * 2 * prec_bytes(d.prec) + (size_t)d.n * 3 * sizeof(uint32_t);
}

int resident_pick_ka(const SolveDims &d, const DevCsr &J, int requested)
{
    (void)J;
    if (d.prec == P_F64) return 0;
    int dev = 0, smax = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const size_t budget = (size_t)smax - 1024;
    auto fits = [&](int ka) { return resident_smem_bytes(d, ka) <= budget; };
    if (requested) return (requested == 8 || requested == 16 || requested == 32) && fits(requested) ? requested : 0;
    // Prefer the tile that gives at least one CTA per SM, then the widest.
    int best = 0;
    for (int ka : {32, 16, 8}) {
        if (!fits(ka)) continue;
        const int64_t ctas = (d.A + ka - 1) / ka;
        if (!best) best = ka;
        if (ctas >= nsm) {
            best = ka;
            break;
        }
        best = ka;
    }
    return best;
}

namespace {

template <class T, int KA>
cudaError_t launch_t(const ResP &P, size_t smem, int threads, int grid, cudaStream_t s, bool pdl)
{
    cudaError_t e = cudaFuncSetAttribute(k_resident<T, KA>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_resident<T, KA>, P);
}

template <class T>
cudaError_t launch_ka(int ka, const ResP &P, size_t smem, int threads, int grid, cudaStream_t s,
                      bool pdl)
{
    if (ka == 8) return launch_t<T, 8>(P, smem, threads, grid, s, pdl);
    if (ka == 16) return launch_t<T, 16>(P, smem, threads, grid, s, pdl);
    return launch_t<T, 32>(P, smem, threads, grid, s, pdl);
}

}  // namespace

cudaError_t launch_resident(const SolveDims &d, const DevCsr &J, Work &w, int ka,
                            int32_t step0, int32_t nsteps, bool first, cudaStream_t s)
{
    ResP P;
    P.rowptr = J.rowptr;
    P.colw = J.colw;
    P.valf = J.valf;
    P.perm = J.perm;
    P.coef = (const float4 *)w.coef32;
    P.x = w.x;
    P.y = w.y;
    P.Wp = w.Wp;
    P.fin = w.fin;
    P.stab = w.stab;
    P.bif = w.bif;
    P.prev = w.prev;
    P.ctl = w.ctl;
    P.wincount = w.wincount;
    P.n = d.n;
    P.A = d.A;
    P.Ap = d.Ap;
    P.W = d.W;
    P.period = d.period;
    P.threshold = d.threshold;
    P.uw = d.uw;
    P.fused = d.fused;
    P.step0 = step0;
    P.nsteps = nsteps;
    P.first = first ? 1 : 0;
    P.unit = J.unit ? 1 : 0;
    P.c0 = (float)d.c0;
    const size_t smem = resident_smem_bytes(d, ka);
    int threads = (int)((d.n + 31) / 32 * 32);
    if (threads > 1024) threads = 1024;
    if (threads < 64) threads = 64;
    const int grid = (d.A + ka - 1) / ka;
    switch (d.prec) {
    case P_F32: return launch_ka<float>(ka, P, smem, threads, grid, s, d.pdl);
    case P_BF16: return launch_ka<__nv_bfloat16>(ka, P, smem, threads, grid, s, d.pdl);
    case P_F16: return launch_ka<__half>(ka, P, smem, threads, grid, s, d.pdl);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace sbx
