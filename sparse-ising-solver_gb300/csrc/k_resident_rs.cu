// k_resident_rs.cu -- resident MaxCut SB kernel for state too large for one
// SM's shared memory: a CTA owns 8 agents of every row and keeps their x, y
// (16-bit storage) partly in registers -- RR rows per thread -- and the rest
// in shared memory, with the rows' 8-bit sign words double-buffered in shared
// memory.  The whole solve (or one window, in the update-window mode) is one
// launch; agents never interact, so a CTA needs no other CTA and one
// __syncthreads() per step gives the Jacobi order of the reference kernel
// (src/kernels.cu:211-269).  The arithmetic is the streaming kernel's
// (sb_update, exact byte-counter force), so the two give identical states.
//
// Thread t owns the slots s = i*NT + t of the degree-sorted row list (row
// perm[s]): slots i < RR in registers, the others in shared memory.  The
// kernel reads the matrix relabelled into slot order (rows and columns), so a
// warp's row pointers are consecutive and sign bytes are indexed by slot;
// perm maps slots back to rows only where the global state is read or
// written.
#include "k_step.cuh"

namespace sbx {

namespace {

struct RsP {
    const int32_t *__restrict__ rowptr;   // slot order
    const uint32_t *__restrict__ colw;    // columns as slots, bit 31 the weight sign
    const float *__restrict__ valf;
    const int32_t *__restrict__ perm;     // slot -> row
    const float4 *__restrict__ coef;    // per step: k1, k2 (clamped), k1, k2 (raw)
    void *x, *y;                        // global [n][Ap]
    uint32_t *Wp, *fin;                 // global planes [n][W]
    int32_t *stab;
    uint8_t *bif, *prev;
    int32_t *ctl;
    int32_t *wincount;                  // bifurcated agents after each window
    int32_t *gbar;                      // co-resident launch: CTAs past each window
    int32_t coop;                       // 1: all windows in one co-resident launch
    int32_t n, A, Ap, W, period, threshold, uw;
    int32_t step0, nsteps, first, unit;
    float c0;
    int32_t giveup;                     // test only: the window barrier gives up at once
};

constexpr int KA = 8;   // agents per CTA: one sign byte per row

// Merge the CTA's 8 bits (at bit offset sh) into a global plane word.
__device__ __forceinline__ void plane_put8(uint32_t *p, uint32_t bits, int sh)
{
    const uint32_t m = 0xffu << sh;
    atomicAnd(p, ~m);
    atomicOr(p, (bits << sh) & m);
}

// One SB step of slot s's 8 agents held in xv, yv (16-bit, packed).
template <class T>
__device__ __forceinline__ uint32_t row_step(const RsP &P, int s, uint4 &xv, uint4 &yv, const uint8_t *Sin,
                                             const float4 &c)
{
    const int32_t e0 = __ldg(&P.rowptr[s]), e1 = __ldg(&P.rowptr[s + 1]);
    const int32_t deg = e1 - e0;
    float tv[KA];
    if (P.unit) {
        // byte counters of 2 * count (deg <= 127), as the streaming kernel
        uint32_t lo = 0, hi = 0;
        auto add = [&](uint32_t cw) {
            const uint32_t b = (uint32_t)Sin[cw & 0x7fffffffu] ^ (0u - (cw >> 31));
            lo += spread2x(b & 0xfu);
            hi += spread2x((b >> 4) & 0xfu);
        };
        if (deg == 4 && (e0 & 3) == 0) {
            // four neighbours on a 16-byte boundary (lattices): one vector load
            const uint4 c4 = __ldg((const uint4 *)(P.colw + e0));
            add(c4.x);
            add(c4.y);
            add(c4.z);
            add(c4.w);
        } else {
#pragma unroll 4
            for (int32_t e = e0; e < e1; e++) add(__ldg(&P.colw[e]));
        }
        const float bias = 8388608.0f + (float)deg;
#pragma unroll
        for (int v = 0; v < KA; v++)
            tv[v] = __uint_as_float(__byte_perm(v < 4 ? lo : hi, 0x4b000000u, 0x7440u + (v & 3))) - bias;
    } else {
#pragma unroll
        for (int v = 0; v < KA; v++) tv[v] = 0.0f;
        for (int32_t e = e0; e < e1; e++) {
            const uint32_t cw = __ldg(&P.colw[e]);
            const float wv = __ldg(&P.valf[e]);
            const uint32_t b = Sin[cw & 0x7fffffffu];
#pragma unroll
            for (int v = 0; v < KA; v++) tv[v] -= wv * (((b >> v) & 1u) ? -1.0f : 1.0f);
        }
    }
    Raw<16> xr, yr;
    xr.u = xv;
    yr.u = yv;
    float x[KA], y[KA];
    to_vals<T, KA>(xr, x);
    to_vals<T, KA>(yr, y);
    sb_update<K_FUSED, false, KA>(x, y, tv, P.c0, c, c);
    uint32_t nb = 0;
#pragma unroll
    for (int v = 0; v < KA; v++) nb |= sbit(x[v]) << v;
    xv = from_vals<T, KA>(x).u;
    yv = from_vals<T, KA>(y).u;
    return nb;
}

template <class T, int NT, int RR>
__global__ void __launch_bounds__(NT, 1) k_resident_rs(const RsP P)
{
    static_assert(sizeof(T) == 2, "16-bit state: 8 agents in 16 bytes");
    extern __shared__ __align__(16) unsigned char smem[];
    const int n = P.n;
    const int ns = n > RR * NT ? n - RR * NT : 0;   // rows kept in shared memory
    uint4 *xs = (uint4 *)smem;
    uint4 *ys = xs + ns;
    uint8_t *Sb0 = (uint8_t *)(ys + ns);
    uint8_t *Sb1 = Sb0 + n;
    uint8_t *Wb = Sb1 + n;
    __shared__ uint32_t s_chg, s_new, s_stop;
    __shared__ int32_t s_stab[KA];
    __shared__ uint8_t s_bif[KA], s_prev[KA];

    pdl_wait();
    const int tid = threadIdx.x;
    const int a0 = blockIdx.x * KA;          // first agent of this CTA
    const int wg = a0 >> 5, sh = a0 & 31;    // its word and bit offset in the planes
    T *xg = (T *)P.x, *yg = (T *)P.y;

    // early exit of the update-window mode (src/ising.cu:200-211)
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

    // Load the state (the pre-step Update_XY at step 0, src/ising.cu:188, as
    // the streaming pre-step computes it) and the sign words of step k0.
    const int32_t k0 = P.step0;
    uint8_t *Scur = (k0 & 1) ? Sb1 : Sb0;
    uint4 xr[RR > 0 ? RR : 1], yr[RR > 0 ? RR : 1];
    const float4 c00 = P.coef[0];
    auto load_row = [&](int s, uint4 &xv, uint4 &yv) {
        const int r = __ldg(&P.perm[s]);
        xv = *(const uint4 *)(xg + (int64_t)r * P.Ap + a0);
        yv = *(const uint4 *)(yg + (int64_t)r * P.Ap + a0);
        Raw<16> xw, yw;
        xw.u = xv;
        yw.u = yv;
        float x[KA], y[KA];
        to_vals<T, KA>(xw, x);
        to_vals<T, KA>(yw, y);
        if (P.first) {
#pragma unroll
            for (int v = 0; v < KA; v++) {
                y[v] = fmaf(c00.w, x[v], y[v]);
                x[v] = fmaf(c00.z, y[v], x[v]);
            }
            xv = from_vals<T, KA>(x).u;
            yv = from_vals<T, KA>(y).u;
        }
        uint32_t bits = 0;
#pragma unroll
        for (int v = 0; v < KA; v++) bits |= sbit(x[v]) << v;
        Scur[s] = (uint8_t)bits;
        Wb[s] = (uint8_t)((P.Wp[(int64_t)r * P.W + wg] >> sh) & 0xffu);
    };
#pragma unroll
    for (int i = 0; i < RR; i++) {
        const int s = i * NT + tid;
        if (s < n) load_row(s, xr[i], yr[i]);
    }
    for (int s = RR * NT + tid; s < n; s += NT) {
        uint4 xv, yv;
        load_row(s, xv, yv);
        xs[s - RR * NT] = xv;
        ys[s - RR * NT] = yv;
    }
    __syncthreads();

    int32_t nrun = P.nsteps;   // steps run (fewer at an update-window exit)
    for (int32_t it = 0; it < P.nsteps; it++) {
        const int32_t k = k0 + it;
        const uint8_t *Sin = (k & 1) ? Sb1 : Sb0;
        uint8_t *Snx = (k & 1) ? Sb0 : Sb1;
        const bool win = ((k + 1) % P.period) == 0;
        const float4 ck = P.coef[k];
        uint32_t chg = 0;
#pragma unroll
        for (int i = 0; i < RR; i++) {
            const int s = i * NT + tid;
            if (s < n) {
                const uint32_t nb = row_step<T>(P, s, xr[i], yr[i], Sin, ck);
                Snx[s] = (uint8_t)nb;
                if (win) {
                    chg |= nb ^ Wb[s];
                    Wb[s] = (uint8_t)nb;
                }
            }
        }
        for (int s = RR * NT + tid; s < n; s += NT) {
            uint4 xv = xs[s - RR * NT], yv = ys[s - RR * NT];
            const uint32_t nb = row_step<T>(P, s, xv, yv, Sin, ck);
            xs[s - RR * NT] = xv;
            ys[s - RR * NT] = yv;
            Snx[s] = (uint8_t)nb;
            if (win) {
                chg |= nb ^ Wb[s];
                Wb[s] = (uint8_t)nb;
            }
        }
        if (win) {
            // per-agent window bookkeeping inside the CTA, src/kernels.cu:46-79
            chg = __reduce_or_sync(FULL, chg);
            if ((tid & 31) == 0 && chg) atomicOr(&s_chg, chg);
            __syncthreads();
            if (tid < KA) {
                const int a = a0 + tid;
                const bool equal = !((s_chg >> tid) & 1u);
                const bool nbf = !s_bif[tid];
                int st = s_stab[tid];
                st += (equal && nbf);
                st = (!equal && nbf) ? 0 : st;
                const bool b = (st == P.threshold - 1);
                const bool newb = b ^ (s_prev[tid] != 0);
                s_prev[tid] = b;
                s_bif[tid] = b;
                s_stab[tid] = st;
                const uint32_t nm = __ballot_sync(0xffu, newb && a < P.A);
                const uint32_t bm = __ballot_sync(0xffu, b && a < P.A);
                if (tid == 0) {
                    s_new = nm;
                    if (P.uw) atomicAdd(&P.wincount[(k + 1) / P.period - 1], __popc(bm));
                }
            }
            __syncthreads();
            if (s_new) {
                for (int s = tid; s < n; s += NT) {
                    uint32_t *p = &P.fin[(int64_t)__ldg(&P.perm[s]) * P.W + wg];
                    atomicAnd(p, ~(s_new << sh));
                    atomicOr(p, ((uint32_t)Wb[s] & s_new) << sh);
                }
            }
            if (tid == 0) s_chg = 0;
            if (P.uw && P.coop) {
                // The update-window exit inside one co-resident launch: after
                // every CTA has counted its bifurcated agents for this window,
                // all of them read the total (src/ising.cu:200-211).  The
                // barrier's wait is bounded; giving up flags an error.
                const int widx = (k + 1) / P.period - 1;
                __syncthreads();
                if (tid == 0) {
                    __threadfence();
                    atomicAdd(P.gbar, 1);
                    // test only (giveup): a target no window reaches and a
                    // short limit, the path of a CTA that never arrives
                    const int target = (int)gridDim.x * (widx + 1 + P.giveup);
                    const uint32_t limit = P.giveup ? (1u << 12) : (1u << 26);
                    uint32_t spins = 0;
                    while (atomicAdd(P.gbar, 0) < target) {
                        if (++spins > limit) {
                            atomicExch(&P.ctl[CTL_ERR], 1);
                            s_stop = 1;
                            break;
                        }
                        __nanosleep(64);
                    }
                    __threadfence();
                    if (!s_stop && atomicAdd(&P.wincount[widx], 0) == P.A) s_stop = 2;
                }
                __syncthreads();
                if (s_stop) {
                    nrun = it + 1;
                    break;
                }
            }
        }
        __syncthreads();
    }

    // write the state back (chunked runs continue from it; get_state reads it)
#pragma unroll
    for (int i = 0; i < RR; i++) {
        const int s = i * NT + tid;
        if (s < n) {
            const int r = __ldg(&P.perm[s]);
            *(uint4 *)(xg + (int64_t)r * P.Ap + a0) = xr[i];
            *(uint4 *)(yg + (int64_t)r * P.Ap + a0) = yr[i];
        }
    }
    for (int s = RR * NT + tid; s < n; s += NT) {
        const int r = __ldg(&P.perm[s]);
        *(uint4 *)(xg + (int64_t)r * P.Ap + a0) = xs[s - RR * NT];
        *(uint4 *)(yg + (int64_t)r * P.Ap + a0) = ys[s - RR * NT];
    }
    for (int s = tid; s < n; s += NT) plane_put8(&P.Wp[(int64_t)__ldg(&P.perm[s]) * P.W + wg], Wb[s], sh);
    if (tid < KA) {
        const int a = a0 + tid;
        P.stab[a] = s_stab[tid];
        P.bif[a] = s_bif[tid];
        P.prev[a] = s_prev[tid];
    }
    if (blockIdx.x == 0 && tid == 0) {
        P.ctl[CTL_STEP] = P.step0 + nrun;
        P.ctl[CTL_WINDOWS] = (P.step0 + nrun) / P.period;
        if (s_stop == 2) P.ctl[CTL_STOP] = 1;
    }
}

// Configurations (threads per CTA, register rows per thread), fewest
// registers first.
struct RsCfg {
    int nt, rr;
};
constexpr RsCfg kRsCfgs[] = {{1024, 0}, {1024, 2}, {1024, 4}};

size_t rs_smem(int64_t n, const RsCfg &c)
{
    const int64_t ns = n > (int64_t)c.rr * c.nt ? n - (int64_t)c.rr * c.nt : 0;
    return (size_t)ns * 32 + (size_t)n * 3;
}

template <class T, int NT, int RR>
cudaError_t launch_rs_t(const RsP &P, size_t smem, int grid, cudaStream_t s, bool pdl)
{
    if (P.coop) {
        // every CTA must be resident at once for the window barrier
        int per_sm = 0, nsm = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaError_t e = cudaFuncSetAttribute(k_resident_rs<T, NT, RR>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_resident_rs<T, NT, RR>, NT, smem);
        if (e != cudaSuccess) return e;
        if ((int64_t)per_sm * nsm < grid) return cudaErrorCooperativeLaunchTooLarge;
    }
    cudaError_t e = cudaFuncSetAttribute(k_resident_rs<T, NT, RR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    if (P.coop) {
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
    } else {
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
    }
    cfg.attrs = at;
    cfg.numAttrs = (pdl || P.coop) ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_resident_rs<T, NT, RR>, P);
}

template <class T>
cudaError_t launch_rs_cfg(int ci, const RsP &P, size_t smem, int grid, cudaStream_t s, bool pdl)
{
    switch (ci) {
    case 0: return launch_rs_t<T, 1024, 0>(P, smem, grid, s, pdl);
    case 1: return launch_rs_t<T, 1024, 2>(P, smem, grid, s, pdl);
    default: return launch_rs_t<T, 1024, 4>(P, smem, grid, s, pdl);
    }
}

}  // namespace

int resident_rs_pick(const SolveDims &d, const DevCsr &J, bool forced)
{
    if (d.prec != P_BF16 && d.prec != P_F16) return 0;
    if (!d.fused || d.n > (1 << 24)) return 0;
    if (J.unit && J.max_deg > kHeavy) return 0;   // byte counters hold 127 neighbours
    int dev = 0, smax = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // one CTA per SM: chosen by itself only when the agents fill half the SMs
    if (!forced && (d.A + KA - 1) / KA < nsm / 2) return 0;
    const size_t budget = (size_t)smax - 1024;
    for (int i = 0; i < (int)(sizeof kRsCfgs / sizeof kRsCfgs[0]); i++)
        if (rs_smem(d.n, kRsCfgs[i]) <= budget) return i + 1;
    return 0;
}

cudaError_t launch_resident_rs(const SolveDims &d, const DevCsr &J, Work &w, int cfg, int32_t step0,
                               int32_t nsteps, bool first, bool coop, cudaStream_t s)
{
    if (cfg < 1) return cudaErrorInvalidValue;
    RsP P;
    if (!J.rs_rowptr) return cudaErrorInvalidValue;
    P.rowptr = J.rs_rowptr;
    P.colw = J.rs_colw;
    P.valf = J.rs_valf;
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
    P.gbar = w.gbar;
    P.coop = (coop && d.uw && w.gbar) ? 1 : 0;
    P.n = (int32_t)d.n;
    P.A = d.A;
    P.Ap = d.Ap;
    P.W = d.W;
    P.period = d.period;
    P.threshold = d.threshold;
    P.uw = d.uw;
    P.step0 = step0;
    P.nsteps = nsteps;
    P.first = first ? 1 : 0;
    P.unit = J.unit ? 1 : 0;
    P.c0 = (float)d.c0;
    P.giveup = d.giveup;
    const size_t smem = rs_smem(d.n, kRsCfgs[cfg - 1]);
    const int grid = (d.A + KA - 1) / KA;
    if (d.prec == P_BF16) return launch_rs_cfg<__nv_bfloat16>(cfg - 1, P, smem, grid, s, d.pdl);
    return launch_rs_cfg<__half>(cfg - 1, P, smem, grid, s, d.pdl);
}

}  // namespace sbx
