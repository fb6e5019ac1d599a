// k_tsp.cu -- TSP-QUBO ballistic SB (src/kernels.cu:543-599) with the
// validity window (src/kernels.cu:461-541).
//
// Structured kernel.  The QUBO of tsp_gpu.cu:76-112 over spins (position i,
// city k) is C/4 between equal cities at different positions, A d_kl/8 between
// cyclically adjacent positions at different cities, B/4 between different
// cities at one position and (B+C)/4 on the diagonal.  Hence, exactly,
//   (J x)[i][k] = C/4 colsum[k] + B/4 rowsum[i] + A/8 sum_l d_kl (x[i-1][l] + x[i+1][l])
// (the diagonal cancels the self terms of the two penalty sums; for N = 2 the
// two neighbours are one position).  A CTA owns KA agents and keeps their x in
// shared memory for the whole run: per step each thread (position i, agent a)
// gathers the two neighbouring rows, one pass computes every row and column
// sum, and the 30x30 distance product runs from shared memory on the FP32
// pipes.  No CTA talks to another, so the whole solve is one launch.
//
// Streaming kernel.  The CSR form of the same QUBO, one launch per step, x
// double-buffered (Jacobi); used in FP64 (which it reproduces operation by
// operation) and when N > 32.
#include "common.cuh"
#include "engine.h"

namespace sbx {

namespace {

struct TspP {
    const float *__restrict__ D;      // [N][N] distances, zero diagonal
    const float *__restrict__ I2;     // [N] linear field per city
    const float2 *__restrict__ sched; // per step: b_t, dt*-(1-a_t)
    void *x, *y;                      // global [n][Ap], n = N*N, row = i*N + k
    uint32_t *Wp;                     // global plane [n][W] (window spins)
    int32_t *tours, *valid;           // [Ap][N], [Ap]
    int32_t *stab;
    uint8_t *bif, *prev;
    int32_t *ctl;
    int32_t N, A, Ap, W, nwin, period, threshold;
    float qa8, qb4, qc4;              // A/8, B/4, C/4
    float dtxi0, dt, k1u, k2u;        // pre-step Update_XY coefficients
};

template <class T> __device__ __forceinline__ float rnd(float v) { return St<T>::ld(St<T>::st(v)); }

template <class T, int NP>
__global__ void __launch_bounds__(512) k_tsp_resident(const TspP P, const int KA)
{
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int NPS = NP + 4;       // padded row: spreads rows over banks
    const int N = P.N;
    float *xs = (float *)smem;                          // [N][KA][NPS]
    float *Ds = xs + (size_t)N * KA * NPS;              // [NP][NP]
    float *colsum = Ds + NP * NP;                       // [NP][KA]
    uint32_t *rowbits = (uint32_t *)(colsum + NP * KA); // [N][KA]
    uint32_t *prevbits = rowbits + N * KA;              // [N][KA]
    int *aflag = (int *)(prevbits + N * KA);            // [KA] valid, [KA] changed
    __shared__ float s_I2[NP];

    pdl_wait();
    const int tid = threadIdx.x;
    const int i = tid / KA, a = tid - (tid / KA) * KA;  // position, local agent
    const int ag = blockIdx.x * KA + a;                 // global agent
    const bool active = i < N;
    const bool real = ag < P.A;                         // padded agents compute on zeros
    T *xg = (T *)P.x, *yg = (T *)P.y;

    for (int t = tid; t < NP * NP; t += blockDim.x) {
        const int k = t / NP, l = t % NP;
        Ds[t] = (k < N && l < N) ? P.D[k * N + l] : 0.f;
    }
    for (int t = tid; t < NP; t += blockDim.x) s_I2[t] = t < N ? P.I2[t] : 0.f;

    // Initial state (x = 0, y from the init stream) and the pre-step
    // Update_XY at step 0 (src/ising_tsp.cu:155).
    float yr[NP], xo[NP];
    uint32_t bits0 = 0;
#pragma unroll
    for (int k = 0; k < NP; k++) {
        float x = 0.f, y = 0.f;
        if (active && k < N && real) {
            const int64_t gi = (int64_t)(i * N + k) * P.Ap + ag;
            x = St<T>::ld(xg[gi]);
            y = St<T>::ld(yg[gi]);
            y = rnd<T>(y + P.k2u * x);
            x = rnd<T>(x + P.k1u * y);
            bits0 |= sbit(x) << k;
        }
        yr[k] = y;
        xo[k] = x;
        if (active) xs[(i * KA + a) * NPS + k] = x;
    }
    if (active) prevbits[i * KA + a] = 0xffffffffu;   // current_spins = -1
    int stab = 0;
    bool bif = false, prv = false;
    if (active && i == 0 && real) {
        stab = P.stab[ag];
        bif = P.bif[ag];
        prv = P.prev[ag];
    }
    (void)bits0;
    __syncthreads();

    const int nwin = P.nwin;
    const uint32_t maskN = N == 32 ? 0xffffffffu : ((1u << N) - 1u);
    int k_step = 0;
    for (int wdx = 0; wdx < nwin; wdx++) {
        for (int it = 0; it < P.period; it++, k_step++) {
            const float2 sc = P.sched[k_step];
            // Phase 1: read neighbours, row sum, one column sum.
            float nb[NP];
            float rs = 0.f;
            if (active) {
                const int im = (i + N - 1) % N, ip = (i + 1) % N;
                const float *rm = &xs[(im * KA + a) * NPS];
                const float *rp = &xs[(ip * KA + a) * NPS];
#pragma unroll
                for (int l = 0; l < NP; l += 4) {
                    const float4 m4 = *(const float4 *)&rm[l];
                    const float4 p4 = N > 2 ? *(const float4 *)&rp[l] : make_float4(0, 0, 0, 0);
                    nb[l] = m4.x + p4.x;
                    nb[l + 1] = m4.y + p4.y;
                    nb[l + 2] = m4.z + p4.z;
                    nb[l + 3] = m4.w + p4.w;
                }
#pragma unroll
                for (int l = 0; l < NP; l++) rs += xo[l];
                float cs = 0.f;   // column (city) i over all positions
                for (int p = 0; p < N; p++) cs += xs[(p * KA + a) * NPS + i];
                colsum[i * KA + a] = cs;
            }
            __syncthreads();
            // Phase 2: forces and the bSB update of this thread's N spins.
            if (active) {
#pragma unroll
                for (int k = 0; k < NP; k++) {
                    if (k < N) {
                        float dk = 0.f;
#pragma unroll
                        for (int l = 0; l < NP; l += 4) {
                            const float4 d4 = *(const float4 *)&Ds[k * NP + l];
                            dk += d4.x * nb[l] + d4.y * nb[l + 1] + d4.z * nb[l + 2] + d4.w * nb[l + 3];
                        }
                        const float jx = P.qc4 * colsum[k * KA + a] + P.qb4 * rs + P.qa8 * dk;
                        float x = xo[k], y = yr[k];
                        if (fabsf(x) > 1.f) {
                            x = spin_of(x);
                            y = 0.f;
                        } else {
                            const float i1 = -1.005f * jx;
                            y = rnd<T>(y + P.dtxi0 * (2.f * i1 + sc.x * s_I2[k]));
                            x = rnd<T>(x + P.dt * y);
                            y = rnd<T>(y + sc.y * x);
                        }
                        xo[k] = x;
                        yr[k] = y;
                    }
                }
#pragma unroll
                for (int l = 0; l < NP; l += 4)
                    *(float4 *)&xs[(i * KA + a) * NPS + l] = make_float4(xo[l], xo[l + 1], xo[l + 2], xo[l + 3]);
            }
            __syncthreads();
        }
        // Window: validity (one +1 per city and per position), stability,
        // tour snapshot of valid agents (src/kernels.cu:473-531).
        uint32_t bits = 0;
        if (active) {
#pragma unroll
            for (int k = 0; k < NP; k++)
                if (k < N) bits |= sbit(xo[k]) << k;
            rowbits[i * KA + a] = bits;
        }
        if (tid < 2 * KA) aflag[tid] = tid < KA ? 1 : 0;
        __syncthreads();
        if (active) {
            const int order_cnt = __popc(~bits & maskN);
            int city_cnt = 0;
            for (int p = 0; p < N; p++) city_cnt += (~rowbits[p * KA + a] >> i) & 1u;
            if (order_cnt != 1 || city_cnt != 1) atomicAnd(&aflag[a], 0);
            if (bits != (prevbits[i * KA + a] & maskN)) atomicOr(&aflag[KA + a], 1);
        }
        __syncthreads();
        if (active) {
            const bool valid = aflag[a] != 0;
            if (valid && real) {
                P.tours[(int64_t)ag * N + i] = __ffs(~bits & maskN) - 1;
                if (i == 0) P.valid[ag] = k_step;
            }
            if (i == 0) {
                const bool equal = aflag[KA + a] == 0;
                const bool nb = !bif;
                stab += (equal && nb);
                stab = (!equal && nb) ? 0 : stab;
                bif = (stab == P.threshold - 1);
                prv = bif;
            }
            prevbits[i * KA + a] = bits;
        }
        __syncthreads();
    }

    // State back to global memory (get_state) and the window spins.
    if (active && real) {
#pragma unroll
        for (int k = 0; k < NP; k++)
            if (k < N) {
                const int64_t gi = (int64_t)(i * N + k) * P.Ap + ag;
                xg[gi] = St<T>::st(xo[k]);
                yg[gi] = St<T>::st(yr[k]);
            }
        const uint32_t bits = prevbits[i * KA + a];
        for (int k = 0; k < N; k++) {
            const int64_t r = i * N + k;
            const uint32_t bit = (bits >> k) & 1u;
            uint32_t *p = &P.Wp[r * P.W + (ag >> 5)];
            if (bit) atomicOr(p, 1u << (ag & 31));
            else atomicAnd(p, ~(1u << (ag & 31)));
        }
        if (i == 0) {
            P.stab[ag] = stab;
            P.bif[ag] = bif;
            P.prev[ag] = prv;
        }
    }
    if (blockIdx.x == 0 && tid == 0) {
        P.ctl[CTL_STEP] = k_step;
        P.ctl[CTL_WINDOWS] = nwin;
    }
}

template <class T, int NP>
cudaError_t launch_res(const TspP &P, int ka, cudaStream_t s, bool pdl)
{
    constexpr int NPS = NP + 4;
    const int N = P.N;
    const size_t smem = sizeof(float) * ((size_t)N * ka * NPS + NP * NP + NP * ka) +
                        sizeof(uint32_t) * 2 * N * ka + sizeof(int) * 2 * ka;
    cudaError_t e = cudaFuncSetAttribute(k_tsp_resident<T, NP>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int threads = (N * ka + 31) / 32 * 32;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((P.A + ka - 1) / ka);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_tsp_resident<T, NP>, P, ka);
}

template <class T>
cudaError_t launch_np(const TspP &P, int ka, cudaStream_t s, bool pdl)
{
    if (P.N <= 16) return launch_res<T, 16>(P, ka, s, pdl);
    return launch_res<T, 32>(P, ka, s, pdl);
}

}  // namespace

int tsp_pick_ka(const SolveDims &d, const DevTsp &t, int requested)
{
    if (d.prec == P_F64 || t.N > 32 || t.N < 2) return 0;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int kmax = 512 / t.N;   // registers: <= 512 threads of ~128 registers
    if (kmax < 1) return 0;
    if (requested > 0) return requested <= kmax ? requested : 0;
    int ka = (d.A + nsm - 1) / nsm;
    if (ka < 1) ka = 1;
    if (ka > kmax) ka = kmax;
    return ka;
}

cudaError_t launch_tsp_resident(const SolveDims &d, const DevTsp &t, Work &w, int ka,
                                cudaStream_t s)
{
    TspP P;
    P.D = t.D;
    P.I2 = t.I2;
    P.sched = w.sched;
    P.x = w.x;
    P.y = w.y;
    P.Wp = w.Wp;
    P.tours = w.tours;
    P.valid = w.valid;
    P.stab = w.stab;
    P.bif = w.bif;
    P.prev = w.prev;
    P.ctl = w.ctl;
    P.N = t.N;
    P.A = d.A;
    P.Ap = d.Ap;
    P.W = d.W;
    P.nwin = d.nwin;
    P.period = d.period;
    P.threshold = d.threshold;
    P.qa8 = (float)(t.A / 8);
    P.qb4 = (float)(t.B / 4);
    P.qc4 = (float)(t.C / 4);
    P.dtxi0 = (float)(d.dt * 0.002);
    P.dt = (float)d.dt;
    const double p0 = 1.025 * 0.0 / d.steps;   // Update_XY pressure at step 0
    P.k1u = (float)(d.dt * (p0 + 1));
    P.k2u = (float)(d.dt * (p0 - 1));
    switch (d.prec) {
    case P_F32: return launch_np<float>(P, ka, s, d.pdl);
    case P_BF16: return launch_np<__nv_bfloat16>(P, ka, s, d.pdl);
    case P_F16: return launch_np<__half>(P, ka, s, d.pdl);
    default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------- streaming

namespace {

struct TspSP {
    const int32_t *__restrict__ rowptr;
    const uint32_t *__restrict__ colw;
    const double *__restrict__ vald;
    const double *__restrict__ I2d;     // [N]
    const double2 *__restrict__ ab;     // per step: a_t, b_t
    const void *xin;
    void *xout, *y;
    int64_t n;
    int32_t N, Ap, W, step;
    double dt, xi0;
};

// One thread of symplectic_kernel_tsp (src/kernels.cu:561-597), Jacobi.
template <class T>
__global__ void __launch_bounds__(256) k_tsp_step(const TspSP P)
{
    using A = typename St<T>::A;
    pdl_wait();
    pdl_trigger();
    const int64_t gw = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (gw >= P.n * P.W) return;
    const int64_t r = gw / P.W;
    const int w = (int)(gw - r * P.W);
    const int64_t idx = r * P.Ap + (int64_t)w * 32 + lane;
    const T *xi = (const T *)P.xin;
    T *xo = (T *)P.xout, *yp = (T *)P.y;
    A x = St<T>::ld(xi[idx]), y = St<T>::ld(yp[idx]);
    if (fabs(x) > A(1)) {
        x = spin_of(x);
        y = A(0);
    } else {
        A i1 = 0;
        for (int32_t e = P.rowptr[r]; e < P.rowptr[r + 1]; e++) {
            const A xv = St<T>::ld(xi[(int64_t)(P.colw[e] & 0x7fffffffu) * P.Ap + (int64_t)w * 32 + lane]);
            const A act = mul(xv, (A)1.005);
            i1 = sub(i1, mul((A)P.vald[e], act));
        }
        const double2 ab = P.ab[P.step];
        const A i2 = (A)P.I2d[r % P.N];
        const A t = mul((A)P.xi0, add(mul((A)2, i1), mul((A)ab.y, i2)));
        y = add(y, mul((A)P.dt, t));
        x = add(x, mul((A)P.dt, y));
        y = add(y, mul((A)mul(P.dt, -sub(1.0, ab.x)), x));
    }
    xo[idx] = St<T>::st(x);
    yp[idx] = St<T>::st(y);
}

// Update_XY at step 0 (the MaxCut kernel the reference reuses, src/ising_tsp.cu:155).
template <class T>
__global__ void k_tsp_prestep(T *x, T *y, int64_t count, double k1, double k2)
{
    using A = typename St<T>::A;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    A xv = St<T>::ld(x[i]), yv = St<T>::ld(y[i]);
    yv = add(yv, mul((A)k2, xv));
    xv = add(xv, mul((A)k1, yv));
    x[i] = St<T>::st(xv);
    y[i] = St<T>::st(yv);
}

struct TspWP {
    const void *x;
    uint32_t *Wp;
    int32_t *visits;   // [2][N][Ap] scratch (city, order)
    int32_t *tours, *valid, *stab;
    uint8_t *bif, *prev;
    int64_t n;
    int32_t N, A, Ap, W, step, threshold;
};

// update_window_tsp, src/kernels.cu:461-541: one thread per agent, serial over
// the N^2 rows, exactly as the reference.
template <class T>
__global__ void k_tsp_window(const TspWP P)
{
    pdl_wait();
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= P.A) return;
    const T *x = (const T *)P.x;
    int32_t *cv = P.visits, *ov = P.visits + (int64_t)P.N * P.Ap;
    bool valid = true, equal = true;
    for (int64_t i = 0; i < P.n; i++) {
        const uint32_t s = sbit(St<T>::ld(x[i * P.Ap + a]));
        const uint32_t cur = (P.Wp[i * P.W + (a >> 5)] >> (a & 31)) & 1u;
        if (s != cur) equal = false;
        if (!s) {
            const int64_t city = i % P.N, order = (i - city) / P.N;
            cv[city * P.Ap + a] += 1;
            ov[order * P.Ap + a] += 1;
        }
    }
    for (int i = 0; i < P.N; i++)
        if (cv[(int64_t)i * P.Ap + a] != 1 || ov[(int64_t)i * P.Ap + a] != 1) {
            valid = false;
            break;
        }
    for (int i = 0; i < P.N; i++) cv[(int64_t)i * P.Ap + a] = ov[(int64_t)i * P.Ap + a] = 0;
    const bool nb = !P.bif[a];
    int st = P.stab[a];
    st += (equal && nb);
    st = (!equal && nb) ? 0 : st;
    const bool b = (st == P.threshold - 1);
    P.stab[a] = st;
    P.bif[a] = b;
    P.prev[a] = b;
    if (valid) {
        P.valid[a] = P.step;
        for (int o = 0; o < P.N; o++)
            for (int c = 0; c < P.N; c++)
                if (!sbit(St<T>::ld(x[((int64_t)o * P.N + c) * P.Ap + a]))) P.tours[(int64_t)a * P.N + o] = c;
    }
    // current_spins = sign(X)
    for (int64_t i = 0; i < P.n; i++) {
        const uint32_t s = sbit(St<T>::ld(x[i * P.Ap + a]));
        uint32_t *p = &P.Wp[i * P.W + (a >> 5)];
        if (s) atomicOr(p, 1u << (a & 31));
        else atomicAnd(p, ~(1u << (a & 31)));
    }
}

template <class T>
cudaError_t stream_t(const SolveDims &d, const DevTsp &t, Work &w, const double2 *ab,
                     const double *I2d, int32_t *visits, cudaStream_t s, int *launches)
{
    const int64_t n = (int64_t)t.N * t.N;
    const double p0 = 1.025 * 0.0 / d.steps;
    k_tsp_prestep<T><<<(unsigned)((n * d.Ap + 255) / 256), 256, 0, s>>>(
        (T *)w.x, (T *)w.y, n * d.Ap, d.dt * (p0 + 1), d.dt * (p0 - 1));
    (*launches)++;
    cudaError_t e = cudaGetLastError();
    TspSP P;
    P.rowptr = t.qubo.rowptr;
    P.colw = t.qubo.colw;
    P.vald = t.qubo.vald;
    P.I2d = I2d;
    P.ab = ab;
    P.y = w.y;
    P.n = n;
    P.N = t.N;
    P.Ap = d.Ap;
    P.W = d.W;
    P.dt = d.dt;
    P.xi0 = 0.002;
    TspWP Q;
    Q.Wp = w.Wp;
    Q.visits = visits;
    Q.tours = w.tours;
    Q.valid = w.valid;
    Q.stab = w.stab;
    Q.bif = w.bif;
    Q.prev = w.prev;
    Q.n = n;
    Q.N = t.N;
    Q.A = d.A;
    Q.Ap = d.Ap;
    Q.W = d.W;
    Q.threshold = d.threshold;
    void *cur = w.x, *nxt = w.x2;
    const int nwin = d.nwin;
    int k = 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)((n * d.W + 7) / 8));
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = d.pdl ? 1 : 0;
    for (int wdx = 0; wdx < nwin && e == cudaSuccess; wdx++) {
        for (int it = 0; it < d.period && e == cudaSuccess; it++, k++) {
            P.xin = cur;
            P.xout = nxt;
            P.step = k;
            e = cudaLaunchKernelEx(&cfg, k_tsp_step<T>, P);
            void *tmp = cur;
            cur = nxt;
            nxt = tmp;
            (*launches)++;
        }
        Q.x = cur;
        Q.step = k;
        k_tsp_window<T><<<(d.A + 127) / 128, 128, 0, s>>>(Q);
        (*launches)++;
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e == cudaSuccess && cur != w.x)
        e = cudaMemcpyAsync(w.x, cur, (size_t)n * d.Ap * sizeof(T), cudaMemcpyDeviceToDevice, s);
    return e;
}

}  // namespace

cudaError_t launch_tsp_stream(const SolveDims &d, const DevTsp &t, Work &w, cudaStream_t s,
                              int *launches)
{
    switch (d.prec) {
    case P_F32: return stream_t<float>(d, t, w, w.ab, t.I2d, w.visits, s, launches);
    case P_BF16: return stream_t<__nv_bfloat16>(d, t, w, w.ab, t.I2d, w.visits, s, launches);
    case P_F16: return stream_t<__half>(d, t, w, w.ab, t.I2d, w.visits, s, launches);
    default: return stream_t<double>(d, t, w, w.ab, t.I2d, w.visits, s, launches);
    }
}

namespace {

// Length of agent a's tour: the packed distance of every consecutive pair,
// the last city back to the first, summed in tour order in FP64 (src/ising_tsp.cu:272-287).
__global__ void __launch_bounds__(128) k_tsp_lengths(const int32_t *__restrict__ tours,
                                                     const int32_t *__restrict__ valid,
                                                     const double *__restrict__ Dd, int32_t N, int32_t A,
                                                     double *len)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    if (valid[a] <= 0) {
        len[a] = __longlong_as_double(0x7ff8000000000000LL);   // NaN: no valid tour
        return;
    }
    const int32_t *t = tours + (int64_t)a * N;
    double s = 0.0;
    for (int i = 0; i < N; i++) {
        const int c1 = t[i], c2 = t[i + 1 < N ? i + 1 : 0];
        s = __dadd_rn(s, Dd[(int64_t)c1 * N + c2]);
    }
    len[a] = s;
}

}  // namespace

namespace {

// TSP_distances_EUC_2D / TSP_distances_GEO (src/kernels.cu:404-442) on the
// device, one thread per pair c1 < c2, with the reference's expressions and
// its (int) truncation (none for the float kind); the packed upper triangle,
// and the symmetric N x N tables of the TSP kernels (float and FP64).
__global__ void __launch_bounds__(256) k_tsp_dist(const double *__restrict__ xc, const double *__restrict__ yc,
                                                  int32_t N, int32_t kind, double *packed, float *D, double *Dd)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * N) return;
    const int c1 = (int)(t / N), c2 = (int)(t - (int64_t)c1 * N);
    if (c2 <= c1) return;
    double d;
    if (kind == 1) {   // GEO, kernels.cu:425-441
        const double R = 6378.388;
        const double q1 = cos(yc[c1] - yc[c2]);
        const double q2 = cos(xc[c1] - xc[c2]);
        const double q3 = cos(xc[c1] + xc[c2]);
        d = (double)(int)(R * acos(0.5 * ((1.0 + q1) * q2 - (1.0 - q1) * q3)) + 1.0);
    } else {           // EUC_2D, kernels.cu:404-423
        const double xd = xc[c1] - xc[c2], yd = yc[c1] - yc[c2];
        d = pow(xd * xd + yd * yd, 0.5);
        if (kind == 0) d = (double)(int)d;
    }
    packed[(int64_t)c2 + (int64_t)c1 * N - (int64_t)(c1 + 2) * (c1 + 1) / 2] = d;
    D[(int64_t)c1 * N + c2] = D[(int64_t)c2 * N + c1] = (float)d;
    Dd[(int64_t)c1 * N + c2] = Dd[(int64_t)c2 * N + c1] = d;
}

// The largest distance (exact in any order).
__global__ void __launch_bounds__(256) k_tsp_max(const double *__restrict__ packed, int64_t nd, double *mx)
{
    double m = 0;
    for (int64_t k = threadIdx.x; k < nd; k += blockDim.x) m = fmax(m, packed[k]);
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(FULL, m, o));
    __shared__ double w[8];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); i++) m = fmax(m, w[i]);
        *mx = fmax(m, w[0]);
    }
}

// Per-city distance sums (src/tsp_gpu.cu:51-68 adds each pair to both of its
// cities walking the packed array, so city c receives its pairs in ascending
// order of the other city), then the linear field of src/kernels.cu:591-592,
// -1 (A rowsum + (N - 2)(B + C)) / 2 with B = C = scale * max distance,
// rounded per operation as the host states it.
__global__ void __launch_bounds__(128) k_tsp_rows(const double *__restrict__ Dd, int32_t N, double A,
                                                  double scale, const double *__restrict__ mx,
                                                  double *rowsum, double *I2d, float *I2)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    double r = 0;
    for (int k = 0; k < N; k++)
        if (k != c) r = __dadd_rn(r, Dd[(int64_t)c * N + k]);
    rowsum[c] = r;
    const double B = __dmul_rn(scale, *mx);
    const double v = __ddiv_rn(__dmul_rn(-1.0, __dadd_rn(__dmul_rn(A, r), __dmul_rn((double)(N - 2), __dadd_rn(B, B)))),
                               2.0);
    I2d[c] = v;
    I2[c] = (float)v;
}

}  // namespace

cudaError_t launch_tsp_setup(const double *xc, const double *yc, int32_t N, int32_t kind, double A, double scale,
                             double *packed, double *mx, double *rowsum, DevTsp &t, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(t.D, 0, sizeof(float) * N * N, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(t.Dd, 0, sizeof(double) * N * N, s);
    if (e != cudaSuccess) return e;
    const int64_t nn = (int64_t)N * N;
    k_tsp_dist<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(xc, yc, N, kind, packed, t.D, t.Dd);
    k_tsp_max<<<1, 256, 0, s>>>(packed, (int64_t)N * (N - 1) / 2, mx);
    k_tsp_rows<<<(N + 127) / 128, 128, 0, s>>>(t.Dd, N, A, scale, mx, rowsum, t.I2d, t.I2);
    return cudaGetLastError();
}

cudaError_t launch_tsp_lengths(const DevTsp &t, const int32_t *tours, const int32_t *valid, int32_t A,
                               double *len, cudaStream_t s)
{
    if (A <= 0) return cudaSuccess;
    k_tsp_lengths<<<(A + 127) / 128, 128, 0, s>>>(tours, valid, t.Dd, t.N, A, len);
    return cudaGetLastError();
}

}  // namespace sbx
