// k_step.cuh -- the streaming MaxCut SB step kernel (one launch per step),
// included by one translation unit per storage precision.
//
// Layout.  x, y: [n][Ap] in the storage precision (Ap = agents rounded up to
// 32).  Sign planes S[2], window plane Wp (the reference's current_spins),
// final plane fin: [n][Ap/32] uint32, bit a%32 of word (r, a/32) = signbit of
// x[r][a] (1 = spin -1).
//
// Semantics (Jacobi): every gather of step k reads the sign plane written by
// step k-1, so each step is the reference kernel run with all threads reading
// the state the launch began with (src/kernels.cu:211-269 for the fused mode;
// src/ising.cu:168-171 for the unfused trio).  The force only needs signs, so
// a neighbour costs one 4-byte word per 32 agents instead of 32 FP64 loads.
#pragma once

#include "common.cuh"
#include "engine.h"

#include <cstring>
#include <type_traits>

namespace sbx {

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
    const int32_t *__restrict__ hchunk;   // heavy rows: first chunk, else -1
    const int32_t *__restrict__ chunk_row;
    uint2 *part;                          // [chunk][segment][lane] byte counters
    const int32_t *__restrict__ order;    // skewed graphs: rows in decreasing degree
    const float *__restrict__ c0r32;      // batched: dt*xi0 per row (else null)
    const double *__restrict__ c0r64;
    int64_t n;
    int32_t W, Ap, nchunks;
    double c0;
};

// One step kernel launch (kind K_*, window step or not) in the precision of
// d.prec; one definition per precision (k_step_<prec>.cu).
cudaError_t step_f32(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win, int offset, cudaStream_t s);
cudaError_t step_bf16(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win, int offset, cudaStream_t s);
cudaError_t step_f16(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win, int offset, cudaStream_t s);
cudaError_t step_f64(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win, int offset, cudaStream_t s);

namespace {

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

__device__ __forceinline__ uint32_t spread4(uint32_t nib) { return (nib * 0x00204081u) & 0x01010101u; }

// V consecutive storage elements moved as one naturally aligned vector.
template <int B> struct Raw;
template <> struct Raw<16> { uint4 u; };
template <> struct Raw<8> { uint2 u; };
template <> struct Raw<4> { uint32_t u; };
template <> struct Raw<2> { unsigned short u; };
template <class T, int V> __device__ __forceinline__ Raw<V * sizeof(T)> vload(const T *p)
{
    Raw<V * sizeof(T)> r;
    r.u = *(const decltype(r.u) *)p;
    return r;
}
template <class T, int V> __device__ __forceinline__ void unpack(const Raw<V * sizeof(T)> &r, T (&o)[V])
{
    memcpy(o, &r.u, V * sizeof(T));
}
template <class T, int V> __device__ __forceinline__ void vstore(T *p, const T (&o)[V])
{
    Raw<V * sizeof(T)> r;
    memcpy(&r.u, o, V * sizeof(T));
    *(decltype(r.u) *)p = r.u;
}

// Raw storage vector <-> arithmetic values.  16-bit types go two at a time
// (one pack instruction per pair); the arithmetic is FP32.
template <class T, int V, class A>
__device__ __forceinline__ void to_vals(const Raw<V * sizeof(T)> &r, A (&o)[V])
{
    if constexpr (sizeof(T) == 2 && V >= 2) {
        uint32_t w[V / 2];
        memcpy(w, &r.u, sizeof w);
#pragma unroll
        for (int i = 0; i < V / 2; i++) {
            if constexpr (std::is_same<T, __nv_bfloat16>::value) {
                o[2 * i] = __uint_as_float(w[i] << 16);
                o[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
            } else {
                const float2 f = __half22float2(*(const __half2 *)&w[i]);
                o[2 * i] = f.x;
                o[2 * i + 1] = f.y;
            }
        }
    } else {
        T t[V];
        memcpy(t, &r.u, sizeof t);
#pragma unroll
        for (int v = 0; v < V; v++) o[v] = St<T>::ld(t[v]);
    }
}
template <class T, int V, class A>
__device__ __forceinline__ Raw<V * sizeof(T)> from_vals(const A (&o)[V])
{
    Raw<V * sizeof(T)> r;
    if constexpr (sizeof(T) == 2 && V >= 2) {
        uint32_t w[V / 2];
#pragma unroll
        for (int i = 0; i < V / 2; i++) {
            if constexpr (std::is_same<T, __nv_bfloat16>::value) {
                const __nv_bfloat162 h = __floats2bfloat162_rn(o[2 * i], o[2 * i + 1]);
                w[i] = *(const uint32_t *)&h;
            } else {
                const __half2 h = __floats2half2_rn(o[2 * i], o[2 * i + 1]);
                w[i] = *(const uint32_t *)&h;
            }
        }
        memcpy(&r.u, w, sizeof w);
    } else {
        T t[V];
#pragma unroll
        for (int v = 0; v < V; v++) t[v] = St<T>::st(o[v]);
        memcpy(&r.u, t, sizeof t);
    }
    return r;
}

// Partial counts of heavy rows (+-1 weights): item = (chunk of kHeavy
// neighbours, segment of 32*V agents); a lane leaves the byte counters of its
// V agents, which the step kernel then sums for the row.
template <int V>
__global__ void __launch_bounds__(256) k_heavy(const StepP P, const int offset)
{
    pdl_wait();
    if (P.ctl[CTL_STOP]) return;
    const int step = P.ctl[CTL_STEP] + offset;
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const uint32_t *Scur = (step & 1) ? P.S1 : P.S0;
    const int nit = P.Ap / (32 * V);
    const int64_t items = (int64_t)P.nchunks * nit;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t item = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); item < items;
         item += nw) {
        const int c = (int)(item / nit), it = (int)(item - (int64_t)c * nit);
        const int32_t r = __ldg(&P.chunk_row[c]);
        const int32_t e0 = __ldg(&P.rowptr[r]) + (c - __ldg(&P.hchunk[r])) * kHeavy;
        const int32_t e1 = min(__ldg(&P.rowptr[r + 1]), e0 + kHeavy);
        const int a0 = it * 32 * V + lane * V;
        const int q = a0 >> 5, off = a0 & 31;
        const uint32_t *Sq = Scur + q;
        uint32_t lo = 0, hi = 0;
        for (int32_t cb = e0; cb < e1; cb += 32) {
            const int m = min(32, e1 - cb);
            const uint32_t mycw = lane < m ? __ldg(&P.colw[cb + lane]) : 0u;
#pragma unroll 4
            for (int k = 0; k < m; k++) {
                const uint32_t cw = __shfl_sync(FULL, mycw, k);
                uint32_t bits = __ldg(Sq + (size_t)(cw & 0x7fffffffu) * (size_t)P.W) >> off;
                bits ^= (uint32_t)((int32_t)cw >> 31);
                lo += spread4(bits & 0xfu);
                if (V == 8) hi += spread4((bits >> 4) & 0xfu);
            }
        }
        P.part[item * 32 + lane] = make_uint2(lo, hi);
    }
}

// One SB step over every (row, agent).  Work item = (row, segment of 32*V
// agents); a warp takes items in turn, lane l owns V consecutive agents of the
// segment (one vector load of x and of y).  Per neighbour j the lane reads the
// sign word of its agents in row j of the plane (lanes of one word share the
// address), XORs the weight's sign and adds the V bits into byte counters
// (bit i of a nibble lands in byte i after multiplying by 0x00204081); the
// force is 2*count - degree, exact (src/kernels.cu:247-255).  A byte counter
// holds up to kHeavy = 128 neighbours; longer rows (+-1 weights) are counted
// in kHeavy chunks by k_heavy and the BIG kernels add those partials.
// The new signs of the V agents are OR-combined across the lanes of a word
// and written once.
// x + a*b: one FMA in FP32; in FP64 two separately rounded operations, the
// reference's arithmetic as the oracle states it.
__device__ __forceinline__ float madd(float a, float b, float x) { return fmaf(a, b, x); }
__device__ __forceinline__ double madd(double a, double b, double x) { return __dadd_rn(x, __dmul_rn(a, b)); }

template <class T, int V, int KIND, bool WIN, int WM, bool BIG, int LR>
__global__ void __launch_bounds__(256) k_row(const StepP P, const int offset)
{
    static_assert(LR == 32 || !BIG, "heavy-row partials are laid out for whole-warp rows");
    static_assert(LR * V >= 32, "a sign word belongs to one row's lanes");
    using A = typename St<T>::A;
    using R = typename std::conditional<WM == W_F64, double, float>::type;
    extern __shared__ uint32_t s_chg[];   // [W] window steps: changed bits of this block
    pdl_wait();
    if (P.ctl[CTL_STOP]) return;          // block-uniform
    const int step = P.ctl[CTL_STEP] + offset;
    const int lane = threadIdx.x & 31;
    if (WIN) {
        for (int q = threadIdx.x; q < P.W; q += blockDim.x) s_chg[q] = 0;
        __syncthreads();
    }
    pdl_trigger();
    T *xp = (T *)P.x, *yp = (T *)P.y;
    uint32_t *Scur = (step & 1) ? P.S1 : P.S0;
    uint32_t *Snext = (step & 1) ? P.S0 : P.S1;
    constexpr int G = 32 / V;   // lanes sharing one sign word
    constexpr int RW = 32 / LR; // rows per warp: LR lanes per row
    constexpr uint32_t VM = (V == 32) ? 0xffffffffu : ((1u << V) - 1u);
    const int rw = lane / LR, sl = lane & (LR - 1);   // row of the warp, lane of the row
    // Items (group of RW rows, segment of LR*V agents) in steps of the warp
    // count, advanced without divisions: g += nw / nit, it += nw % nit with
    // carry.  Below 32 lanes per row a row is one segment (nit = 1).
    const int nit = P.Ap / (LR * V);
    const int64_t ng = (P.n + RW - 1) / RW;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t w0 = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t dr = nw / nit;
    const int dit = (int)(nw - dr * nit);
    int64_t g = w0 / nit;
    int it = (int)(w0 - g * nit);
    for (; g < ng; g += dr, it += dit) {
        if (it >= nit) {
            it -= nit;
            g++;
            if (g >= ng) break;
        }
        // Lanes of a group past the last row repeat row n-1 and store nothing.
        const int64_t gi = g * RW + rw;
        const bool live = RW == 1 || gi < P.n;
        const int64_t ri = live ? gi : P.n - 1;
        // Skewed graphs are visited in decreasing degree, so every warp's
        // share holds the same mix of long and short rows.
        const int64_t r = P.order ? (int64_t)__ldg(&P.order[ri]) : ri;
        const int a0 = it * LR * V + sl * V;
        const int q = a0 >> 5, off = a0 & 31;
        const int64_t base = r * P.Ap + a0;
        uint32_t wp_old = 0;   // window steps: the previous window's word, fetched early
        if (WIN && (lane & (G - 1)) == 0) wp_old = P.Wp[r * P.W + q];
        const auto xr = vload<T, V>(xp + base);
        const auto yr = vload<T, V>(yp + base);
        A x[V], y[V];
        if (KIND == K_XY) {
            // Update_XY, src/kernels.cu:8-22 (pressure not clamped)
            const auto c = Coef<A>::get(P, step);
            to_vals<T, V>(xr, x);
            to_vals<T, V>(yr, y);
#pragma unroll
            for (int v = 0; v < V; v++) {
                y[v] = madd((A)c.w, x[v], y[v]);
                x[v] = madd((A)c.z, y[v], x[v]);
            }
        } else {
            const int32_t e0 = __ldg(&P.rowptr[r]), e1 = __ldg(&P.rowptr[r + 1]);
            const int deg = e1 - e0;
            uint32_t lo = 0, hi = 0;
            int cnt[BIG ? V : 1];
            R tot[WM == W_UNIT ? 1 : V];
#pragma unroll
            for (int v = 0; v < (BIG ? V : 1); v++) cnt[v] = 0;
#pragma unroll
            for (int v = 0; v < (WM == W_UNIT ? 1 : V); v++) tot[v] = R(0);
            // Heavy rows (BIG kernels only) take their counts from k_heavy.
            // With several rows per warp the walk runs to the longest row of
            // the warp; shuffles stay warp-wide, loads and sums per row.
            const int32_t dw = (BIG && WM == W_UNIT && deg > kHeavy) ? 0 : deg;
            int32_t dmax = dw;
            if constexpr (LR < 32) dmax = __reduce_max_sync(FULL, dw);
            for (int32_t cb = 0; cb < dmax; cb += LR) {
                const int m = min(LR, dmax - cb);
                const int32_t idx = cb + sl;
                const uint32_t mycw = idx < dw ? __ldg(&P.colw[e0 + idx]) : 0u;
                R myv = R(0);
                if (WM == W_F32) myv = idx < dw ? __ldg(&P.valf[e0 + idx]) : 0.f;
                if (WM == W_F64) myv = idx < dw ? __ldg(&P.vald[e0 + idx]) : 0.0;
                const uint32_t *Sq = Scur + q;
#pragma unroll 4
                for (int k = 0; k < m; k++) {
                    const uint32_t cw = __shfl_sync(FULL, mycw, k, LR);
                    R wv = R(0);
                    if (WM != W_UNIT) wv = __shfl_sync(FULL, myv, k, LR);
                    if (LR == 32 || cb + k < dw) {
                        const uint32_t word = __ldg(Sq + (size_t)(cw & 0x7fffffffu) * (size_t)P.W);
                        uint32_t bits = word >> off;
                        if (WM == W_UNIT) {
                            // weight sign -> all-ones mask; unused high bits
                            // only reach counter bytes that are never read
                            bits ^= (uint32_t)((int32_t)cw >> 31);
                            lo += spread4(bits & 0xfu);
                            if (V == 8) hi += spread4((bits >> 4) & 0xfu);
                        } else {
                            bits &= VM;
#pragma unroll
                            for (int v = 0; v < V; v++) {
                                const R sv = ((bits >> v) & 1u) ? R(-1) : R(1);
                                if (WM == W_F64) tot[v] = sub(tot[v], mul(wv, sv));
                                else tot[v] -= wv * sv;
                            }
                        }
                    }
                }
            }
            if (BIG && WM == W_UNIT) {
                if (deg > kHeavy) {
                    // a heavy row: its neighbours were counted in chunks by
                    // k_heavy; the loop above did not run for it
                    const int c0i = __ldg(&P.hchunk[r]), nc = (deg + kHeavy - 1) / kHeavy;
                    for (int cc = 0; cc < nc; cc++) {
                        const uint2 pr = P.part[((int64_t)(c0i + cc) * nit + it) * 32 + lane];
#pragma unroll
                        for (int v = 0; v < (BIG ? V : 1); v++)
                            cnt[v] += ((v < 4 ? pr.x : pr.y) >> (8 * (v & 3))) & 0xffu;
                    }
                } else {
#pragma unroll
                    for (int v = 0; v < (BIG ? V : 1); v++)
                        cnt[v] += ((v < 4 ? lo : hi) >> (8 * (v & 3))) & 0xffu;
                }
            }
            const auto c = Coef<A>::get(P, step);
            A c0 = (A)P.c0;
            if (P.c0r32) c0 = std::is_same<A, double>::value ? (A)__ldg(&P.c0r64[r]) : (A)__ldg(&P.c0r32[r]);
            // FP32 totals straight from the byte counters: PRMT builds the
            // float 2^23 + count; fma(2, f, -2^24) is 2*count exactly, and
            // subtracting the degree gives the exact integer 2*count - deg.
            const float fdeg = (float)deg;
            to_vals<T, V>(xr, x);
            to_vals<T, V>(yr, y);
#pragma unroll
            for (int v = 0; v < V; v++) {
                A total;
                if (WM != W_UNIT) {
                    total = (A)tot[WM == W_UNIT ? 0 : v];
                } else if (BIG) {
                    total = (A)(2 * cnt[v < (BIG ? V : 1) ? v : 0] - deg);
                } else if (std::is_same<A, float>::value) {
                    const uint32_t f = __byte_perm(v < 4 ? lo : hi, 0x4b000000u, 0x7440u + (v & 3));
                    total = (A)(fmaf(2.0f, __uint_as_float(f), -16777216.0f) - fdeg);
                } else {
                    total = (A)(2 * (int)(((v < 4 ? lo : hi) >> (8 * (v & 3))) & 0xffu) - deg);
                }
                const bool clamp = fabs(x[v]) > A(1);
                const A xc = spin_of(x[v]);
                if (KIND == K_FUSED) {
                    // src/kernels.cu:236-262: clamp or kick, then the drift /
                    // kick pair that runs unconditionally (a clamped oscillator
                    // leaves with y = dt (p-1) sign(x)).
                    y[v] = clamp ? A(0) : madd(c0, total, y[v]);
                    x[v] = clamp ? xc : x[v];
                    x[v] = madd((A)c.x, y[v], x[v]);
                    y[v] = madd((A)c.y, x[v], y[v]);
                } else {
                    // mat_mult (:207) and confine (:158-165) of this step, then
                    // Update_XY of the next one unless the window closes here.
                    y[v] = clamp ? A(0) : madd(c0, total, y[v]);
                    x[v] = clamp ? xc : x[v];
                    if (!WIN) {
                        const auto cn = Coef<A>::get(P, step + 1);
                        y[v] = madd((A)cn.w, x[v], y[v]);
                        x[v] = madd((A)cn.z, y[v], x[v]);
                    }
                }
            }
        }
        // Signs of the new x (rounding to the storage type keeps the sign).
        uint32_t b = 0;
#pragma unroll
        for (int v = 0; v < V; v++) b |= sbit(x[v]) << v;
        const auto xw = from_vals<T, V>(x);
        const auto yw = from_vals<T, V>(y);
        if (live) {
            *(decltype(xw.u) *)(xp + base) = xw.u;
            *(decltype(yw.u) *)(yp + base) = yw.u;
        }
        b <<= off;
#pragma unroll
        for (int sft = 1; sft < G; sft <<= 1) b |= __shfl_xor_sync(FULL, b, sft);
        if (live && (lane & (G - 1)) == 0) {
            const int64_t wi = r * P.W + q;
            if (KIND == K_XY) Scur[wi] = b;
            else if (KIND == K_FUSED || !WIN) Snext[wi] = b;
            if (WIN) {
                // window compare, src/kernels.cu:37-46 + :84-90
                const uint32_t ch = b ^ wp_old;
                P.Wp[wi] = b;
                if (ch) atomicOr(&s_chg[q], ch);
            }
        }
    }
    if (WIN) {
        __syncthreads();
        for (int qq = threadIdx.x; qq < P.W; qq += blockDim.x)
            if (s_chg[qq]) atomicOr(&P.chg[qq], s_chg[qq]);
    }
}

template <class K, class... Args>
cudaError_t launch(K kern, dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool pdl, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}


// Grid of a persistent grid-stride kernel: as many resident CTAs of bt
// threads as the occupancy allows on every SM, fewer when the items run out.
template <class K>
cudaError_t launch_grid(K kern, const SolveDims &d, int64_t items, int bt, size_t smem, cudaStream_t s,
                        const StepP &P, int offset)
{
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, bt, smem);
    if (per_sm < 1) per_sm = 1;
    const int wpb = bt / 32;
    int64_t blocks = (items + wpb - 1) / wpb;
    if (blocks > (int64_t)nsm * per_sm) blocks = (int64_t)nsm * per_sm;
    if (blocks < 1) blocks = 1;
    return launch(kern, dim3((unsigned)blocks), dim3(bt), smem, s, d.pdl, P, offset);
}

// One step with V agents per lane and LR lanes per row.
template <class T, int V, int LR, int KIND, bool WIN>
cudaError_t step_vl(const SolveDims &d, const DevCsr &J, const StepP &P, int offset, cudaStream_t s)
{
    constexpr int RW = 32 / LR;
    const int64_t items = (d.n + RW - 1) / RW * (d.Ap / (LR * V));
    const size_t smem = WIN ? sizeof(uint32_t) * d.W : 0;
    const int bt = d.tbt;
    const bool big = J.unit && J.nchunks > 0 && KIND != K_XY;
    if constexpr (LR == 32) {
        if (big) {
            cudaError_t e = launch_grid(k_heavy<V>, d, (int64_t)J.nchunks * (d.Ap / (32 * V)), 256, 0, s, P,
                                        offset);
            if (e != cudaSuccess) return e;
            return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, true, 32>, d, items, bt, smem, s, P, offset);
        }
    } else {
        if (big) return cudaErrorInvalidValue;
    }
    if (KIND == K_XY || J.unit)
        return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, false, LR>, d, items, bt, smem, s, P, offset);
    if constexpr (sizeof(T) == 8)
        return launch_grid(k_row<T, V, KIND, WIN, W_F64, false, LR>, d, items, bt, smem, s, P, offset);
    else
        return launch_grid(k_row<T, V, KIND, WIN, W_F32, false, LR>, d, items, bt, smem, s, P, offset);
}

// Agents per lane by default: a 16-byte vector when the padded agent count
// allows.
template <class T> int pick_v(int Ap)
{
    int v = 16 / (int)sizeof(T);
    while (v > 1 && Ap % (32 * v)) v >>= 1;
    return v;
}

// The tile (d.tv agents per lane, d.tlr lanes per row) picks the kernel.
// Whole-warp rows take any V that divides the padded agent count; fewer
// lanes per row are built for the two widest vectors (VM, VM/2) and need
// LR*V = Ap.  The host validates tiles (tile_ok) before they get here.
template <class T, int KIND, bool WIN>
cudaError_t step_kw(const SolveDims &d, const DevCsr &J, const StepP &P, int offset, cudaStream_t s)
{
    constexpr int VM = 16 / (int)sizeof(T);
    const int lr = (KIND == K_XY || d.tlr == 0) ? 32 : d.tlr;
    const int v = (KIND == K_XY || d.tv == 0) ? pick_v<T>(d.Ap) : d.tv;
    if (lr == 32) {
        switch (v) {
        case 8:
            if constexpr (VM >= 8) return step_vl<T, 8, 32, KIND, WIN>(d, J, P, offset, s);
            else return cudaErrorInvalidValue;
        case 4:
            if constexpr (VM >= 4) return step_vl<T, 4, 32, KIND, WIN>(d, J, P, offset, s);
            else return cudaErrorInvalidValue;
        case 2: return step_vl<T, 2, 32, KIND, WIN>(d, J, P, offset, s);
        case 1: return step_vl<T, 1, 32, KIND, WIN>(d, J, P, offset, s);
        default: return cudaErrorInvalidValue;
        }
    }
    if constexpr (KIND != K_XY) {
        if (v == VM) {
            switch (lr) {
            case 16: return step_vl<T, VM, 16, KIND, WIN>(d, J, P, offset, s);
            case 8:
                if constexpr (VM * 8 >= 32) return step_vl<T, VM, 8, KIND, WIN>(d, J, P, offset, s);
                else return cudaErrorInvalidValue;
            case 4:
                if constexpr (VM * 4 >= 32) return step_vl<T, VM, 4, KIND, WIN>(d, J, P, offset, s);
                else return cudaErrorInvalidValue;
            default: return cudaErrorInvalidValue;
            }
        }
        if constexpr (VM >= 2) {
            if (v == VM / 2) {
                switch (lr) {
                case 16:
                    if constexpr (VM / 2 * 16 >= 32) return step_vl<T, VM / 2, 16, KIND, WIN>(d, J, P, offset, s);
                    else return cudaErrorInvalidValue;
                case 8:
                    if constexpr (VM / 2 * 8 >= 32) return step_vl<T, VM / 2, 8, KIND, WIN>(d, J, P, offset, s);
                    else return cudaErrorInvalidValue;
                default: return cudaErrorInvalidValue;
                }
            }
        }
    }
    return cudaErrorInvalidValue;
}

template <class T>
cudaError_t step_t(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win,
                   int offset, cudaStream_t s)
{
    if (kind == K_XY) return step_kw<T, K_XY, false>(d, J, P, offset, s);
    if (kind == K_FUSED)
        return win ? step_kw<T, K_FUSED, true>(d, J, P, offset, s)
                   : step_kw<T, K_FUSED, false>(d, J, P, offset, s);
    return win ? step_kw<T, K_FC, true>(d, J, P, offset, s) : step_kw<T, K_FC, false>(d, J, P, offset, s);
}

}  // namespace

}  // namespace sbx
