// k_tsp_tc.cu -- TSP-QUBO ballistic SB (src/kernels.cu:543-599, window
// src/kernels.cu:461-541) with the distance product on the tensor cores
// (tcgen05), 16-bit state (BF16 or FP16).
//
// The structured force of the QUBO of src/tsp_gpu.cu:76-112 is
//   (J x)[i][k] = C/4 colsum[k] + B/4 rowsum[i]
//                 + A/8 (sum_l d_kl x[i-1][l] + sum_l d_kl x[i+1][l]).
// Over the rows m = i*8 + a (position i, agent a of the CTA's 8 agents) the
// last term is a product of two matrices, P[m][k] = sum_l X-[m][l] d_kl +
// sum_l X+[m][l] d_kl, X-/X+ the rows of the neighbouring positions.  The CTA
// keeps its agents' x in shared memory in the storage type, already in the
// tensor cores' operand layout (K-major, no swizzle: 8-row x 16-byte core
// matrices), with a halo position on each side (position -1 holds N-1,
// position N holds 0).  X- and X+ are then the same array seen from two start
// rows 16 apart, two operand descriptors and no copy.  D enters as three
// 16-bit matrices whose sum is D exactly (hi, mid, lo; FP16 after an exact
// power-of-two scale), stacked along N, so every product is exact and the
// sums are FP32 in the tensor core.  Per step one thread issues 4 MMAs
// (M = 128, N = 96, K = 16) per 128-row tile into TMEM, while the threads sum
// the state's columns and rows; each thread then reads its row's products
// with the three parts back (tcgen05.ld), adds them, and updates its spins on
// the FP32 pipes as the CUDA-core kernel does.
//
// The MMA completion is a bounded mbarrier wait: a wait that runs out flags
// CTL_ERR, waits (bounded) for the MMAs in flight, frees TMEM and returns.
#include "common.cuh"
#include "engine.h"

namespace sbx {

namespace {

constexpr int KA = 8;                 // agents per CTA: rows m = i*KA + a
constexpr int NP = 32;                // cities padded: the MMA's N and K
constexpr int ROWB = NP * 2;          // operand row: 32 16-bit values
constexpr int SBO = 8 * ROWB;         // bytes between 8-row core-matrix groups
constexpr int LBO = 128;              // bytes between 16-byte K chunks of a group
constexpr int XROWS = 256 + 2 * KA;   // two tiles of rows and the halo
constexpr int DPART = NP * ROWB;      // one 32 x 32 part of D
constexpr uint32_t kTcLimit = 1u << 22;

struct TcP {
    const float *__restrict__ D;      // [N][N] distances, zero diagonal
    const float *__restrict__ I2;     // [N] linear field per city
    const float2 *__restrict__ sched; // per step: b_t, dt*-(1-a_t)
    void *x, *y;                      // global [n][Ap], n = N*N, row = i*N + k
    uint32_t *Wp;                     // global plane [n][W] (window spins)
    int32_t *tours, *valid;           // [Ap][N], [Ap]
    int32_t *stab;
    uint8_t *bif, *prev;
    int32_t *ctl;
    int32_t N, A, Ap, W, nwin, period, threshold, tiles, giveup;
    float qa8, qb4, qc4;              // A/8, B/4, C/4
    float dtxi0, dt, k1u, k2u;        // pre-step Update_XY coefficients
    float dscale, dunscale;           // D scaled by 2^-s into the operand range, and 2^s
};

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of (row r, element c) in the operand layout
__device__ __forceinline__ uint32_t opoff(int r, int c)
{
    return (uint32_t)((r >> 3) * SBO + (c >> 3) * LBO + (r & 7) * 16 + (c & 7) * 2);
}

// shared-memory matrix descriptor: start, leading (K) and stride (8-row)
// byte offsets, the descriptor version bit, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(LBO >> 4) << 16) |
           ((uint64_t)(SBO >> 4) << 32) | (1ull << 46);
}

template <class T> struct TcType;
template <> struct TcType<__nv_bfloat16> {
    static constexpr uint32_t code = 1;   // BF16 operands
    static __device__ __forceinline__ unsigned short bits(float v) {
        return __bfloat16_as_ushort(__float2bfloat16_rn(v));
    }
    static __device__ __forceinline__ float val(unsigned short b) {
        return __bfloat162float(__ushort_as_bfloat16(b));
    }
};
template <> struct TcType<__half> {
    static constexpr uint32_t code = 0;   // FP16 operands
    static __device__ __forceinline__ unsigned short bits(float v) { return __half_as_ushort(__float2half_rn(v)); }
    static __device__ __forceinline__ float val(unsigned short b) { return __half2float(__ushort_as_half(b)); }
};

// instruction descriptor: FP32 accumulator, A and B of the state's type,
// both K-major, N = 96 (the three parts of D stacked), M = 128
template <class T> __device__ __forceinline__ uint32_t idesc()
{
    return (1u << 4) | (TcType<T>::code << 7) | (TcType<T>::code << 10) | ((uint32_t)(3 * NP >> 3) << 17) |
           ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma16(uint32_t dtm, uint64_t a, uint64_t b, uint32_t id, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtm),
                 "l"(a), "l"(b), "r"(id), "r"(acc)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_n(uint32_t bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t k = 0; k < limit; k++)
        if (mbar_try(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// C FP32 columns of this thread's TMEM lane (C = 32, 16 or 8)
template <int C> __device__ __forceinline__ void tmem_ld(uint32_t ta, float *v);
template <> __device__ __forceinline__ void tmem_ld<32>(uint32_t ta, float *v)
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
                   "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
                   "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
                   "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
                   "=r"(r[31])
                 : "r"(ta));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; k++) v[k] = __uint_as_float(r[k]);
}
template <> __device__ __forceinline__ void tmem_ld<16>(uint32_t ta, float *v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
                   "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(ta));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}
template <> __device__ __forceinline__ void tmem_ld<8>(uint32_t ta, float *v)
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(ta));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = __uint_as_float(r[k]);
}

template <class T> __device__ __forceinline__ float rnd(float v) { return St<T>::ld(St<T>::st(v)); }

// two values rounded to the storage type and back (one packed conversion)
template <class T> __device__ __forceinline__ float2 rnd2(float2 v);
template <> __device__ __forceinline__ float2 rnd2<__nv_bfloat16>(float2 v)
{
    return __bfloat1622float2(__float22bfloat162_rn(v));
}
template <> __device__ __forceinline__ float2 rnd2<__half>(float2 v) { return __half22float2(__float22half2_rn(v)); }

// H threads share a row m = (i, a): thread part hh owns the cities
// [32 hh / H, 32 (hh + 1) / H).  Warp w reads TMEM lanes 32 (w mod 4) of
// tile (w / 4) mod T, part (w / 4) / T; 128 T H threads.
template <class T, int H>
__global__ void __launch_bounds__(128 * 2 * H, 1) k_tsp_tc(const TcP P)
{
    using TT = TcType<T>;
    constexpr int CPT = NP / H;                     // cities of a thread
    __shared__ __align__(1024) unsigned char xs[XROWS * ROWB];   // X with halo, operand layout
    __shared__ __align__(1024) unsigned char ds[3 * DPART];      // D = hi + mid + lo
    __shared__ float colsum[NP * KA], rsum[NP * KA];
    __shared__ uint32_t rowbits[NP * KA], prevbits[NP * KA];
    __shared__ int aflag[2 * KA];
    __shared__ float s_I2[NP];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t s_tmem;

    pdl_wait();
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = P.N, T2 = P.tiles;
    const int tile = (warp >> 2) % T2, hh = (warp >> 2) / T2;
    const int m = 128 * tile + 32 * (warp & 3) + lane;   // this thread's row
    const int i = m / KA, a = m % KA;                    // position, local agent
    const int k0 = CPT * hh;                             // first city of this thread
    const int ag = blockIdx.x * KA + a;                  // global agent
    const bool active = i < N;
    const bool real = active && ag < P.A;                // padded agents compute on zeros
    T *xg = (T *)P.x, *yg = (T *)P.y;
    const uint32_t xs0 = saddr(xs), ds0 = saddr(ds), bar = saddr(&mbar);

    // operands: X all zero (halo, padding rows and columns), D split exactly
    for (int t = tid; t < XROWS * ROWB / 16; t += blockDim.x) ((uint4 *)xs)[t] = make_uint4(0, 0, 0, 0);
    for (int t = tid; t < NP * NP; t += blockDim.x) {
        const int k = t / NP, l = t % NP;
        const float d = (k < N && l < N) ? P.D[k * N + l] * P.dscale : 0.f;
        const unsigned short h = TT::bits(d);
        const float r1 = d - TT::val(h);
        const unsigned short md = TT::bits(r1);
        const unsigned short lo = TT::bits(r1 - TT::val(md));
        const uint32_t o = opoff(k, l);
        *(unsigned short *)(ds + o) = h;
        *(unsigned short *)(ds + DPART + o) = md;
        *(unsigned short *)(ds + 2 * DPART + o) = lo;
    }
    for (int t = tid; t < NP; t += blockDim.x) s_I2[t] = t < N ? P.I2[t] : 0.f;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // TMEM: 96 columns a tile (the products with hi, mid, lo), tile t at 128 t
    const uint32_t ncols = 128u * (uint32_t)T2;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&s_tmem)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = s_tmem;

    // Initial state (x = 0, y from the init stream) and the pre-step
    // Update_XY at step 0 (src/ising_tsp.cu:155).
    float yr[CPT], xo[CPT];
#pragma unroll
    for (int j = 0; j < CPT; j++) {
        const int k = k0 + j;
        float x = 0.f, y = 0.f;
        if (real && k < N) {
            const int64_t gi = (int64_t)(i * N + k) * P.Ap + ag;
            x = St<T>::ld(xg[gi]);
            y = St<T>::ld(yg[gi]);
            y = rnd<T>(y + P.k2u * x);
            x = rnd<T>(x + P.k1u * y);
        }
        yr[j] = y;
        xo[j] = x;
    }
    // this thread's part of its row of X (and the halo copies of positions
    // 0 and N-1)
    auto put_row = [&]() {
        uint32_t w[CPT / 2];
#pragma unroll
        for (int c = 0; c < CPT / 2; c++)
            w[c] = (uint32_t)TT::bits(xo[2 * c]) | ((uint32_t)TT::bits(xo[2 * c + 1]) << 16);
        const int rows[3] = {(i + 1) * KA + a, i == 0 ? (N + 1) * KA + a : -1, i == N - 1 ? a : -1};
#pragma unroll
        for (int h = 0; h < 3; h++) {
            if (rows[h] < 0) continue;
#pragma unroll
            for (int c = 0; c < CPT / 8; c++)
                *(uint4 *)(xs + opoff(rows[h], k0 + 8 * c)) =
                    make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
        }
    };
    if (active) {
        put_row();
        if (hh == 0) prevbits[m] = 0xffffffffu;   // current_spins = -1
    }
    int stab = 0;
    bool bif = false, prv = false;
    if (real && i == 0 && hh == 0) {
        stab = P.stab[ag];
        bif = P.bif[ag];
        prv = P.prev[ag];
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_before();
    __syncthreads();
    tc_after();

    const uint32_t id = idesc<T>();
    const float qa8u = P.qa8 * P.dunscale;
    float i2r[CPT];   // the linear field of this thread's cities
#pragma unroll
    for (int j = 0; j < CPT; j++) i2r[j] = s_I2[k0 + j];
    // this thread's TMEM lane and its columns
    const uint32_t tlane = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + 128u * (uint32_t)tile + (uint32_t)k0;
    const int nwin = P.nwin;
    const uint32_t maskN = N == 32 ? 0xffffffffu : ((1u << N) - 1u);
    int k_step = 0;
    uint32_t phase = 0;
    bool failed = false;
    for (int wdx = 0; wdx < nwin && !failed; wdx++) {
        for (int it = 0; it < P.period; it++, k_step++) {
            const float2 sc = P.sched[k_step];
            // the distance product of the current X: 4 MMAs per tile (both
            // neighbour positions, two K halves), N = 96 covering the three
            // parts of D at once
            if (tid == 0) {
                for (int t = 0; t < T2; t++) {
                    uint32_t acc = 0;
#pragma unroll
                    for (int h = 0; h < 2; h++)
#pragma unroll
                        for (int s = 0; s < 2; s++) {
                            const uint32_t ao = xs0 + (uint32_t)((128 * t + 2 * KA * h) / 8 * SBO + 2 * LBO * s);
                            const uint32_t bo = ds0 + (uint32_t)(2 * LBO * s);
                            mma16(tmem + 128u * (uint32_t)t, sdesc(ao), sdesc(bo), id, acc);
                            acc = 1;
                        }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                             : "memory");
            }
            // meanwhile: the column sum of city i (part 0) and the row sum
            // (part 1 from the stored row, or part 0 alone from its
            // registers), each in the CUDA-core kernel's order
            float rs = 0.f;
            if (active) {
                if (hh == 0) {
                    float cs = 0.f;
#pragma unroll
                    for (int p = 0; p < NP; p++)
                        if (p < N) cs += TT::val(*(const unsigned short *)(xs + opoff((p + 1) * KA + a, i)));
                    colsum[m] = cs;
                    if (H == 1) {
#pragma unroll
                        for (int l = 0; l < NP; l++) rs += xo[l];
                    }
                } else if (hh == 1) {
                    const int r = (i + 1) * KA + a;
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        const uint4 v = *(const uint4 *)(xs + opoff(r, 8 * c));
                        const uint32_t u[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            rs += TT::val((unsigned short)(u[e] & 0xffffu));
                            rs += TT::val((unsigned short)(u[e] >> 16));
                        }
                    }
                    rsum[m] = rs;
                }
            }
            // the products are in TMEM once every thread's wait ends; the
            // barrier also publishes colsum and rsum and ends this step's
            // reads of X, so X may be rewritten after it
            const bool ok = mbar_wait_n(bar, phase, P.giveup ? 0u : kTcLimit);
            if (__syncthreads_or(!ok)) {
                // flag it, let the MMAs in flight finish (bounded), stop
                if (tid == 0) atomicExch(&P.ctl[CTL_ERR], 1);
                mbar_wait_n(bar, phase, kTcLimit);
                failed = true;
                break;
            }
            phase ^= 1u;
            tc_after();
            // the products with hi, mid and lo, summed (hi + mid) + lo
            float dk[CPT], dm[CPT], dl[CPT];
            tmem_ld<CPT>(tlane, dk);
            tmem_ld<CPT>(tlane + NP, dm);
            tmem_ld<CPT>(tlane + 2 * NP, dl);
#pragma unroll
            for (int j = 0; j < CPT; j++) dk[j] = (dk[j] + dm[j]) + dl[j];
            if (active) {
                if (H > 1) rs = rsum[m];
                // two cities at a time in packed FP32 (per component the
                // roundings of fmaf / __fmul_rn), both clamp branches
                // computed and selected; cities past N stay zero
                const float2 qc = make_float2(P.qc4, P.qc4), qb = make_float2(P.qb4, P.qb4);
                const float2 rs2 = make_float2(rs, rs);
                const float2 qa = make_float2(qa8u, qa8u), m1005 = make_float2(-1.005f, -1.005f);
                const float2 two = make_float2(2.f, 2.f), bt = make_float2(sc.x, sc.x);
                const float2 cxi = make_float2(P.dtxi0, P.dtxi0), cdt = make_float2(P.dt, P.dt);
                const float2 cy = make_float2(sc.y, sc.y);
#pragma unroll
                for (int j = 0; j < CPT; j += 2) {
                    const int k = k0 + j;
                    const float2 cs2 = make_float2(colsum[k * KA + a], colsum[(k + 1) * KA + a]);
                    // jx = (qc4 colsum + qb4 rs) + qa8u dk as the CUDA-core
                    // kernel contracts it; qa8u = A/8 times the FP16 operand
                    // scale 2^s (exact), so qa8u dk is A/8 (2^s dk) bit for bit
                    const float2 jx = __ffma2_rn(qa, make_float2(dk[j], dk[j + 1]),
                                                 __ffma2_rn(qb, rs2, __fmul2_rn(qc, cs2)));
                    const float2 i1 = __fmul2_rn(m1005, jx);
                    const float2 x0 = make_float2(xo[j], xo[j + 1]), y0 = make_float2(yr[j], yr[j + 1]);
                    float2 y = rnd2<T>(__ffma2_rn(cxi, __ffma2_rn(bt, make_float2(i2r[j], i2r[j + 1]),
                                                                   __fmul2_rn(two, i1)), y0));
                    const float2 x = rnd2<T>(__ffma2_rn(cdt, y, x0));
                    y = rnd2<T>(__ffma2_rn(cy, x, y));
                    const bool c0 = fabsf(x0.x) > 1.f, c1 = fabsf(x0.y) > 1.f;
                    if (k < N) {
                        xo[j] = c0 ? spin_of(x0.x) : x.x;
                        yr[j] = c0 ? 0.f : y.x;
                    }
                    if (k + 1 < N) {
                        xo[j + 1] = c1 ? spin_of(x0.y) : x.y;
                        yr[j + 1] = c1 ? 0.f : y.y;
                    }
                }
                put_row();
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc_before();
            __syncthreads();
            tc_after();
        }
        if (failed) break;
        // Window: validity (one +1 per city and per position), stability,
        // tour snapshot of valid agents (src/kernels.cu:473-531); each part
        // stores its cities' sign bits, part 0 of the row decides.
        uint32_t part = 0;
        if (active) {
#pragma unroll
            for (int j = 0; j < CPT; j++)
                if (k0 + j < N) part |= sbit(xo[j]) << j;
            if (H == 1) rowbits[m] = part;
            else if (H == 2) ((unsigned short *)rowbits)[2 * m + hh] = (unsigned short)part;
            else ((unsigned char *)rowbits)[4 * m + hh] = (unsigned char)part;
        }
        if (tid < 2 * KA) aflag[tid] = tid < KA ? 1 : 0;
        __syncthreads();
        const uint32_t bits = active ? rowbits[m] : 0u;
        if (active && hh == 0) {
            const int order_cnt = __popc(~bits & maskN);
            int city_cnt = 0;
            for (int p = 0; p < N; p++) city_cnt += (~rowbits[p * KA + a] >> i) & 1u;
            if (order_cnt != 1 || city_cnt != 1) atomicAnd(&aflag[a], 0);
            if (bits != (prevbits[m] & maskN)) atomicOr(&aflag[KA + a], 1);
        }
        __syncthreads();
        if (active && hh == 0) {
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
            prevbits[m] = bits;
        }
        __syncthreads();
    }

    // State back to global memory (get_state) and the window spins.
    if (real) {
#pragma unroll
        for (int j = 0; j < CPT; j++) {
            const int k = k0 + j;
            if (k < N) {
                const int64_t gi = (int64_t)(i * N + k) * P.Ap + ag;
                xg[gi] = St<T>::st(xo[j]);
                yg[gi] = St<T>::st(yr[j]);
            }
        }
        const uint32_t bits = prevbits[m];
        for (int k = k0; k < k0 + CPT && k < N; k++) {
            const int64_t r = i * N + k;
            const uint32_t bit = (bits >> k) & 1u;
            uint32_t *p = &P.Wp[r * P.W + (ag >> 5)];
            if (bit) atomicOr(p, 1u << (ag & 31));
            else atomicAnd(p, ~(1u << (ag & 31)));
        }
        if (i == 0 && hh == 0) {
            P.stab[ag] = stab;
            P.bif[ag] = bif;
            P.prev[ag] = prv;
        }
    }
    if (blockIdx.x == 0 && tid == 0 && !failed) {
        P.ctl[CTL_STEP] = k_step;
        P.ctl[CTL_WINDOWS] = nwin;
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

template <class T>
cudaError_t launch_h(int H, const cudaLaunchConfig_t &cfg0, const TcP &P)
{
    cudaLaunchConfig_t cfg = cfg0;
    cfg.blockDim = dim3(128 * P.tiles * H);
    if (H == 4) return cudaLaunchKernelEx(&cfg, k_tsp_tc<T, 4>, P);
    if (H == 2) return cudaLaunchKernelEx(&cfg, k_tsp_tc<T, 2>, P);
    return cudaLaunchKernelEx(&cfg, k_tsp_tc<T, 1>, P);
}

}  // namespace

int tsp_tensor_threads_per_row(int requested)
{
    // 4 measured fastest on GB300 (TSP-30, 1024 agents: 3.3 us a step against
    // 3.8 with 2 and 5.3 with 1)
    return requested == 1 || requested == 2 || requested == 4 ? requested : 4;
}

bool tsp_tensor_fits(const SolveDims &d, const DevTsp &t)
{
    return (d.prec == P_BF16 || d.prec == P_F16) && t.N >= 3 && t.N <= NP;
}

cudaError_t launch_tsp_tensor(const SolveDims &d, const DevTsp &t, Work &w, int threads_per_row, cudaStream_t s)
{
    if (!tsp_tensor_fits(d, t)) return cudaErrorInvalidValue;
    TcP P;
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
    P.tiles = (t.N * KA + 127) / 128;
    P.giveup = d.giveup;
    P.qa8 = (float)(t.A / 8);
    P.qb4 = (float)(t.B / 4);
    P.qc4 = (float)(t.C / 4);
    P.dtxi0 = (float)(d.dt * 0.002);
    P.dt = (float)d.dt;
    const double p0 = 1.025 * 0.0 / d.steps;   // Update_XY pressure at step 0
    P.k1u = (float)(d.dt * (p0 + 1));
    P.k2u = (float)(d.dt * (p0 - 1));
    // FP16 operands: D scaled by a power of two so its largest entry lies in
    // [2^13, 2^14) (exact; the product is scaled back); BF16 has FP32's range
    int e = 0;
    if (d.prec == P_F16) {
        double mx = 0;
        for (double v : t.packed) mx = v > mx ? v : mx;
        if (mx > 0) {
            std::frexp(mx, &e);   // mx = f * 2^e, f in [0.5, 1)
            e -= 14;
        }
    }
    P.dscale = (float)std::ldexp(1.0, -e);
    P.dunscale = (float)std::ldexp(1.0, e);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)((d.A + KA - 1) / KA));
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = d.pdl ? 1 : 0;
    // threads per row: the CUDA-core share of a step splits over them
    const int H = tsp_tensor_threads_per_row(threads_per_row);
    if (d.prec == P_BF16) return launch_h<__nv_bfloat16>(H, cfg, P);
    return launch_h<__half>(H, cfg, P);
}

}  // namespace sbx
