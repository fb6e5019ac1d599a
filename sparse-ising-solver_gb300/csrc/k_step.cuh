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
    int32_t *hcount;                      // [first chunk][segment]: chunks of a heavy row done
    const int32_t *__restrict__ order;    // rows in decreasing degree (or null: natural order)
    int64_t row0;                         // first entry of order the row items visit
    const float *__restrict__ c0r32;      // batched: dt*xi0 per row (else null)
    const double *__restrict__ c0r64;
    int64_t n;
    int32_t W, Ap, nchunks;
    uint32_t zrow;                        // n: the sign planes' all-zero row (column of no neighbour)
    int32_t stream_state;                 // state larger than L2: x, y loads/stores evict first
    int32_t allpos;                       // every weight is +1: no sign bits in colw
    int32_t bits_min;                     // heavy-row kernels: light rows of this degree or more
                                          // are counted in bit planes (INT32_MAX: none)
    int64_t niso;                         // isolated rows left to k_iso: the last niso entries of
                                          // order, which the row items then skip
    double c0;
    int32_t giveup;                       // test only: the staged-row wait gives up at once
};

// One step kernel launch (kind K_*, window step or not) in the precision of
// d.prec; one definition per precision (k_step_<prec>.cu).
cudaError_t step_f32(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win, int offset, cudaStream_t s);
cudaError_t step_bf16(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win, int offset, cudaStream_t s);
cudaError_t step_f16(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win, int offset, cudaStream_t s);
cudaError_t step_f64(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win, int offset, cudaStream_t s);
// One window of fused steps (d.period) of the isolated rows (k_iso).
cudaError_t iso_f32(const SolveDims &d, const DevCsr &J, const StepP &P, cudaStream_t s);
cudaError_t iso_bf16(const SolveDims &d, const DevCsr &J, const StepP &P, cudaStream_t s);
cudaError_t iso_f16(const SolveDims &d, const DevCsr &J, const StepP &P, cudaStream_t s);
cudaError_t iso_f64(const SolveDims &d, const DevCsr &J, const StepP &P, cudaStream_t s);

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
// State passes that do not fit in L2 stream through it: loads and stores
// marked evict-first keep the sign planes (the gathered data) resident.
template <class T, int V> __device__ __forceinline__ Raw<V * sizeof(T)> vload_s(const T *p, bool cs)
{
    Raw<V * sizeof(T)> r;
    if (cs) r.u = __ldcs((const decltype(r.u) *)p);
    else r.u = *(const decltype(r.u) *)p;
    return r;
}
template <class U> __device__ __forceinline__ void vstore_s(void *p, const U &u, bool cs)
{
    if (cs) __stcs((U *)p, u);
    else *(U *)p = u;
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

// Bulk asynchronous copies global -> shared with an mbarrier (sm_90+ PTX).
// Addresses 16-byte aligned, sizes multiples of 16 (the callers' segments are
// 32 agents x 16 bytes per lane row pieces).
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// Bounded wait for phase `parity` of the barrier: false when it did not
// complete within `limit` checks (the caller flags the error).
constexpr uint32_t kMbarLimit = 1u << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit = kMbarLimit)
{
    for (uint32_t k = 0; k < limit; k++) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(smem_u32(bar)), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}

// x + a*b: one FMA in FP32; in FP64 two separately rounded operations, the
// reference's arithmetic as the oracle states it.
__device__ __forceinline__ float madd(float a, float b, float x) { return fmaf(a, b, x); }
__device__ __forceinline__ double madd(double a, double b, double x) { return __dadd_rn(x, __dmul_rn(a, b)); }

// Word of a sign-plane row: row col, word offset already in Sq.  The byte
// offset is a 32 x 32 -> 64-bit product (col * 4W), one widening multiply-add
// with the base.
__device__ __forceinline__ uint32_t plane_ld(const uint32_t *Sq, uint32_t col, int32_t W)
{
    const uint32_t wb = (uint32_t)W * 4u;
    return __ldg((const uint32_t *)((const char *)Sq + (uint64_t)col * (uint64_t)wb));
}

// Full adder over 32 bit lanes: a + b + e -> sum into a, carry returned.
__device__ __forceinline__ uint32_t fadd(uint32_t &a, uint32_t b, uint32_t e)
{
    const uint32_t c = (a & b) | (e & (a ^ b));
    a = a ^ b ^ e;
    return c;
}

// Twice the sign bits of a nibble, one per byte: byte i of the result is
// 2 * bit i.  Byte counters of +-1 neighbours then hold 2 * count (<= 254 for
// up to kHeavy = 127 neighbours).
__device__ __forceinline__ uint32_t spread2x(uint32_t nib) { return (nib * 0x00408102u) & 0x02020202u; }

// Walk m neighbours (+-1 weights) of one row starting at CSR entry e0, all 32
// lanes of the warp together: lane l reads the sign word of its V agents in
// each neighbour's row of the plane and adds 2 * (bit ^ weight sign) into
// byte counters lo (agents 0..3) / hi (4..7).  Counts agents whose neighbour
// term is -1: the force is 2 * count - degree (src/kernels.cu:247-255).
template <int V, int LR, bool NEG>
__device__ __forceinline__ void count_unit_s(const StepP &P, const uint32_t *Sq, int off, int32_t e0,
                                             int32_t dw, int sl, uint32_t &lo, uint32_t &hi)
{
    int32_t dmax = dw;
    if constexpr (LR < 32) dmax = __reduce_max_sync(FULL, dw);
    const uint32_t *cwp = P.colw + e0 + sl;   // this lane's column words, from one base
    for (int32_t cb = 0; cb < dmax; cb += LR) {
        const int m = min(LR, dmax - cb);
        const int32_t idx = cb + sl;
        // past the row's end: the all-zero row, whose terms vanish
        const uint32_t mycw = idx < dw ? __ldg(cwp + cb) : P.zrow;
#pragma unroll 4
        for (int k = 0; k < m; k++) {
            const uint32_t cw = __shfl_sync(FULL, mycw, k, LR);
            // all weights +1: bit 31 is clear, no sign to apply
            const uint32_t word = plane_ld(Sq, NEG ? (cw & 0x7fffffffu) : cw, P.W);
            // weight sign -> all-ones mask; unused high bits only reach
            // counter bytes that are never read
            uint32_t bits = word >> off;
            if (NEG) bits ^= (uint32_t)((int32_t)cw >> 31);
            lo += spread2x(bits & 0xfu);
            if (V == 8) hi += spread2x((bits >> 4) & 0xfu);
        }
    }
}
template <int V, int LR>
__device__ __forceinline__ void count_unit(const StepP &P, const uint32_t *Sq, int off, int32_t e0,
                                           int32_t dw, int sl, uint32_t &lo, uint32_t &hi)
{
    if (P.allpos) count_unit_s<V, LR, false>(P, Sq, off, e0, dw, sl, lo, hi);
    else count_unit_s<V, LR, true>(P, Sq, off, e0, dw, sl, lo, hi);
}

// Bit-sliced counting of the same quantity for rows with many neighbours:
// the G = 32/V lanes sharing a sign word split the row's neighbours (lane j
// of the group takes every G-th); each adds whole 32-agent words (bit ^
// weight sign) into bit planes -- bit a of plane i is bit i of agent a's
// count -- with a ripple of two logic operations per plane.  The planes are
// then summed across the group (butterfly of shuffles and bit-sliced adds)
// and each lane takes out its V agents as byte counters holding 2 * count,
// the form count_unit leaves.  Counts stay below 128 (kHeavy = 127).
template <int V, int LR, bool NEG>
__device__ __forceinline__ void count_bits_s(const StepP &P, const uint32_t *Sq, int off, int32_t e0,
                                             int32_t dw, int sl, uint32_t &lo, uint32_t &hi)
{
    constexpr int G = 32 / V;
    static_assert(LR % G == 0, "a row's lanes hold whole words");
    // planes one lane needs for ceil(127 / G) neighbours; 7 after the sum
    constexpr int BL = G == 4 ? 6 : G == 8 ? 5 : G == 16 ? 4 : 3;
    constexpr int NP = 7;
    const int j = sl & (G - 1);
    uint32_t p[NP];
#pragma unroll
    for (int i = 0; i < NP; i++) p[i] = 0;
    int32_t dmax = dw;
    if constexpr (LR < 32) dmax = __reduce_max_sync(FULL, dw);
    // Blocks of 32 neighbours: the row's lanes load 32/LR column words each,
    // every lane issues its 32/G sign-word loads, then adds them -- one
    // memory latency per block.  Sub-blocks past the longest row of the
    // warp are skipped (warp-uniform).
    constexpr int T = 32 / LR;     // column words per lane per block
    constexpr int KPL = LR / G;    // neighbours per lane per column word
    const uint32_t *cwp = P.colw + e0 + sl;   // this lane's column words, from one base
    for (int32_t cb = 0; cb < dmax; cb += 32) {
        // past a row's end: the zero row (word 0, weight sign clear), so
        // those terms vanish without a test per word
        uint32_t mycw[T];
#pragma unroll
        for (int t = 0; t < T; t++) {
            const int32_t idx = cb + t * LR + sl;
            mycw[t] = idx < dw ? __ldg(cwp + cb + t * LR) : P.zrow;
        }
        uint32_t w[T * KPL];
#pragma unroll
        for (int t = 0; t < T; t++) {
#pragma unroll
            for (int kk = 0; kk < KPL; kk++) {
                const int src = kk * G + j;
                const uint32_t cw = __shfl_sync(FULL, mycw[t], src, LR);
                w[t * KPL + kk] = 0u;
                if (cb + t * LR < dmax) {
                    const uint32_t word = plane_ld(Sq, NEG ? (cw & 0x7fffffffu) : cw, P.W);
                    w[t * KPL + kk] = NEG ? word ^ (uint32_t)((int32_t)cw >> 31) : word;
                }
            }
        }
        static_assert(T * KPL == V, "V words per lane per block");
        if constexpr (V >= 4) {
            // carry-save tree: the block's V words (zero past the rows'
            // ends) meet the planes in full adders, level by level, and
            // only the top carry ripples
            uint32_t c2[V / 4], c4;
#pragma unroll
            for (int h = 0; h < V / 4; h++) {
                uint32_t c1[2];
#pragma unroll
                for (int i = 0; i < 2; i++)
                    c1[i] = fadd(p[0], w[4 * h + 2 * i], w[4 * h + 2 * i + 1]);
                c2[h] = fadd(p[1], c1[0], c1[1]);
            }
            int k0;
            if constexpr (V == 8) {
                c4 = fadd(p[2], c2[0], c2[1]);
                k0 = 3;
            } else {
                c4 = c2[0];
                k0 = 2;
            }
#pragma unroll
            for (int k = k0; k < BL; k++) {
                const uint32_t t = p[k] & c4;
                p[k] ^= c4;
                c4 = t;
            }
        } else {
            // pairs of words through a full adder into plane 0, the carry
            // rippling up the planes
#pragma unroll
            for (int i = 0; i < T * KPL; i += 2) {
                if (cb + (i / KPL) * LR >= dmax) break;   // warp-uniform
                uint32_t c;
                if (i + 1 < T * KPL) {
                    c = fadd(p[0], w[i], w[i + 1]);
                } else {
                    c = p[0] & w[i];
                    p[0] ^= w[i];
                }
#pragma unroll
                for (int k = 1; k < BL; k++) {
                    const uint32_t t = p[k] & c;
                    p[k] ^= c;
                    c = t;
                }
            }
        }
    }
    // sum over the group: planes grow by one per round, capped at 7
#pragma unroll
    for (int s = 1, np = BL; s < G; s <<= 1, np = np + 1 < NP ? np + 1 : NP) {
        uint32_t c = 0;
#pragma unroll
        for (int i = 0; i < NP; i++) {
            if (i <= np) {
                const uint32_t a = p[i], b = __shfl_xor_sync(FULL, p[i], s);
                p[i] = a ^ b ^ c;
                c = (a & b) | (c & (a ^ b));
            }
        }
    }
    if constexpr (V == 8) {
        // this lane's byte of every plane, gathered into 64 bits (byte i =
        // plane i), then an 8x8 bit transpose: byte k = agent k's count
        static_assert(NP <= 8, "planes fit the 8x8 block");
        const uint32_t sel = (uint32_t)off >> 3;
        const uint32_t s01 = sel | ((sel + 4) << 4);
        const uint32_t g0 = __byte_perm(__byte_perm(p[0], p[1], s01), __byte_perm(p[2], p[3], s01), 0x5410);
        const uint32_t g1 = __byte_perm(__byte_perm(p[4], p[5], s01), __byte_perm(p[6], 0u, sel | 0x4440u), 0x5410);
        uint64_t x = ((uint64_t)g1 << 32) | g0;
        uint64_t t;
        t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull;
        x ^= t ^ (t << 7);
        t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull;
        x ^= t ^ (t << 14);
        t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull;
        x ^= t ^ (t << 28);
        // counts < 128: doubling stays inside each byte
        lo += (uint32_t)x << 1;
        hi += (uint32_t)(x >> 32) << 1;
    } else {
        // this lane's V agents: bit k of plane i -> 2^(i+1) in byte k
#pragma unroll
        for (int i = 0; i < NP; i++) {
            const uint32_t b = p[i] >> off;
            lo += ((b & 0xfu) * (0x00204081u << (i + 1))) & (0x01010101u << (i + 1));
        }
    }
}
template <int V, int LR>
__device__ __forceinline__ void count_bits(const StepP &P, const uint32_t *Sq, int off, int32_t e0,
                                           int32_t dw, int sl, uint32_t &lo, uint32_t &hi)
{
    if (P.allpos) count_bits_s<V, LR, false>(P, Sq, off, e0, dw, sl, lo, hi);
    else count_bits_s<V, LR, true>(P, Sq, off, e0, dw, sl, lo, hi);
}

// The SB update of V agents from their totals (the force sum_j J_ij s_j):
// src/kernels.cu:236-262 in the fused mode -- clamp or kick, then the drift /
// kick pair that runs unconditionally, so a clamped oscillator leaves with
// y = dt (p-1) sign(x) -- or the unfused trio's mat_mult (:207) and confine
// (:158-165), then Update_XY of the next step unless the window closes.
// FP32 pairs go through the packed FMA (per component the same rounding as
// fmaf); FP64 keeps separately rounded operations.
template <int KIND, bool WIN, int V, class C4>
__device__ __forceinline__ void sb_update(float (&x)[V], float (&y)[V], const float (&tv)[V], float c0,
                                          const C4 &c, const C4 &cn)
{
    if constexpr (V % 2 == 0) {
        const float2 c02 = make_float2(c0, c0);
#pragma unroll
        for (int i = 0; i < V; i += 2) {
            float2 X = make_float2(x[i], x[i + 1]), Y = make_float2(y[i], y[i + 1]);
            const float2 K = __ffma2_rn(c02, make_float2(tv[i], tv[i + 1]), Y);
            const bool k0 = fabsf(X.x) > 1.0f, k1 = fabsf(X.y) > 1.0f;
            Y.x = k0 ? 0.0f : K.x;
            Y.y = k1 ? 0.0f : K.y;
            X.x = k0 ? spin_of(X.x) : X.x;
            X.y = k1 ? spin_of(X.y) : X.y;
            if (KIND == K_FUSED) {
                X = __ffma2_rn(make_float2(c.x, c.x), Y, X);
                Y = __ffma2_rn(make_float2(c.y, c.y), X, Y);
            } else if (!WIN) {
                Y = __ffma2_rn(make_float2(cn.w, cn.w), X, Y);
                X = __ffma2_rn(make_float2(cn.z, cn.z), Y, X);
            }
            x[i] = X.x;
            x[i + 1] = X.y;
            y[i] = Y.x;
            y[i + 1] = Y.y;
        }
    } else {
#pragma unroll
        for (int v = 0; v < V; v++) {
            const bool clamp = fabsf(x[v]) > 1.0f;
            const float xc = spin_of(x[v]);
            y[v] = clamp ? 0.0f : fmaf(c0, tv[v], y[v]);
            x[v] = clamp ? xc : x[v];
            if (KIND == K_FUSED) {
                x[v] = fmaf(c.x, y[v], x[v]);
                y[v] = fmaf(c.y, x[v], y[v]);
            } else if (!WIN) {
                y[v] = fmaf(cn.w, x[v], y[v]);
                x[v] = fmaf(cn.z, y[v], x[v]);
            }
        }
    }
}
template <int KIND, bool WIN, int V, class C4>
__device__ __forceinline__ void sb_update(double (&x)[V], double (&y)[V], const double (&tv)[V], double c0,
                                          const C4 &c, const C4 &cn)
{
#pragma unroll
    for (int v = 0; v < V; v++) {
        const bool clamp = fabs(x[v]) > 1.0;
        const double xc = spin_of(x[v]);
        y[v] = clamp ? 0.0 : madd(c0, tv[v], y[v]);
        x[v] = clamp ? xc : x[v];
        if (KIND == K_FUSED) {
            x[v] = madd(c.x, y[v], x[v]);
            y[v] = madd(c.y, x[v], y[v]);
        } else if (!WIN) {
            y[v] = madd(cn.w, x[v], y[v]);
            x[v] = madd(cn.z, y[v], x[v]);
        }
    }
}

// One SB step over every (row, agent).  Work item = (group of 32/LR rows,
// segment of LR*V agents); lane l of a row owns V consecutive agents (one
// vector load of x and of y).  Per neighbour j the lane reads the sign word
// of its agents in row j of the plane (lanes of one word share the address)
// and counts into byte counters (count_unit, CM = 0) or bit planes
// (count_bits, CM = 1); the new signs of the V agents are OR-combined across
// the lanes of a word and written once.
//
// Heavy rows (BIG kernels: +-1 weights, degree > kHeavy) come first, as
// items of kHeavy neighbours: each leaves its byte counters in P.part, and
// the warp completing a row's last chunk (a per-row counter, re-armed by that
// warp) sums them and updates the row.  The other rows follow, in decreasing
// degree when P.order is set; in a BIG byte-counter kernel those of
// P.bits_min or more neighbours are counted in bit planes (mixed mode).
// Isolated rows (the last P.niso entries of the order) are left to k_iso.
// Resident CTAs per SM asked of the register allocator (measured on GB300):
// 4 for bit-plane counting without heavy rows (its loads in flight need
// registers), 5 otherwise (heavy-row kernels: 6 spilled more and ran 2%
// slower on R-MAT 2^20, 7 ran 11% slower).
template <class T, int V, int KIND, bool WIN, int WM, bool BIG, int LR, int CM, int ST>
__global__ void __launch_bounds__(256, (CM && !BIG) ? 4 : 5) k_row(const StepP P, const int offset)
{
    static_assert(LR == 32 || !BIG, "heavy rows are counted by whole warps");
    static_assert(!ST || (LR == 32 && !WIN && KIND != K_XY), "staged rows: whole-warp rows, plain steps");
    static_assert(LR * V >= 32, "a sign word belongs to one row's lanes");
    using A = typename St<T>::A;
    using R = typename std::conditional<WM == W_F64, double, float>::type;
    using RawT = Raw<V * sizeof(T)>;
    // window steps: [W] changed bits of this block; staged steps: the warps'
    // x, y stages
    extern __shared__ __align__(16) uint32_t s_chg[];
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
    const bool cs = P.stream_state != 0;
    // coefficients of this step and of the next (the unfused mode's
    // Update_XY), loop-invariant
    const auto c = Coef<A>::get(P, step);
    const auto cn = Coef<A>::get(P, step + 1);
    uint32_t *Scur = (step & 1) ? P.S1 : P.S0;
    uint32_t *Snext = (step & 1) ? P.S0 : P.S1;
    constexpr int G = 32 / V;   // lanes sharing one sign word
    constexpr int RW = 32 / LR; // rows per warp
    constexpr uint32_t VM = (V == 32) ? 0xffffffffu : ((1u << V) - 1u);
    const int rw = lane / LR, sl = lane & (LR - 1);   // row of the warp, lane of the row
    const int nit = P.Ap / (LR * V);                  // segments per row (1 when LR < 32)
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t w0 = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);

    // The item's update from the totals tv of its agents; x, y stored, the
    // new sign word written (and compared with the previous window's).
    auto finish = [&](int64_t r, int q, int off, int64_t base, bool live, const RawT &xr, const RawT &yr,
                      const A (&tv)[V], A c0, uint32_t wp_old) {
        A x[V], y[V];
        to_vals<T, V>(xr, x);
        to_vals<T, V>(yr, y);
        if (KIND == K_XY) {
            // Update_XY, src/kernels.cu:8-22 (pressure not clamped)
#pragma unroll
            for (int v = 0; v < V; v++) {
                y[v] = madd((A)c.w, x[v], y[v]);
                x[v] = madd((A)c.z, y[v], x[v]);
            }
        } else {
            sb_update<KIND, WIN, V>(x, y, tv, c0, c, cn);
        }
        // signs of the new x (rounding to the storage type keeps the sign)
        uint32_t b = 0;
#pragma unroll
        for (int v = 0; v < V; v++) b |= sbit(x[v]) << v;
        const auto xw = from_vals<T, V>(x);
        const auto yw = from_vals<T, V>(y);
        if (live) {
            vstore_s(xp + base, xw.u, cs);
            vstore_s(yp + base, yw.u, cs);
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
    };
    // dt * xi0 of the row's instance (batched) or of the problem
    auto row_c0 = [&](int64_t r) -> A {
        if (P.c0r32) return std::is_same<A, double>::value ? (A)__ldg(&P.c0r64[r]) : (A)__ldg(&P.c0r32[r]);
        return (A)P.c0;
    };

    if constexpr (BIG) {
        const int64_t hitems = (int64_t)P.nchunks * nit;
        for (int64_t item = w0; item < hitems; item += nw) {
            const int ci = (int)(item / nit), it = (int)(item - (int64_t)ci * nit);
            const int64_t r = __ldg(&P.chunk_row[ci]);
            const int32_t h0 = __ldg(&P.hchunk[r]);
            const int32_t rb = __ldg(&P.rowptr[r]), re = __ldg(&P.rowptr[r + 1]);
            const int32_t e0 = rb + (ci - h0) * kHeavy;
            const int a0 = it * 32 * V + lane * V;
            const int q = a0 >> 5, off = a0 & 31;
            uint32_t lo = 0, hi = 0;
            count_bits<V, 32>(P, Scur + q, off, e0, min(re - e0, (int32_t)kHeavy), lane, lo, hi);
            P.part[item * 32 + lane] = make_uint2(lo, hi);
            // publish the partial, then count the row's finished chunks
            __threadfence();
            const int deg = re - rb, nc = (deg + kHeavy - 1) / kHeavy;
            int last = 0;
            if (lane == 0) last = atomicAdd(&P.hcount[(int64_t)h0 * nit + it], 1) == nc - 1;
            if (!__shfl_sync(FULL, last, 0)) continue;   // warp-uniform
            __threadfence();
            if (lane == 0) P.hcount[(int64_t)h0 * nit + it] = 0;   // armed for the next step
            int s[V];
#pragma unroll
            for (int v = 0; v < V; v++) s[v] = 0;
            for (int cc = 0; cc < nc; cc++) {
                const uint2 pr = __ldcg(&P.part[((int64_t)(h0 + cc) * nit + it) * 32 + lane]);
#pragma unroll
                for (int v = 0; v < V; v++) s[v] += ((v < 4 ? pr.x : pr.y) >> (8 * (v & 3))) & 0xffu;
            }
            A tv[V];
#pragma unroll
            for (int v = 0; v < V; v++) tv[v] = (A)(s[v] - deg);
            const int64_t base = r * P.Ap + a0;
            uint32_t wp_old = 0;
            if (WIN && (lane & (G - 1)) == 0) wp_old = P.Wp[r * P.W + q];
            const RawT xr = vload_s<T, V>(xp + base, cs);
            const RawT yr = vload_s<T, V>(yp + base, cs);
            finish(r, q, off, base, true, xr, yr, tv, row_c0(r), wp_old);
        }
    }

    // Row items (group g, segment it) in steps of the warp count, advanced
    // without divisions: g += nw / nit, it += nw % nit with carry.
    const int64_t nrows = P.n - P.row0 - P.niso;
    const int64_t ng = (nrows + RW - 1) / RW;
    const int64_t dr = nw / nit;
    const int dit = (int)(nw - dr * nit);
    // Totals (the force sum_j J_ij s_j) of the item's V agents of row r.
    auto item_totals = [&](int64_t r, int q, int off, A (&tv)[V]) {
        if (KIND != K_XY) {
            const int32_t e0 = __ldg(&P.rowptr[r]), e1 = __ldg(&P.rowptr[r + 1]);
            const int32_t deg = e1 - e0;
            if (WM == W_UNIT) {
                uint32_t lo = 0, hi = 0;
                if (CM) {
                    count_bits<V, LR>(P, Scur + q, off, e0, deg, sl, lo, hi);
                } else if constexpr (BIG) {
                    // one row per warp: the choice is warp-uniform
                    if (deg >= P.bits_min) count_bits<V, LR>(P, Scur + q, off, e0, deg, sl, lo, hi);
                    else count_unit<V, LR>(P, Scur + q, off, e0, deg, sl, lo, hi);
                } else {
                    count_unit<V, LR>(P, Scur + q, off, e0, deg, sl, lo, hi);
                }
                if constexpr (std::is_same<A, float>::value) {
                    // PRMT builds the float 2^23 + 2*count from a byte
                    // counter; minus (2^23 + deg) it is 2*count - deg exactly
                    const float bias = 8388608.0f + (float)deg;
#pragma unroll
                    for (int v = 0; v < V; v++)
                        tv[v] = __uint_as_float(__byte_perm(v < 4 ? lo : hi, 0x4b000000u, 0x7440u + (v & 3))) - bias;
                } else {
#pragma unroll
                    for (int v = 0; v < V; v++)
                        tv[v] = (A)((int)(((v < 4 ? lo : hi) >> (8 * (v & 3))) & 0xffu) - deg);
                }
            } else {
                R tot[V];
#pragma unroll
                for (int v = 0; v < V; v++) tot[v] = R(0);
                int32_t dmax = deg;
                if constexpr (LR < 32) dmax = __reduce_max_sync(FULL, deg);
                const uint32_t *Sq = Scur + q;
                for (int32_t cb = 0; cb < dmax; cb += LR) {
                    const int m = min(LR, dmax - cb);
                    const int32_t idx = cb + sl;
                    const uint32_t mycw = idx < deg ? __ldg(&P.colw[e0 + idx]) : 0u;
                    R myv = R(0);
                    if (WM == W_F32) myv = idx < deg ? __ldg(&P.valf[e0 + idx]) : 0.f;
                    if (WM == W_F64) myv = idx < deg ? __ldg(&P.vald[e0 + idx]) : 0.0;
#pragma unroll 4
                    for (int k = 0; k < m; k++) {
                        const uint32_t cw = __shfl_sync(FULL, mycw, k, LR);
                        const R wv = __shfl_sync(FULL, myv, k, LR);
                        if (LR == 32 || cb + k < deg) {
                            const uint32_t word = plane_ld(Sq, cw & 0x7fffffffu, P.W);
                            const uint32_t bits = (word >> off) & VM;
#pragma unroll
                            for (int v = 0; v < V; v++) {
                                const R sv = ((bits >> v) & 1u) ? R(-1) : R(1);
                                if (WM == W_F64) tot[v] = sub(tot[v], mul(wv, sv));
                                else tot[v] -= wv * sv;
                            }
                        }
                    }
                }
#pragma unroll
                for (int v = 0; v < V; v++) tv[v] = (A)tot[v];
            }
        }
    };

    if constexpr (ST) {
        // Staged rows (state larger than L2): each warp copies the x, y
        // segments of its next item into shared memory (bulk asynchronous
        // copies completing on an mbarrier) while it works on the current
        // one, so the state's DRAM latency is off the item's critical path.
        constexpr int SEGB = 32 * V * (int)sizeof(T);
        static_assert(SEGB % 16 == 0, "bulk copies move 16-byte multiples");
        __shared__ __align__(8) uint64_t s_bar[8][2];   // 256-thread blocks at most
        const int wid = threadIdx.x >> 5;
        unsigned char *stg = (unsigned char *)s_chg + (size_t)wid * 4 * SEGB;
        if (lane == 0) {
            mbar_init(&s_bar[wid][0], 1);
            mbar_init(&s_bar[wid][1], 1);
            mbar_fence_init();
        }
        __syncwarp();
        auto row_of = [&](int64_t gg) -> int64_t {
            const int64_t ri = P.row0 + gg;
            return P.order ? (int64_t)__ldg(&P.order[ri]) : ri;
        };
        auto issue = [&](int stage, int64_t rr, int itx) {
            if (lane == 0) {
                const int64_t e = rr * P.Ap + (int64_t)itx * 32 * V;
                mbar_expect_tx(&s_bar[wid][stage], 2 * SEGB);
                bulk_g2s(stg + stage * 2 * SEGB, xp + e, SEGB, &s_bar[wid][stage]);
                bulk_g2s(stg + stage * 2 * SEGB + SEGB, yp + e, SEGB, &s_bar[wid][stage]);
            }
        };
        int64_t g = w0 / nit;
        int it = (int)(w0 - g * nit);
        int64_t r = 0;
        if (g < ng) {
            r = row_of(g);
            issue(0, r, it);
        }
        uint32_t j = 0;
        while (g < ng) {
            int64_t gn = g + dr;
            int itn = it + dit;
            if (itn >= nit) {
                itn -= nit;
                gn++;
            }
            const int64_t rn = gn < ng ? row_of(gn) : 0;
            if (gn < ng) issue((j + 1) & 1, rn, itn);
            if (!mbar_wait(&s_bar[wid][j & 1], (j >> 1) & 1, P.giveup ? 0u : kMbarLimit)) {
                // never expected: flag it, let the copies in flight (this
                // stage's and the next one's) land, within the limit, stop
                if (lane == 0) atomicExch(&P.ctl[CTL_ERR], 1);
                mbar_wait(&s_bar[wid][j & 1], (j >> 1) & 1);
                if (gn < ng) mbar_wait(&s_bar[wid][(j + 1) & 1], ((j + 1) >> 1) & 1);
                break;
            }
            const int a0 = it * 32 * V + lane * V;
            const int q = a0 >> 5, off = a0 & 31;
            const unsigned char *sx = stg + (j & 1) * 2 * SEGB + lane * V * (int)sizeof(T);
            RawT xr, yr;
            xr.u = *(const decltype(xr.u) *)sx;
            yr.u = *(const decltype(yr.u) *)(sx + SEGB);
            A tv[V];
            item_totals(r, q, off, tv);
            finish(r, q, off, r * P.Ap + a0, true, xr, yr, tv, row_c0(r), 0u);
            __syncwarp();   // this stage is free for the copy two items on
            g = gn;
            it = itn;
            r = rn;
            j++;
        }
    } else {
    // 32-bit row arithmetic (rows < 2^31); 64-bit only for state offsets
    const int32_t nr32 = (int32_t)nrows, ng32 = (int32_t)ng, dr32 = (int32_t)dr, row0 = (int32_t)P.row0;
    int32_t g = (int32_t)(w0 / nit);
    int it = (int)(w0 - (int64_t)g * nit);
    for (; g < ng32; g += dr32, it += dit) {
        if (it >= nit) {
            it -= nit;
            g++;
            if (g >= ng32) break;
        }
        // lanes of a group past the last row repeat the last row, store nothing
        const int32_t gi = g * RW + rw;
        const bool live = RW == 1 || gi < nr32;
        const int32_t ri = row0 + (live ? gi : nr32 - 1);
        const int32_t r = P.order ? __ldg(&P.order[ri]) : ri;
        const int a0 = it * LR * V + sl * V;
        const int q = a0 >> 5, off = a0 & 31;
        const int64_t base = (int64_t)r * P.Ap + a0;
        uint32_t wp_old = 0;   // window steps: the previous window's word, fetched early
        if (WIN && (lane & (G - 1)) == 0) wp_old = P.Wp[(int64_t)r * P.W + q];
        RawT xr, yr;
        A tv[V];
        bool wide = false;   // mixed mode: a bit-plane row (warp-uniform)
        if constexpr (BIG && !CM && KIND != K_XY) wide = __ldg(&P.rowptr[r + 1]) - __ldg(&P.rowptr[r]) >= P.bits_min;
        if (wide) {
            // x, y fetched after the count: the planes need the registers
            item_totals(r, q, off, tv);
            xr = vload_s<T, V>(xp + base, cs);
            yr = vload_s<T, V>(yp + base, cs);
        } else {
            xr = vload_s<T, V>(xp + base, cs);
            yr = vload_s<T, V>(yp + base, cs);
            item_totals(r, q, off, tv);
        }
        finish(r, q, off, base, live, xr, yr, tv, row_c0(r), wp_old);
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
    const int nsm = std::max(1, dev_attr(cudaDevAttrMultiProcessorCount));
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
    const size_t smem = WIN ? sizeof(uint32_t) * d.W : 0;
    const int bt = d.tbt;
    const int nit = d.Ap / (LR * V);
    const bool big = J.unit && J.nchunks > 0 && KIND != K_XY;
    // Row order: heavy rows first (their chunk items), then the rest in
    // decreasing degree when rows differ much in length or share a warp.
    StepP Q = P;
    Q.order = nullptr;
    Q.row0 = 0;
    if (big) {
        Q.order = J.perm;
        Q.row0 = J.nheavy;
    } else if (KIND != K_XY && (J.skewed || LR < 32 || P.niso)) {
        Q.order = J.perm;
    }
    // isolated rows (P.niso, left to k_iso) are the end of the degree order
    if (P.niso && !Q.order) return cudaErrorInvalidValue;
    const int64_t items = ((d.n - Q.row0 - P.niso + RW - 1) / RW + (big ? J.nchunks : 0)) * nit;
    // count mode of the +-1 rows: byte counters per lane (0), bit planes (1),
    // or mixed (2: the byte-counter kernel with P.bits_min set, heavy rows
    // only); staged rows (x, y copied ahead into shared memory) for
    // whole-warp rows of plain steps
    const bool cm = d.tcm == 1;
    constexpr bool can_st = LR == 32 && !WIN && KIND != K_XY;
    const bool st = can_st && d.tst != 0 && J.unit;
    const size_t smem_st = (size_t)(bt / 32) * 4 * 32 * V * sizeof(T);
    if constexpr (LR == 32) {
        if (big) {
            if constexpr (can_st) {
                if (st) {
                    if (cm) return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, true, 32, 1, 1>, d, items, bt, smem_st, s, Q, offset);
                    return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, true, 32, 0, 1>, d, items, bt, smem_st, s, Q, offset);
                }
            }
            if (cm) return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, true, 32, 1, 0>, d, items, bt, smem, s, Q, offset);
            return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, true, 32, 0, 0>, d, items, bt, smem, s, Q, offset);
        }
    } else {
        if (big) return cudaErrorInvalidValue;
    }
    if (KIND == K_XY) return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, false, LR, 0, 0>, d, items, bt, smem, s, Q, offset);
    if (J.unit) {
        if constexpr (KIND != K_XY) {
            if constexpr (can_st) {
                if (st) {
                    if (cm) return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, false, LR, 1, 1>, d, items, bt, smem_st, s, Q, offset);
                    return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, false, LR, 0, 1>, d, items, bt, smem_st, s, Q, offset);
                }
            }
            if (cm) return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, false, LR, 1, 0>, d, items, bt, smem, s, Q, offset);
        }
        return launch_grid(k_row<T, V, KIND, WIN, W_UNIT, false, LR, 0, 0>, d, items, bt, smem, s, Q, offset);
    }
    if constexpr (sizeof(T) == 8)
        return launch_grid(k_row<T, V, KIND, WIN, W_F64, false, LR, 0, 0>, d, items, bt, smem, s, Q, offset);
    else
        return launch_grid(k_row<T, V, KIND, WIN, W_F32, false, LR, 0, 0>, d, items, bt, smem, s, Q, offset);
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

// Isolated rows (degree 0, the last P.niso entries of P.order) have no
// neighbour and are no row's neighbour: the force on them is zero at every
// step and no step reads their signs.  One launch advances them through a
// whole window of fused steps in registers -- each step the step kernel's
// arithmetic (sb_update with a zero force) followed by the rounding to the
// storage type that storing and reloading the state between launches does
// -- and writes the signs of the window's last two steps to the planes the
// step kernel would have written, with the window compare of its last
// step.  The state it leaves is bit-identical to stepping the rows one
// launch per step.  Thread item: V agents of one row; warps stride over
// groups of 32 items (warp-uniform trip counts for the sign shuffles).
template <class T, int V, int NT>
__global__ void __launch_bounds__(NT) k_iso(const StepP P, const int nsteps)
{
    using A = typename St<T>::A;
    using RawT = Raw<V * sizeof(T)>;
    extern __shared__ __align__(16) uint32_t s_chg[];
    pdl_wait();
    if (P.ctl[CTL_STOP]) return;   // grid-uniform
    for (int q = threadIdx.x; q < P.W; q += NT) s_chg[q] = 0;
    __syncthreads();
    constexpr int G = 32 / V;   // lanes sharing one sign word
    const int lane = threadIdx.x & 31;
    const int step0 = P.ctl[CTL_STEP];
    const int nseg = P.Ap / V;   // items per row (a multiple of G)
    const int64_t total = P.niso * nseg;
    const int64_t nwarp = (int64_t)gridDim.x * (NT / 32);
    T *xp = (T *)P.x, *yp = (T *)P.y;
    const bool cs = P.stream_state != 0;
    A zero[V];
#pragma unroll
    for (int v = 0; v < V; v++) zero[v] = A(0);
    const int last = step0 + nsteps - 1;   // step k writes plane (k & 1) ^ 1
    uint32_t *Sl = (last & 1) ? P.S0 : P.S1, *Sp = (last & 1) ? P.S1 : P.S0;
    for (int64_t wg = (int64_t)blockIdx.x * (NT / 32) + (threadIdx.x >> 5); wg * 32 < total; wg += nwarp) {
        // lanes past the last item repeat it and store nothing
        const int64_t t = wg * 32 + lane;
        const bool live = t < total;
        const int64_t tt = live ? t : total - 1;
        const int64_t i = tt / nseg;
        const int seg = (int)(tt - i * nseg);
        const int64_t r = __ldg(&P.order[P.n - P.niso + i]);
        const int a0 = seg * V, q = a0 >> 5, off = a0 & 31;
        const int64_t base = r * P.Ap + a0;
        A x[V], y[V];
        RawT xw = vload_s<T, V>(xp + base, cs), yw = vload_s<T, V>(yp + base, cs);
        to_vals<T, V>(xw, x);
        to_vals<T, V>(yw, y);
        A c0 = (A)P.c0;
        if (P.c0r32) c0 = std::is_same<A, double>::value ? (A)__ldg(&P.c0r64[r]) : (A)__ldg(&P.c0r32[r]);
        auto one = [&](int k) {
            const auto c = Coef<A>::get(P, step0 + k);
            sb_update<K_FUSED, false, V>(x, y, zero, c0, c, c);
            xw = from_vals<T, V>(x);
            yw = from_vals<T, V>(y);
            to_vals<T, V>(xw, x);
            to_vals<T, V>(yw, y);
        };
        auto signs = [&]() {
            uint32_t b = 0;
#pragma unroll
            for (int v = 0; v < V; v++) b |= sbit(x[v]) << v;
            return b << off;
        };
        const int body = nsteps > 2 ? nsteps - 2 : 0;
#pragma unroll 1
        for (int k = 0; k < body; k++) one(k);
        uint32_t bprev = 0, b = 0;
        for (int k = body; k < nsteps; k++) {
            one(k);
            bprev = b;
            b = signs();
        }
        if (nsteps > 0 && live) {
            vstore_s(xp + base, xw.u, cs);
            vstore_s(yp + base, yw.u, cs);
        }
#pragma unroll
        for (int sft = 1; sft < G; sft <<= 1) {
            b |= __shfl_xor_sync(FULL, b, sft);
            bprev |= __shfl_xor_sync(FULL, bprev, sft);
        }
        if (nsteps > 0 && live && (lane & (G - 1)) == 0) {
            const int64_t wi = r * P.W + q;
            Sl[wi] = b;
            if (nsteps > 1) Sp[wi] = bprev;
            // window compare of the last step, src/kernels.cu:37-46 + :84-90
            const uint32_t ch = b ^ P.Wp[wi];
            P.Wp[wi] = b;
            if (ch) atomicOr(&s_chg[q], ch);
        }
    }
    __syncthreads();
    for (int qq = threadIdx.x; qq < P.W; qq += NT)
        if (s_chg[qq]) atomicOr(&P.chg[qq], s_chg[qq]);
    // late: the next step's CTAs would otherwise wait on SMs these need
    pdl_trigger();
}

// 256-thread blocks, each warp four groups of 32 items.
template <class T>
cudaError_t iso_t(const SolveDims &d, const DevCsr &J, const StepP &P, cudaStream_t s)
{
    constexpr int V = 16 / (int)sizeof(T);
    if (!P.niso || !P.order || d.Ap % 32) return cudaErrorInvalidValue;
    const int nsm = std::max(1, dev_attr(cudaDevAttrMultiProcessorCount));
    const size_t smem = sizeof(uint32_t) * d.W;
    const int64_t warps = (P.niso * (d.Ap / V) + 31) / 32;
    const int64_t blocks = std::min<int64_t>((warps + 4 * 8 - 1) / (4 * 8), (int64_t)nsm * 64);
    return launch(k_iso<T, V, 256>, dim3((unsigned)std::max<int64_t>(blocks, 1)), dim3(256), smem, s, d.pdl, P,
                  (int)d.period);
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
