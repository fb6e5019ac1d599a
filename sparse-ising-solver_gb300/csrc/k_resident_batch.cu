// k_resident_batch.cu -- resident kernel for batched MaxCut: the rows of the
// block-diagonal matrix are packed into bins (whole instances, first-fit
// decreasing), and one CTA owns 4 agents of every row of one bin for the
// whole solve: their x, y (16-bit) in registers (RR rows per thread) and
// shared memory, the rows' 4-bit sign words in one shared byte per row
// (low nibble for even steps, high nibble for odd steps).  Instances never
// interact and neither do agents, so a CTA needs no other CTA; one
// __syncthreads() per step gives the Jacobi order of the reference kernel
// (src/kernels.cu:211-269), and the arithmetic is the streaming kernel's
// (sb_update, exact byte-counter force), so the per-agent results are
// identical to the streaming batch.
//
// The matrix is read relabelled into slot order (bins concatenated, rows of
// a bin by decreasing degree): thread t of a CTA owns the bin's slots t,
// t + NT, ...; perm maps slots to rows where the global state is read or
// written.
#include "k_step.cuh"

namespace sbx {

namespace {

constexpr int KB = 4;   // agents per CTA

struct RbP {
    const int32_t *__restrict__ rowptr;   // slot order
    const uint32_t *__restrict__ colw;    // columns as slots, bit 31 the weight sign
    const float *__restrict__ valf;
    const float *__restrict__ c0;         // dt * xi0 of each slot's instance
    const int32_t *__restrict__ perm;     // slot -> row
    const int32_t *__restrict__ bin_off;  // [nbins + 1] first slot of each bin
    const int32_t *__restrict__ cta_bin;  // [grid / groups] bin of each CTA row, largest first
    const float4 *__restrict__ coef;
    void *x, *y;                          // global [rows][Ap]
    uint32_t *Wp;                         // global plane [rows][W]: signs of the last step
    int32_t *ctl;
    int32_t Ap, W, groups, nsteps, unit;
};

template <class T, int NT, int RR>
__global__ void __launch_bounds__(NT, 1) k_resident_batch(const RbP P)
{
    static_assert(sizeof(T) == 2, "16-bit state: 4 agents in 8 bytes");
    extern __shared__ __align__(16) unsigned char smem[];
    pdl_wait();
    const int tid = threadIdx.x;
    const int bin = P.cta_bin[blockIdx.x / P.groups];
    const int a0 = (blockIdx.x % P.groups) * KB;
    const int wg = a0 >> 5, sh = a0 & 31;
    const int s0 = P.bin_off[bin], n = P.bin_off[bin + 1] - s0;   // the bin's slots
    const int ns = n > RR * NT ? n - RR * NT : 0;
    uint2 *xs = (uint2 *)smem;
    uint2 *ys = xs + ns;
    uint8_t *Sb = (uint8_t *)(ys + ns);   // [n]: bits 0-3 even steps, 4-7 odd steps
    T *xg = (T *)P.x, *yg = (T *)P.y;

    uint2 xr[RR > 0 ? RR : 1], yr[RR > 0 ? RR : 1];
    const float4 c00 = P.coef[0];
    // the state, after the pre-step Update_XY of step 0 (src/ising.cu:188),
    // computed and rounded as the streaming pre-step does
    auto load_row = [&](int s, uint2 &xv, uint2 &yv) {
        const int r = __ldg(&P.perm[s0 + s]);
        xv = *(const uint2 *)(xg + (int64_t)r * P.Ap + a0);
        yv = *(const uint2 *)(yg + (int64_t)r * P.Ap + a0);
        Raw<8> xw, yw;
        xw.u = xv;
        yw.u = yv;
        float x[KB], y[KB];
        to_vals<T, KB>(xw, x);
        to_vals<T, KB>(yw, y);
#pragma unroll
        for (int v = 0; v < KB; v++) {
            y[v] = fmaf(c00.w, x[v], y[v]);
            x[v] = fmaf(c00.z, y[v], x[v]);
        }
        xv = from_vals<T, KB>(x).u;
        yv = from_vals<T, KB>(y).u;
        uint32_t bits = 0;
#pragma unroll
        for (int v = 0; v < KB; v++) bits |= sbit(x[v]) << v;
        Sb[s] = (uint8_t)bits;   // step 0 reads the low nibble
    };
#pragma unroll
    for (int i = 0; i < RR; i++) {
        const int s = i * NT + tid;
        if (s < n) load_row(s, xr[i], yr[i]);
    }
    for (int s = RR * NT + tid; s < n; s += NT) {
        uint2 xv, yv;
        load_row(s, xv, yv);
        xs[s - RR * NT] = xv;
        ys[s - RR * NT] = yv;
    }
    __syncthreads();

    // one SB step of slot s (state in xv, yv); k: the step index
    auto row_step = [&](int s, uint2 &xv, uint2 &yv, int k, const float4 &c) {
        const int sg = s0 + s;
        const int32_t e0 = __ldg(&P.rowptr[sg]), e1 = __ldg(&P.rowptr[sg + 1]);
        const int32_t deg = e1 - e0;
        const int rd = 4 * (k & 1);   // nibble of this step's signs
        float tv[KB];
        if (P.unit) {
            uint32_t lo = 0;
#pragma unroll 4
            for (int32_t e = e0; e < e1; e++) {
                const uint32_t cw = __ldg(&P.colw[e]);
                const uint32_t b = ((uint32_t)Sb[(cw & 0x7fffffffu) - s0] >> rd) ^ (0u - (cw >> 31));
                lo += spread2x(b & 0xfu);
            }
            const float bias = 8388608.0f + (float)deg;
#pragma unroll
            for (int v = 0; v < KB; v++)
                tv[v] = __uint_as_float(__byte_perm(lo, 0x4b000000u, 0x7440u + v)) - bias;
        } else {
#pragma unroll
            for (int v = 0; v < KB; v++) tv[v] = 0.0f;
            for (int32_t e = e0; e < e1; e++) {
                const uint32_t cw = __ldg(&P.colw[e]);
                const float wv = __ldg(&P.valf[e]);
                const uint32_t b = (uint32_t)Sb[(cw & 0x7fffffffu) - s0] >> rd;
#pragma unroll
                for (int v = 0; v < KB; v++) tv[v] -= wv * (((b >> v) & 1u) ? -1.0f : 1.0f);
            }
        }
        Raw<8> xw, yw;
        xw.u = xv;
        yw.u = yv;
        float x[KB], y[KB];
        to_vals<T, KB>(xw, x);
        to_vals<T, KB>(yw, y);
        sb_update<K_FUSED, false, KB>(x, y, tv, __ldg(&P.c0[sg]), c, c);
        uint32_t nb = 0;
#pragma unroll
        for (int v = 0; v < KB; v++) nb |= sbit(x[v]) << v;
        xv = from_vals<T, KB>(x).u;
        yv = from_vals<T, KB>(y).u;
        // keep this step's nibble (others read it), replace the next one
        const int wr = 4 - rd;
        Sb[s] = (uint8_t)(((uint32_t)Sb[s] & (0xfu << rd)) | (nb << wr));
    };

    for (int32_t k = 0; k < P.nsteps; k++) {
        const float4 ck = P.coef[k];
#pragma unroll
        for (int i = 0; i < RR; i++) {
            const int s = i * NT + tid;
            if (s < n) row_step(s, xr[i], yr[i], k, ck);
        }
        for (int s = RR * NT + tid; s < n; s += NT) {
            uint2 xv = xs[s - RR * NT], yv = ys[s - RR * NT];
            row_step(s, xv, yv, k, ck);
            xs[s - RR * NT] = xv;
            ys[s - RR * NT] = yv;
        }
        __syncthreads();
    }

    // the state and the signs of the last step back to global memory
    const int last = 4 * (P.nsteps & 1);
    auto store_row = [&](int s, const uint2 &xv, const uint2 &yv) {
        const int r = __ldg(&P.perm[s0 + s]);
        *(uint2 *)(xg + (int64_t)r * P.Ap + a0) = xv;
        *(uint2 *)(yg + (int64_t)r * P.Ap + a0) = yv;
        uint32_t *p = &P.Wp[(int64_t)r * P.W + wg];
        const uint32_t m = 0xfu << sh;
        atomicAnd(p, ~m);
        atomicOr(p, (((uint32_t)Sb[s] >> last) & 0xfu) << sh);
    };
#pragma unroll
    for (int i = 0; i < RR; i++) {
        const int s = i * NT + tid;
        if (s < n) store_row(s, xr[i], yr[i]);
    }
    for (int s = RR * NT + tid; s < n; s += NT) store_row(s, xs[s - RR * NT], ys[s - RR * NT]);
    if (blockIdx.x == 0 && tid == 0) {
        P.ctl[CTL_STEP] = P.nsteps;
        P.ctl[CTL_WINDOWS] = 0;
    }
}

constexpr int kRbNT = 1024, kRbRR = 8;

size_t rb_smem(int64_t rows)
{
    const int64_t ns = rows > (int64_t)kRbRR * kRbNT ? rows - (int64_t)kRbRR * kRbNT : 0;
    return (size_t)ns * 16 + (size_t)rows;
}

}  // namespace

int64_t resident_batch_max_rows()
{
    int dev = 0, smax = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const int64_t budget = (int64_t)smax - 1024;
    // rows r with rb_smem(r) <= budget
    int64_t r = (int64_t)kRbRR * kRbNT;
    r += (budget - r > 0 ? (budget - r) / 17 : 0);
    while (r > 0 && rb_smem(r) > (size_t)budget) r--;
    return r;
}

cudaError_t launch_resident_batch(const SolveDims &d, const DevRb &B, Work &w, cudaStream_t s)
{
    RbP P;
    P.rowptr = B.rowptr;
    P.colw = B.colw;
    P.valf = B.valf;
    P.c0 = B.c0;
    P.perm = B.perm;
    P.bin_off = B.bin_off;
    P.cta_bin = B.cta_bin;
    P.coef = (const float4 *)w.coef32;
    P.x = w.x;
    P.y = w.y;
    P.Wp = w.Wp;
    P.ctl = w.ctl;
    P.Ap = d.Ap;
    P.W = d.W;
    P.groups = d.Ap / KB;
    P.nsteps = d.steps_run;
    P.unit = B.unit ? 1 : 0;
    const size_t smem = rb_smem(B.max_bin_rows);
    const int grid = B.nbins * P.groups;
    auto kern = d.prec == P_BF16 ? k_resident_batch<__nv_bfloat16, kRbNT, kRbRR> : k_resident_batch<__half, kRbNT, kRbRR>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kRbNT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = d.pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, P);
}

}  // namespace sbx
