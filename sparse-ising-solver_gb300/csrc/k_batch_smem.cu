// k_batch_smem.cu -- the batched MaxCut step with each instance's sign plane
// in shared memory (one launch per SB step, all instances).
//
// A batch packs many small instances into one block-diagonal matrix, so a
// row's neighbours all lie in its own instance.  Each CTA (one per SM) owns a
// contiguous run of rows, cut into segments at instance boundaries; for each
// segment it copies the instance's whole sign plane (n_i rows x W words, plus
// an all-zero row) from global memory into shared memory, and every neighbour
// gather of the segment's rows is then a shared-memory load instead of an L2
// round trip.  Instances of up to ~27,000 rows fit at 64 agents.
//
// A lane owns one 32-agent sign word of one row (W lanes per row, 32 / W rows
// per warp item): it walks all of the row's neighbours itself and adds their
// words into seven bit planes with a carry-save (Harley-Seal) tree -- about
// one full adder per neighbour word, no cross-lane sums -- then transposes
// the planes into per-agent counts and updates its 32 agents (four 16-byte
// vectors of x and of y).  The arithmetic is the streaming kernel's (k_row):
// the force 2 count - degree is exact, the update is sb_update in FP32, one
// rounding to the storage type per store, so the state is bit-identical.
//
// Columns are 16-bit local rows (instances of at most 32,767 rows) with the
// weight's sign in bit 15, each row's list padded to whole blocks of eight
// with the all-zero row and 16-byte aligned, so a block of neighbours is one
// 16-byte load; one word per row packs its first block and its degree.
//
// At 64 agents (two words per row) the two lanes of a row interleave their
// 8-agent chunks of x and y: in each of the four vector loads they read the
// two halves of one 32-byte sector, which halves the sectors the state moves
// through L1.  A lane counts its own 32-agent word, the pair swaps the counts
// of the chunks the other updates, and swaps the new sign bytes back into
// words.
#include "k_step.cuh"

namespace sbx {

namespace {

struct BsmP {
    const uint4 *__restrict__ lcol;       // blocks of eight 16-bit entries: local column | sign << 15
    const uint32_t *__restrict__ rinfo;   // per row: first block of eight entries << 7 | degree
    const int32_t *__restrict__ seg;      // per segment: instance, first row, end row (global)
    const int32_t *__restrict__ cta_seg;  // per CTA: first segment (grid + 1 entries)
    const int32_t *__restrict__ ioff;     // per instance: first row
    const int32_t *__restrict__ in;       // per instance: rows
};

// a + b + e -> a (sum), returns the carry
__device__ __forceinline__ uint32_t fa(uint32_t &a, uint32_t b, uint32_t e)
{
    const uint32_t c = (a & b) | (e & (a ^ b));
    a ^= b ^ e;
    return c;
}

template <class T, int W, int KIND, bool WIN, int NT>
__global__ void __launch_bounds__(NT, 1) k_bsm(const StepP P, const BsmP B, const int offset)
{
    static_assert(sizeof(T) == 2, "16-bit state: 32 agents in four 16-byte vectors");
    static_assert(W == 1 || W == 2 || W == 4, "W words per row");
    constexpr int RPW = 32 / W;          // rows per warp item
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) uint32_t s_plane[];   // [rows + 1][W], then s_chg[W]
    __shared__ uint32_t s_chg[W];
    pdl_wait();
    if (P.ctl[CTL_STOP]) return;          // grid-uniform
    const int step = P.ctl[CTL_STEP] + offset;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (WIN) {
        if (tid < W) s_chg[tid] = 0;
    }
    pdl_trigger();
    using A = float;
    const float4 c = __ldg(&P.coef32[step]);
    const float4 cn = __ldg(&P.coef32[step + 1]);
    const uint32_t *Scur = (step & 1) ? P.S1 : P.S0;
    uint32_t *Snext = (step & 1) ? P.S0 : P.S1;
    T *xp = (T *)P.x, *yp = (T *)P.y;
    const bool cs = P.stream_state != 0;
    const int q = lane % W;                  // this lane's word of its row
    const uint32_t qbase = (uint32_t)__cvta_generic_to_shared(s_plane) + 4u * (uint32_t)q;
    constexpr bool IL = W == 2;              // interleaved chunks (see above)
    int loaded = -1;
    for (int s = __ldg(&B.cta_seg[blockIdx.x]); s < __ldg(&B.cta_seg[blockIdx.x + 1]); s++) {
        const int inst = __ldg(&B.seg[3 * s]);
        const int r0 = __ldg(&B.seg[3 * s + 1]), r1 = __ldg(&B.seg[3 * s + 2]);
        const int ni = __ldg(&B.in[inst]);
        if (inst != loaded) {
            // the instance's plane (written by the previous step) and the
            // all-zero row that padded neighbours read
            __syncthreads();
            // (cp.async: a thread issues all its word copies back to back and
            // waits once, instead of a load-to-store round trip per word)
            const uint32_t *src = Scur + (int64_t)__ldg(&B.ioff[inst]) * W;
            const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(s_plane);
            for (int i = tid; i < ni * W; i += NT)
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4;"
                             :: "r"(sbase + 4u * (uint32_t)i), "l"(src + i) : "memory");
            asm volatile("cp.async.wait_all;" ::: "memory");
            if (tid < W) s_plane[ni * W + tid] = 0u;
            __syncthreads();
            loaded = inst;
        }
        // dt * xi0 is one value per instance
        const float c0 = __ldg(&P.c0r32[r0]);
        const int ngroups = (r1 - r0 + RPW - 1) / RPW;
        for (int g = wid; g < ngroups; g += NW) {
            const int rr = r0 + g * RPW + lane / W;
            const bool live = rr < r1;
            const int r = live ? rr : r1 - 1;    // lanes past the segment repeat its last row
            const int64_t rbase = (int64_t)r * P.Ap;
            // the lane's four 8-agent chunks: its word's (32 q + 8 k), or
            // interleaved with its partner's (8 (2 k + q))
            auto chunk = [&](int k) { return IL ? 8 * (2 * k + q) : 32 * q + 8 * k; };
            // x of the lane's 32 agents in flight during the count (y after
            // it: both at once would spill the count's registers)
            Raw<16> xr[4], yr[4];
#pragma unroll
            for (int k = 0; k < 4; k++) xr[k] = vload_s<T, 8>(xp + rbase + chunk(k), cs);
            uint32_t wp_old = 0;
            if (WIN) wp_old = P.Wp[(int64_t)r * W + q];
            const uint32_t ri = __ldg(&B.rinfo[r]);
            const int32_t deg = live ? (int32_t)(ri & 127u) : 0;
            const int32_t dmax = __reduce_max_sync(FULL, deg);
            // seven bit planes of the count of agents whose neighbour term is
            // -1 (bit a of p[k] = bit k of agent a's count), Harley-Seal
            // blocks of eight neighbour words
            uint32_t p[7];
#pragma unroll
            for (int k = 0; k < 7; k++) p[k] = 0;
            const uint4 *cp = B.lcol + (ri >> 7);
            const uint32_t zpair = (uint32_t)ni * 0x10001u;   // two entries of the zero row
            for (int32_t kb = 0; kb < dmax; kb += 8) {
                uint4 cv = make_uint4(zpair, zpair, zpair, zpair);
                if (kb < deg) cv = __ldg(cp + kb / 8);
                const uint32_t pv[4] = {cv.x, cv.y, cv.z, cv.w};
                uint32_t w[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const uint32_t v = pv[j / 2];
                    const uint32_t col = (j & 1) ? (v >> 16) & 0x7fffu : v & 0x7fffu;
                    uint32_t word;
                    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(word) : "r"(qbase + col * (uint32_t)(4 * W)));
                    if (!P.allpos) {
                        // the sign bit (15 or 31) replicated over the word
                        uint32_t neg;
                        if (j & 1) asm("prmt.b32 %0, %1, 0, 0xbbbb;" : "=r"(neg) : "r"(v));
                        else asm("prmt.b32 %0, %1, 0, 0x9999;" : "=r"(neg) : "r"(v));
                        word ^= neg;
                    }
                    w[j] = word;
                }
                const uint32_t a1 = fa(p[0], w[0], w[1]);
                const uint32_t b1 = fa(p[0], w[2], w[3]);
                const uint32_t a2 = fa(p[1], a1, b1);
                const uint32_t c1 = fa(p[0], w[4], w[5]);
                const uint32_t d1 = fa(p[0], w[6], w[7]);
                const uint32_t b2 = fa(p[1], c1, d1);
                uint32_t e = fa(p[2], a2, b2);
#pragma unroll
                for (int k = 3; k < 7; k++) {
                    const uint32_t t = p[k] & e;
                    p[k] ^= e;
                    e = t;
                }
            }
            // the planes as byte counters: byte v of cnt[2k + v / 4] = 2 * count
            // of agent 8k + v of the word.  Byte k of each plane goes to one
            // byte of a 64-bit value shifted up a byte (which doubles the
            // counts), then an 8x8 bit transpose (rows = bytes).
            uint32_t cnt[8];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint32_t s01 = (uint32_t)k | (((uint32_t)k + 4) << 4);
                uint32_t lo = __byte_perm(__byte_perm(0u, p[0], s01), __byte_perm(p[1], p[2], s01), 0x5410);
                uint32_t hi = __byte_perm(__byte_perm(p[3], p[4], s01), __byte_perm(p[5], p[6], s01), 0x5410);
                uint32_t t;
                t = (lo ^ (lo >> 7)) & 0x00AA00AAu;
                lo ^= t ^ (t << 7);
                t = (hi ^ (hi >> 7)) & 0x00AA00AAu;
                hi ^= t ^ (t << 7);
                t = (lo ^ (lo >> 14)) & 0x0000CCCCu;
                lo ^= t ^ (t << 14);
                t = (hi ^ (hi >> 14)) & 0x0000CCCCu;
                hi ^= t ^ (t << 14);
                t = (lo ^ (hi << 4)) & 0xF0F0F0F0u;
                lo ^= t;
                hi ^= t >> 4;
                cnt[2 * k] = lo;
                cnt[2 * k + 1] = hi;
            }
            if (IL) {
                // lane q updates the chunks c = q, q + 2 of both words: its
                // own word's, and the partner's sent across (the partner
                // sends its chunks 1 - q, 3 - q)
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    const uint32_t s0 = q ? cnt[4 * j] : cnt[4 * j + 2];
                    const uint32_t s1 = q ? cnt[4 * j + 1] : cnt[4 * j + 3];
                    const uint32_t r0v = __shfl_xor_sync(FULL, s0, 1);
                    const uint32_t r1v = __shfl_xor_sync(FULL, s1, 1);
                    // chunk k = j (word 0) and k = 2 + j (word 1)
                    const uint32_t o0 = q ? cnt[4 * j + 2] : cnt[4 * j];
                    const uint32_t o1 = q ? cnt[4 * j + 3] : cnt[4 * j + 1];
                    // word 0 holds lane 0's own counts, word 1 lane 1's
                    cnt[4 * j] = q ? r0v : o0;        // k = j (word 0)
                    cnt[4 * j + 1] = q ? r1v : o1;
                    cnt[4 * j + 2] = q ? o0 : r0v;    // k = 2 + j (word 1)
                    cnt[4 * j + 3] = q ? o1 : r1v;
                }
            }
            // PRMT builds the float 2^23 + 2 count; minus 2^23 + degree it is
            // the force 2 count - degree, exactly
            const float bias = 8388608.0f + (float)deg;
            uint32_t b = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                yr[k] = vload_s<T, 8>(yp + rbase + chunk(k), cs);
                // the counts of chunk k: cnt[2k], cnt[2k + 1] (word order), or
                // in the interleaved order cnt[4 (k % 2) + 2 (k / 2)] ...
                const int ci = IL ? 4 * (k % 2) + 2 * (k / 2) : 2 * k;
                float tv[8], x[8], y[8];
#pragma unroll
                for (int v = 0; v < 8; v++)
                    tv[v] = __uint_as_float(__byte_perm(cnt[ci + v / 4], 0x4b000000u, 0x7440u + (v & 3))) - bias;
                to_vals<T, 8>(xr[k], x);
                to_vals<T, 8>(yr[k], y);
                sb_update<KIND, WIN, 8>(x, y, tv, c0, c, cn);
#pragma unroll
                for (int v = 0; v < 8; v++) b |= sbit(x[v]) << (8 * k + v);
                xr[k] = from_vals<T, 8>(x);
                yr[k] = from_vals<T, 8>(y);
            }
            if (IL) {
                // byte k of b: the signs of chunk 2 k + q; word q is the
                // chunks 4 q .. 4 q + 3, alternately the two lanes' bytes
                const uint32_t pb = __shfl_xor_sync(FULL, b, 1);
                b = q ? __byte_perm(b, pb, 0x3726) : __byte_perm(b, pb, 0x5140);
            }
            if (live) {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    vstore_s(xp + rbase + chunk(k), xr[k].u, cs);
                    vstore_s(yp + rbase + chunk(k), yr[k].u, cs);
                }
                const int64_t wi = (int64_t)r * W + q;
                if (KIND == K_FUSED || !WIN) Snext[wi] = b;
                if (WIN) {
                    // window compare, src/kernels.cu:37-46 + :84-90
                    P.Wp[wi] = b;
                    const uint32_t ch = b ^ wp_old;
                    if (ch) atomicOr(&s_chg[q], ch);
                }
            }
        }
    }
    if (WIN) {
        __syncthreads();
        if (tid < W && s_chg[tid]) atomicOr(&P.chg[tid], s_chg[tid]);
    }
}

template <class T, int W, int KIND, bool WIN, int NT>
cudaError_t launch_n(const StepP &P, const BsmP &B, int grid, size_t smem, int offset, cudaStream_t s,
                     bool pdl)
{
    auto kern = k_bsm<T, W, KIND, WIN, NT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return launch(kern, dim3((unsigned)grid), dim3(NT), smem, s, pdl, P, B, offset);
}

// CTA size: 1024 threads (64 registers each), 640 (96) or 512 (128)
template <class T, int W, int KIND, bool WIN>
cudaError_t launch_w(const StepP &P, const BsmP &B, int grid, size_t smem, int offset, cudaStream_t s,
                     bool pdl, int nt)
{
    if (nt == 512) return launch_n<T, W, KIND, WIN, 512>(P, B, grid, smem, offset, s, pdl);
    if (nt == 640) return launch_n<T, W, KIND, WIN, 640>(P, B, grid, smem, offset, s, pdl);
    return launch_n<T, W, KIND, WIN, 1024>(P, B, grid, smem, offset, s, pdl);
}

template <class T, int KIND, bool WIN>
cudaError_t launch_t(int W, const StepP &P, const BsmP &B, int grid, size_t smem, int offset, cudaStream_t s,
                     bool pdl, int nt)
{
    switch (W) {
    case 1: return launch_w<T, 1, KIND, WIN>(P, B, grid, smem, offset, s, pdl, nt);
    case 2: return launch_w<T, 2, KIND, WIN>(P, B, grid, smem, offset, s, pdl, nt);
    case 4: return launch_w<T, 4, KIND, WIN>(P, B, grid, smem, offset, s, pdl, nt);
    default: return cudaErrorInvalidValue;
    }
}

template <class T>
cudaError_t launch_k(int kind, bool win, int W, const StepP &P, const BsmP &B, int grid, size_t smem,
                     int offset, cudaStream_t s, bool pdl, int nt)
{
    if (kind == K_FUSED)
        return win ? launch_t<T, K_FUSED, true>(W, P, B, grid, smem, offset, s, pdl, nt)
                   : launch_t<T, K_FUSED, false>(W, P, B, grid, smem, offset, s, pdl, nt);
    if (kind == K_FC)
        return win ? launch_t<T, K_FC, true>(W, P, B, grid, smem, offset, s, pdl, nt)
                   : launch_t<T, K_FC, false>(W, P, B, grid, smem, offset, s, pdl, nt);
    return cudaErrorInvalidValue;
}

}  // namespace

size_t bsm_smem_bytes(int64_t max_rows, int W) { return (size_t)(max_rows + 1) * W * 4; }

cudaError_t launch_batch_smem(const SolveDims &d, const DevBsm &M, const StepP &P, int kind, bool win,
                              int offset, cudaStream_t s)
{
    BsmP B;
    B.lcol = (const uint4 *)M.lcol;
    B.rinfo = M.rinfo;
    B.seg = M.seg;
    B.cta_seg = M.cta_seg;
    B.ioff = M.ioff;
    B.in = M.in;
    const size_t smem = bsm_smem_bytes(M.max_rows, d.W);
    const int nt = d.tbsm == 512 || d.tbsm == 640 ? d.tbsm : 1024;
    if (d.prec == P_BF16) return launch_k<__nv_bfloat16>(kind, win, d.W, P, B, M.grid, smem, offset, s, d.pdl, nt);
    if (d.prec == P_F16) return launch_k<__half>(kind, win, d.W, P, B, M.grid, smem, offset, s, d.pdl, nt);
    return cudaErrorInvalidValue;
}

}  // namespace sbx
