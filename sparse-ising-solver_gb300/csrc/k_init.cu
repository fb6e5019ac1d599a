// k_init.cu -- the reference's initial state, generated on the device.
//
// The reference fills X and Y on the host with glibc rand() after
// srand(seed), interleaved X[i], Y[i] (src/ising.cu:91-95), or Y only with
// X = 0 for TSP (src/ising_tsp.cu:55-59).  glibc's rand() (TYPE_3 additive
// feedback generator) is the linear recurrence over Z/2^32
//     u[i] = u[i-31] + u[i-3],   output_k = u[344+k] >> 1,
// seeded by u[0] = seed (0 -> 1), u[i] = 16807 u[i-1] mod (2^31-1) for
// i = 1..30, u[31..33] = u[0..2].  Its 31-word window therefore advances by a
// fixed 31x31 matrix M, and M^k jumps k outputs at once.  Each device thread
// jumps to the start of its own chunk of outputs with precomputed powers
// M^(L*2^b) and then runs the recurrence serially, so the whole stream is
// produced in parallel and equals, value for value, what rand() returns.
// The powers do not depend on the seed; one launch can fill many instances,
// each from its own seed (its own 31-word starting window).
#include "common.cuh"
#include "engine.h"

#include <cstring>

namespace sbx {

namespace {

constexpr int R = 31;

void matmul31(const uint32_t *a, const uint32_t *b, uint32_t *c)
{
    uint32_t t[R * R];
    for (int i = 0; i < R; i++)
        for (int j = 0; j < R; j++) {
            uint32_t s = 0;
            for (int k = 0; k < R; k++) s += a[i * R + k] * b[k * R + j];
            t[i * R + j] = s;
        }
    memcpy(c, t, sizeof t);
}

}  // namespace

void rand_seed_window(uint32_t seed, uint32_t *V0)
{
    // the minimal-standard LCG, then the lag-31 recurrence up to the first
    // returned value; V0 = u[313..343], the window before output 0
    uint32_t u[344];
    uint64_t word = seed ? seed : 1u;
    u[0] = (uint32_t)word;
    for (int i = 1; i < 31; i++) {
        word = (16807u * word) % 2147483647u;
        u[i] = (uint32_t)word;
    }
    for (int i = 31; i < 34; i++) u[i] = u[i - 31];
    for (int i = 34; i < 344; i++) u[i] = u[i - 31] + u[i - 3];
    for (int i = 0; i < R; i++) V0[i] = u[313 + i];
}

void rand_jump_matrices(int64_t L, int nbits, std::vector<uint32_t> &out)
{
    // M: window (u[i-31..i-1]) -> (u[i-30..i]); out[b] = M^(L*2^b)
    uint32_t M[R * R] = {0}, P[R * R], Acc[R * R];
    for (int i = 0; i < R - 1; i++) M[i * R + i + 1] = 1;
    M[(R - 1) * R + 0] = 1;
    M[(R - 1) * R + 28] = 1;
    for (int i = 0; i < R * R; i++) Acc[i] = (i % (R + 1)) == 0;
    memcpy(P, M, sizeof P);
    for (int64_t e = L; e; e >>= 1) {
        if (e & 1) matmul31(Acc, P, Acc);
        matmul31(P, P, P);
    }
    out.assign((size_t)nbits * R * R, 0);
    for (int b = 0; b < nbits; b++) {
        memcpy(&out[(size_t)b * R * R], Acc, sizeof Acc);
        matmul31(Acc, Acc, Acc);
    }
}

int rand_threads_bits(int64_t outputs, int64_t L)
{
    int64_t threads = (outputs + L - 1) / L;
    int b = 0;
    while ((1ll << b) < threads) b++;
    return b;
}

namespace {

template <class T>
__device__ __forceinline__ void put(T *p, int64_t i, double v) { p[i] = St<T>::st((typename St<T>::A)v); }

// One thread: find its instance, jump to its chunk start, emit L outputs.
// slot (MaxCut only, may be null): the row of the state that takes the
// instance's row r, as a global row (row_off + r -> slot[row_off + r]).
template <class T>
__global__ void __launch_bounds__(128) k_rand_init(T *x, T *y, int32_t Ap, int tsp, int64_t L,
                                                   const uint32_t *__restrict__ mats,
                                                   const RandInst *__restrict__ inst, int count,
                                                   int64_t total_threads,
                                                   const int32_t *__restrict__ slot)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total_threads) return;
    int lo = 0, hi = count - 1;   // last instance with thread_base <= t
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst[mid].thread_base <= t) lo = mid;
        else hi = mid - 1;
    }
    const RandInst &I = inst[lo];
    const int64_t lt = t - I.thread_base;
    const int64_t outputs = I.n * I.A * (tsp ? 1 : 2);
    const int64_t o0 = lt * L;
    if (o0 >= outputs) return;
    uint32_t v[R];
#pragma unroll
    for (int i = 0; i < R; i++) v[i] = I.V0[i];
    for (int b = 0; (lt >> b) != 0; b++) {
        if (!((lt >> b) & 1)) continue;
        const uint32_t *P = mats + (size_t)b * R * R;
        uint32_t nv[R];
#pragma unroll
        for (int i = 0; i < R; i++) {
            uint32_t s = 0;
#pragma unroll
            for (int k = 0; k < R; k++) s += __ldg(&P[i * R + k]) * v[k];
            nv[i] = s;
        }
#pragma unroll
        for (int i = 0; i < R; i++) v[i] = nv[i];
    }
    const int64_t o1 = min(o0 + L, outputs);
    const int64_t A = I.A;
    T *xi = x + I.row_off * Ap, *yi = y + I.row_off * Ap;
    int64_t o = o0;
    // Circular window: at phase q, v[q] holds u[i-31] and v[(q+28)%31] u[i-3].
    while (o < o1) {
#pragma unroll
        for (int q = 0; q < R; q++) {
            const uint32_t nu = v[q] + v[(q + 28) % R];
            v[q] = nu;
            if (o < o1) {
                const double r = (double)(nu >> 1);
                // (((double)rand() / RAND_MAX) * 2 - 1) / 10, each op rounded
                const double val =
                    __ddiv_rn(__dsub_rn(__dmul_rn(__ddiv_rn(r, 2147483647.0), 2.0), 1.0), 10.0);
                if (tsp) {
                    const int64_t row = o / A, a = o - row * A, idx = row * Ap + a;
                    put(xi, idx, 0.0);
                    put(yi, idx, val);
                } else {
                    const int64_t e = o >> 1, row = e / A, a = e - row * A;
                    const int64_t srow = slot ? (int64_t)__ldg(&slot[I.row_off + row]) - I.row_off : row;
                    const int64_t idx = srow * Ap + a;
                    if (o & 1) put(yi, idx, val);
                    else put(xi, idx, val);
                }
            }
            o++;
        }
    }
}

template <class T>
cudaError_t launch_t(void *x, void *y, int32_t Ap, int tsp, int64_t L, const uint32_t *mats,
                     const RandInst *inst, int count, int64_t total_threads, const int32_t *slot,
                     cudaStream_t s)
{
    const int blk = 128;
    const int64_t grid = (total_threads + blk - 1) / blk;
    if (grid == 0) return cudaSuccess;
    k_rand_init<T><<<(unsigned)grid, blk, 0, s>>>((T *)x, (T *)y, Ap, tsp, L, mats, inst, count,
                                                 total_threads, slot);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_rand_init(int prec, void *x, void *y, int32_t Ap, bool tsp, int64_t L,
                             const uint32_t *mats, const RandInst *inst, int count,
                             int64_t total_threads, const int32_t *slot, cudaStream_t s)
{
    if (tsp) slot = nullptr;
    switch (prec) {
    case P_F32: return launch_t<float>(x, y, Ap, tsp, L, mats, inst, count, total_threads, slot, s);
    case P_BF16:
        return launch_t<__nv_bfloat16>(x, y, Ap, tsp, L, mats, inst, count, total_threads, slot, s);
    case P_F16: return launch_t<__half>(x, y, Ap, tsp, L, mats, inst, count, total_threads, slot, s);
    default: return launch_t<double>(x, y, Ap, tsp, L, mats, inst, count, total_threads, slot, s);
    }
}

}  // namespace sbx
