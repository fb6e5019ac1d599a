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

void rand_jump_tables(uint32_t seed, int64_t L, int nbits, std::vector<uint32_t> &out)
{
    // Seeding: the minimal-standard LCG, then the lag-31 recurrence up to the
    // first returned value.
    uint32_t u[344];
    uint64_t word = seed ? seed : 1u;
    u[0] = (uint32_t)word;
    for (int i = 1; i < 31; i++) {
        word = (16807u * word) % 2147483647u;
        u[i] = (uint32_t)word;
    }
    for (int i = 31; i < 34; i++) u[i] = u[i - 31];
    for (int i = 34; i < 344; i++) u[i] = u[i - 31] + u[i - 3];
    out.assign(R + (size_t)nbits * R * R, 0);
    for (int i = 0; i < R; i++) out[i] = u[313 + i];   // window before output 0
    // M: window (u[i-31..i-1]) -> (u[i-30..i]).
    uint32_t M[R * R] = {0}, P[R * R], Acc[R * R];
    for (int i = 0; i < R - 1; i++) M[i * R + i + 1] = 1;
    M[(R - 1) * R + 0] = 1;
    M[(R - 1) * R + 28] = 1;
    // P = M^L by square-and-multiply.
    for (int i = 0; i < R * R; i++) Acc[i] = (i % (R + 1)) == 0;
    memcpy(P, M, sizeof P);
    for (int64_t e = L; e; e >>= 1) {
        if (e & 1) matmul31(Acc, P, Acc);
        matmul31(P, P, P);
    }
    for (int b = 0; b < nbits; b++) {
        memcpy(&out[R + (size_t)b * R * R], Acc, sizeof Acc);
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

// One thread: jump to output t*L, then emit L outputs.
template <class T>
__global__ void __launch_bounds__(128) k_rand_init(T *x, T *y, int64_t outputs, int32_t A,
                                                   int32_t Ap, int tsp, int64_t L, int nbits,
                                                   const uint32_t *__restrict__ tab)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t o0 = t * L;
    if (o0 >= outputs) return;
    uint32_t v[R];
#pragma unroll
    for (int i = 0; i < R; i++) v[i] = __ldg(&tab[i]);
    for (int b = 0; b < nbits; b++) {
        if (!((t >> b) & 1)) continue;
        const uint32_t *P = tab + R + (size_t)b * R * R;
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
    int64_t o = o0;
    // Circular window: at phase q, v[q] holds u[i-31] and v[(q+28)%31] u[i-3].
    while (o < o1) {
#pragma unroll
        for (int q = 0; q < R; q++) {
            uint32_t nu = v[q] + v[(q + 28) % R];
            v[q] = nu;
            if (o < o1) {
                const double r = (double)(nu >> 1);
                // (((double)rand() / RAND_MAX) * 2 - 1) / 10, each op rounded
                const double val =
                    __ddiv_rn(__dsub_rn(__dmul_rn(__ddiv_rn(r, 2147483647.0), 2.0), 1.0), 10.0);
                if (tsp) {
                    const int64_t e = o, row = e / A, a = e - row * A, idx = row * Ap + a;
                    put(x, idx, 0.0);
                    put(y, idx, val);
                } else {
                    const int64_t e = o >> 1, row = e / A, a = e - row * A, idx = row * Ap + a;
                    if (o & 1) put(y, idx, val);
                    else put(x, idx, val);
                }
            }
            o++;
        }
    }
}

template <class T>
cudaError_t launch_t(const SolveDims &d, Work &w, bool tsp, int64_t L, int nbits,
                     cudaStream_t s)
{
    const int64_t outputs = d.n * d.A * (tsp ? 1 : 2);
    const int64_t threads = (outputs + L - 1) / L;
    const int blk = 128;
    const int64_t grid = (threads + blk - 1) / blk;
    // padded agents start (and stay) at zero
    if (d.Ap != d.A) {
        cudaError_t e = cudaMemsetAsync(w.x, 0, (size_t)d.n * d.Ap * sizeof(T), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(w.y, 0, (size_t)d.n * d.Ap * sizeof(T), s);
        if (e != cudaSuccess) return e;
    }
    k_rand_init<T><<<(unsigned)grid, blk, 0, s>>>((T *)w.x, (T *)w.y, outputs, d.A, d.Ap,
                                                 tsp ? 1 : 0, L, nbits, w.rjump);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_rand_init(const SolveDims &d, Work &w, bool tsp, int64_t L, int nbits,
                             cudaStream_t s)
{
    switch (d.prec) {
    case P_F32: return launch_t<float>(d, w, tsp, L, nbits, s);
    case P_BF16: return launch_t<__nv_bfloat16>(d, w, tsp, L, nbits, s);
    case P_F16: return launch_t<__half>(d, w, tsp, L, nbits, s);
    default: return launch_t<double>(d, w, tsp, L, nbits, s);
    }
}

}  // namespace sbx
