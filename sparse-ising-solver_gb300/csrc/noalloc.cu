// noalloc.cu -- fused SB steps for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: a serving process that has handed all
// of the device's memory to its own arena or caching allocator has none left
// to give, and a latency-critical loop cannot take the device-wide
// synchronisation that cudaMalloc/cudaFree may perform.  For them
// sbx_fused_steps_noalloc runs fused SB steps on buffers the caller already
// owns and keeps its only scratch -- the two sign planes the steps gather
// from -- in the file-scope array below, which every GPU that loads the
// library holds until the process exits.
//
// The array's name is a host-side stand-in in host code, not a device
// address: the entry point asks for the address with cudaGetSymbolAddress,
// once per device, with that device current, on its first call there.  That
// first call on each device should therefore come before any stream capture.
// Every call shares the array and finds the previous call's contents in it;
// each call rebuilds the plane it reads first, and calls that overlap on the
// GPU (other streams, other threads) race on it.  The looked-up address is
// kept for the life of the process: after cudaDeviceReset (or anything else
// that tears down the device's primary context) it is stale, and the entry
// point must not be called again in that process.
#include "../../include/sbx.h"

#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "common.cuh"

namespace sbx {
void set_last_error(const std::string &m);   // api.cpp
}

namespace {

// Two sign planes of SBX_NOALLOC_MAX_WORDS words each (16 MiB).
static __device__ __align__(256) uint32_t g_noalloc_planes[2 * (size_t)SBX_NOALLOC_MAX_WORDS];

constexpr int kMaxDevices = 64;
uint32_t *g_planes_addr[kMaxDevices] = {};
std::mutex g_planes_mutex;

// Bit a%32 of word (r, a/32) = sign bit of x[r][a].
__global__ void k_noalloc_signs(const float *__restrict__ x, uint32_t *__restrict__ S, int64_t n,
                                int32_t W)
{
    const int64_t gw = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (gw >= n * W) return;
    const uint32_t b = __ballot_sync(sbx::FULL, sbx::sbit(x[gw * 32 + lane]));
    if (lane == 0) S[gw] = b;
}

// One fused step (src/kernels.cu:211-269, Jacobi order), FP32 state, any
// float weights: a warp owns (row, 32-agent word), lane = agent.
__global__ void k_noalloc_step(const int32_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                               const float *__restrict__ val, float *__restrict__ x,
                               float *__restrict__ y, const uint32_t *__restrict__ Sin,
                               uint32_t *__restrict__ Sout, int64_t n, int32_t W, float c0,
                               float k1, float k2)
{
    const int64_t gw = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (gw >= n * W) return;
    const int64_t r = gw / W;
    const int w = (int)(gw - r * W);
    const int64_t idx = gw * 32 + lane;
    float xv = x[idx], yv = y[idx];
    float total = 0.f;
    for (int32_t e = rowptr[r]; e < rowptr[r + 1]; e++) {
        const uint32_t word = Sin[(int64_t)col[e] * W + w];
        total -= val[e] * (((word >> lane) & 1u) ? -1.f : 1.f);
    }
    if (fabsf(xv) > 1.f) {
        xv = sbx::spin_of(xv);
        yv = 0.f;
    } else {
        yv = fmaf(c0, total, yv);
    }
    xv = fmaf(k1, yv, xv);
    yv = fmaf(k2, xv, yv);
    x[idx] = xv;
    y[idx] = yv;
    const uint32_t b = __ballot_sync(sbx::FULL, sbx::sbit(xv));
    if (lane == 0) Sout[gw] = b;
}

int fail(int code, const std::string &m)
{
    sbx::set_last_error("sbx_fused_steps_noalloc: " + m);
    return code;
}

}  // namespace

extern "C" int sbx_fused_steps_noalloc(const int32_t *d_rowptr, const int32_t *d_col,
                                       const float *d_val, int64_t n, int32_t agents, float *d_x,
                                       float *d_y, double dt, double xi0, int32_t step0,
                                       int32_t nsteps, int32_t max_steps, void *cuda_stream)
{
    // d_col and d_val are checked even when the matrix has no entries: the
    // number of entries is on the device, out of this call's sight.
    if (!d_rowptr || !d_col || !d_val || !d_x || !d_y || n <= 0 || agents <= 0 || step0 < 0 ||
        nsteps < 0 || max_steps <= 0)
        return fail(SBX_ERR_ARG, "null pointer or non-positive size");
    if (agents % 32)
        return fail(SBX_ERR_ARG, "agents must be a multiple of 32 (x, y are [n][agents])");
    const int64_t W = agents / 32;
    if (n * W > (int64_t)SBX_NOALLOC_MAX_WORDS)
        return fail(SBX_ERR_ARG, "n * agents / 32 = " + std::to_string(n * W) +
                                     " exceeds SBX_NOALLOC_MAX_WORDS = " +
                                     std::to_string((long long)SBX_NOALLOC_MAX_WORDS));
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SBX_ERR_NODEVICE, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(SBX_ERR_UNSUPPORTED, "device index too large");
    uint32_t *planes;
    {
        std::lock_guard<std::mutex> lock(g_planes_mutex);
        if (!g_planes_addr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_planes);
            if (e != cudaSuccess || !p) return fail(SBX_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_planes_addr[dev] = (uint32_t *)p;
        }
        planes = g_planes_addr[dev];
    }
    // Each launch reports its own error (cudaLaunchKernelEx returns it), so
    // an error left pending by the caller's earlier work is neither consumed
    // nor blamed on this call.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)((n * W + 7) / 8));
    cfg.blockDim = dim3(256);
    cfg.stream = (cudaStream_t)cuda_stream;
    uint32_t *S[2] = {planes, planes + SBX_NOALLOC_MAX_WORDS};
    const int32_t W32 = (int32_t)W;
    // The plane the first step gathers from is rebuilt from x: nothing is
    // read that a previous call left behind.
    e = cudaLaunchKernelEx(&cfg, k_noalloc_signs, (const float *)d_x, S[step0 & 1], n, W32);
    if (e != cudaSuccess) return fail(SBX_ERR_CUDA, cudaGetErrorString(e));
    const float c0 = (float)(dt * xi0);
    for (int32_t i = 0; i < nsteps; i++) {
        const int32_t k = step0 + i;
        double p = 1.025 * (double)k / max_steps;   // src/kernels.cu:225-226
        p = p < 1.0 ? p : 1.0;
        e = cudaLaunchKernelEx(&cfg, k_noalloc_step, d_rowptr, d_col, d_val, d_x, d_y,
                               (const uint32_t *)S[k & 1], S[(k + 1) & 1], n, W32, c0,
                               (float)(dt * (p + 1)), (float)(dt * (p - 1)));
        if (e != cudaSuccess) return fail(SBX_ERR_CUDA, cudaGetErrorString(e));
    }
    return SBX_OK;
}
