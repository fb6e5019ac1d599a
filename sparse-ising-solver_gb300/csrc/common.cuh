// common.cuh -- device helpers shared by the SB kernels (sm_103a).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sbx {

constexpr unsigned FULL = 0xffffffffu;

// Storage type <-> arithmetic type.  BF16/FP16/FP32 state is updated in FP32;
// FP64 state in FP64 (the bit-exact parity mode).
template <class T> struct St;
template <> struct St<float> {
    using A = float;
    static __device__ __forceinline__ float ld(float v) { return v; }
    static __device__ __forceinline__ float st(float v) { return v; }
};
template <> struct St<double> {
    using A = double;
    static __device__ __forceinline__ double ld(double v) { return v; }
    static __device__ __forceinline__ double st(double v) { return v; }
};
template <> struct St<__nv_bfloat16> {
    using A = float;
    static __device__ __forceinline__ float ld(__nv_bfloat16 v) { return __bfloat162float(v); }
    static __device__ __forceinline__ __nv_bfloat16 st(float v) { return __float2bfloat16_rn(v); }
};
template <> struct St<__half> {
    using A = float;
    static __device__ __forceinline__ float ld(__half v) { return __half2float(v); }
    static __device__ __forceinline__ __half st(float v) { return __float2half_rn(v); }
};

// IEEE sign bit of the stored value: (signbit(val) * -2) + 1 of the
// reference, as a bit (1 = spin -1).
__device__ __forceinline__ uint32_t sbit(float v) { return __float_as_uint(v) >> 31; }
__device__ __forceinline__ uint32_t sbit(double v) {
    return (uint32_t)(__double_as_longlong(v) >> 63) & 1u;
}
__device__ __forceinline__ float spin_of(float v) { return sbit(v) ? -1.0f : 1.0f; }
__device__ __forceinline__ double spin_of(double v) { return sbit(v) ? -1.0 : 1.0; }

// Separately rounded FP64 operations: the FP64 path must not contract a*b+c,
// so that it reproduces the reference's FP64 arithmetic as the oracle states
// it (one rounding per operation).
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }

// MaxCut pressure, src/kernels.cu:225-226 (clamped) and :15 (not clamped).
__device__ __forceinline__ double pressure(int step, int max_steps, bool clamp) {
    double p = __ddiv_rn(__dmul_rn(1.025, (double)step), (double)max_steps);
    if (clamp) p = p < 1.0 ? p : 1.0;
    return p;
}

// Programmatic dependent launch: wait for the preceding grid's memory, and
// let the next grid begin its launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

}  // namespace sbx
