// k_step_bf16.cu -- the step kernels with BF16 state (one translation unit per
// precision, so they compile in parallel).
#include "k_step.cuh"

namespace sbx {

cudaError_t step_bf16(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win,
                 int offset, cudaStream_t s)
{
    return step_t<__nv_bfloat16>(d, J, P, kind, win, offset, s);
}

cudaError_t iso_bf16(const SolveDims &d, const DevCsr &J, const StepP &P, cudaStream_t s)
{
    return iso_t<__nv_bfloat16>(d, J, P, s);
}

}  // namespace sbx
