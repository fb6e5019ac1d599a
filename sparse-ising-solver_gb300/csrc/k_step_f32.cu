// k_step_f32.cu -- the step kernels with F32 state (one translation unit per
// precision, so they compile in parallel).
#include "k_step.cuh"

namespace sbx {

cudaError_t step_f32(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win,
                 int offset, cudaStream_t s)
{
    return step_t<float>(d, J, P, kind, win, offset, s);
}

cudaError_t iso_f32(const SolveDims &d, const DevCsr &J, const StepP &P, cudaStream_t s)
{
    return iso_t<float>(d, J, P, s);
}

}  // namespace sbx
