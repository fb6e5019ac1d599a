// k_step_f16.cu -- the step kernels with F16 state (one translation unit per
// precision, so they compile in parallel).
#include "k_step.cuh"

namespace sbx {

cudaError_t step_f16(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win,
                 int offset, cudaStream_t s)
{
    return step_t<__half>(d, J, P, kind, win, offset, s);
}

cudaError_t iso_f16(const SolveDims &d, const DevCsr &J, const StepP &P, cudaStream_t s)
{
    return iso_t<__half>(d, J, P, s);
}

}  // namespace sbx
