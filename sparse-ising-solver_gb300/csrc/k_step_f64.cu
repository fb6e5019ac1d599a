// k_step_f64.cu -- the step kernels with F64 state (one translation unit per
// precision, so they compile in parallel).
#include "k_step.cuh"

namespace sbx {

cudaError_t step_f64(const SolveDims &d, const DevCsr &J, const StepP &P, int kind, bool win,
                 int offset, cudaStream_t s)
{
    return step_t<double>(d, J, P, kind, win, offset, s);
}

cudaError_t iso_f64(const SolveDims &d, const DevCsr &J, const StepP &P, cudaStream_t s)
{
    return iso_t<double>(d, J, P, s);
}

}  // namespace sbx
