// Batched sweep instantiations for Scheme=MUSCL, the FP32 compensated form, all tile shapes.
// One translation unit per scheme and precision so the library builds in parallel.
#include "batch_impl.cuh"

namespace ibtfo {

BatchKernel batch_kernel_muscl_f32(int riemann, int limiter, int shape)
{
    return batch_kernel_scheme<MUSCL, 2>(riemann, limiter, shape);
}

} // namespace ibtfo
