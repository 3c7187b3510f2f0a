// Batched sweep instantiations for Scheme=GODUNOV, fp64_fast, all tile shapes.
// One translation unit per scheme and precision so the library builds in parallel.
#include "batch_impl.cuh"

namespace ibtfo {

BatchKernel batch_kernel_godunov_fast(int riemann, int limiter, int shape)
{
    return batch_kernel_scheme<GODUNOV, 1>(riemann, limiter, shape);
}

} // namespace ibtfo
