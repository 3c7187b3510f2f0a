// Batched sweep instantiations for Scheme=MHM, fp64_fast, all tile shapes.
// One translation unit per scheme and precision so the library builds in parallel.
#include "batch_impl.cuh"

namespace ibtfo {

BatchKernel batch_kernel_mhm_fast(int riemann, int limiter, int shape)
{
    return batch_kernel_scheme<MHM, 1>(riemann, limiter, shape);
}

} // namespace ibtfo
