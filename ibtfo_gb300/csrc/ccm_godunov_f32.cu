// Cut-cell sweep instantiations for Scheme=GODUNOV, the FP32 compensated form.
// One translation unit per scheme and precision so the library builds in parallel.
#include "ccm_impl.cuh"

namespace ibtfo {

CcmLaunch ccm_launcher_godunov_f32(int riemann, int limiter)
{
    return ccm_launcher_scheme<GODUNOV, 2>(riemann, limiter);
}

} // namespace ibtfo
