// Cut-cell sweep instantiations for Scheme=GODUNOV, FP64.
// One translation unit per scheme and precision so the library builds in parallel.
#include "ccm_impl.cuh"

namespace ibtfo {

CcmLaunch ccm_launcher_godunov_fast(int riemann, int limiter)
{
    return ccm_launcher_scheme<GODUNOV, 1>(riemann, limiter);
}

} // namespace ibtfo
