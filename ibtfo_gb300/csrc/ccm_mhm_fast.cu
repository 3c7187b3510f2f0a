// Cut-cell sweep instantiations for Scheme=MHM, FP64.
// One translation unit per scheme and precision so the library builds in parallel.
#include "ccm_impl.cuh"

namespace ibtfo {

CcmLaunch ccm_launcher_mhm_fast(int riemann, int limiter)
{
    return ccm_launcher_scheme<MHM, 1>(riemann, limiter);
}

} // namespace ibtfo
