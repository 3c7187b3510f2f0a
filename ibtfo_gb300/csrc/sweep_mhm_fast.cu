// Instantiations of the fused sweep for Scheme=MHM, fp64_fast (compiled with contraction).
// One translation unit per scheme and precision so the library builds in parallel.
#include "sweep_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_mhm_fast(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<MHM, PVRS, VANLEER, 1> : &launch_sweep<MHM, PVRS, MINMOD, 1>;
    case SW: return vl ? &launch_sweep<MHM, SW, VANLEER, 1> : &launch_sweep<MHM, SW, MINMOD, 1>;
    case HLLCT: return vl ? &launch_sweep<MHM, HLLCT, VANLEER, 1> : &launch_sweep<MHM, HLLCT, MINMOD, 1>;
    default: return vl ? &launch_sweep<MHM, HLL, VANLEER, 1> : &launch_sweep<MHM, HLL, MINMOD, 1>;
    }
}

} // namespace ibtfo
