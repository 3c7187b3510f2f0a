// Instantiations of the fused sweep for Scheme=MUSCL, fp64_fast (compiled with contraction).
// One translation unit per scheme and precision so the library builds in parallel.
#include "sweep_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_muscl_fast(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<MUSCL, PVRS, VANLEER, 1> : &launch_sweep<MUSCL, PVRS, MINMOD, 1>;
    case SW: return vl ? &launch_sweep<MUSCL, SW, VANLEER, 1> : &launch_sweep<MUSCL, SW, MINMOD, 1>;
    case HLLCT: return vl ? &launch_sweep<MUSCL, HLLCT, VANLEER, 1> : &launch_sweep<MUSCL, HLLCT, MINMOD, 1>;
    default: return vl ? &launch_sweep<MUSCL, HLL, VANLEER, 1> : &launch_sweep<MUSCL, HLL, MINMOD, 1>;
    }
}

} // namespace ibtfo
