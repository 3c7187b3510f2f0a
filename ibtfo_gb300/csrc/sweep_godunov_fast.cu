// Instantiations of the fused sweep for Scheme=GODUNOV, fp64_fast (compiled with contraction).
// One translation unit per scheme and precision so the library builds in parallel.
#include "sweep_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_godunov_fast(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<GODUNOV, PVRS, VANLEER, 1> : &launch_sweep<GODUNOV, PVRS, MINMOD, 1>;
    case SW: return vl ? &launch_sweep<GODUNOV, SW, VANLEER, 1> : &launch_sweep<GODUNOV, SW, MINMOD, 1>;
    case HLLCT: return vl ? &launch_sweep<GODUNOV, HLLCT, VANLEER, 1> : &launch_sweep<GODUNOV, HLLCT, MINMOD, 1>;
    default: return vl ? &launch_sweep<GODUNOV, HLL, VANLEER, 1> : &launch_sweep<GODUNOV, HLL, MINMOD, 1>;
    }
}

} // namespace ibtfo
