// Instantiations of the fused sweep for Scheme=GODUNOV, strict FP64 (compiled without contraction).
// One translation unit per scheme and precision so the library builds in parallel.
#include "sweep_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_godunov(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<GODUNOV, PVRS, VANLEER, 0> : &launch_sweep<GODUNOV, PVRS, MINMOD, 0>;
    case SW: return vl ? &launch_sweep<GODUNOV, SW, VANLEER, 0> : &launch_sweep<GODUNOV, SW, MINMOD, 0>;
    case HLLCT: return vl ? &launch_sweep<GODUNOV, HLLCT, VANLEER, 0> : &launch_sweep<GODUNOV, HLLCT, MINMOD, 0>;
    case HLLT: return vl ? &launch_sweep<GODUNOV, HLLT, VANLEER, 0> : &launch_sweep<GODUNOV, HLLT, MINMOD, 0>;
    default: return vl ? &launch_sweep<GODUNOV, HLL, VANLEER, 0> : &launch_sweep<GODUNOV, HLL, MINMOD, 0>;
    }
}

} // namespace ibtfo
