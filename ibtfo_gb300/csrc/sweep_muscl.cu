// Instantiations of the fused sweep for Scheme=MUSCL, strict FP64 (compiled without contraction).
// One translation unit per scheme and precision so the library builds in parallel.
#include "sweep_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_muscl(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<MUSCL, PVRS, VANLEER, 0> : &launch_sweep<MUSCL, PVRS, MINMOD, 0>;
    case SW: return vl ? &launch_sweep<MUSCL, SW, VANLEER, 0> : &launch_sweep<MUSCL, SW, MINMOD, 0>;
    case HLLCT: return vl ? &launch_sweep<MUSCL, HLLCT, VANLEER, 0> : &launch_sweep<MUSCL, HLLCT, MINMOD, 0>;
    case HLLT: return vl ? &launch_sweep<MUSCL, HLLT, VANLEER, 0> : &launch_sweep<MUSCL, HLLT, MINMOD, 0>;
    default: return vl ? &launch_sweep<MUSCL, HLL, VANLEER, 0> : &launch_sweep<MUSCL, HLL, MINMOD, 0>;
    }
}

} // namespace ibtfo
