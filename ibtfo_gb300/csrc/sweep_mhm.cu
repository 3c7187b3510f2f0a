// Instantiations of the fused sweep for Scheme=MHM, strict FP64 (compiled without contraction).
// One translation unit per scheme and precision so the library builds in parallel.
#include "sweep_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_mhm(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<MHM, PVRS, VANLEER, 0> : &launch_sweep<MHM, PVRS, MINMOD, 0>;
    case SW: return vl ? &launch_sweep<MHM, SW, VANLEER, 0> : &launch_sweep<MHM, SW, MINMOD, 0>;
    case HLLCT: return vl ? &launch_sweep<MHM, HLLCT, VANLEER, 0> : &launch_sweep<MHM, HLLCT, MINMOD, 0>;
    case HLLT: return vl ? &launch_sweep<MHM, HLLT, VANLEER, 0> : &launch_sweep<MHM, HLLT, MINMOD, 0>;
    default: return vl ? &launch_sweep<MHM, HLL, VANLEER, 0> : &launch_sweep<MHM, HLL, MINMOD, 0>;
    }
}

} // namespace ibtfo
