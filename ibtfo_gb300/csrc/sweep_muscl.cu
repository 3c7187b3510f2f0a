// Instantiations of the fused sweep for Scheme=MUSCL (one translation unit per
// scheme so the library builds in parallel).
#include "sweep_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_muscl(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<MUSCL, PVRS, VANLEER> : &launch_sweep<MUSCL, PVRS, MINMOD>;
    case SW: return vl ? &launch_sweep<MUSCL, SW, VANLEER> : &launch_sweep<MUSCL, SW, MINMOD>;
    default: return vl ? &launch_sweep<MUSCL, HLL, VANLEER> : &launch_sweep<MUSCL, HLL, MINMOD>;
    }
}

} // namespace ibtfo
