// Instantiations of the fused sweep for Scheme=GODUNOV (one translation unit per
// scheme so the library builds in parallel).
#include "sweep_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_godunov(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<GODUNOV, PVRS, VANLEER> : &launch_sweep<GODUNOV, PVRS, MINMOD>;
    case SW: return vl ? &launch_sweep<GODUNOV, SW, VANLEER> : &launch_sweep<GODUNOV, SW, MINMOD>;
    default: return vl ? &launch_sweep<GODUNOV, HLL, VANLEER> : &launch_sweep<GODUNOV, HLL, MINMOD>;
    }
}

} // namespace ibtfo
