// Instantiations of the fused sweep for Scheme=MHM (one translation unit per
// scheme so the library builds in parallel).
#include "sweep_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_mhm(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<MHM, PVRS, VANLEER> : &launch_sweep<MHM, PVRS, MINMOD>;
    case SW: return vl ? &launch_sweep<MHM, SW, VANLEER> : &launch_sweep<MHM, SW, MINMOD>;
    default: return vl ? &launch_sweep<MHM, HLL, VANLEER> : &launch_sweep<MHM, HLL, MINMOD>;
    }
}

} // namespace ibtfo
