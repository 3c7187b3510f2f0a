// Instantiations of the FP32 compensated sweep for Scheme=MHM (HLL/HLLC, HLLC_Toro and
// Steger-Warming; compiled with contraction on).
#include "sweep_f32_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_mhm_f32(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    if (riemann == SW)
        return vl ? &launch_sweep_f32<MHM, SW, VANLEER> : &launch_sweep_f32<MHM, SW, MINMOD>;
    if (riemann == HLLCT)
        return vl ? &launch_sweep_f32<MHM, HLLCT, VANLEER> : &launch_sweep_f32<MHM, HLLCT, MINMOD>;
    if (riemann == HLL)
        return vl ? &launch_sweep_f32<MHM, HLL, VANLEER> : &launch_sweep_f32<MHM, HLL, MINMOD>;
    return nullptr; // PVRS: FP64 precisions only
}

} // namespace ibtfo
