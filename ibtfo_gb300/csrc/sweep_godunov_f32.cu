// Instantiations of the FP32 compensated sweep for Scheme=GODUNOV (HLL/HLLC, HLLC_Toro and
// Steger-Warming; compiled with contraction on).
#include "sweep_f32_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_godunov_f32(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    if (riemann == SW)
        return vl ? &launch_sweep_f32<GODUNOV, SW, VANLEER> : &launch_sweep_f32<GODUNOV, SW, MINMOD>;
    if (riemann == HLLCT)
        return vl ? &launch_sweep_f32<GODUNOV, HLLCT, VANLEER> : &launch_sweep_f32<GODUNOV, HLLCT, MINMOD>;
    if (riemann == HLL)
        return vl ? &launch_sweep_f32<GODUNOV, HLL, VANLEER> : &launch_sweep_f32<GODUNOV, HLL, MINMOD>;
    return nullptr; // PVRS: FP64 precisions only
}

} // namespace ibtfo
