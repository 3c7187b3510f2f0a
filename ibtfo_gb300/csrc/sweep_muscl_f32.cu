// Instantiations of the FP32 compensated sweep for Scheme=MUSCL (HLL/HLLC, HLLC_Toro and
// Steger-Warming; compiled with contraction on).
#include "sweep_f32_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_muscl_f32(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    if (riemann == SW)
        return vl ? &launch_sweep_f32<MUSCL, SW, VANLEER> : &launch_sweep_f32<MUSCL, SW, MINMOD>;
    if (riemann == HLLCT)
        return vl ? &launch_sweep_f32<MUSCL, HLLCT, VANLEER> : &launch_sweep_f32<MUSCL, HLLCT, MINMOD>;
    if (riemann == HLL)
        return vl ? &launch_sweep_f32<MUSCL, HLL, VANLEER> : &launch_sweep_f32<MUSCL, HLL, MINMOD>;
    return nullptr; // PVRS: FP64 precisions only
}

} // namespace ibtfo
