// Instantiations of the FP32 compensated sweep for Scheme=GODUNOV (HLL/HLLC, HLLC_Toro and
// Steger-Warming; compiled with contraction on).
#include "sweep_f32_impl.cuh"

namespace ibtfo {

SweepLaunch sweep_launcher_godunov_f32(int riemann, int limiter, int ty)
{
    const bool vl = (limiter == VANLEER);
    return ty == TILE_Y ? select_f32<GODUNOV, TILE_Y>(riemann, vl) : select_f32<GODUNOV, FAST_TILE_Y>(riemann, vl);
}

} // namespace ibtfo
