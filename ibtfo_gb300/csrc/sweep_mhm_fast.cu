// Instantiations of the fused sweep for Scheme=MHM, fp64_fast (compiled with contraction):
// 32x16 tiles (FAST_TILE_Y rows) or 32x8, 32x8 with the PVRS solvers.
// One translation unit per scheme and precision so the library builds in parallel.
#include "sweep_impl.cuh"

namespace ibtfo {

template <int TY>
static SweepLaunch select(int riemann, bool vl)
{
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<MHM, PVRS, VANLEER, 1> : &launch_sweep<MHM, PVRS, MINMOD, 1>;
    case SW: return vl ? prepared_sweep_launcher<MHM, SW, VANLEER, 1, TY>() : prepared_sweep_launcher<MHM, SW, MINMOD, 1, TY>();
    case HLLCT: return vl ? prepared_sweep_launcher<MHM, HLLCT, VANLEER, 1, TY>() : prepared_sweep_launcher<MHM, HLLCT, MINMOD, 1, TY>();
    case HLLT: return vl ? prepared_sweep_launcher<MHM, HLLT, VANLEER, 1, TY>() : prepared_sweep_launcher<MHM, HLLT, MINMOD, 1, TY>();
    default: return vl ? prepared_sweep_launcher<MHM, HLL, VANLEER, 1, TY>() : prepared_sweep_launcher<MHM, HLL, MINMOD, 1, TY>();
    }
}

SweepLaunch sweep_launcher_mhm_fast(int riemann, int limiter, int ty)
{
    const bool vl = (limiter == VANLEER);
    if (ty == TILE_Y || riemann == PVRS)
        return select<TILE_Y>(riemann, vl);
    return select<FAST_TILE_Y>(riemann, vl);
}

} // namespace ibtfo
