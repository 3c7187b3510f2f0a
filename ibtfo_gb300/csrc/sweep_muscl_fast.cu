// Instantiations of the fused sweep for Scheme=MUSCL, fp64_fast (compiled with contraction):
// 32x16 tiles (FAST_TILE_Y rows) or 32x8, 32x8 with the PVRS solvers.
// One translation unit per scheme and precision so the library builds in parallel.
#include "sweep_impl.cuh"

namespace ibtfo {

template <int TY>
static SweepLaunch select(int riemann, bool vl)
{
    switch (riemann)
    {
    case PVRS: return vl ? &launch_sweep<MUSCL, PVRS, VANLEER, 1> : &launch_sweep<MUSCL, PVRS, MINMOD, 1>;
    case SW: return vl ? prepared_sweep_launcher<MUSCL, SW, VANLEER, 1, TY>() : prepared_sweep_launcher<MUSCL, SW, MINMOD, 1, TY>();
    case HLLCT: return vl ? prepared_sweep_launcher<MUSCL, HLLCT, VANLEER, 1, TY>() : prepared_sweep_launcher<MUSCL, HLLCT, MINMOD, 1, TY>();
    case HLLT: return vl ? prepared_sweep_launcher<MUSCL, HLLT, VANLEER, 1, TY>() : prepared_sweep_launcher<MUSCL, HLLT, MINMOD, 1, TY>();
    default: return vl ? prepared_sweep_launcher<MUSCL, HLL, VANLEER, 1, TY>() : prepared_sweep_launcher<MUSCL, HLL, MINMOD, 1, TY>();
    }
}

SweepLaunch sweep_launcher_muscl_fast(int riemann, int limiter, int ty)
{
    const bool vl = (limiter == VANLEER);
    if (ty == TILE_Y || riemann == PVRS)
        return select<TILE_Y>(riemann, vl);
    return select<FAST_TILE_Y>(riemann, vl);
}

} // namespace ibtfo
