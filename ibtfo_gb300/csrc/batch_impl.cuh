// The persistent batched sweep: CTAs (a fixed grid of resident CTAs) walk
// one tile table that holds the active tiles of every case of a batch.  Each
// tile runs the same tile body as the one-case kernels (sweep_tile64 /
// sweep_tile32), so a case advances bit for bit as it does alone with the
// same tile shape; its statistics go to its own device state, and the last
// of its tiles to finish computes its next dt (per-case dt and loop
// accounting, Test/Sod/Sod.cpp:123-176).  Cases whose loop has ended
// (now_t >= t_end or iter >= max_iter) are skipped tile by tile.
#pragma once

#include "sweep_f32_impl.cuh"
#include "sweep_impl.cuh"

namespace ibtfo {

template <int SCH, int RIE, int LIM, int PREC, int TX, int TY>
__global__ void __launch_bounds__(BATCH_THREADS, (PREC == 2 && RIE == HLLT) ? 3 : 1)
    batch_sweep_kernel(const BatchHeader *__restrict__ h, int stage)
{
    constexpr int NT = BATCH_THREADS;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int ntiles = h->ntiles;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
    {
        const BatchTile e = h->tiles[t];
        const BatchCase &bc = h->cases[e.z];
        const SweepArgs &a = bc.s;
        DevState *st = a.st;
        if (e.y == 0 && threadIdx.x == 0)
            st->fill_pending = 0;
        // the case's tiles of this launch all read the same state: its
        // accounting changes only when the last of them has finished
        if (!(st->now_t < a.t_end && st->iter < a.max_iter))
            continue;
        const double dt = st->dt;
        const int cur = st->cur;
        const GridDesc &g = a.g;
        const int i0 = g.ng + tile_ix(e.x) * TX;
        const int j0 = g.ng + tile_jy(e.x) * TY;
        const bool interior = (e.x & TILE_INTERIOR) != 0;
        // the case's own tensor maps describe boxes of its one-case tiles
        // (32x16 except under PVRS): the 32x16 shape stages tiles with them
        const CUtensorMap *tm = nullptr;
        if constexpr (TX == TILE_X && TY == FAST_TILE_Y && RIE != PVRS)
            if (a.tma)
            {
                tm = &a.tmap[cur];
                if (threadIdx.x == 0)
                    tensormap_acquire(tm);
            }
        int *status = tm ? &st->status : nullptr;
        if constexpr (PREC == 2)
        {
            const float *U = reinterpret_cast<const float *>(cur ? a.buf1 : a.buf0);
            float *V = reinterpret_cast<float *>(cur ? a.buf0 : a.buf1);
            CellStats32 cs;
            if constexpr (RIE == HLLT)
                sweep_tile32_delta<SCH, RIE, LIM, TX, TY, NT>(*reinterpret_cast<SweepSmem32D<TX, TY> *>(smem_raw), g,
                                                              U, V, a.type, i0, j0, dt, cs, stage, tm, status,
                                                              interior);
            else
                sweep_tile32<SCH, RIE, LIM, TX, TY, NT>(*reinterpret_cast<SweepSmem32<TX, TY> *>(smem_raw), g, U, V,
                                                        a.type, i0, j0, dt, cs, stage, tm, status, interior);
            block_reduce_finalize32<NT>(cs, st, a.partial, g, (unsigned)bc.ntiles, e.y, stage == 1);
        }
        else
        {
            auto &s = *reinterpret_cast<SweepSmem64<TX, TY> *>(smem_raw);
            const double *U = cur ? a.buf1 : a.buf0;
            double *V = cur ? a.buf0 : a.buf1;
            CellStats cs;
            sweep_tile64<SCH, RIE, LIM, 1, TX, TY, NT>(s, g, U, V, a.type, i0, j0, dt, cs, stage, tm, status,
                                                       interior);
            block_reduce_finalize<NT>(cs, st, a.partial, g, true, false, (unsigned)bc.ntiles, e.y, stage == 1);
        }
    }
}

template <int SCH, int RIE, int LIM, int PREC, int TX, int TY>
struct BatchVariant
{
    static constexpr size_t smem()
    {
        return PREC == 2 ? sizeof(Smem32<RIE, TX, TY>) : sizeof(SweepSmem64<TX, TY>);
    }
    static void launch(const BatchHeader *h, int grid, cudaStream_t s, int stage)
    {
        batch_sweep_kernel<SCH, RIE, LIM, PREC, TX, TY><<<grid, BATCH_THREADS, smem(), s>>>(h, stage);
    }
    static int prepare()
    {
        auto k = batch_sweep_kernel<SCH, RIE, LIM, PREC, TX, TY>;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem()) != cudaSuccess)
            return 0;
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, BATCH_THREADS, smem()) != cudaSuccess)
            return 0;
        return n;
    }
};

template <int SCH, int RIE, int LIM, int PREC>
BatchKernel batch_kernel_shape(int shape)
{
    switch (shape)
    {
    case SHAPE_32x16:
        return {&BatchVariant<SCH, RIE, LIM, PREC, 32, 16>::launch, &BatchVariant<SCH, RIE, LIM, PREC, 32, 16>::prepare};
    case SHAPE_64x8:
        return {&BatchVariant<SCH, RIE, LIM, PREC, 64, 8>::launch, &BatchVariant<SCH, RIE, LIM, PREC, 64, 8>::prepare};
    default:
        return {&BatchVariant<SCH, RIE, LIM, PREC, 32, 8>::launch, &BatchVariant<SCH, RIE, LIM, PREC, 32, 8>::prepare};
    }
}

// every (Riemann solver, limiter) of one scheme and precision; PVRS has no
// FP32 form
template <int SCH, int PREC>
BatchKernel batch_kernel_scheme(int riemann, int limiter, int shape)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case PVRS:
        if constexpr (PREC == 2)
            return {nullptr, nullptr};
        else
            return vl ? batch_kernel_shape<SCH, PVRS, VANLEER, PREC>(shape)
                      : batch_kernel_shape<SCH, PVRS, MINMOD, PREC>(shape);
    case SW:
        return vl ? batch_kernel_shape<SCH, SW, VANLEER, PREC>(shape) : batch_kernel_shape<SCH, SW, MINMOD, PREC>(shape);
    case HLLCT:
        return vl ? batch_kernel_shape<SCH, HLLCT, VANLEER, PREC>(shape)
                  : batch_kernel_shape<SCH, HLLCT, MINMOD, PREC>(shape);
    case HLLT:
        return vl ? batch_kernel_shape<SCH, HLLT, VANLEER, PREC>(shape)
                  : batch_kernel_shape<SCH, HLLT, MINMOD, PREC>(shape);
    default:
        return vl ? batch_kernel_shape<SCH, HLL, VANLEER, PREC>(shape) : batch_kernel_shape<SCH, HLL, MINMOD, PREC>(shape);
    }
}

} // namespace ibtfo
