// Scheme = Lax: the Lax-Friedrichs update of the reference's Lax scheme
// (Src/Base/Euler/Advection/Lax/Lax_Scheme.cpp:15-60), one CTA per active
// tile, strict FP64 (this unit compiles without contraction for both FP64
// precision keys).
//
// The reference copies U_OLD into scratch, evaluates Conserve2Flux
// (Src/Base/Common/Conserve2Flux.cpp:2-37) on every cell, then sets each
// fluid cell to the average of its four neighbours minus the centred flux
// differences.  Here a tile stages its cells and a one-cell halo in shared
// memory, evaluates F and G once per staged cell, and updates its fluid
// cells; the CFL maxima and the mass sum of the new state are folded into
// the epilogue as in the other schemes.  Time = RK2 stages work as in the
// other sweeps (stage 1 stores the first stage, stage 2 the average).
#include "sweep_impl.cuh"

namespace ibtfo {

namespace {

constexpr int LX = TILE_X + 2, LY = TILE_Y + 2;

struct LaxSmem
{
    double sU[4][LY][LX];
    double sF[4][LY][LX];
    double sG[4][LY][LX];
};

__global__ void __launch_bounds__(TILE_X *TILE_Y) lax_kernel(const SweepArgs a)
{
    constexpr int NT = TILE_X * TILE_Y;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    auto &s = *reinterpret_cast<LaxSmem *>(smem_raw);

    const GridDesc &g = a.g;
    DevState *st = a.st;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        st->fill_pending = 0;
    // reference loop condition, Test/Sod/Sod.cpp:123
    if (a.guard && !(st->now_t < a.t_end && st->iter < a.max_iter))
        return;
    const double dt = st->dt;
    const int cur = st->cur;
    const double *U = cur ? a.buf1 : a.buf0;
    double *V = cur ? a.buf0 : a.buf1;
    const unsigned bid = a.tile0 + blockIdx.x;
    const unsigned tile = a.tiles[bid];
    const int i0 = g.ng + tile_ix(tile) * TILE_X;
    const int j0 = g.ng + tile_jy(tile) * TILE_Y;
    const long long P = g.plane;
    const int pitch = g.pitch;
    const double gam = g.gamma;

    // stage the tile with a one-cell halo (inside the padded array: ng >= 2)
    // and evaluate Conserve2Flux on each staged cell
    for (int q = threadIdx.x; q < LX * LY; q += NT)
    {
        const int ly = q / LX, lx = q - ly * LX;
        const int gi = i0 - 1 + lx, gj = j0 - 1 + ly;
        double u4[4] = {0.0, 0.0, 0.0, 0.0};
        if (gi < g.M && gj < g.N)
        {
#pragma unroll
            for (int k = 0; k < 4; k++)
                u4[k] = U[k * P + (long long)gj * pitch + gi];
        }
        // Conserve2Flux.cpp:21-35
        double rho = u4[0];
        double u = u4[1] / rho;
        double v = u4[2] / rho;
        double p = (gam - 1) * (u4[3] - 0.5 * rho * (u * u + v * v));
#pragma unroll
        for (int k = 0; k < 4; k++)
            s.sU[k][ly][lx] = u4[k];
        s.sF[0][ly][lx] = rho * u;
        s.sF[1][ly][lx] = rho * u * u + p;
        s.sF[2][ly][lx] = rho * u * v;
        s.sF[3][ly][lx] = (u4[3] + p) * u;
        s.sG[0][ly][lx] = rho * v;
        s.sG[1][ly][lx] = rho * u * v;
        s.sG[2][ly][lx] = rho * v * v + p;
        s.sG[3][ly][lx] = (u4[3] + p) * v;
    }
    __syncthreads();

    CellStats cs;
    const int c = threadIdx.x % TILE_X, r = threadIdx.x / TILE_X;
    const int i = i0 + c, j = j0 + r;
    const int lx = c + 1, ly = r + 1;
    if (i < g.ng + g.n_x && j < g.ng + g.n_y && a.type[(long long)j * pitch + i] == 0)
    {
        double v[4];
        // Lax_Scheme.cpp:51-55, evaluated left to right
#pragma unroll
        for (int k = 0; k < 4; k++)
            v[k] = 0.25 * (s.sU[k][ly][lx - 1] + s.sU[k][ly][lx + 1] + s.sU[k][ly + 1][lx] + s.sU[k][ly - 1][lx]) -
                   0.5 * dt * (s.sF[k][ly][lx + 1] - s.sF[k][ly][lx - 1]) / g.dx -
                   0.5 * dt * (s.sG[k][ly + 1][lx] - s.sG[k][ly - 1][lx]) / g.dy;
        const long long o = (long long)j * pitch + i;
        if (a.stage == 2)
            rk2_average(V, o, P, v);
#pragma unroll
        for (int k = 0; k < 4; k++)
            V[k * P + o] = v[k];
        if (a.stage != 1)
            cell_stats(v, gam, g.dx, g.dy, cs);
    }
    block_reduce_finalize<NT>(cs, st, a.partial, g, true, false, a.nblocks ? a.nblocks : gridDim.x, bid,
                              a.stage == 1);
}

void launch_lax(const SweepArgs &a, dim3 grid, dim3 block, cudaStream_t s)
{
    lax_kernel<<<grid, block, sizeof(LaxSmem), s>>>(a);
}

} // namespace

SweepLaunch sweep_launcher_lax() { return &launch_lax; }

} // namespace ibtfo
