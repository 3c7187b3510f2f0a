// The fused per-step sweep: one CTA advances a TILE_X x TILE_Y block of
// interior cells by one time step.
//
// It restates, in one pass over shared memory, the reference Advance
// (MUSCL_Scheme.cpp:6-152 / MHM_Scheme.cpp:5-203 / Godunov_Scheme.cpp:6-140):
// face reconstruction, MHM predictor, X and Y Riemann solves, the X update
// followed by the Y update (both from the old state), restricted to fluid
// cells; then the CFL maxima (ComputeDt.cpp:28-49) and the mass sum
// (CaculateMass.cpp:27-38) of the new state, folded into the epilogue.
//
// The reference's Y solver shares its output slot with the X solver
// (MUSCL/EQDefine.H:35-36) and skips the store in some branches; the
// kernel keeps both face fluxes in shared memory and takes the X-face flux
// of the same cell where the reference would have left it in place.
#pragma once

#include "internal.h"
#include "physics.cuh"
#include "physics_fast.cuh"

namespace ibtfo {

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *addr, double v)
{
    // non-negative doubles order like their bit patterns
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// Block-wide reduction of (max a, max |u|, max |v|, sum mass, nan count),
// then the last block to finish computes the next dt and advances the
// reference loop accounting.  Deterministic: the mass partials are summed
// in a fixed order whichever block finishes last.
// WARP_DONE: the caller has already reduced each warp into its lane 0 (the
// FP32 form does that in FP32 so no per-cell FP64 work remains).
template <int NT, bool WARP_DONE = false>
__device__ __forceinline__ void block_reduce_finalize(double amax, double umax, double vmax, double mass, int nans,
                                                      DevState *st, double *partial, const GridDesc &g,
                                                      bool step_accounting, bool set_start)
{
    __shared__ double red[4][NT / 32];
    __shared__ int rnan[NT / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (!WARP_DONE)
    {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
            umax = fmax(umax, __shfl_xor_sync(0xffffffffu, umax, o));
            vmax = fmax(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
            mass += __shfl_xor_sync(0xffffffffu, mass, o);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        nans += __shfl_xor_sync(0xffffffffu, nans, o);
    if (lane == 0)
    {
        red[0][wid] = amax;
        red[1][wid] = umax;
        red[2][wid] = vmax;
        red[3][wid] = mass;
        rnan[wid] = nans;
    }
    __syncthreads();
    const unsigned nblocks = gridDim.x * gridDim.y;
    const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
    if (threadIdx.x == 0)
    {
        double a = red[0][0], u = red[1][0], v = red[2][0], m = red[3][0];
        int n = rnan[0];
        for (int w = 1; w < NT / 32; w++)
        {
            a = fmax(a, red[0][w]);
            u = fmax(u, red[1][w]);
            v = fmax(v, red[2][w]);
            m += red[3][w];
            n += rnan[w];
        }
        if (a > 0) atomic_max_nonneg(&st->amax_bits, a);
        if (u > 0) atomic_max_nonneg(&st->umax_bits, u);
        if (v > 0) atomic_max_nonneg(&st->vmax_bits, v);
        if (n) atomicAdd(&st->nan_cells, n);
        partial[bid] = m;
        __threadfence();
        unsigned t = atomicAdd(&st->ticket, 1u);
        last = (t == nblocks - 1);
    }
    __syncthreads();
    if (!last)
        return;
    __threadfence();
    // fixed-order sum of the per-block mass partials
    __shared__ double msum[NT];
    double s = 0.0;
    for (unsigned b = threadIdx.x; b < nblocks; b += NT)
        s += ((volatile double *)partial)[b];
    msum[threadIdx.x] = s;
    __syncthreads();
    for (int h = NT / 2; h > 0; h >>= 1)
    {
        if (threadIdx.x < h)
            msum[threadIdx.x] += msum[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        volatile DevState *vs = st;
        double a_max = __longlong_as_double((long long)vs->amax_bits);
        double u_max = __longlong_as_double((long long)vs->umax_bits);
        double v_max = __longlong_as_double((long long)vs->vmax_bits);
        // ComputeDt.cpp:49
        double dt_new = g.cfl * g.dx / (a_max + ((u_max < v_max) ? v_max : u_max));
        vs->last_amax = a_max;
        vs->last_umax = u_max;
        vs->last_vmax = v_max;
        vs->dt = dt_new;
        vs->mass = msum[0];
        if (set_start)
            vs->mass_start = msum[0];
        if (step_accounting)
        {
            vs->now_t = vs->now_t + dt_new; // Test/Sod/Sod.cpp:176
            vs->iter = vs->iter + 1;
            vs->cur = vs->cur ^ 1;
            vs->fill_pending = 1;
        }
        if (vs->nan_cells)
            vs->status |= STATUS_NAN;
        vs->amax_bits = 0ull;
        vs->umax_bits = 0ull;
        vs->vmax_bits = 0ull;
        vs->ticket = 0u;
        __threadfence();
    }
}

// CFL and mass contributions of one fluid cell of the new state
// (ComputeDt.cpp:38-45, CaculateMass.cpp:36)
__device__ __forceinline__ void cell_stats(const double v[4], double gam, double dx, double dy, double &amax,
                                           double &umax, double &vmax, double &mass, int &nans)
{
    double rho = v[0];
    double u = v[1] / v[0];
    double w = v[2] / v[0];
    double p = (gam - 1) * (v[3] - 0.5 * rho * (u * u + w * w));
    double a = pow_half(gam * p / rho);
    amax = fmax(amax, a);
    umax = fmax(umax, fabs(u));
    vmax = fmax(vmax, fabs(w));
    mass += v[0] * dx * dy;
    nans += (isnan(v[0]) || isnan(v[1]) || isnan(v[2]) || isnan(v[3])) ? 1 : 0;
}

// the same statistics with a shared reciprocal (fp64_fast)
__device__ __forceinline__ void cell_stats_fast(const double v[4], const GasConst<double> &K, double dxdy,
                                                double &amax, double &umax, double &vmax, double &mass, int &nans)
{
    const double ir = rcp_t(v[0]);
    const double u = v[1] * ir, w = v[2] * ir;
    const double p = K.gm1 * (v[3] - 0.5 * v[0] * (u * u + w * w));
    const double a = pow_half(K.g * p * ir);
    amax = fmax(amax, a);
    umax = fmax(umax, fabs(u));
    vmax = fmax(vmax, fabs(w));
    mass += v[0] * dxdy;
    nans += (isnan(v[0]) || isnan(v[1]) || isnan(v[2]) || isnan(v[3])) ? 1 : 0;
}

template <int SCH, int RIE, int LIM, int FAST>
__global__ void __launch_bounds__(TILE_X *TILE_Y) sweep_kernel(const SweepArgs a)
{
    constexpr int TX = TILE_X, TY = TILE_Y, NT = TX * TY;
    constexpr int WX = TX + 4, WY = TY + 4; // tile plus two halo cells each side
    __shared__ double sU[4][WY][WX];
    __shared__ double sF[4][TY + 1][TX + 1]; // X faces (i+1/2, j), i in [i0-1, i0+TX), j in [j0-1, j0+TY)
    __shared__ double sG[4][TY + 1][TX];     // Y faces (i, j+1/2), i in [i0, i0+TX), j in [j0-1, j0+TY)
    __shared__ unsigned char sKeep[TY + 1][TX];
    __shared__ double sC[4]; // fp64_fast: dt/dx, dt/dy, dt/(2dx), dt/(2dy), computed once per block

    const GridDesc &g = a.g;
    DevState *st = a.st;
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0)
        st->fill_pending = 0;
    // reference loop condition, Test/Sod/Sod.cpp:123
    if (a.guard && !(st->now_t < a.t_end && st->iter < a.max_iter))
        return;
    const double dt = st->dt;
    const int cur = st->cur;
    const double *__restrict__ U = cur ? a.buf1 : a.buf0;
    double *__restrict__ V = cur ? a.buf0 : a.buf1;
    const long long P = g.plane;
    const int pitch = g.pitch;
    // tiles without fluid cells are skipped: nothing in them is updated or
    // counted by the reference (updates, ComputeDt and CaculateMass all test
    // the cell type), so the launch covers the active tiles only
    const unsigned tile = a.tiles[blockIdx.x];
    const int i0 = g.ng + (int)(tile & 0xFFFFu) * TX;
    const int j0 = g.ng + (int)(tile >> 16) * TY;
    const int tid = threadIdx.x;
    constexpr bool FASTPHYS = FAST || RIE == HLLCT; // faces evaluated by physics_fast.cuh
    if (FASTPHYS && tid == 0)
    {
        sC[0] = dt / g.dx;
        sC[1] = dt / g.dy;
        sC[2] = 0.5 * dt / g.dx;
        sC[3] = 0.5 * dt / g.dy;
    }

    // stage the tile and its halo (always inside the padded array: ng >= 2)
    for (int q = tid; q < 4 * WX * WY; q += NT)
    {
        int k = q / (WX * WY);
        int r = q - k * (WX * WY);
        int ly = r / WX, lx = r - ly * WX;
        int gi = i0 - 2 + lx, gj = j0 - 2 + ly;
        double v = 0.0;
        if (gi < g.M && gj < g.N)
            v = U[k * P + (long long)gj * pitch + gi];
        sU[k][ly][lx] = v;
    }
    __syncthreads();

    const double gam = g.gamma;
    const GasConst<double> K(gam, g.gm1, g.c1, g.c2);
    const double hx2 = FASTPHYS ? sC[2] : 0.0, hy2 = FASTPHYS ? sC[3] : 0.0; // MHM predictor of physics_fast
    constexpr int NXF = (TX + 1) * (TY + 1);
    constexpr int NYF = TX * (TY + 1);
    for (int q = tid; q < NXF + NYF; q += NT)
    {
        double c0[4], c1[4], c2[4], c3[4], f[4];
        if (q < NXF)
        {
            int r = q / (TX + 1), fc = q - r * (TX + 1);
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                c0[k] = sU[k][r + 1][fc];
                c1[k] = sU[k][r + 1][fc + 1];
                c2[k] = sU[k][r + 1][fc + 2];
                c3[k] = sU[k][r + 1][fc + 3];
            }
            if (FASTPHYS)
                x_face_fast<double, SCH, RIE, LIM>(c0, c1, c2, c3, K, hx2, f);
            else
                x_face<SCH, RIE, LIM>(c0, c1, c2, c3, gam, dt, g.dx, f);
#pragma unroll
            for (int k = 0; k < 4; k++)
                sF[k][r][fc] = f[k];
        }
        else
        {
            int qq = q - NXF;
            int r = qq / TX, c = qq - r * TX;
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                c0[k] = sU[k][r][c + 2];
                c1[k] = sU[k][r + 1][c + 2];
                c2[k] = sU[k][r + 2][c + 2];
                c3[k] = sU[k][r + 3][c + 2];
            }
            double stray = 0.0;
            int keep = FASTPHYS ? y_face_fast<double, SCH, RIE, LIM>(c0, c1, c2, c3, K, hy2, f, &stray)
                            : y_face<SCH, RIE, LIM>(c0, c1, c2, c3, gam, dt, g.dy, f, &stray);
#pragma unroll
            for (int k = 0; k < 4; k++)
                sG[k][r][c] = f[k];
            sKeep[r][c] = (unsigned char)keep;
        }
    }
    __syncthreads();

    // update (X then Y, MUSCL_Scheme.cpp:74-88 and :136-150) on fluid cells
    double amax = 0.0, umax = 0.0, vmax = 0.0, mass = 0.0;
    int nans = 0;
    {
        const int c = tid % TX, r = tid / TX;
        const int i = i0 + c, j = j0 + r;
        if (i < g.ng + g.n_x && j < g.ng + g.n_y && a.type[(long long)j * pitch + i] == 0)
        {
            const int kp = sKeep[r + 1][c], km = sKeep[r][c];
            const double lx = FAST ? sC[0] : 0.0, ly = FAST ? sC[1] : 0.0;
            double v[4];
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                double gp = ((kp >> k) & 1) ? sF[k][r + 1][c + 1] : sG[k][r + 1][c];
                double gm = ((km >> k) & 1) ? sF[k][r][c + 1] : sG[k][r][c];
                if (FAST)
                {
                    double x = sU[k][r + 2][c + 2] - lx * (sF[k][r + 1][c + 1] - sF[k][r + 1][c]);
                    v[k] = x - ly * (gp - gm);
                }
                else
                {
                    double x = sU[k][r + 2][c + 2] - dt * (sF[k][r + 1][c + 1] - sF[k][r + 1][c]) / g.dx;
                    v[k] = x - dt * (gp - gm) / g.dy;
                }
                V[k * P + (long long)j * pitch + i] = v[k];
            }
            if (FAST)
                cell_stats_fast(v, K, g.dx * g.dy, amax, umax, vmax, mass, nans);
            else
                cell_stats(v, gam, g.dx, g.dy, amax, umax, vmax, mass, nans);
        }
    }
    block_reduce_finalize<NT>(amax, umax, vmax, mass, nans, st, a.partial, g, true, false);
}

template <int SCH, int RIE, int LIM, int FAST>
void launch_sweep(const SweepArgs &a, dim3 grid, dim3 block, cudaStream_t s)
{
    sweep_kernel<SCH, RIE, LIM, FAST><<<grid, block, 0, s>>>(a);
}

} // namespace ibtfo
