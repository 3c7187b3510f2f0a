// The fused per-step sweep: one CTA advances a TX x TY tile of interior
// cells by one time step.
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
//
// The tile body (sweep_tile64) is shared by two frames: sweep_kernel (one
// case, one CTA per active tile) and the persistent batched kernel of
// batch.cu (many cases, CTAs loop over one tile table).
#pragma once

#include <atomic>

#include "internal.h"
#include "physics.cuh"
#include "physics_fast.cuh"
#include "tile_faces.cuh"
#include "tma.cuh"

namespace ibtfo {

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *addr, double v)
{
    // non-negative doubles order like their bit patterns
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// Commit one block's (max a, max |u|, max |v|, mass, nan count), held by
// thread 0, to the step's device state; the last of the case's `nblocks`
// blocks to finish computes the next dt and advances the reference loop
// accounting.  Deterministic: the mass partials are summed in a fixed order
// (by block index `bid`) whichever block finishes last.  Called by every
// thread of the block.  A first RK2 stage (`first_stage`) commits nothing:
// its last block only hands the stage's buffer to the boundary pass.
template <int NT>
__device__ __forceinline__ void block_commit_finalize(double a, double u, double v, double m, int n, DevState *st,
                                                      double *partial, const GridDesc &g, bool step_accounting,
                                                      bool set_start, unsigned nblocks, unsigned bid,
                                                      bool first_stage = false)
{
    __shared__ bool last;
    if (first_stage)
    {
        if (threadIdx.x == 0)
        {
            __threadfence();
            unsigned t = atomicAdd(&st->ticket, 1u);
            if (t == nblocks - 1)
            {
                volatile DevState *vs = st;
                vs->cur = vs->cur ^ 1;
                vs->fill_pending = 1;
                vs->ticket = 0u;
                __threadfence();
            }
        }
        return;
    }
    if (threadIdx.x == 0)
    {
        if (a > 0) atomic_max_nonneg(&st->amax_bits, a);
        if (u > 0) atomic_max_nonneg(&st->umax_bits, u);
        if (v > 0) atomic_max_nonneg(&st->vmax_bits, v);
        if (n) atomicAdd(&st->nan_step, n);
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
        vs->nan_cells = vs->nan_step;
        vs->nan_step = 0;
        if (vs->nan_cells)
            vs->status |= STATUS_NAN; // sticky: some step held a NaN
        vs->amax_bits = 0ull;
        vs->umax_bits = 0ull;
        vs->vmax_bits = 0ull;
        vs->ticket = 0u;
        __threadfence();
    }
    __syncthreads(); // msum and `last` are reused by the next tile of a persistent CTA
}

// Second RK2 stage: the cell's new state is 0.5 (U0 + w), w the advanced
// first-stage state and U0 the state at the start of the step, which the
// output buffer still holds at this cell (RK2.cpp:41-43 without the
// reference's stride mix-up; the first stage never writes that buffer)
__device__ __forceinline__ void rk2_average(const double *V, long long o, long long P, double v[4])
{
#pragma unroll
    for (int k = 0; k < 4; k++)
        v[k] = 0.5 * (V[k * P + o] + v[k]);
}

// Per-thread CFL maxima, mass and NaN count of the cells a thread updated.
// The sound speed enters as its square (a2max); the block takes one square
// root of the maximum, which equals the maximum of the roots (the root is
// monotone and correctly rounded; NaN and negative squares drop out of both).
struct CellStats
{
    double amax = 0.0, a2max = 0.0, umax = 0.0, vmax = 0.0, mass = 0.0;
    int nans = 0;
};

// Block-wide FP64 reduction of the per-thread statistics, then
// block_commit_finalize.
template <int NT>
__device__ __forceinline__ void block_reduce_finalize(CellStats cs, DevState *st, double *partial, const GridDesc &g,
                                                      bool step_accounting, bool set_start, unsigned nblocks,
                                                      unsigned bid, bool first_stage = false)
{
    if (first_stage)
    {
        __syncthreads(); // every thread of the block has stored its cells
        block_commit_finalize<NT>(0, 0, 0, 0, 0, st, partial, g, false, false, nblocks, bid, true);
        return;
    }
    __shared__ double red[5][NT / 32];
    __shared__ int rnan[NT / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        cs.amax = fmax(cs.amax, __shfl_xor_sync(0xffffffffu, cs.amax, o));
        cs.a2max = fmax(cs.a2max, __shfl_xor_sync(0xffffffffu, cs.a2max, o));
        cs.umax = fmax(cs.umax, __shfl_xor_sync(0xffffffffu, cs.umax, o));
        cs.vmax = fmax(cs.vmax, __shfl_xor_sync(0xffffffffu, cs.vmax, o));
        cs.mass += __shfl_xor_sync(0xffffffffu, cs.mass, o);
        cs.nans += __shfl_xor_sync(0xffffffffu, cs.nans, o);
    }
    if (lane == 0)
    {
        red[0][wid] = cs.amax;
        red[1][wid] = cs.umax;
        red[2][wid] = cs.vmax;
        red[3][wid] = cs.mass;
        red[4][wid] = cs.a2max;
        rnan[wid] = cs.nans;
    }
    __syncthreads();
    double a = 0.0, u = 0.0, v = 0.0, m = 0.0;
    int n = 0;
    if (threadIdx.x == 0)
    {
        double a2 = red[4][0];
        a = red[0][0], u = red[1][0], v = red[2][0], m = red[3][0];
        n = rnan[0];
        for (int w = 1; w < NT / 32; w++)
        {
            a = fmax(a, red[0][w]);
            a2 = fmax(a2, red[4][w]);
            u = fmax(u, red[1][w]);
            v = fmax(v, red[2][w]);
            m += red[3][w];
            n += rnan[w];
        }
        a = fmax(a, sqrt(a2));
    }
    block_commit_finalize<NT>(a, u, v, m, n, st, partial, g, step_accounting, set_start, nblocks, bid);
}

// max(m, x) for m >= 0 as fmax gives it (NaN and negative x leave m), with
// the compare on the integer pipe: non-negative doubles order like their bits
__device__ __forceinline__ double max_nonneg(double m, double x)
{
    const long long bm = __double_as_longlong(m), bx = __double_as_longlong(x);
    return (bx > bm && bx <= 0x7ff0000000000000LL) ? x : m;
}

// any of four values NaN, tested on the integer pipe
__device__ __forceinline__ int any_nan4(const double v[4])
{
    const long long inf = 0x7ff0000000000000LL, mask = 0x7fffffffffffffffLL;
    return ((__double_as_longlong(v[0]) & mask) > inf || (__double_as_longlong(v[1]) & mask) > inf ||
            (__double_as_longlong(v[2]) & mask) > inf || (__double_as_longlong(v[3]) & mask) > inf)
               ? 1
               : 0;
}

// CFL and mass contributions of one fluid cell of the new state
// (ComputeDt.cpp:38-45, CaculateMass.cpp:36)
__device__ __forceinline__ void cell_stats(const double v[4], double gam, double dx, double dy, CellStats &cs)
{
    double rho = v[0];
    double u = v[1] / v[0];
    double w = v[2] / v[0];
    double p = (gam - 1) * (v[3] - 0.5 * rho * (u * u + w * w));
    cs.a2max = max_nonneg(cs.a2max, gam * p / rho); // pow(gam p / rho, 0.5) taken once per block
    cs.umax = max_nonneg(cs.umax, fabs(u));
    cs.vmax = max_nonneg(cs.vmax, fabs(w));
    cs.mass += v[0] * dx * dy;
    cs.nans += any_nan4(v);
}

// the same statistics with a shared reciprocal (fp64_fast)
__device__ __forceinline__ void cell_stats_fast(const double v[4], const GasConst<double> &K, double dxdy,
                                                CellStats &cs)
{
    const double ir = rcp_t(v[0]);
    const double u = v[1] * ir, w = v[2] * ir;
    const double p = K.gm1 * fma(-0.5, fma(v[1], u, v[2] * w), v[3]);
    cs.a2max = max_nonneg(cs.a2max, K.g * ir * p);
    cs.umax = max_nonneg(cs.umax, fabs(u));
    cs.vmax = max_nonneg(cs.vmax, fabs(w));
    cs.mass += v[0] * dxdy;
    cs.nans += any_nan4(v);
}

// shared memory of one FP64 tile: the tile plus two halo cells each side,
// X faces (i+1/2, j) for i in [i0-1, i0+TX), j in [j0-1, j0+TY), Y faces
// (i, j+1/2) for i in [i0, i0+TX), j in [j0-1, j0+TY)
template <int TX, int TY>
struct SweepSmem64
{
    double sU[4][TY + 4][TX + 4];
    double sF[4][TY + 1][TX + 1];
    double sG[4][TY + 1][TX];
    double sC[4]; // fp64_fast: dt/dx, dt/dy, dt/(2dx), dt/(2dy), computed once per tile
    unsigned char sKeep[TY + 1][TX];
    TileFaces<TX, TY> tf; // the faces some fluid cell of the tile reads
};

// Advance the tile whose first interior cell is (i0, j0) from U into V and
// accumulate the statistics of the updated cells.  All NT threads call it.
// stage 2 (the second RK2 stage) stores 0.5 (V + the advanced state) instead,
// V holding the state at the start of the step; stage 1 gathers no statistics.
// With `tmap` the tile and halo are staged by one bulk tensor copy (the box
// starts at column i0 - 2, which must be a multiple of 2); a copy that does
// not complete within the bounded wait sets STATUS_STALL in *status and the
// tile is staged element-wise.
template <int SCH, int RIE, int LIM, int FAST, int TX, int TY, int NT>
__device__ __forceinline__ void sweep_tile64(SweepSmem64<TX, TY> &s, const GridDesc &g, const double *__restrict__ U,
                                             double *__restrict__ V, const uint8_t *__restrict__ type, int i0, int j0,
                                             double dt, CellStats &cs, int stage = 0,
                                             const CUtensorMap *tmap = nullptr, int *status = nullptr,
                                             bool interior = false)
{
    constexpr int WX = TX + 4, WY = TY + 4;
    const long long P = g.plane;
    const int pitch = g.pitch;
    const int tid = threadIdx.x;
    constexpr bool FASTPHYS = FAST || safeguarded(RIE); // faces evaluated by physics_fast.cuh
    if (FASTPHYS && tid == 0)
    {
        s.sC[0] = dt * g.idx;
        s.sC[1] = dt * g.idy;
        s.sC[2] = 0.5 * s.sC[0];
        s.sC[3] = 0.5 * s.sC[1];
    }

    bool staged = false;
    __shared__ uint64_t bar;
    if (tmap)
    {
        if (tid == 0)
            mbar_init(&bar, 1);
        __syncthreads();
        if (tid == 0)
        {
            mbar_expect_tx(&bar, (unsigned)sizeof(s.sU));
            tma_load_3d(&s.sU[0][0][0], tmap, i0 - 2, j0 - 2, 0, &bar);
        }
    }
    // cell flags and the face list while the copy is in flight
    tile_faces_build<TX, TY, NT>(s.tf, s.sKeep, g, type, i0, j0, interior);
    if (tmap)
    {
        staged = __syncthreads_and(mbar_wait(&bar, 0));
        // a copy that missed the bounded wait: the step is reported as failed
        // (STATUS_STALL makes the host return IBTFO_ETIMEOUT); the tile is
        // staged element-wise and, before the CTA leaves the tile, the copy is
        // waited for once more, so that a late copy lands while this CTA
        // still owns the shared memory (it brings the values staged here)
        if (!staged && tid == 0 && status)
            atomicOr(status, STATUS_STALL);
    }
    // stage the tile and its halo (always inside the padded array: ng >= 2),
    // one index computation per cell for the four planes
    if (!staged)
        for (int q = tid; q < WX * WY; q += NT)
    {
        const int ly = q / WX, lx = q - ly * WX;
        const int gi = i0 - 2 + lx, gj = j0 - 2 + ly;
        double v[4] = {0.0, 0.0, 0.0, 0.0};
        if (gi < g.M && gj < g.N)
        {
            const double *src = U + (long long)gj * pitch + gi;
#pragma unroll
            for (int k = 0; k < 4; k++)
                v[k] = src[k * P];
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
            s.sU[k][ly][lx] = v[k];
    }
    __syncthreads();

    const double gam = g.gamma;
    const GasConst<double> K(gam, g.gm1, g.c1, g.c2, g.igm1, g.ig2);
    const double hx2 = FASTPHYS ? s.sC[2] : 0.0, hy2 = FASTPHYS ? s.sC[3] : 0.0; // MHM predictor of physics_fast
    // X faces of the tile's rows (sF rows 1..TY) and all Y faces; the X faces
    // of the row below the tile (sF row 0) follow below, where needed
    constexpr int NXF = TileFaces<TX, TY>::NXF;
    const int nfaces = s.tf.n;
    for (int t = tid; t < nfaces; t += NT)
    {
        const int q = tile_face(s.tf, t);
        double c0[4], c1[4], c2[4], c3[4], f[4];
        if (q < NXF)
        {
            int r, fc;
            x_face_of<TX, TY>(q, r, fc);
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                c0[k] = s.sU[k][r + 1][fc];
                c1[k] = s.sU[k][r + 1][fc + 1];
                c2[k] = s.sU[k][r + 1][fc + 2];
                c3[k] = s.sU[k][r + 1][fc + 3];
            }
            if (FASTPHYS)
                x_face_fast<double, SCH, RIE, LIM>(c0, c1, c2, c3, K, hx2, f);
            else
                x_face<SCH, RIE, LIM>(c0, c1, c2, c3, gam, dt, g.dx, f);
#pragma unroll
            for (int k = 0; k < 4; k++)
                s.sF[k][r][fc] = f[k];
        }
        else
        {
            int r, c;
            y_face_of<TX, TY>(q, r, c);
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                c0[k] = s.sU[k][r][c + 2];
                c1[k] = s.sU[k][r + 1][c + 2];
                c2[k] = s.sU[k][r + 2][c + 2];
                c3[k] = s.sU[k][r + 3][c + 2];
            }
            double stray = 0.0;
            int keep = FASTPHYS ? y_face_fast<double, SCH, RIE, LIM>(c0, c1, c2, c3, K, hy2, f, &stray)
                                : y_face<SCH, RIE, LIM>(c0, c1, c2, c3, gam, dt, g.dy, f, &stray);
            if constexpr (RIE == PVRS)
            {
                // the reference's PVRS stray store from cell 7 c' + 2 into this face's
                // energy flux (physics.cuh, pvrs_stray_source)
                const long long lin = (long long)g.M * (j0 - 1 + r) + (i0 + c);
                const long long src = 7 * lin + 2;
                double sv;
                if (i0 + c < g.M && src < (long long)g.M * g.N &&
                    pvrs_stray_source<SCH, LIM>(U, P, pitch, g.M, g.N, g.ng, gam, dt, g.dx, g.dy,
                                                (int)(src % g.M), (int)(src / g.M), &sv))
                {
                    f[3] = sv;
                    keep &= ~8;
                }
            }
#pragma unroll
            for (int k = 0; k < 4; k++)
                s.sG[k][r][c] = f[k];
            s.sKeep[r][c] = (unsigned char)keep;
        }
    }
    __syncthreads();
    // a Y face (i, j - 1/2) that kept the X-face flux of its slot, as the
    // reference's Y solver does in some branches, reads the X face
    // (i + 1/2, j - 1): solved here where the list did not (always for the
    // row below the tile)
    for (int q = tid; q < TX * TY; q += NT)
    {
        const int r = q / TX, c = q - r * TX, fc = c + 1;
        if (!s.sKeep[r][c] || x_face_listed(s.tf, r, fc))
            continue;
        double c0[4], c1[4], c2[4], c3[4], f[4];
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            c0[k] = s.sU[k][r + 1][fc];
            c1[k] = s.sU[k][r + 1][fc + 1];
            c2[k] = s.sU[k][r + 1][fc + 2];
            c3[k] = s.sU[k][r + 1][fc + 3];
        }
        if (FASTPHYS)
            x_face_fast<double, SCH, RIE, LIM>(c0, c1, c2, c3, K, hx2, f);
        else
            x_face<SCH, RIE, LIM>(c0, c1, c2, c3, gam, dt, g.dx, f);
#pragma unroll
        for (int k = 0; k < 4; k++)
            s.sF[k][r][fc] = f[k];
    }
    __syncthreads();

    // update (X then Y, MUSCL_Scheme.cpp:74-88 and :136-150) on fluid cells
    for (int cell = tid; cell < TX * TY; cell += NT)
    {
        const int c = cell % TX, r = cell / TX;
        const int i = i0 + c, j = j0 + r;
        if (tile_cell_fluid(s.tf, r, c))
        {
            const int kp = s.sKeep[r + 1][c], km = s.sKeep[r][c];
            const double lx = FAST ? s.sC[0] : 0.0, ly = FAST ? s.sC[1] : 0.0;
            double v[4];
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                double gp = ((kp >> k) & 1) ? s.sF[k][r + 1][c + 1] : s.sG[k][r + 1][c];
                double gm = ((km >> k) & 1) ? s.sF[k][r][c + 1] : s.sG[k][r][c];
                if (FAST)
                {
                    double x = s.sU[k][r + 2][c + 2] - lx * (s.sF[k][r + 1][c + 1] - s.sF[k][r + 1][c]);
                    v[k] = x - ly * (gp - gm);
                }
                else
                {
                    double x = s.sU[k][r + 2][c + 2] - dt * (s.sF[k][r + 1][c + 1] - s.sF[k][r + 1][c]) / g.dx;
                    v[k] = x - dt * (gp - gm) / g.dy;
                }
            }
            if constexpr (safeguarded(RIE))
                pressure_floor(v);
            if (stage == 2)
                rk2_average(V, (long long)j * pitch + i, P, v);
#pragma unroll
            for (int k = 0; k < 4; k++)
                V[k * P + (long long)j * pitch + i] = v[k];
            if (stage == 1)
                continue;
            if (FAST)
                cell_stats_fast(v, K, g.dxdy, cs);
            else
                cell_stats(v, gam, g.dx, g.dy, cs);
        }
    }
    // a copy that missed the first wait is waited for once more (bounded);
    // the barrier is then released for the next tile of a persistent CTA
    if (tmap && tid == 0 && (staged || mbar_wait(&bar, 0)))
        mbar_inval(&bar);
}

// one case: one CTA of TILE_X x TILE_Y threads per active tile of TILE_X x TY
// cells.  fp64_fast with HLL or Steger-Warming: 32x8 tiles in 64 registers
// (4 CTAs per SM); 32x16 tiles in 85 registers (3 CTAs per SM, 59 KB of
// shared memory each), which measured 4% faster than 512 threads per tile.
template <int SCH, int RIE, int LIM, int FAST, int TY>
__global__ void __launch_bounds__(TILE_X *TILE_Y, (FAST && (RIE == HLL || RIE == SW)) ? (TY == TILE_Y ? 4 : 3) : 1)
    sweep_kernel(const __grid_constant__ SweepArgs a)
{
    constexpr int NT = TILE_X * TILE_Y;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    auto &s = *reinterpret_cast<SweepSmem64<TILE_X, TY> *>(smem_raw);

    const GridDesc &g = a.g;
    DevState *st = a.st;
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0)
        st->fill_pending = 0;
    // reference loop condition, Test/Sod/Sod.cpp:123
    if (a.guard && !(st->now_t < a.t_end && st->iter < a.max_iter))
        return;
    const double dt = st->dt;
    const int cur = st->cur;
    const double *U = cur ? a.buf1 : a.buf0;
    double *V = cur ? a.buf0 : a.buf1;
    // tiles without fluid cells are skipped: nothing in them is updated or
    // counted by the reference (updates, ComputeDt and CaculateMass all test
    // the cell type), so the launch covers the active tiles only
    const unsigned bid = a.tile0 + blockIdx.x;
    const unsigned tile = a.tiles[bid];
    const int i0 = g.ng + tile_ix(tile) * TILE_X;
    const int j0 = g.ng + tile_jy(tile) * TY;
    const bool interior = (tile & TILE_INTERIOR) != 0;
    CellStats cs;
    sweep_tile64<SCH, RIE, LIM, FAST, TILE_X, TY, NT>(s, g, U, V, a.type, i0, j0, dt, cs, a.stage,
                                                      a.tma ? &a.tmap[cur] : nullptr, &st->status, interior);
    block_reduce_finalize<NT>(cs, st, a.partial, g, true, false, a.nblocks ? a.nblocks : gridDim.x, bid,
                              a.stage == 1);
}

template <int SCH, int RIE, int LIM, int FAST, int TY = TILE_Y>
void launch_sweep(const SweepArgs &a, dim3 grid, dim3 block, cudaStream_t s)
{
    sweep_kernel<SCH, RIE, LIM, FAST, TY><<<grid, block, sizeof(SweepSmem64<TILE_X, TY>), s>>>(a);
}

// The launcher of one instantiation.  A 32 x FAST_TILE_Y tile's shared memory
// (59 KB) exceeds the default 48 KB limit: the limit is raised on the current
// device, once per device, when a case picks the launcher (outside any
// stream capture).
template <int SCH, int RIE, int LIM, int FAST, int TY>
SweepLaunch prepared_sweep_launcher()
{
    constexpr int smem = (int)sizeof(SweepSmem64<TILE_X, TY>);
    if (smem > 48 * 1024)
    {
        static std::atomic<unsigned long long> ready{0};
        int dev = 0;
        cudaGetDevice(&dev);
        const unsigned long long bit = 1ull << (dev & 63);
        if (!(ready.load() & bit))
        {
            cudaFuncSetAttribute(sweep_kernel<SCH, RIE, LIM, FAST, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem);
            ready.fetch_or(bit);
        }
    }
    return &launch_sweep<SCH, RIE, LIM, FAST, TY>;
}

} // namespace ibtfo
