// The fused sweep of the FP32 compensated precision form.
//
// Same tile structure, face reuse and reference semantics as sweep_impl.cuh
// (including the Y-face slot aliasing of the HLL solver), with the state
// held as float (hi, lo) pairs: faces are reconstructed and solved in FP32
// from the hi parts, and the update
//   U_new = U - dt/dx (F(i+1/2) - F(i-1/2)) - dt/dy (G(j+1/2) - G(j-1/2))
// adds the FP32 increment to the (hi, lo) pair with an error-free sum
// (TwoSum, then renormalisation), so the stored state keeps about 48
// significant bits across steps instead of accumulating one FP32 rounding
// per step.  The mass sum and the CFL time step are formed in FP64 once per
// block, from FP32 (compensated for the mass) block reductions.
//
// Memory per cell update: 32 B read (hi, lo x 4) + 32 B write + 1 B type,
// the same bytes as the FP64 path, with the arithmetic on the FP32 pipes.
#pragma once

#include <type_traits>

#include "internal.h"
#include "physics_delta.cuh"
#include "physics_fast.cuh"
#include "sweep_impl.cuh"

namespace ibtfo {

// (hi, lo) - d with an error-free FP32 sum: returns the renormalised pair
__device__ __forceinline__ void two_float_sub(float &hi, float &lo, float d)
{
    const float s = hi - d;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (-d - bb);
    const float l2 = lo + err;
    const float h3 = s + l2;
    lo = l2 - (h3 - s);
    hi = h3;
}

// (h, l) += (oh, ol), error-free on the hi parts (TwoSum)
__device__ __forceinline__ void two_float_acc(float &h, float &l, float oh, float ol)
{
    const float s = h + oh, bb = s - h;
    const float err = (h - (s - bb)) + (oh - bb);
    h = s;
    l = l + ol + err;
}

// (h, l) = ((h, l) + (oh, ol)) / 2 for the second RK2 stage: TwoSum of the
// hi parts, the halving is exact, then renormalisation
__device__ __forceinline__ void two_float_average(float &h, float &l, float oh, float ol)
{
    two_float_acc(h, l, oh, ol);
    h *= 0.5f;
    l *= 0.5f;
    const float s = h + l;
    l = l - (s - h);
    h = s;
}

// per-thread statistics in FP32; the mass as a compensated (hi, lo) pair
struct CellStats32
{
    float amax = 0.0f, umax = 0.0f, vmax = 0.0f, mhi = 0.0f, mlo = 0.0f;
    int nans = 0;
};

template <int TX, int TY>
struct SweepSmem32
{
    float sU[4][TY + 4][TX + 4];
    float sF[4][TY + 1][TX + 1];
    float sG[4][TY + 1][TX];
    float sC[4]; // dt/dx, dt/dy, dt/(2dx), dt/(2dy) of this step (one thread computes them)
    unsigned char sKeep[TY + 1][TX];
    TileFaces<TX, TY> tf; // the faces some fluid cell of the tile reads
};

// Advance the tile whose first interior cell is (i0, j0) from U into V (float
// planes: 0-3 hi, 4-7 lo) and accumulate the statistics of the updated cells.
// Time = RK2: stage 1 gathers no statistics; stage 2 stores the average of
// the advanced state and the pair the output buffer holds (the state at the
// start of the step).
// With `tmap` the tile and halo (hi planes) are staged by one bulk tensor
// copy (column i0 - 2 must be a multiple of 4); a copy that does not
// complete within the bounded wait sets STATUS_STALL and the tile is staged
// element-wise.
template <int SCH, int RIE, int LIM, int TX, int TY, int NT>
__device__ __forceinline__ void sweep_tile32(SweepSmem32<TX, TY> &s, const GridDesc &g, const float *__restrict__ U,
                                             float *__restrict__ V, const uint8_t *__restrict__ type, int i0, int j0,
                                             double dt, CellStats32 &cs, int stage = 0,
                                             const CUtensorMap *tmap = nullptr, int *status = nullptr,
                                             bool interior = false)
{
    constexpr int WX = TX + 4, WY = TY + 4;
    const long long P = g.plane;
    const int pitch = g.pitch;
    const int tid = threadIdx.x;
    if (tid == 0)
    {
        const float dtf = (float)dt;
        s.sC[0] = dtf * g.idxf;
        s.sC[1] = dtf * g.idyf;
        s.sC[2] = 0.5f * s.sC[0];
        s.sC[3] = 0.5f * s.sC[1];
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
    // stage the tile and its halo: one index computation per cell, four planes
    if (!staged)
        for (int q = tid; q < WX * WY; q += NT)
    {
        const int ly = q / WX, lx = q - ly * WX;
        const int gi = i0 - 2 + lx, gj = j0 - 2 + ly;
        float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (gi < g.M && gj < g.N)
        {
            const float *src = U + (long long)gj * pitch + gi;
#pragma unroll
            for (int k = 0; k < 4; k++)
                v[k] = src[k * P];
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
            s.sU[k][ly][lx] = v[k];
    }
    __syncthreads();

    const GasConst<float> K(g.gf, g.gm1f, g.c1f, g.c2f, g.igm1f, g.ig2f);
    const float hx2 = s.sC[2], hy2 = s.sC[3];
    // X faces of the tile's rows (sF rows 1..TY; a warp reads one row of sU:
    // columns 0..TX-1 first, the last column after) and all Y faces; the X
    // faces of the row below the tile follow below, where needed
    constexpr int NXF = TileFaces<TX, TY>::NXF;
    const int nfaces = s.tf.n;
    for (int t = tid; t < nfaces; t += NT)
    {
        const int q = tile_face(s.tf, t);
        float c0[4], c1[4], c2[4], c3[4], f[4];
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
            x_face_fast<float, SCH, RIE, LIM>(c0, c1, c2, c3, K, hx2, f);
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
            float stray = 0.0f;
            int keep = y_face_fast<float, SCH, RIE, LIM>(c0, c1, c2, c3, K, hy2, f, &stray);
#pragma unroll
            for (int k = 0; k < 4; k++)
                s.sG[k][r][c] = f[k];
            s.sKeep[r][c] = (unsigned char)keep;
        }
    }
    __syncthreads();
    // a Y face (i, j - 1/2) that kept the X-face flux of its slot (the
    // reference's Y-solver aliasing) reads the X face (i + 1/2, j - 1): solved
    // here where the list did not (always for the row below the tile)
    for (int q = tid; q < TX * TY; q += NT)
    {
        const int r = q / TX, c = q - r * TX, fc = c + 1;
        if (!s.sKeep[r][c] || x_face_listed(s.tf, r, fc))
            continue;
        float c0[4], c1[4], c2[4], c3[4], f[4];
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            c0[k] = s.sU[k][r + 1][fc];
            c1[k] = s.sU[k][r + 1][fc + 1];
            c2[k] = s.sU[k][r + 1][fc + 2];
            c3[k] = s.sU[k][r + 1][fc + 3];
        }
        x_face_fast<float, SCH, RIE, LIM>(c0, c1, c2, c3, K, hx2, f);
#pragma unroll
        for (int k = 0; k < 4; k++)
            s.sF[k][r][fc] = f[k];
    }
    __syncthreads();

    for (int cell = tid; cell < TX * TY; cell += NT)
    {
        const int c = cell % TX, r = cell / TX;
        const int i = i0 + c, j = j0 + r;
        if (tile_cell_fluid(s.tf, r, c))
        {
            const long long o = (long long)j * pitch + i;
            const int kp = s.sKeep[r + 1][c], km = s.sKeep[r][c];
            const float lx = s.sC[0], ly = s.sC[1];
            float hi[4], lo[4];
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                const float gp = ((kp >> k) & 1) ? s.sF[k][r + 1][c + 1] : s.sG[k][r + 1][c];
                const float gm = ((km >> k) & 1) ? s.sF[k][r][c + 1] : s.sG[k][r][c];
                const float d = fmaf(lx, s.sF[k][r + 1][c + 1] - s.sF[k][r + 1][c], ly * (gp - gm));
                hi[k] = s.sU[k][r + 2][c + 2];
                lo[k] = U[(4 + k) * P + o];
                two_float_sub(hi[k], lo[k], d);
            }
            if constexpr (safeguarded(RIE))
            {
                float e;
                if (pressure_floor_energy(hi, e))
                {
                    hi[3] = e;
                    lo[3] = 0.0f;
                }
            }
            if (stage == 2)
            {
#pragma unroll
                for (int k = 0; k < 4; k++)
                    two_float_average(hi[k], lo[k], V[k * P + o], V[(4 + k) * P + o]);
            }
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                V[k * P + o] = hi[k];
                V[(4 + k) * P + o] = lo[k];
            }
            if (stage == 1)
                continue;
            // CFL statistics (ComputeDt.cpp:38-45) from the hi parts
            const float ir = rcp_t(hi[0]);
            const float u = hi[1] * ir, w = hi[2] * ir;
            const float p = K.gm1 * (hi[3] - 0.5f * hi[0] * (u * u + w * w));
            cs.amax = fmaxf(cs.amax, sqrt_t(K.g * p * ir)); // NaN (ignored by the maximum) where p < 0
            cs.umax = fmaxf(cs.umax, fabsf(u));
            cs.vmax = fmaxf(cs.vmax, fabsf(w));
            two_float_acc(cs.mhi, cs.mlo, hi[0], lo[0]);
            cs.nans += (isnan(hi[0]) || isnan(hi[1]) || isnan(hi[2]) || isnan(hi[3])) ? 1 : 0;
        }
    }
    // a copy that missed the first wait is waited for once more (bounded);
    // the barrier is then released for the next tile of a persistent CTA
    if (tmap && tid == 0 && (staged || mbar_wait(&bar, 0)))
        mbar_inval(&bar);
}

// Shared memory of one FP32 tile in difference form (HLL_Toro): the hi and lo
// planes of the tile and its two-cell halo, and per face P = F - F(lower /
// left cell) and Q = F - F(upper / right cell) (physics_delta.cuh).
template <int TX, int TY>
struct SweepSmem32D
{
    float sU[8][TY + 4][TX + 4]; // planes 0-3 hi, 4-7 lo (the buffer's plane order)
    float sFP[4][TY + 1][TX + 1];
    float sFQ[4][TY + 1][TX + 1];
    float sGP[4][TY + 1][TX];
    float sGQ[4][TY + 1][TX];
    float sC[4];
    unsigned char sKeep[TY + 1][TX]; // no slot reuse under HLL_Toro: cleared, kept for the face list
    TileFaces<TX, TY> tf;
};

// the FP32 tile's shared memory for a Riemann key
template <int RIE, int TX, int TY>
using Smem32 = typename std::conditional<RIE == HLLT, SweepSmem32D<TX, TY>, SweepSmem32<TX, TY>>::type;

// sweep_tile32 for HLL_Toro in difference form: the same tile, face list,
// update, floor, RK2 stages and statistics; the faces store (P, Q) and the
// update takes P_east - Q_west and P_north - Q_south.  With `tmap` the hi
// and lo planes of the box come by two bulk tensor copies (planes 0-3 and
// 4-7 of the case's 8-plane tensor map).
template <int SCH, int RIE, int LIM, int TX, int TY, int NT>
__device__ __forceinline__ void sweep_tile32_delta(SweepSmem32D<TX, TY> &s, const GridDesc &g,
                                                   const float *__restrict__ U, float *__restrict__ V,
                                                   const uint8_t *__restrict__ type, int i0, int j0, double dt,
                                                   CellStats32 &cs, int stage = 0, const CUtensorMap *tmap = nullptr,
                                                   int *status = nullptr, bool interior = false)
{
    constexpr int WX = TX + 4, WY = TY + 4;
    const long long P = g.plane;
    const int pitch = g.pitch;
    const int tid = threadIdx.x;
    if (tid == 0)
    {
        const float dtf = (float)dt;
        s.sC[0] = dtf * g.idxf;
        s.sC[1] = dtf * g.idyf;
        s.sC[2] = 0.5f * s.sC[0];
        s.sC[3] = 0.5f * s.sC[1];
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
            tma_load_3d(&s.sU[4][0][0], tmap, i0 - 2, j0 - 2, 4, &bar);
        }
    }
    tile_faces_build<TX, TY, NT>(s.tf, s.sKeep, g, type, i0, j0, interior);
    if (tmap)
    {
        staged = __syncthreads_and(mbar_wait(&bar, 0));
        // as in sweep_tile32: a missed wait fails the step, the tile is staged
        // element-wise, and the copy is waited for again before the CTA leaves
        if (!staged && tid == 0 && status)
            atomicOr(status, STATUS_STALL);
    }
    if (!staged)
        for (int q = tid; q < WX * WY; q += NT)
        {
            const int ly = q / WX, lx = q - ly * WX;
            const int gi = i0 - 2 + lx, gj = j0 - 2 + ly;
            float v[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            if (gi < g.M && gj < g.N)
            {
                const float *src = U + (long long)gj * pitch + gi;
#pragma unroll
                for (int k = 0; k < 8; k++)
                    v[k] = src[k * P];
            }
#pragma unroll
            for (int k = 0; k < 8; k++)
                s.sU[k][ly][lx] = v[k];
        }
    __syncthreads();

    const GasConst<float> K(g.gf, g.gm1f, g.c1f, g.c2f, g.igm1f, g.ig2f);
    const float hx2 = s.sC[2], hy2 = s.sC[3];
    constexpr int NXF = TileFaces<TX, TY>::NXF;
    const int nfaces = s.tf.n;
    for (int t = tid; t < nfaces; t += NT)
    {
        const int q = tile_face(s.tf, t);
        float h[4][4], l[4][4], fp[4], fq[4];
        if (q < NXF)
        {
            int r, fc;
            x_face_of<TX, TY>(q, r, fc);
#pragma unroll
            for (int n = 0; n < 4; n++)
#pragma unroll
                for (int k = 0; k < 4; k++)
                {
                    h[n][k] = s.sU[k][r + 1][fc + n];
                    l[n][k] = s.sU[4 + k][r + 1][fc + n];
                }
            face_delta<SCH, LIM, 1>(h[0], l[0], h[1], l[1], h[2], l[2], h[3], l[3], K, hx2, fp, fq);
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                s.sFP[k][r][fc] = fp[k];
                s.sFQ[k][r][fc] = fq[k];
            }
        }
        else
        {
            int r, c;
            y_face_of<TX, TY>(q, r, c);
#pragma unroll
            for (int n = 0; n < 4; n++)
#pragma unroll
                for (int k = 0; k < 4; k++)
                {
                    h[n][k] = s.sU[k][r + n][c + 2];
                    l[n][k] = s.sU[4 + k][r + n][c + 2];
                }
            face_delta<SCH, LIM, 2>(h[0], l[0], h[1], l[1], h[2], l[2], h[3], l[3], K, hy2, fp, fq);
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                s.sGP[k][r][c] = fp[k];
                s.sGQ[k][r][c] = fq[k];
            }
        }
    }
    __syncthreads();

    for (int cell = tid; cell < TX * TY; cell += NT)
    {
        const int c = cell % TX, r = cell / TX;
        if (tile_cell_fluid(s.tf, r, c))
        {
            const long long o = (long long)(j0 + r) * pitch + (i0 + c);
            const float lx = s.sC[0], ly = s.sC[1];
            float hi[4], lo[4];
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                // F_e - F_w = P_e - Q_w, G_n - G_s = P_n - Q_s
                const float d = fmaf(lx, s.sFP[k][r + 1][c + 1] - s.sFQ[k][r + 1][c],
                                     ly * (s.sGP[k][r + 1][c] - s.sGQ[k][r][c]));
                hi[k] = s.sU[k][r + 2][c + 2];
                lo[k] = s.sU[4 + k][r + 2][c + 2];
                two_float_sub(hi[k], lo[k], d);
            }
            float e;
            if (pressure_floor_energy(hi, e))
            {
                hi[3] = e;
                lo[3] = 0.0f;
            }
            if (stage == 2)
            {
#pragma unroll
                for (int k = 0; k < 4; k++)
                    two_float_average(hi[k], lo[k], V[k * P + o], V[(4 + k) * P + o]);
            }
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                V[k * P + o] = hi[k];
                V[(4 + k) * P + o] = lo[k];
            }
            if (stage == 1)
                continue;
            const float ir = rcp_t(hi[0]);
            const float u = hi[1] * ir, w = hi[2] * ir;
            const float p = K.gm1 * (hi[3] - 0.5f * hi[0] * (u * u + w * w));
            cs.amax = fmaxf(cs.amax, sqrt_t(K.g * p * ir));
            cs.umax = fmaxf(cs.umax, fabsf(u));
            cs.vmax = fmaxf(cs.vmax, fabsf(w));
            two_float_acc(cs.mhi, cs.mlo, hi[0], lo[0]);
            cs.nans += (isnan(hi[0]) || isnan(hi[1]) || isnan(hi[2]) || isnan(hi[3])) ? 1 : 0;
        }
    }
    // a copy that missed the first wait is waited for once more (bounded);
    // the barrier is then released for the next tile of a persistent CTA
    if (tmap && tid == 0 && (staged || mbar_wait(&bar, 0)))
        mbar_inval(&bar);
}

// Block reduction in FP32 (compensated for the mass); thread 0 converts the
// block's values to FP64 once (an FP64 instruction costs 64 FP32 ones on
// this part), then block_commit_finalize.
template <int NT>
__device__ __forceinline__ void block_reduce_finalize32(CellStats32 cs, DevState *st, double *partial,
                                                        const GridDesc &g, unsigned nblocks, unsigned bid,
                                                        bool first_stage = false)
{
    if (first_stage)
    {
        __syncthreads(); // every thread of the block has stored its cells
        block_commit_finalize<NT>(0, 0, 0, 0, 0, st, partial, g, false, false, nblocks, bid, true);
        return;
    }
    __shared__ float red[5][NT / 32];
    __shared__ int rnan[NT / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        cs.amax = fmaxf(cs.amax, __shfl_xor_sync(0xffffffffu, cs.amax, o));
        cs.umax = fmaxf(cs.umax, __shfl_xor_sync(0xffffffffu, cs.umax, o));
        cs.vmax = fmaxf(cs.vmax, __shfl_xor_sync(0xffffffffu, cs.vmax, o));
        const float oh = __shfl_xor_sync(0xffffffffu, cs.mhi, o), ol = __shfl_xor_sync(0xffffffffu, cs.mlo, o);
        two_float_acc(cs.mhi, cs.mlo, oh, ol);
        cs.nans += __shfl_xor_sync(0xffffffffu, cs.nans, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
    {
        red[0][wid] = cs.amax;
        red[1][wid] = cs.umax;
        red[2][wid] = cs.vmax;
        red[3][wid] = cs.mhi;
        red[4][wid] = cs.mlo;
        rnan[wid] = cs.nans;
    }
    __syncthreads();
    double amax = 0.0, umax = 0.0, vmax = 0.0, mass = 0.0;
    int n = 0;
    if (threadIdx.x == 0)
    {
        float fa = red[0][0], fu = red[1][0], fv = red[2][0], h = red[3][0], l = red[4][0];
        n = rnan[0];
        for (int w = 1; w < NT / 32; w++)
        {
            fa = fmaxf(fa, red[0][w]);
            fu = fmaxf(fu, red[1][w]);
            fv = fmaxf(fv, red[2][w]);
            two_float_acc(h, l, red[3][w], red[4][w]);
            n += rnan[w];
        }
        amax = (double)fa;
        umax = (double)fu;
        vmax = (double)fv;
        mass = ((double)h + (double)l) * g.dxdy;
    }
    block_commit_finalize<NT>(amax, umax, vmax, mass, n, st, partial, g, true, false, nblocks, bid);
}

// one case: one 256-thread CTA per active tile of TILE_X x TY cells (32x8:
// 40 registers, 6 CTAs per SM; 32x16: 5 CTAs per SM; the difference form of
// HLL_Toro: 3 CTAs per SM, its 32x16 tile holding 62 KB of shared memory)
template <int SCH, int RIE, int LIM, int TY>
__global__ void __launch_bounds__(TILE_X *TILE_Y, RIE == HLLT ? 3 : (TY == TILE_Y ? 6 : 5))
    sweep_f32_kernel(const __grid_constant__ SweepArgs a)
{
    constexpr int NT = TILE_X * TILE_Y;
    extern __shared__ __align__(128) unsigned char smem_raw[];

    const GridDesc &g = a.g;
    DevState *st = a.st;
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0)
        st->fill_pending = 0;
    if (a.guard && !(st->now_t < a.t_end && st->iter < a.max_iter))
        return;
    const double dt = st->dt;
    const int cur = st->cur;
    const float *U = reinterpret_cast<const float *>(cur ? a.buf1 : a.buf0);
    float *V = reinterpret_cast<float *>(cur ? a.buf0 : a.buf1);
    const unsigned bid = a.tile0 + blockIdx.x;
    const unsigned tile = a.tiles[bid];
    const int i0 = g.ng + tile_ix(tile) * TILE_X;
    const int j0 = g.ng + tile_jy(tile) * TY;
    const bool interior = (tile & TILE_INTERIOR) != 0;
    CellStats32 cs;
    if constexpr (RIE == HLLT)
        sweep_tile32_delta<SCH, RIE, LIM, TILE_X, TY, NT>(*reinterpret_cast<SweepSmem32D<TILE_X, TY> *>(smem_raw), g,
                                                          U, V, a.type, i0, j0, dt, cs, a.stage,
                                                          a.tma ? &a.tmap[cur] : nullptr, &st->status, interior);
    else
        sweep_tile32<SCH, RIE, LIM, TILE_X, TY, NT>(*reinterpret_cast<SweepSmem32<TILE_X, TY> *>(smem_raw), g, U, V,
                                                    a.type, i0, j0, dt, cs, a.stage, a.tma ? &a.tmap[cur] : nullptr,
                                                    &st->status, interior);
    block_reduce_finalize32<NT>(cs, st, a.partial, g, a.nblocks ? a.nblocks : gridDim.x, bid, a.stage == 1);
}

template <int SCH, int RIE, int LIM, int TY>
void launch_sweep_f32(const SweepArgs &a, dim3 grid, dim3 block, cudaStream_t s)
{
    sweep_f32_kernel<SCH, RIE, LIM, TY><<<grid, block, sizeof(Smem32<RIE, TILE_X, TY>), s>>>(a);
}

// The launcher of one instantiation; a tile whose shared memory exceeds the
// default 48 KB (the difference form's 32x16 tile) has the limit raised on the
// current device, once per device, when a case picks the launcher (outside
// any stream capture).
template <int SCH, int RIE, int LIM, int TY>
SweepLaunch prepared_f32_launcher()
{
    constexpr int smem = (int)sizeof(Smem32<RIE, TILE_X, TY>);
    if (smem > 48 * 1024)
    {
        static std::atomic<unsigned long long> ready{0};
        int dev = 0;
        cudaGetDevice(&dev);
        const unsigned long long bit = 1ull << (dev & 63);
        if (!(ready.load() & bit))
        {
            cudaFuncSetAttribute(sweep_f32_kernel<SCH, RIE, LIM, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem);
            ready.fetch_or(bit);
        }
    }
    return &launch_sweep_f32<SCH, RIE, LIM, TY>;
}

// the launchers of one scheme over TILE_X x TY tiles (nullptr: PVRS, FP64 precisions only)
template <int SCH, int TY>
SweepLaunch select_f32(int riemann, bool vl)
{
    if (riemann == SW)
        return vl ? &launch_sweep_f32<SCH, SW, VANLEER, TY> : &launch_sweep_f32<SCH, SW, MINMOD, TY>;
    if (riemann == HLLCT)
        return vl ? &launch_sweep_f32<SCH, HLLCT, VANLEER, TY> : &launch_sweep_f32<SCH, HLLCT, MINMOD, TY>;
    if (riemann == HLLT)
        return vl ? prepared_f32_launcher<SCH, HLLT, VANLEER, TY>() : prepared_f32_launcher<SCH, HLLT, MINMOD, TY>();
    if (riemann == HLL)
        return vl ? &launch_sweep_f32<SCH, HLL, VANLEER, TY> : &launch_sweep_f32<SCH, HLL, MINMOD, TY>;
    return nullptr;
}

} // namespace ibtfo
