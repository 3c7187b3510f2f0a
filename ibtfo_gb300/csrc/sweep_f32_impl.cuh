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
// per step.  The mass sum and the CFL time step are formed in FP64.
//
// Memory per cell update: 32 B read (hi, lo x 4) + 32 B write + 1 B type,
// the same bytes as the FP64 path but a quarter of the FP64 instructions run
// on the FP32 pipes, so this form can approach the HBM bound.
#pragma once

#include "internal.h"
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

template <int SCH, int RIE, int LIM>
__global__ void __launch_bounds__(TILE_X *TILE_Y) sweep_f32_kernel(const SweepArgs a)
{
    constexpr int TX = TILE_X, TY = TILE_Y, NT = TX * TY;
    constexpr int WX = TX + 4, WY = TY + 4;
    __shared__ float sU[4][WY][WX];
    __shared__ float sF[4][TY + 1][TX + 1];
    __shared__ float sG[4][TY + 1][TX];
    __shared__ unsigned char sKeep[TY + 1][TX];
    __shared__ float sC[4]; // dt/dx, dt/dy, dt/(2dx), dt/(2dy) of this step (one thread computes them)

    const GridDesc &g = a.g;
    DevState *st = a.st;
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0)
        st->fill_pending = 0;
    if (a.guard && !(st->now_t < a.t_end && st->iter < a.max_iter))
        return;
    const double dt = st->dt; // read by thread 0 into sC
    const int cur = st->cur;
    const float *__restrict__ U = reinterpret_cast<const float *>(cur ? a.buf1 : a.buf0);
    float *__restrict__ V = reinterpret_cast<float *>(cur ? a.buf0 : a.buf1);
    const long long P = g.plane;
    const int pitch = g.pitch;
    const unsigned tile = a.tiles[blockIdx.x];
    const int i0 = g.ng + (int)(tile & 0xFFFFu) * TX;
    const int j0 = g.ng + (int)(tile >> 16) * TY;
    const int tid = threadIdx.x;
    if (tid == 0)
    {
        sC[0] = (float)(dt / g.dx);
        sC[1] = (float)(dt / g.dy);
        sC[2] = (float)(0.5 * dt / g.dx);
        sC[3] = (float)(0.5 * dt / g.dy);
    }

    for (int q = tid; q < 4 * WX * WY; q += NT)
    {
        int k = q / (WX * WY);
        int r = q - k * (WX * WY);
        int ly = r / WX, lx = r - ly * WX;
        int gi = i0 - 2 + lx, gj = j0 - 2 + ly;
        float v = 0.0f;
        if (gi < g.M && gj < g.N)
            v = U[k * P + (long long)gj * pitch + gi];
        sU[k][ly][lx] = v;
    }
    __syncthreads();

    const GasConst<float> K(g.gf, g.gm1f, g.c1f, g.c2f);
    const float hx2 = sC[2], hy2 = sC[3];
    constexpr int NXF = (TX + 1) * (TY + 1);
    constexpr int NYF = TX * (TY + 1);
    for (int q = tid; q < NXF + NYF; q += NT)
    {
        float c0[4], c1[4], c2[4], c3[4], f[4];
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
            x_face_fast<float, SCH, RIE, LIM>(c0, c1, c2, c3, K, hx2, f);
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
            float stray = 0.0f;
            int keep = y_face_fast<float, SCH, RIE, LIM>(c0, c1, c2, c3, K, hy2, f, &stray);
#pragma unroll
            for (int k = 0; k < 4; k++)
                sG[k][r][c] = f[k];
            sKeep[r][c] = (unsigned char)keep;
        }
    }
    __syncthreads();

    // per-cell statistics in FP32; the mass as a compensated (hi, lo) float
    // pair, converted to FP64 once per warp
    float famax = 0.0f, fumax = 0.0f, fvmax = 0.0f, mhi = 0.0f, mlo = 0.0f;
    int nans = 0;
    {
        const int c = tid % TX, r = tid / TX;
        const int i = i0 + c, j = j0 + r;
        if (i < g.ng + g.n_x && j < g.ng + g.n_y && a.type[(long long)j * pitch + i] == 0)
        {
            const long long o = (long long)j * pitch + i;
            const int kp = sKeep[r + 1][c], km = sKeep[r][c];
            const float lx = sC[0], ly = sC[1];
            float hi[4], lo[4];
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                const float gp = ((kp >> k) & 1) ? sF[k][r + 1][c + 1] : sG[k][r + 1][c];
                const float gm = ((km >> k) & 1) ? sF[k][r][c + 1] : sG[k][r][c];
                const float d = fmaf(lx, sF[k][r + 1][c + 1] - sF[k][r + 1][c], ly * (gp - gm));
                hi[k] = sU[k][r + 2][c + 2];
                lo[k] = U[(4 + k) * P + o];
                two_float_sub(hi[k], lo[k], d);
                V[k * P + o] = hi[k];
                V[(4 + k) * P + o] = lo[k];
            }
            // CFL statistics (ComputeDt.cpp:38-45) from the hi parts
            const float ir = rcp_t(hi[0]);
            const float u = hi[1] * ir, w = hi[2] * ir;
            const float p = K.gm1 * (hi[3] - 0.5f * hi[0] * (u * u + w * w));
            famax = sqrtf(K.g * p * ir); // NaN (ignored by the maximum) where p < 0
            fumax = fabsf(u);
            fvmax = fabsf(w);
            mhi = hi[0];
            mlo = lo[0];
            nans = (isnan(hi[0]) || isnan(hi[1]) || isnan(hi[2]) || isnan(hi[3])) ? 1 : 0;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        famax = fmaxf(famax, __shfl_xor_sync(0xffffffffu, famax, o));
        fumax = fmaxf(fumax, __shfl_xor_sync(0xffffffffu, fumax, o));
        fvmax = fmaxf(fvmax, __shfl_xor_sync(0xffffffffu, fvmax, o));
        // (mhi, mlo) += the partner's pair, error-free on the hi parts
        const float oh = __shfl_xor_sync(0xffffffffu, mhi, o), ol = __shfl_xor_sync(0xffffffffu, mlo, o);
        const float s = mhi + oh, bb = s - mhi;
        const float err = (mhi - (s - bb)) + (oh - bb);
        mhi = s;
        mlo = mlo + ol + err;
    }
    // one FP64 value per warp: the lane-0 value carries the warp's sums
    const bool lead = (threadIdx.x & 31) == 0;
    const double amax = lead ? (double)famax : 0.0, umax = lead ? (double)fumax : 0.0,
                 vmax = lead ? (double)fvmax : 0.0;
    const double mass = lead ? ((double)mhi + (double)mlo) * (g.dx * g.dy) : 0.0;
    block_reduce_finalize<NT, true>(amax, umax, vmax, mass, nans, st, a.partial, g, true, false);
}

template <int SCH, int RIE, int LIM>
void launch_sweep_f32(const SweepArgs &a, dim3 grid, dim3 block, cudaStream_t s)
{
    sweep_f32_kernel<SCH, RIE, LIM><<<grid, block, 0, s>>>(a);
}

} // namespace ibtfo
