// The fused sweep of a cut-cell case (BC_CCM).  No counterpart in the
// reference, which has no cut-cell method: this is a Cartesian cut-cell
// finite-volume update written from the literature.
//
// One CTA per active 32x8 tile, as in sweep_impl.cuh, with the cell types of
// the tile and its halo staged beside the state:
//   * faces: every X and Y face of the tile; a face whose four-cell stencil
//     touches a cut or solid cell takes the first-order pair (the two cell
//     averages), the others the scheme's reconstruction (and MHM predictor);
//     plain HLL in both directions, Steger-Warming or the contact-restoring HLLC;
//   * full fluid cells: the usual update, in the precision's arithmetic;
//   * cut cells, in FP64 (they divide by the volume fraction):
//       alpha U' = alpha U - dt/dx (A_e F_e - A_w F_w) - dt/dy (A_n G_n - A_s G_s)
//                  - dt/(dx dy) L W,
//     A the face apertures, (n L) = ((A_w - A_e) dy, (A_s - A_n) dx) the
//     outward wall normal times the wall length, W the wall flux of the
//     mirrored-state Riemann problem (ccm_wall_flux);
//   * statistics: mass sum alpha rho over full and cut cells; CFL maxima over
//     full cells and cut cells with alpha >= 0.5 (smaller cells are mixed with
//     their neighbours right after the sweep, so they do not limit dt).
// The small-cell mixing that follows is in ccm_geometry.cu.
#pragma once

#include <type_traits>

#include "sweep_f32_impl.cuh"
#include "sweep_impl.cuh"

namespace ibtfo {

template <typename T, int TX, int TY>
struct CcmSmem
{
    T sU[4][TY + 4][TX + 4];
    T sF[4][TY + 1][TX + 1];
    T sG[4][TY + 1][TX];
    T sC[4];
    uint8_t sT[TY + 4][TX + 4];
};

__device__ __forceinline__ bool low_order_cell(uint8_t t) { return t == CELL_SOLID || t == CELL_CUT; }

// a face term A F where only A > 0 faces carry a flux (faces beside solid
// cells have A = 0 and a meaningless F)
__device__ __forceinline__ double face_term(double A, double F) { return (A > 0.0) ? A * F : 0.0; }

// rows of a cut-cell tile: 32x16 in the FP32 form (256 threads, two cells
// each: fewer faces and staged cells per cell), 32x8 in FP64
template <int PREC>
constexpr int ccm_tile_rows()
{
    return PREC == 2 ? FAST_TILE_Y : TILE_Y;
}

template <int SCH, int RIE, int LIM, int PREC>
__global__ void __launch_bounds__(TILE_X *TILE_Y, PREC == 2 ? 4 : 1) ccm_sweep_kernel(const CcmArgs ca)
{
    using T = typename std::conditional<PREC == 2, float, double>::type;
    constexpr int TX = TILE_X, TY = ccm_tile_rows<PREC>(), NT = TILE_X * TILE_Y, WX = TX + 4, WY = TY + 4;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    auto &s = *reinterpret_cast<CcmSmem<T, TX, TY> *>(smem_raw);

    const SweepArgs &a = ca.s;
    const GridDesc &g = a.g;
    DevState *st = a.st;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        st->fill_pending = 0;
    if (a.guard && !(st->now_t < a.t_end && st->iter < a.max_iter))
        return;
    const double dt = st->dt;
    const int cur = st->cur;
    const double *Ud = cur ? a.buf1 : a.buf0;
    double *Vd = cur ? a.buf0 : a.buf1;
    const T *U = reinterpret_cast<const T *>(Ud); // FP64 planes, or the FP32 hi planes 0-3
    T *V = reinterpret_cast<T *>(Vd);
    const long long P = g.plane;
    const int pitch = g.pitch;
    const unsigned tile = a.tiles[blockIdx.x];
    const int i0 = g.ng + tile_ix(tile) * TX;
    const int j0 = g.ng + tile_jy(tile) * TY;
    const int tid = threadIdx.x;
    if (tid == 0)
    {
        if constexpr (PREC == 2)
        {
            const float dtf = (float)dt;
            s.sC[0] = dtf * g.idxf;
            s.sC[1] = dtf * g.idyf;
        }
        else
        {
            s.sC[0] = dt * g.idx;
            s.sC[1] = dt * g.idy;
        }
        s.sC[2] = (T)0.5 * s.sC[0];
        s.sC[3] = (T)0.5 * s.sC[1];
    }
    // stage the tile, its halo and their cell types: one index computation per cell
    for (int q = tid; q < WX * WY; q += NT)
    {
        const int ly = q / WX, lx = q - ly * WX;
        const int gi = i0 - 2 + lx, gj = j0 - 2 + ly;
        T v[4] = {(T)0, (T)0, (T)0, (T)0};
        uint8_t t = (uint8_t)CELL_SOLID;
        if (gi < g.M && gj < g.N)
        {
            const long long o = (long long)gj * pitch + gi;
#pragma unroll
            for (int k = 0; k < 4; k++)
                v[k] = U[k * P + o];
            t = a.type[o];
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
            s.sU[k][ly][lx] = v[k];
        s.sT[ly][lx] = t;
    }
    __syncthreads();

    GasConst<T> K = (PREC == 2) ? GasConst<T>(g.gf, g.gm1f, g.c1f, g.c2f, g.igm1f, g.ig2f)
                                : GasConst<T>(g.gamma, g.gm1, g.c1, g.c2, g.igm1, g.ig2);
    const T hx2 = s.sC[2], hy2 = s.sC[3];
    // X faces of the tile's rows (sF rows 1..TY; a warp reads one row of sU:
    // columns 0..TX-1 first, the last column after) and all Y faces
    constexpr int NXF = (TX + 1) * TY;
    constexpr int NYF = TX * (TY + 1);
    for (int q = tid; q < NXF + NYF; q += NT)
    {
        T c0[4], c1[4], c2[4], c3[4], f[4];
        if (q < NXF)
        {
            int r, fc;
            if (q < TX * TY)
                r = q / TX + 1, fc = q - (r - 1) * TX;
            else
                r = q - TX * TY + 1, fc = TX;
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                c0[k] = s.sU[k][r + 1][fc];
                c1[k] = s.sU[k][r + 1][fc + 1];
                c2[k] = s.sU[k][r + 1][fc + 2];
                c3[k] = s.sU[k][r + 1][fc + 3];
            }
            const bool lo = low_order_cell(s.sT[r + 1][fc]) || low_order_cell(s.sT[r + 1][fc + 1]) ||
                            low_order_cell(s.sT[r + 1][fc + 2]) || low_order_cell(s.sT[r + 1][fc + 3]);
            ccm_face<T, 1, SCH, RIE, LIM>(c0, c1, c2, c3, K, hx2, lo, f);
#pragma unroll
            for (int k = 0; k < 4; k++)
                s.sF[k][r][fc] = f[k];
        }
        else
        {
            const int qq = q - NXF;
            const int r = qq / TX, c = qq - r * TX;
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                c0[k] = s.sU[k][r][c + 2];
                c1[k] = s.sU[k][r + 1][c + 2];
                c2[k] = s.sU[k][r + 2][c + 2];
                c3[k] = s.sU[k][r + 3][c + 2];
            }
            const bool lo = low_order_cell(s.sT[r][c + 2]) || low_order_cell(s.sT[r + 1][c + 2]) ||
                            low_order_cell(s.sT[r + 2][c + 2]) || low_order_cell(s.sT[r + 3][c + 2]);
            ccm_face<T, 2, SCH, RIE, LIM>(c0, c1, c2, c3, K, hy2, lo, f);
#pragma unroll
            for (int k = 0; k < 4; k++)
                s.sG[k][r][c] = f[k];
        }
    }
    __syncthreads();

    using Stats = typename std::conditional<PREC == 2, CellStats32, CellStats>::type;
    Stats cs;
#pragma unroll 1
    for (int q = tid; q < TX * TY; q += NT)
    {
        const int c = q % TX, r = q / TX;
        const int i = i0 + c, j = j0 + r;
        const uint8_t t = s.sT[r + 2][c + 2];
        const long long o = (long long)j * pitch + i;
        if (i < g.ng + g.n_x && j < g.ng + g.n_y && t == CELL_FLUID)
        {
            const T lx = s.sC[0], ly = s.sC[1];
            if constexpr (PREC == 2)
            {
                float hi[4], lo[4];
#pragma unroll
                for (int k = 0; k < 4; k++)
                {
                    const float d = fmaf(lx, s.sF[k][r + 1][c + 1] - s.sF[k][r + 1][c],
                                         ly * (s.sG[k][r + 1][c] - s.sG[k][r][c]));
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
#pragma unroll
                for (int k = 0; k < 4; k++)
                {
                    V[k * P + o] = hi[k];
                    V[(4 + k) * P + o] = lo[k];
                }
                const float ir = rcp_t(hi[0]);
                const float u = hi[1] * ir, w = hi[2] * ir;
                const float p = K.gm1 * (hi[3] - 0.5f * hi[0] * (u * u + w * w));
                cs.amax = fmaxf(cs.amax, sqrt_t(K.g * p * ir));
                cs.umax = fmaxf(cs.umax, fabsf(u));
                cs.vmax = fmaxf(cs.vmax, fabsf(w));
                two_float_acc(cs.mhi, cs.mlo, hi[0], lo[0]);
                cs.nans += (isnan(hi[0]) || isnan(hi[1]) || isnan(hi[2]) || isnan(hi[3])) ? 1 : 0;
            }
            else
            {
                double v[4];
#pragma unroll
                for (int k = 0; k < 4; k++)
                {
                    const double x = s.sU[k][r + 2][c + 2] - lx * (s.sF[k][r + 1][c + 1] - s.sF[k][r + 1][c]);
                    v[k] = x - ly * (s.sG[k][r + 1][c] - s.sG[k][r][c]);
                }
                if constexpr (safeguarded(RIE))
                    pressure_floor(v);
#pragma unroll
                for (int k = 0; k < 4; k++)
                    V[k * P + o] = v[k];
                cell_stats_fast(v, K, g.dxdy, cs);
            }
        }
        else if (i < g.ng + g.n_x && j < g.ng + g.n_y && t == CELL_CUT)
        {
            // FP64: the cell's full state (hi + lo in the FP32 form), apertures,
            // volume fraction and the wall
            const double al = ca.alpha[o];
            const double aw = ca.ax[o - 1], ae = ca.ax[o], as = ca.ay[o - pitch], an = ca.ay[o];
            const double nLx = (aw - ae) * g.dy, nLy = (as - an) * g.dx;
            const double L = sqrt(nLx * nLx + nLy * nLy);
            double W[4] = {0.0, 0.0, 0.0, 0.0};
            if (L > 0.0)
            {
                T Uc[4], Wt[4];
#pragma unroll
                for (int k = 0; k < 4; k++)
                    Uc[k] = s.sU[k][r + 2][c + 2];
                ccm_wall_flux<T, RIE>(Uc, (T)(nLx / L), (T)(nLy / L), K, Wt);
#pragma unroll
                for (int k = 0; k < 4; k++)
                    W[k] = (double)Wt[k];
            }
            const double lxd = dt / g.dx, lyd = dt / g.dy, lw = dt / (g.dx * g.dy) * L;
            double v[4];
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                const double u0 = state_ld(Ud, k, o, g);
                const double fx = face_term(ae, (double)s.sF[k][r + 1][c + 1]) - face_term(aw, (double)s.sF[k][r + 1][c]);
                const double gy = face_term(an, (double)s.sG[k][r + 1][c]) - face_term(as, (double)s.sG[k][r][c]);
                v[k] = (al * u0 - lxd * fx - lyd * gy - lw * W[k]) / al;
            }
            // the floor only where no mixing follows: a small cell's swept state
            // is provisional (divided by a small alpha) until it is mixed
            if constexpr (safeguarded(RIE))
                if (al >= 0.5)
                    pressure_floor(v);
#pragma unroll
            for (int k = 0; k < 4; k++)
                state_st(Vd, k, o, v[k], g);
            // statistics: mass alpha rho; CFL only from cells that are not mixed
            const double m = al * v[0];
            const bool cfl = al >= 0.5;
            const double ir = 1.0 / v[0];
            const double uu = v[1] * ir, ww = v[2] * ir;
            const double p = (g.gamma - 1.0) * (v[3] - 0.5 * v[0] * (uu * uu + ww * ww));
            const double snd = sqrt(g.gamma * p * ir);
            const int bad = (isnan(v[0]) || isnan(v[1]) || isnan(v[2]) || isnan(v[3])) ? 1 : 0;
            if constexpr (PREC == 2)
            {
                const float mh = (float)m;
                two_float_acc(cs.mhi, cs.mlo, mh, (float)(m - (double)mh));
                if (cfl)
                {
                    cs.amax = fmaxf(cs.amax, (float)snd);
                    cs.umax = fmaxf(cs.umax, (float)fabs(uu));
                    cs.vmax = fmaxf(cs.vmax, (float)fabs(ww));
                }
                cs.nans += bad;
            }
            else
            {
                cs.mass += m * g.dxdy;
                if (cfl)
                {
                    cs.amax = fmax(cs.amax, snd);
                    cs.umax = fmax(cs.umax, fabs(uu));
                    cs.vmax = fmax(cs.vmax, fabs(ww));
                }
                cs.nans += bad;
            }
        }
    }
    if constexpr (PREC == 2)
        block_reduce_finalize32<NT>(cs, st, a.partial, g, gridDim.x * gridDim.y, blockIdx.y * gridDim.x + blockIdx.x);
    else
        block_reduce_finalize<NT>(cs, st, a.partial, g, true, false, gridDim.x * gridDim.y,
                                  blockIdx.y * gridDim.x + blockIdx.x);
}

template <int SCH, int RIE, int LIM, int PREC>
void launch_ccm_sweep(const CcmArgs &a, dim3 grid, dim3 block, cudaStream_t s)
{
    using T = typename std::conditional<PREC == 2, float, double>::type;
    ccm_sweep_kernel<SCH, RIE, LIM, PREC><<<grid, block, sizeof(CcmSmem<T, TILE_X, ccm_tile_rows<PREC>()>), s>>>(a);
}

// every Riemann solver and limiter of one scheme and precision: HLL_Toro,
// Steger-Warming, HLLC_Toro (the reference's HLL and PVRS have no cut-cell
// form)
template <int SCH, int PREC>
CcmLaunch ccm_launcher_scheme(int riemann, int limiter)
{
    const bool vl = (limiter == VANLEER);
    switch (riemann)
    {
    case SW: return vl ? &launch_ccm_sweep<SCH, SW, VANLEER, PREC> : &launch_ccm_sweep<SCH, SW, MINMOD, PREC>;
    case HLLCT: return vl ? &launch_ccm_sweep<SCH, HLLCT, VANLEER, PREC> : &launch_ccm_sweep<SCH, HLLCT, MINMOD, PREC>;
    case HLLT: return vl ? &launch_ccm_sweep<SCH, HLLT, VANLEER, PREC> : &launch_ccm_sweep<SCH, HLLT, MINMOD, PREC>;
    default: return nullptr;
    }
}

} // namespace ibtfo
