// FP64 physics with fewer FP64 instructions, for the `fp64_fast` precision.
//
// Same algorithm and branches as physics.cuh (the reference's), evaluated
// with shared reciprocals, precomputed gamma constants, fused multiply-adds
// (this header is compiled with contraction on) and the limiter's sign and
// magnitude tests done on integer bit patterns.  The results differ from the
// reference in rounding only: relative differences of order 1e-15 per step,
// inside the plain path's 1e-12 parity bar (checked by the GPU parity tests
// for this precision).  Degenerate inputs (zero or non-finite density or
// pressure) may produce a different mix of inf and NaN than the reference.
#pragma once

#include "physics.cuh"

namespace ibtfo {

// gamma-dependent constants, computed once per thread
struct GasConst
{
    double g, gm1, c1, c2, g_over_gm1;
    __device__ __forceinline__ explicit GasConst(double gamma)
    {
        g = gamma;
        gm1 = gamma - 1;
        c1 = (gamma + 1) / (2 * gamma); // HLL wave speed: (g+1)/(2g) * p*/p + (g-1)/(2g)
        c2 = (gamma - 1) / (2 * gamma);
        g_over_gm1 = gamma / (gamma - 1);
    }
};

// 1/x: hardware seed + two Newton steps (within an ulp of the rounded value)
__device__ __forceinline__ double rcp_nr(double x)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

// minmod with the sign and magnitude tests on the integer pipe:
// (a*b > 0) ? (|a| > |b| ? b : a) : 0, treating a product that would
// underflow to zero as positive (only for |a|,|b| below ~1e-154)
__device__ __forceinline__ double minmod_int(double a, double b)
{
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long ma = ia & 0x7fffffffffffffffLL, mb = ib & 0x7fffffffffffffffLL;
    const bool ok = ((ia ^ ib) >= 0) && ma != 0 && mb != 0 && ma <= 0x7ff0000000000000LL &&
                    mb <= 0x7ff0000000000000LL;
    return ok ? ((ma > mb) ? b : a) : 0.0;
}

template <int SCH, int LIM>
__device__ __forceinline__ void face_states_fast(const double c0[4], const double c1[4], const double c2[4],
                                                 const double c3[4], double UL[4], double UR[4])
{
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        if (SCH == GODUNOV)
        {
            UL[k] = c1[k];
            UR[k] = c2[k];
        }
        else if (LIM == VANLEER)
        {
            UL[k] = c1[k] + half_slope<LIM>(c1[k], c0[k], c2[k], c1[k]);
            UR[k] = c2[k] - half_slope<LIM>(c3[k], c2[k], c2[k], c1[k]);
        }
        else
        {
            const double dm = c1[k] - c0[k], d0 = c2[k] - c1[k], dp = c3[k] - c2[k];
            UL[k] = fma(0.5, minmod_int(dm, d0), c1[k]);
            UR[k] = fma(-0.5, minmod_int(dp, d0), c2[k]);
        }
    }
}

// primitive variables and sound speed of one state
struct Prim
{
    double r, ir, un, ut, p, a;
};

// n = index of the face-normal momentum (1 for X, 2 for Y)
template <int NRM>
__device__ __forceinline__ Prim prim_fast(const double U[4], const GasConst &K)
{
    Prim s;
    s.r = U[0];
    s.ir = rcp_nr(U[0]);
    s.un = U[NRM] * s.ir;
    s.ut = U[3 - NRM] * s.ir;
    s.p = K.gm1 * (U[3] - 0.5 * s.r * (s.un * s.un + s.ut * s.ut));
    s.a = sqrt(K.g * s.p * s.ir);
    return s;
}

// physical flux normal to the face; components in state order
template <int NRM>
__device__ __forceinline__ void flux_fast(const double U[4], const Prim &s, double F[4])
{
    const double m = s.r * s.un;
    F[0] = m;
    F[NRM] = m * s.un + s.p;
    F[3 - NRM] = m * s.ut;
    F[3] = (U[3] + s.p) * s.un;
}

// HLL face flux (HLL/Riemann_solver.cpp:131-169 X, :202-235 Y).  For Y,
// returns false when S_D >= 0 (the reference keeps the X-face flux).
template <int NRM>
__device__ __forceinline__ bool hll_fast(const double UL[4], const double UR[4], const GasConst &K, double F[4])
{
    const Prim L = prim_fast<NRM>(UL, K), R = prim_fast<NRM>(UR, K);
    const double p_star = 0.5 * (L.p + R.p) + 0.125 * (L.un - R.un) * ((L.r + R.r) * (L.a + R.a));
    const double t = K.c1 * p_star;
    const double S_L = L.un - L.a * sqrt(fma(t, rcp_nr(L.p), K.c2));
    const double S_R = R.un + R.a * sqrt(fma(t, rcp_nr(R.p), K.c2));
    if (NRM == 2 && S_L >= 0)
        return false;
    double FL[4], FR[4];
    flux_fast<NRM>(UL, L, FL);
    flux_fast<NRM>(UR, R, FR);
    if (S_L >= 0)
    {
#pragma unroll
        for (int k = 0; k < 4; k++)
            F[k] = FL[k];
    }
    else if (S_R <= 0)
    {
#pragma unroll
        for (int k = 0; k < 4; k++)
            F[k] = FR[k];
    }
    else
    {
        const double inv = rcp_nr(S_R - S_L), srsl = S_R * S_L;
#pragma unroll
        for (int k = 0; k < 4; k++)
            F[k] = (S_R * FL[k] - S_L * FR[k] + srsl * (UR[k] - UL[k])) * inv;
    }
    return true;
}

// MHM predictor with h2 = 0.5 * dt / h precomputed
template <int NRM>
__device__ __forceinline__ void mhm_predict_fast(double UL[4], double UR[4], const GasConst &K, double h2)
{
    double FL[4], FR[4];
    const Prim L = prim_fast<NRM>(UL, K), R = prim_fast<NRM>(UR, K);
    flux_fast<NRM>(UL, L, FL);
    flux_fast<NRM>(UR, R, FR);
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        const double d = h2 * (FL[k] - FR[k]);
        UL[k] += d;
        UR[k] += d;
    }
}

template <int SCH, int RIE, int LIM>
__device__ __forceinline__ void x_face_fast(const double c0[4], const double c1[4], const double c2[4],
                                            const double c3[4], const GasConst &K, double dt, double h2, double F[4])
{
    double UL[4], UR[4];
    face_states_fast<SCH, LIM>(c0, c1, c2, c3, UL, UR);
    if (SCH == MHM)
        mhm_predict_fast<1>(UL, UR, K, h2);
    if (RIE == PVRS)
        pvrs_x(UL, UR, K.g, F);
    else if (RIE == SW)
        sw_x(UL, UR, K.g, F);
    else
        hll_fast<1>(UL, UR, K, F);
}

template <int SCH, int RIE, int LIM>
__device__ __forceinline__ int y_face_fast(const double c0[4], const double c1[4], const double c2[4],
                                           const double c3[4], const GasConst &K, double dt, double h2, double G[4],
                                           double *stray)
{
    double UD[4], UU[4];
    face_states_fast<SCH, LIM>(c0, c1, c2, c3, UD, UU);
    if (SCH == MHM)
        mhm_predict_fast<2>(UD, UU, K, h2);
    if (RIE == PVRS)
        return pvrs_y(UD, UU, K.g, G, stray);
    if (RIE == SW)
    {
        sw_y(UD, UU, K.g, G);
        return 0;
    }
    return hll_fast<2>(UD, UU, K, G) ? 0 : 0xF;
}

} // namespace ibtfo
