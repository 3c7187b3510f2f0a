// Device-side physics of the IBTFO update: limiters, physical fluxes and the
// three Riemann solvers, written so that every expression is evaluated in
// the same order as the reference (the parity build compiles with
// -fmad=false, so no multiply-add is fused and each result is the IEEE
// binary64 value of the reference expression).
//
// pow(x, 0.5) of the reference is evaluated as a correctly rounded square
// root; both agree except where the library pow is off by its last bit.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace ibtfo {

enum Scheme { MUSCL = 0, MHM = 1, GODUNOV = 2, LAX = 3 };
enum Riemann { HLL = 0, HLLC = 1, PVRS = 2, SW = 3, HLLCT = 4, HLLT = 5 };
// the solver keys with no reference counterpart that carry the positivity
// safeguards (first-order fallback of unphysical face pairs, pressure floor)
constexpr bool safeguarded(int rie) { return rie == HLLCT || rie == HLLT; }
enum Limiter { MINMOD = 0, VANLEER = 1 };

// pow(x, 0.5): +0 for a zero of either sign (as pow gives), sqrt otherwise
__device__ __forceinline__ double pow_half(double x) { return (x == 0.0) ? 0.0 : sqrt(x); }

// Src/Base/Slope_limiter/minmod/Slope_limiter.H:4:
//   ((a*b) > 0) ? ((a/b > 1) ? b : a) : 0
// evaluated on the integer pipe with the same result:
// * a*b > 0 holds when a and b are non-zero, not NaN, of the same sign, and
//   the product does not underflow to zero; for biased exponents
//   ea + eb >= 972 (both normal) |a*b| >= 2^-1074 cannot underflow, below
//   that the product itself is evaluated;
// * where a*b > 0, the rounded quotient a/b exceeds 1 exactly when |a| > |b|:
//   for doubles |a| > |b| implies |a|/|b| >= 1 + ulp(b)/|b| > 1 + 2^-53,
//   which rounds above 1, and |a| <= |b| gives a quotient <= 1; magnitudes of
//   non-NaN doubles order like their bit patterns.
__device__ __forceinline__ double lim_minmod(double a, double b)
{
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long ma = ia & 0x7fffffffffffffffLL, mb = ib & 0x7fffffffffffffffLL;
    bool pos = ((ia ^ ib) >= 0) && ma != 0 && mb != 0 && ma <= 0x7ff0000000000000LL && mb <= 0x7ff0000000000000LL;
    if (pos)
    {
        const int ea = (int)(ma >> 52), eb = (int)(mb >> 52);
        if (!(ea != 0 && eb != 0 && ea + eb >= 972))
            pos = (a * b) > 0;
    }
    return pos ? ((ma > mb) ? b : a) : 0.0;
}

// Src/Base/Slope_limiter/VanLeer/Slope_limiter.H:4 as the macro expands at its
// call sites, where b is the text `P - Q`: (r*r + r) * P - Q / (r*r + 1)
__device__ __forceinline__ double lim_vanleer(double a, double P, double Q)
{
    double b = P - Q;
    double r = (a + 1e-7) / (b + 1e-7);
    return (r > 0) ? ((r * r + r) * P - Q / (r * r + 1)) : 0.0;
}

// 0.5 * limiter(hi - lo, P - Q)
template <int LIM>
__device__ __forceinline__ double half_slope(double hi, double lo, double P, double Q)
{
    double a = hi - lo;
    if (LIM == VANLEER)
        return 0.5 * lim_vanleer(a, P, Q);
    return 0.5 * lim_minmod(a, P - Q);
}

// Face states of one interface from the four cells c0..c3 along the sweep
// (interface between c1 and c2).  MUSCL_Scheme.cpp:39-41 and :55-57 (and the
// Y forms :100-102, :116-118): U_L = c1 + 0.5 lim(c1-c0, c2-c1),
// U_R = c2 - 0.5 lim(c3-c2, c2-c1).  Godunov: U_L = c1, U_R = c2.
template <int SCH, int LIM>
__device__ __forceinline__ void face_states(const double c0[4], const double c1[4], const double c2[4],
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
        else
        {
            UL[k] = c1[k] + half_slope<LIM>(c1[k], c0[k], c2[k], c1[k]);
            UR[k] = c2[k] - half_slope<LIM>(c3[k], c2[k], c2[k], c1[k]);
        }
    }
}

// Conserve2FluxX (Src/Base/Common/Conserve2Flux.cpp:66-74)
__device__ __forceinline__ void flux_x(const double U[4], double g, double F[4])
{
    double rho = U[0];
    double u = U[1] / rho;
    double v = U[2] / rho;
    double p = (g - 1) * (U[3] - 0.5 * rho * (u * u + v * v));
    F[0] = rho * u;
    F[1] = rho * u * u + p;
    F[2] = rho * u * v;
    F[3] = (U[3] + p) * u;
}

// Conserve2FluxY (Src/Base/Common/Conserve2Flux.cpp:101-109)
__device__ __forceinline__ void flux_y(const double U[4], double g, double G[4])
{
    double rho = U[0];
    double u = U[1] / rho;
    double v = U[2] / rho;
    double p = (g - 1) * (U[3] - 0.5 * rho * (u * u + v * v));
    G[0] = rho * v;
    G[1] = rho * u * v;
    G[2] = rho * v * v + p;
    G[3] = (U[3] + p) * v;
}

// MHM half-step predictor on the two states of one interface,
// MHM_Scheme.cpp:73-93 (X, h = dx) and :160-180 (Y, h = dy):
// U += 0.5 * (F(U_L) - F(U_R)) * dt / h for both states.
template <int YDIR>
__device__ __forceinline__ void mhm_predict(double UL[4], double UR[4], double g, double dt, double h)
{
    double FL[4], FR[4];
    if (YDIR)
    {
        flux_y(UL, g, FL);
        flux_y(UR, g, FR);
    }
    else
    {
        flux_x(UL, g, FL);
        flux_x(UR, g, FR);
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        double d = 0.5 * (FL[k] - FR[k]) * dt / h;
        UL[k] = UL[k] + d;
        UR[k] = UR[k] + d;
    }
}

// ----------------------------------------------------------------- HLL

// HLL/Riemann_solver.cpp:131-169 (X).  Returns the face flux.
__device__ __forceinline__ void hll_x(const double UL[4], const double UR[4], double g, double F[4])
{
    double rho_L = UL[0], rho_R = UR[0];
    double u_L = UL[1] / rho_L;
    double v_L = UL[2] / rho_L;
    double p_L = (g - 1) * (UL[3] - 0.5 * rho_L * (u_L * u_L + v_L * v_L));
    double u_R = UR[1] / rho_R;
    double v_R = UR[2] / rho_R;
    double p_R = (g - 1) * (UR[3] - 0.5 * rho_R * (u_R * u_R + v_R * v_R));
    double a_L = pow_half(g * p_L / rho_L);
    double a_R = pow_half(g * p_R / rho_R);
    double rho_bar = 0.5 * (rho_L + rho_R);
    double a_bar = 0.5 * (a_L + a_R);
    double p_star = 0.5 * (p_L + p_R) + 0.5 * (u_L - u_R) * (rho_bar * a_bar);
    double S_L = u_L - a_L * sqrt((g + 1) * p_star / 2 / g / p_L + (g - 1) / 2 / g);
    double S_R = u_R + a_R * sqrt((g + 1) * p_star / 2 / g / p_R + (g - 1) / 2 / g);
    double FL[4], FR[4];
    flux_x(UL, g, FL);
    flux_x(UR, g, FR);
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        if (S_L >= 0)
            F[k] = FL[k];
        else if (S_R <= 0)
            F[k] = FR[k];
        else
            F[k] = (S_R * FL[k] - S_L * FR[k] + S_R * S_L * (UR[k] - UL[k])) / (S_R - S_L);
    }
}

// HLL/Riemann_solver.cpp:202-235 (Y).  Returns false when S_D >= 0: the
// reference then stores nothing and the slot keeps the X-face flux (:224-227).
__device__ __forceinline__ bool hll_y(const double UD[4], const double UU[4], double g, double G[4])
{
    double rho_U = UU[0], rho_D = UD[0];
    double u_U = UU[1] / rho_U;
    double v_U = UU[2] / rho_U;
    double p_U = (g - 1) * (UU[3] - 0.5 * rho_U * (u_U * u_U + v_U * v_U));
    double u_D = UD[1] / rho_D;
    double v_D = UD[2] / rho_D;
    double p_D = (g - 1) * (UD[3] - 0.5 * rho_D * (u_D * u_D + v_D * v_D));
    double a_U = pow_half(g * p_U / rho_U);
    double a_D = pow_half(g * p_D / rho_D);
    double rho_bar = 0.5 * (rho_U + rho_D);
    double a_bar = 0.5 * (a_U + a_D);
    double p_star = 0.5 * (p_U + p_D) + 0.5 * (v_D - v_U) * (rho_bar * a_bar);
    double S_D = v_D - a_D * sqrt((g + 1) * p_star / 2 / g / p_D + (g - 1) / 2 / g);
    double S_U = v_U + a_U * sqrt((g + 1) * p_star / 2 / g / p_U + (g - 1) / 2 / g);
    if (S_D >= 0)
        return false;
    double GD[4], GU[4];
    flux_y(UD, g, GD);
    flux_y(UU, g, GU);
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        if (S_U <= 0)
            G[k] = GU[k];
        else
            G[k] = (S_U * GD[k] - S_D * GU[k] + S_U * S_D * (UU[k] - UD[k])) / (S_U - S_D);
    }
    return true;
}

// ----------------------------------------------------------------- PVRS

// PVRS/Riemann_solver.cpp:308-435 (X), with the reference's S_TL/S_TR (both use
// p_star/p_R, :331,:334) and fan states (rho in place of u, :375-377).
__device__ __forceinline__ void pvrs_x(const double UL[4], const double UR[4], double g, double F[4])
{
    double rho_L = UL[0], rho_R = UR[0];
    double u_L = UL[1] / rho_L;
    double v_L = UL[2] / rho_L;
    double p_L = (g - 1) * (UL[3] - 0.5 * rho_L * (u_L * u_L + v_L * v_L));
    double u_R = UR[1] / rho_R;
    double v_R = UR[2] / rho_R;
    double p_R = (g - 1) * (UR[3] - 0.5 * rho_R * (u_R * u_R + v_R * v_R));
    double a_L = pow_half(g * p_L / rho_L);
    double a_R = pow_half(g * p_R / rho_R);
    double rho_bar = 0.5 * (rho_L + rho_R);
    double a_bar = 0.5 * (a_L + a_R);
    double p_star = 0.5 * (p_L + p_R) + 0.5 * (u_L - u_R) * (rho_bar * a_bar);
    double u_star = 0.5 * (u_L + u_R) + 0.5 * (p_L - p_R) / (rho_bar * a_bar);
    double rhoL_star = rho_L + (p_star - p_L) / a_L / a_L;
    double rhoR_star = rho_R + (p_star - p_R) / a_R / a_R;
    double S_L = u_L - a_L * sqrt((g + 1) * p_star / 2 / g / p_L + (g - 1) / 2 / g);
    double S_R = u_R + a_R * sqrt((g + 1) * p_star / 2 / g / p_R + (g - 1) / 2 / g);
    double S_HL = u_L - a_L;
    double S_TL = u_star - pow(a_L * (p_star / p_R), ((g - 1) / 2 / g));
    double S_HR = u_R + a_R;
    double S_TR = u_star + pow(a_R * (p_star / p_R), ((g - 1) / 2 / g));
    // 0: left direct, 1: left star, 2: left fan, 3: right direct, 4: right star, 5: right fan
    int br;
    if (u_star > 0)
    {
        if (p_star > p_L)
            br = (S_L > 0) ? 0 : 1;
        else
            br = (S_HL > 0) ? 0 : ((S_TL < 0) ? 1 : 2);
    }
    else
    {
        if (p_star > p_R)
            br = (S_R < 0) ? 3 : 4;
        else
            br = (S_HR < 0) ? 3 : ((S_TR > 0) ? 4 : 5);
    }
    if (br == 0)
    {
        F[0] = rho_L * u_L;
        F[1] = rho_L * u_L * u_L + p_L;
        F[2] = rho_L * u_L * v_L;
        F[3] = (UL[3] + p_L) * u_L;
    }
    else if (br == 3)
    {
        F[0] = rho_R * u_R;
        F[1] = rho_R * u_R * u_R + p_R;
        F[2] = rho_R * u_R * v_R;
        F[3] = (UR[3] + p_R) * u_R;
    }
    else if (br == 1 || br == 4)
    {
        double rs = (br == 1) ? rhoL_star : rhoR_star;
        double vt = (br == 1) ? v_L : v_R;
        F[0] = rs * u_star;
        F[1] = rs * u_star * u_star + p_star;
        F[2] = rs * u_star * vt;
        F[3] = (g * p_star / (g - 1) + 0.5 * rs * (u_star * u_star + vt * vt)) * u_star;
    }
    else
    {
        double rho_s = (br == 2) ? rho_L : rho_R;
        double a_s = (br == 2) ? a_L : a_R;
        double u_s = (br == 2) ? u_L : u_R;
        double p_s = (br == 2) ? p_L : p_R;
        double vt = (br == 2) ? v_L : v_R;
        double rho_f = rho_s * pow(2 / (g + 1) + (g - 1) * (rho_s) / (g + 1) / a_s, 2 / (g - 1));
        double u_f = 2 * (a_s + (g - 1) * u_s / 2) / (g + 1);
        double p_f = p_s * pow((2 / (g + 1) + (g - 1) * (rho_s) / (g + 1) / a_s), 2 * g / (g - 1));
        F[0] = rho_f * u_f;
        F[1] = rho_f * u_f * u_f + p_f;
        F[2] = rho_f * u_f * vt;
        F[3] = (g * p_f / (g - 1) + 0.5 * rho_f * (u_f * u_f + vt * vt)) * u_f;
    }
}

// PVRS/Riemann_solver.cpp:463-590 (Y).  Returns a mask of components the
// reference leaves unchanged in the shared flux slot: the branch at :547-550
// stores its energy flux elsewhere, so component 3 keeps the X-face flux.
// *stray receives that energy flux when the branch fires.
__device__ __forceinline__ int pvrs_y(const double UD[4], const double UU[4], double g, double G[4], double *stray)
{
    double rho_U = UU[0], rho_D = UD[0];
    double u_U = UU[1] / rho_U;
    double v_U = UU[2] / rho_U;
    double p_U = (g - 1) * (UU[3] - 0.5 * rho_U * (u_U * u_U + v_U * v_U));
    double u_D = UD[1] / rho_D;
    double v_D = UD[2] / rho_D;
    double p_D = (g - 1) * (UD[3] - 0.5 * rho_D * (u_D * u_D + v_D * v_D));
    double a_U = pow_half(g * p_U / rho_U);
    double a_D = pow_half(g * p_D / rho_D);
    double rho_bar = 0.5 * (rho_U + rho_D);
    double a_bar = 0.5 * (a_U + a_D);
    double p_star = 0.5 * (p_U + p_D) + 0.5 * (v_D - v_U) * (rho_bar * a_bar);
    double v_star = 0.5 * (v_D + v_U) + 0.5 * (p_D - p_U) / (rho_bar * a_bar);
    double rhoD_star = rho_D + (p_star - p_D) / a_D / a_D;
    double rhoU_star = rho_U + (p_star - p_U) / a_U / a_U;
    double S_D = v_D - a_D * sqrt((g + 1) * p_star / 2 / g / p_D + (g - 1) / 2 / g);
    double S_U = v_U + a_U * sqrt((g + 1) * p_star / 2 / g / p_U + (g - 1) / 2 / g);
    double S_HD = v_D - a_D;
    double S_TD = v_star - pow(a_D * (p_star / p_U), ((g - 1) / 2 / g));
    double S_HU = v_U + a_U;
    double S_TU = v_star + pow(a_U * (p_star / p_U), ((g - 1) / 2 / g));
    // 0: down direct, 1: down star, 2: down fan, 3: up direct, 4: up star, 5: up fan, 6: up direct (:547-550)
    int br;
    if (v_star > 0)
    {
        if (p_star > p_D)
            br = (S_D > 0) ? 0 : 1;
        else
            br = (S_HD > 0) ? 0 : ((S_TD < 0) ? 1 : 2);
    }
    else
    {
        if (p_star > p_U)
            br = (S_U < 0) ? 6 : 4;
        else
            br = (S_HU < 0) ? 3 : ((S_TU > 0) ? 4 : 5);
    }
    int keep = 0;
    if (br == 0)
    {
        G[0] = rho_D * v_D;
        G[1] = rho_D * u_D * v_D;
        G[2] = rho_D * v_D * v_D + p_D;
        G[3] = (UD[3] + p_D) * v_D;
    }
    else if (br == 3 || br == 6)
    {
        G[0] = rho_U * v_U;
        G[1] = rho_U * u_U * v_U;
        G[2] = rho_U * v_U * v_U + p_U;
        G[3] = (UU[3] + p_U) * v_U;
        if (br == 6)
        {
            *stray = G[3];
            keep = 1 << 3;
        }
    }
    else if (br == 1 || br == 4)
    {
        double rs = (br == 1) ? rhoD_star : rhoU_star;
        double ut = (br == 1) ? u_D : u_U;
        G[0] = rs * v_star;
        G[1] = rs * v_star * ut;
        G[2] = rs * v_star * v_star + p_star;
        G[3] = (g * p_star / (g - 1) + 0.5 * rs * (v_star * v_star + ut * ut)) * v_star;
    }
    else
    {
        double rho_s = (br == 2) ? rho_D : rho_U;
        double a_s = (br == 2) ? a_D : a_U;
        double v_s = (br == 2) ? v_D : v_U;
        double p_s = (br == 2) ? p_D : p_U;
        double ut = (br == 2) ? u_D : u_U;
        double rho_f = rho_s * pow(2 / (g + 1) + (g - 1) * (rho_s) / (g + 1) / a_s, 2 / (g - 1));
        double v_f = 2 * (a_s + (g - 1) * v_s / 2) / (g + 1);
        double p_f = p_s * pow((2 / (g + 1) + (g - 1) * (rho_s) / (g + 1) / a_s), 2 * g / (g - 1));
        G[0] = rho_f * v_f;
        G[1] = rho_f * v_f * ut;
        G[2] = rho_f * v_f * v_f + p_f;
        G[3] = (g * p_f / (g - 1) + 0.5 * rho_f * (v_f * v_f + ut * ut)) * v_f;
    }
    return keep;
}

// ----------------------------------------------------------- Steger-Warming

#define IBTFO_SW_LAM(x, sgn) (0.5 * ((x)sgn sqrt((x) * (x) + delta * delta)))

// StegerWarming/Riemann_solver.cpp:173-234 (X): F = F+(U_L) + F-(U_R)
__device__ __forceinline__ void sw_x(const double UL[4], const double UR[4], double g, double F[4])
{
    double rho_L = UL[0], rho_R = UR[0];
    double u_L = UL[1] / rho_L;
    double v_L = UL[2] / rho_L;
    double p_L = (g - 1) * (UL[3] - 0.5 * rho_L * (u_L * u_L + v_L * v_L));
    double u_R = UR[1] / rho_R;
    double v_R = UR[2] / rho_R;
    double p_R = (g - 1) * (UR[3] - 0.5 * rho_R * (u_R * u_R + v_R * v_R));
    double a_L = pow_half(g * p_L / rho_L);
    double a_R = pow_half(g * p_R / rho_R);
    double e_L = p_L / (g - 1) / rho_L;
    double e_R = p_R / (g - 1) / rho_R;
    double h_L = e_L + u_L * u_L / 2 + v_L * v_L / 2 + p_L / rho_L;
    double h_R = e_R + u_R * u_R / 2 + v_R * v_R / 2 + p_R / rho_R;
    const double delta = 1e-6;
    double l1p = IBTFO_SW_LAM(u_L, +), l3p = IBTFO_SW_LAM((u_L - a_L), +), l4p = IBTFO_SW_LAM((u_L + a_L), +);
    double l1n = IBTFO_SW_LAM(u_R, -), l3n = IBTFO_SW_LAM((u_R - a_R), -), l4n = IBTFO_SW_LAM((u_R + a_R), -);
    double f1p = rho_L * (2 * (g - 1) * l1p + l3p + l4p) / 2 / g;
    double f2p = rho_L * (2 * (g - 1) * u_L * l1p + (u_L - a_L) * l3p + (u_L + a_L) * l4p) / 2 / g;
    double f3p = rho_L * (2 * (g - 1) * v_L * l1p + l3p * v_L + l4p * v_L) / 2 / g;
    double f4p = rho_L * ((g - 1) * (u_L * u_L + v_L * v_L) * l1p + (h_L - a_L * u_L) * l3p + (h_L + a_L * u_L) * l4p) / 2 / g;
    double f1n = rho_R * (2 * (g - 1) * l1n + l3n + l4n) / 2 / g;
    double f2n = rho_R * (2 * (g - 1) * u_R * l1n + (u_R - a_R) * l3n + (u_R + a_R) * l4n) / 2 / g;
    double f3n = rho_R * (2 * (g - 1) * v_R * l1n + l3n * v_R + l4n * v_R) / 2 / g;
    double f4n = rho_R * ((g - 1) * (u_R * u_R + v_R * v_R) * l1n + (h_R - a_R * u_R) * l3n + (h_R + a_R * u_R) * l4n) / 2 / g;
    F[0] = f1p + f1n;
    F[1] = f2p + f2n;
    F[2] = f3p + f3n;
    F[3] = f4p + f4n;
}

// StegerWarming/Riemann_solver.cpp:262-325 (Y): G = G+(U_D) + G-(U_U)
__device__ __forceinline__ void sw_y(const double UD[4], const double UU[4], double g, double G[4])
{
    double rho_U = UU[0], rho_D = UD[0];
    double u_U = UU[1] / rho_U;
    double v_U = UU[2] / rho_U;
    double p_U = (g - 1) * (UU[3] - 0.5 * rho_U * (u_U * u_U + v_U * v_U));
    double u_D = UD[1] / rho_D;
    double v_D = UD[2] / rho_D;
    double p_D = (g - 1) * (UD[3] - 0.5 * rho_D * (u_D * u_D + v_D * v_D));
    double a_U = pow_half(g * p_U / rho_U);
    double a_D = pow_half(g * p_D / rho_D);
    double e_U = p_U / (g - 1) / rho_U;
    double e_D = p_D / (g - 1) / rho_D;
    double h_U = e_U + u_U * u_U / 2 + v_U * v_U / 2 + p_U / rho_U;
    double h_D = e_D + u_D * u_D / 2 + v_D * v_D / 2 + p_D / rho_D;
    const double delta = 1e-6;
    double m1p = IBTFO_SW_LAM(v_D, +), m3p = IBTFO_SW_LAM((v_D - a_D), +), m4p = IBTFO_SW_LAM((v_D + a_D), +);
    double m1n = IBTFO_SW_LAM(v_U, -), m3n = IBTFO_SW_LAM((v_U - a_U), -), m4n = IBTFO_SW_LAM((v_U + a_U), -);
    double g1p = rho_D * (2 * (g - 1) * m1p + m3p + m4p) / 2 / g;
    double g2p = rho_D * (2 * (g - 1) * u_D * m1p + m3p * u_D + m4p * u_D) / 2 / g;
    double g3p = rho_D * (2 * (g - 1) * v_D * m1p + (v_D - a_D) * m3p + (v_D + a_D) * m4p) / 2 / g;
    double g4p = rho_D * ((g - 1) * (u_D * u_D + v_D * v_D) * m1p + (h_D - a_D * v_D) * m3p + (h_D + a_D * v_D) * m4p) / 2 / g;
    double g1n = rho_U * (2 * (g - 1) * m1n + m3n + m4n) / 2 / g;
    double g2n = rho_U * (2 * (g - 1) * u_U * m1n + m3n * u_U + m4n * u_U) / 2 / g;
    double g3n = rho_U * (2 * (g - 1) * v_U * m1n + (v_U - a_U) * m3n + (v_U + a_U) * m4n) / 2 / g;
    double g4n = rho_U * ((g - 1) * (u_U * u_U + v_U * v_U) * m1n + (h_U - a_U * v_U) * m3n + (h_U + a_U * v_U) * m4n) / 2 / g;
    G[0] = g1p + g1n;
    G[1] = g2p + g2n;
    G[2] = g3p + g3n;
    G[3] = g4p + g4n;
}

#undef IBTFO_SW_LAM

// ---------------------------------------------------------------- PVRS stray store
//
// In the reference's PVRS Y solver the branch at PVRS/Riemann_solver.cpp:547-550
// stores the energy flux (E_U + p_U) v_U of cell c at U_TMP[c*4 + 3]: the
// state's indexing applied to the 28-double scratch records, i.e. component 3
// of scratch slot c mod 7 of cell c/7.  With the serial row-major loop the
// target cell is already solved; for c mod 7 == 2 the store replaces the
// energy component of that cell's Y-face flux (slot 2), which the Y update
// then uses.  The sweep reproduces this in pull form: the Y face of cell c'
// recomputes the solve of its only possible source, cell 7 c' + 2.
//
// That solve reads the face states the reference's scratch slots hold at
// that point (MUSCL_Scheme.cpp / MHM_Scheme.cpp / Godunov_Scheme.cpp loop
// ranges, with the harness's zero-initialised scratch): slot 5 (U_D) is the
// Y reconstruction for rows [ng-1, N-1), else the X stage's U_L (columns
// [il0, M-1), il0 = ng-1 for MHM and 1 otherwise; MHM-predicted), else 0;
// slot 6 (U_U) the Y reconstruction for rows [0, N-2), else the X stage's
// U_R (columns [0, M-2)), else 0; MHM then predicts each slot in its row
// range from the fluxes of both.  Returns whether the branch fires at (i, j)
// and the value it stores.
template <int SCH, int LIM>
__device__ bool pvrs_stray_source(const double *__restrict__ U, long long P, int pitch, int M, int N, int ng,
                                  double g, double dt, double dx, double dy, int i, int j, double *value)
{
    auto cell = [&](int ii, int jj, double v[4]) {
#pragma unroll
        for (int k = 0; k < 4; k++)
            v[k] = U[k * P + (long long)jj * pitch + ii];
    };
    const int il0 = (SCH == MHM) ? ng - 1 : 1;
    const bool x5 = i >= il0 && i < M - 1, x6 = i < M - 2;
    const bool y5 = j >= ng - 1 && j < N - 1, y6 = j < N - 2;
    double s5[4] = {0.0, 0.0, 0.0, 0.0}, s6[4] = {0.0, 0.0, 0.0, 0.0};
    if (!y5 || !y6)
    {
        // the X stage's U_L and U_R at (i, j): MUSCL_Scheme.cpp:30-60 / MHM_Scheme.cpp:28-96
        double a[4], b[4], c[4], d[4];
        if (x5 || x6)
            cell(i, j, b);
        if (x5)
        {
            cell(i - 1, j, a);
            cell(i + 1, j, c);
#pragma unroll
            for (int k = 0; k < 4; k++)
                s5[k] = (SCH == GODUNOV) ? b[k] : b[k] + half_slope<LIM>(b[k], a[k], c[k], b[k]);
        }
        if (x6)
        {
            cell(i + 1, j, c);
            cell(i + 2, j, d);
#pragma unroll
            for (int k = 0; k < 4; k++)
                s6[k] = (SCH == GODUNOV) ? c[k] : c[k] - half_slope<LIM>(d[k], c[k], c[k], b[k]);
        }
        if (SCH == MHM)
        {
            double FL[4], FR[4];
            flux_x(s5, g, FL);
            flux_x(s6, g, FR);
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                double dd = 0.5 * (FL[k] - FR[k]) * dt / dx;
                if (x5)
                    s5[k] = s5[k] + dd;
                if (x6)
                    s6[k] = s6[k] + dd;
            }
        }
    }
    if (y5 || y6)
    {
        // the Y stage: MUSCL_Scheme.cpp:91-121 / MHM_Scheme.cpp:98-183
        double a[4], b[4], c[4], d[4];
        cell(i, j, b);
        cell(i, j + 1, c);
        if (y5)
        {
            cell(i, j - 1, a);
#pragma unroll
            for (int k = 0; k < 4; k++)
                s5[k] = (SCH == GODUNOV) ? b[k] : b[k] + half_slope<LIM>(b[k], a[k], c[k], b[k]);
        }
        if (y6)
        {
            cell(i, j + 2, d);
#pragma unroll
            for (int k = 0; k < 4; k++)
                s6[k] = (SCH == GODUNOV) ? c[k] : c[k] - half_slope<LIM>(d[k], c[k], c[k], b[k]);
        }
    }
    if (SCH == MHM)
    {
        double FL[4], FR[4];
        flux_y(s5, g, FL);
        flux_y(s6, g, FR);
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            double dd = 0.5 * (FL[k] - FR[k]) * dt / dy;
            if (y5)
                s5[k] = s5[k] + dd;
            if (y6)
                s6[k] = s6[k] + dd;
        }
    }
    double G[4], stray = 0.0;
    if (!(pvrs_y(s5, s6, g, G, &stray) & 8))
        return false;
    *value = stray;
    return true;
}

// One X face: states from four cells, MHM predictor, Riemann solver.
template <int SCH, int RIE, int LIM>
__device__ __forceinline__ void x_face(const double c0[4], const double c1[4], const double c2[4], const double c3[4],
                                       double g, double dt, double dx, double F[4])
{
    double UL[4], UR[4];
    face_states<SCH, LIM>(c0, c1, c2, c3, UL, UR);
    if (SCH == MHM)
        mhm_predict<0>(UL, UR, g, dt, dx);
    if (RIE == PVRS)
        pvrs_x(UL, UR, g, F);
    else if (RIE == SW)
        sw_x(UL, UR, g, F);
    else
        hll_x(UL, UR, g, F);
}

// One Y face.  Returns the mask of components that keep the X-face flux of
// the same cell (all four for HLL with S_D >= 0, component 3 for the PVRS
// branch at :547-550, none otherwise).
template <int SCH, int RIE, int LIM>
__device__ __forceinline__ int y_face(const double c0[4], const double c1[4], const double c2[4], const double c3[4],
                                      double g, double dt, double dy, double G[4], double *stray)
{
    double UD[4], UU[4];
    face_states<SCH, LIM>(c0, c1, c2, c3, UD, UU);
    if (SCH == MHM)
        mhm_predict<1>(UD, UU, g, dt, dy);
    if (RIE == PVRS)
        return pvrs_y(UD, UU, g, G, stray);
    if (RIE == SW)
    {
        sw_y(UD, UU, g, G);
        return 0;
    }
    return hll_y(UD, UU, g, G) ? 0 : 0xF;
}

} // namespace ibtfo
