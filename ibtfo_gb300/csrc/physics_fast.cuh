// Physics with fewer floating-point instructions, templated on the
// arithmetic type: T = double for the `fp64_fast` precision, T = float for
// the FP32 compensated precision form.
//
// Same algorithm and branches as physics.cuh (the reference's), evaluated
// with shared reciprocals, precomputed gamma constants, fused multiply-adds
// (these units are compiled with contraction on) and the limiter's sign and
// magnitude tests done on integer bit patterns.  For T = double the results
// differ from the reference in rounding only: relative differences of order
// 1e-15 per step, inside the plain path's 1e-12 parity bar (checked by the GPU
// parity tests for this precision).  Degenerate inputs (zero or non-finite
// density or pressure) may produce a different mix of inf and NaN than the
// reference.
#pragma once

#include "physics.cuh"

namespace ibtfo {

// gamma-dependent constants (precomputed on the host, see GridDesc)
template <typename T>
struct GasConst
{
    T g, gm1, c1, c2; // gamma, gamma - 1, (gamma+1)/(2 gamma), (gamma-1)/(2 gamma)
    T igm1, ig2;      // 1/(gamma - 1), 1/(2 gamma)
    __device__ __forceinline__ GasConst(T g_, T gm1_, T c1_, T c2_, T igm1_, T ig2_)
        : g(g_), gm1(gm1_), c1(c1_), c2(c2_), igm1(igm1_), ig2(ig2_)
    {
    }
};

// 1/x: hardware seed + two Newton steps (within an ulp of the rounded value)
__device__ __forceinline__ double rcp_t(double x)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}
// FP32 form: hardware reciprocal seed + one Newton step (within ~1 ulp; no
// correctly-rounded slow path), and the hardware square root approximation
// (relative error ~2^-23); the FP32 form makes no bitwise claim
__device__ __forceinline__ float rcp_t(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    const float e = fmaf(-x, y, 1.0f);
    return fmaf(y, e, y);
}
// sqrt(x) for positive normal finite x from the hardware reciprocal square
// root estimate y0 = (1 + e)/sqrt(x), |e| <= 2^-20 (measured on GB300): one
// Newton step folded into t = x y0 gives s0 = t (1 + r/2), r = 1 - x y0^2,
// with relative error 1.5 e^2; one residual correction s1 = s0 + (y0/2)(x -
// s0^2) leaves 1.5 e^3 (< 2^-59), so s1 is within about an ulp of sqrt(x).
// Seven FP64 operations; zero, negative, subnormal and non-finite x take the
// library square root.
__device__ __forceinline__ double sqrt_t(double x)
{
    const long long ix = __double_as_longlong(x);
    if (ix < 0x0010000000000000LL || ix >= 0x7ff0000000000000LL)
        return sqrt(x);
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double t = x * y;
    const double r = fma(-t, y, 1.0);
    const double s0 = fma(0.5 * t, r, t);
    const double d = fma(-s0, s0, x);
    return fma(0.5 * y, d, s0);
}
__device__ __forceinline__ float sqrt_t(float x)
{
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }

// minmod with the sign and magnitude tests on the integer pipe:
// (a*b > 0) ? (|a| > |b| ? b : a) : 0, treating a product that would
// underflow to zero as positive (only for |a|,|b| below ~1e-154 in double)
__device__ __forceinline__ double minmod_t(double a, double b)
{
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long ma = ia & 0x7fffffffffffffffLL, mb = ib & 0x7fffffffffffffffLL;
    const bool ok = ((ia ^ ib) >= 0) && ma != 0 && mb != 0 && ma <= 0x7ff0000000000000LL &&
                    mb <= 0x7ff0000000000000LL;
    return ok ? ((ma > mb) ? b : a) : 0.0;
}
// FP32: the reference's form, a product and two compares on the FP32 pipes
// (a product below the smallest float counts as not positive)
__device__ __forceinline__ float minmod_t(float a, float b)
{
    return (a * b > 0.0f) ? ((fabsf(a) > fabsf(b)) ? b : a) : 0.0f;
}

// VanLeer as the reference macro expands (physics.cuh lim_vanleer)
template <typename T>
__device__ __forceinline__ T vanleer_t(T a, T P, T Q)
{
    T b = P - Q;
    T r = (a + (T)1e-7) / (b + (T)1e-7);
    return (r > 0) ? ((r * r + r) * P - Q / (r * r + 1)) : (T)0;
}

template <typename T, int SCH, int LIM>
__device__ __forceinline__ void face_states_fast(const T c0[4], const T c1[4], const T c2[4], const T c3[4], T UL[4],
                                                 T UR[4])
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
            UL[k] = c1[k] + (T)0.5 * vanleer_t<T>(c1[k] - c0[k], c2[k], c1[k]);
            UR[k] = c2[k] - (T)0.5 * vanleer_t<T>(c3[k] - c2[k], c2[k], c1[k]);
        }
        else
        {
            const T dm = c1[k] - c0[k], d0 = c2[k] - c1[k], dp = c3[k] - c2[k];
            UL[k] = fma_t((T)0.5, minmod_t(dm, d0), c1[k]);
            UR[k] = fma_t((T)-0.5, minmod_t(dp, d0), c2[k]);
        }
    }
}

// primitive variables and sound speed of one state
template <typename T>
struct Prim
{
    T r, ir, un, ut, p, a, gi; // gi = gamma / rho, a = sqrt(gi p)
};

// NRM = index of the face-normal momentum (1 for X, 2 for Y)
template <typename T, int NRM>
__device__ __forceinline__ Prim<T> prim_fast(const T U[4], const GasConst<T> &K)
{
    Prim<T> s;
    s.r = U[0];
    s.ir = rcp_t(U[0]);
    s.un = U[NRM] * s.ir;
    s.ut = U[3 - NRM] * s.ir;
    // rho (un^2 + ut^2) = m_n un + m_t ut
    s.p = K.gm1 * fma_t((T)-0.5, fma_t(U[NRM], s.un, U[3 - NRM] * s.ut), U[3]);
    s.gi = K.g * s.ir;
    s.a = sqrt_t(s.gi * s.p);
    return s;
}

// physical flux normal to the face; components in state order
// (the mass flux rho un is the normal momentum itself)
template <typename T, int NRM>
__device__ __forceinline__ void flux_fast(const T U[4], const Prim<T> &s, T F[4])
{
    const T m = U[NRM];
    F[0] = m;
    F[NRM] = fma_t(m, s.un, s.p);
    F[3 - NRM] = m * s.ut;
    F[3] = (U[3] + s.p) * s.un;
}

// HLL face flux (HLL/Riemann_solver.cpp:131-169 X, :202-235 Y).  For Y,
// returns false when S_D >= 0 (the reference keeps the X-face flux).
template <typename T, int NRM>
__device__ __forceinline__ bool hll_fast(const T UL[4], const T UR[4], const GasConst<T> &K, T F[4])
{
    const Prim<T> L = prim_fast<T, NRM>(UL, K), R = prim_fast<T, NRM>(UR, K);
    const T p_star = (T)0.5 * (L.p + R.p) + (T)0.125 * (L.un - R.un) * ((L.r + R.r) * (L.a + R.a));
    const T t = K.c1 * p_star;
    // a_K sqrt(c1 p*/p_K + c2) = sqrt((gamma/rho_K)(c1 p* + c2 p_K)): one root, no 1/p_K
    const T S_L = L.un - sqrt_t(L.gi * fma_t(K.c2, L.p, t));
    const T S_R = R.un + sqrt_t(R.gi * fma_t(K.c2, R.p, t));
    if (NRM == 2 && S_L >= 0)
        return false;
    T FL[4], FR[4];
    flux_fast<T, NRM>(UL, L, FL);
    flux_fast<T, NRM>(UR, R, FR);
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
        // (S_R F_L - S_L F_R + S_R S_L (U_R - U_L)) / (S_R - S_L) with the three weights formed once
        const T inv = rcp_t(S_R - S_L);
        const T wl = S_R * inv, wr = -S_L * inv, wu = wl * S_L;
#pragma unroll
        for (int k = 0; k < 4; k++)
            F[k] = fma_t(wl, FL[k], fma_t(wr, FR[k], wu * (UR[k] - UL[k])));
    }
    return true;
}

// Steger-Warming flux-vector splitting (StegerWarming/Riemann_solver.cpp:173-234
// X, :262-325 Y): F = F+(U_L) + F-(U_R) with lambda+- = (lambda +- sqrt(lambda^2 + delta^2))/2
template <typename T, int NRM, int SIGN>
__device__ __forceinline__ void sw_split(const T U[4], const GasConst<T> &K, T F[4])
{
    const Prim<T> s = prim_fast<T, NRM>(U, K);
    const T d2 = (T)1e-12; // delta = 1e-6 (:193)
    auto lam = [&](T x) { return (T)0.5 * (x + (T)SIGN * sqrt_t(x * x + d2)); };
    const T l1 = lam(s.un), l3 = lam(s.un - s.a), l4 = lam(s.un + s.a);
    const T h = s.p * K.igm1 * s.ir + (T)0.5 * (s.un * s.un + s.ut * s.ut) + s.p * s.ir; // e + |u|^2/2 + p/rho
    const T w = s.r * K.ig2;
    F[0] = w * ((T)2 * K.gm1 * l1 + l3 + l4);
    F[NRM] = w * ((T)2 * K.gm1 * s.un * l1 + (s.un - s.a) * l3 + (s.un + s.a) * l4);
    F[3 - NRM] = w * s.ut * ((T)2 * K.gm1 * l1 + l3 + l4);
    F[3] = w * (K.gm1 * (s.un * s.un + s.ut * s.ut) * l1 + (h - s.a * s.un) * l3 + (h + s.a * s.un) * l4);
}

template <typename T, int NRM>
__device__ __forceinline__ void sw_fast(const T UL[4], const T UR[4], const GasConst<T> &K, T F[4])
{
    T Fp[4], Fm[4];
    sw_split<T, NRM, 1>(UL, K, Fp);
    sw_split<T, NRM, -1>(UR, K, Fm);
#pragma unroll
    for (int k = 0; k < 4; k++)
        F[k] = Fp[k] + Fm[k];
}

// Contact-restoring HLLC (Toro, Riemann Solvers and Numerical Methods for
// Fluid Dynamics, 3rd ed., eqs. 10.37-10.39 and 10.71-10.73), offered under its
// own key: the reference's HLLC directory holds the HLL solver (see also the
// HLLC_Toro safeguards below).  Wave speeds
// from the PVRS pressure estimate with Toro's q_K = 1 for p* <= p_K; no face
// leaves its flux slot unchanged (always returns a flux).
template <typename T, int NRM>
__device__ __forceinline__ void hllc_toro(const T UL[4], const T UR[4], const GasConst<T> &K, T F[4])
{
    const Prim<T> L = prim_fast<T, NRM>(UL, K), R = prim_fast<T, NRM>(UR, K);
    T p_star = (T)0.5 * (L.p + R.p) + (T)0.125 * (L.un - R.un) * ((L.r + R.r) * (L.a + R.a));
    p_star = p_star > (T)0 ? p_star : (T)0;
    const T t = K.c1 * p_star;
    // a_K q_K = sqrt((gamma/rho_K)(c1 p* + c2 p_K)) where p* > p_K, else a_K
    const T S_L = L.un - ((p_star > L.p) ? sqrt_t(L.gi * fma_t(K.c2, L.p, t)) : L.a);
    const T S_R = R.un + ((p_star > R.p) ? sqrt_t(R.gi * fma_t(K.c2, R.p, t)) : R.a);
    T FL[4], FR[4];
    flux_fast<T, NRM>(UL, L, FL);
    flux_fast<T, NRM>(UR, R, FR);
    if (S_L >= 0)
    {
#pragma unroll
        for (int k = 0; k < 4; k++)
            F[k] = FL[k];
        return;
    }
    if (S_R <= 0)
    {
#pragma unroll
        for (int k = 0; k < 4; k++)
            F[k] = FR[k];
        return;
    }
    const T mL = L.r * (S_L - L.un), mR = R.r * (S_R - R.un);
    const T S_s = (R.p - L.p + L.un * mL - R.un * mR) * rcp_t(mL - mR);
    const bool left = S_s >= 0;
    const Prim<T> &s = left ? L : R;
    const T *U = left ? UL : UR;
    const T *Fk = left ? FL : FR;
    const T S = left ? S_L : S_R, m = left ? mL : mR;
    const T fac = m * rcp_t(S - S_s);
    T Us[4];
    Us[0] = fac;
    Us[NRM] = fac * S_s;
    Us[3 - NRM] = fac * s.ut;
    Us[3] = fac * (U[3] * s.ir + (S_s - s.un) * (S_s + s.p * rcp_t(m)));
#pragma unroll
    for (int k = 0; k < 4; k++)
        F[k] = Fk[k] + S * (Us[k] - U[k]);
}

// HLL flux in either direction with Toro's PVRS wave-speed estimates
// (the HLL_Toro key, in the ghost-fluid and the cut-cell sweeps)
// (p* >= 0, q_K = 1 for p* <= p_K; Toro 2009, eqs. 10.59-10.60), which stay
// defined in strong expansions where the reference's HLL estimate takes the
// square root of a negative number
template <typename T, int NRM>
__device__ __forceinline__ void hll_plain(const T UL[4], const T UR[4], const GasConst<T> &K, T F[4])
{
    const Prim<T> L = prim_fast<T, NRM>(UL, K), R = prim_fast<T, NRM>(UR, K);
    T p_star = (T)0.5 * (L.p + R.p) + (T)0.125 * (L.un - R.un) * ((L.r + R.r) * (L.a + R.a));
    p_star = p_star > (T)0 ? p_star : (T)0;
    const T t = K.c1 * p_star;
    const T S_L = L.un - ((p_star > L.p) ? sqrt_t(L.gi * fma_t(K.c2, L.p, t)) : L.a);
    const T S_R = R.un + ((p_star > R.p) ? sqrt_t(R.gi * fma_t(K.c2, R.p, t)) : R.a);
    T FL[4], FR[4];
    flux_fast<T, NRM>(UL, L, FL);
    flux_fast<T, NRM>(UR, R, FR);
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
        const T inv = rcp_t(S_R - S_L), srsl = S_R * S_L;
#pragma unroll
        for (int k = 0; k < 4; k++)
            F[k] = (S_R * FL[k] - S_L * FR[k] + srsl * (UR[k] - UL[k])) * inv;
    }
}

// MHM predictor with h2 = 0.5 * dt / h precomputed
template <typename T, int NRM>
__device__ __forceinline__ void mhm_predict_fast(T UL[4], T UR[4], const GasConst<T> &K, T h2)
{
    T FL[4], FR[4];
    const Prim<T> L = prim_fast<T, NRM>(UL, K), R = prim_fast<T, NRM>(UR, K);
    flux_fast<T, NRM>(UL, L, FL);
    flux_fast<T, NRM>(UR, R, FR);
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        const T d = h2 * (FL[k] - FR[k]);
        UL[k] += d;
        UR[k] += d;
    }
}

// ---------------------------------------------------------------- HLLC_Toro safeguards
//
// MUSCL on conserved variables keeps each variable between its neighbours
// but not the pressure: in the fast, low-pressure expansion behind a body hit
// by a strong shock (a cylinder at Mach >= 2.5) a reconstructed face state can
// have p < 0, and the conservative update can leave a cell with p < 0, where
// the kinetic energy is tens of times the internal energy.  The reference's
// solvers turn such cases to NaN (its HLL takes the square root of a negative
// p*, reproduced by the oracle).  Under the HLLC_Toro key two safeguards keep
// the pressure positive.  Their thresholds are fractions of E, the same in
// FP64 and FP32 so that both precisions run one algorithm; they sit well above
// FP32 rounding of E - E_kin (about 1e-7 E), so whatever way an expression
// rounds, the solver never meets a non-positive pressure.

// internal energy E - rho (u^2 + v^2) / 2, evaluated as prim_fast does
template <typename T>
__device__ __forceinline__ T internal_energy(const T U[4])
{
    const T ir = rcp_t(U[0]);
    const T u = U[1] * ir, v = U[2] * ir;
    return fma_t((T)-0.5, fma_t(U[1], u, U[2] * v), U[3]);
}

// positive density and an internal energy above 1e-6 E (NaN fails)
template <typename T>
__device__ __forceinline__ bool physical(const T U[4])
{
    return U[0] > (T)0 && internal_energy(U) > (T)1e-6 * fabs(U[3]);
}

// a face whose reconstructed (or predicted) pair is not physical takes the
// first-order pair, the two cell averages; faces next to solid cells are
// left alone (their fluxes are not used)
template <typename T>
__device__ __forceinline__ void positivity_fallback(const T c1[4], const T c2[4], T UL[4], T UR[4])
{
    if (!physical(c1) || !physical(c2) || (physical(UL) && physical(UR)))
        return;
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        UL[k] = c1[k];
        UR[k] = c2[k];
    }
}

// after the update of a fluid cell: where the internal energy falls below
// 1e-5 E, E becomes E_kin + 1e-5 E (the energy added is at most 1e-5 E, in
// the few cells where the conservative update lost positivity).  Returns
// whether the floor applied and the energy to store.
template <typename T>
__device__ __forceinline__ bool pressure_floor_energy(const T U[4], T &E)
{
    if (!(U[0] > (T)0))
        return false; // density not positive: nothing sensible to floor
    const T f = (T)1e-5 * fabs(U[3]);
    const T e = internal_energy(U);
    if (e >= f)
        return false;
    E = (U[3] - e) + f;
    return true;
}

template <typename T>
__device__ __forceinline__ void pressure_floor(T U[4])
{
    T e;
    if (pressure_floor_energy(U, e))
        U[3] = e;
}

template <typename T, int SCH, int RIE, int LIM>
__device__ __forceinline__ void x_face_fast(const T c0[4], const T c1[4], const T c2[4], const T c3[4],
                                            const GasConst<T> &K, T h2, T F[4])
{
    T UL[4], UR[4];
    face_states_fast<T, SCH, LIM>(c0, c1, c2, c3, UL, UR);
    if (SCH == MHM)
        mhm_predict_fast<T, 1>(UL, UR, K, h2);
    if constexpr (safeguarded(RIE))
        if (SCH != GODUNOV)
            positivity_fallback(c1, c2, UL, UR);
    if constexpr (RIE == PVRS)
        pvrs_x(UL, UR, (double)K.g, F); // double only (FP32 form rejects PVRS)
    else if constexpr (RIE == SW)
        sw_fast<T, 1>(UL, UR, K, F);
    else if constexpr (RIE == HLLCT)
        hllc_toro<T, 1>(UL, UR, K, F);
    else if constexpr (RIE == HLLT)
        hll_plain<T, 1>(UL, UR, K, F);
    else
        hll_fast<T, 1>(UL, UR, K, F);
}

template <typename T, int SCH, int RIE, int LIM>
__device__ __forceinline__ int y_face_fast(const T c0[4], const T c1[4], const T c2[4], const T c3[4],
                                           const GasConst<T> &K, T h2, T G[4], T *stray)
{
    T UD[4], UU[4];
    face_states_fast<T, SCH, LIM>(c0, c1, c2, c3, UD, UU);
    if (SCH == MHM)
        mhm_predict_fast<T, 2>(UD, UU, K, h2);
    if constexpr (safeguarded(RIE))
        if (SCH != GODUNOV)
            positivity_fallback(c1, c2, UD, UU);
    if constexpr (RIE == PVRS)
        return pvrs_y(UD, UU, (double)K.g, G, stray);
    else if constexpr (RIE == SW)
    {
        sw_fast<T, 2>(UD, UU, K, G);
        return 0;
    }
    else if constexpr (RIE == HLLCT)
    {
        hllc_toro<T, 2>(UD, UU, K, G);
        return 0;
    }
    else if constexpr (RIE == HLLT)
    {
        hll_plain<T, 2>(UD, UU, K, G);
        return 0;
    }
    else
        return hll_fast<T, 2>(UD, UU, K, G) ? 0 : 0xF;
}

// ---------------------------------------------------------------- cut cells
//
// The cut-cell method has no reference counterpart, so its faces use the
// HLL flux with Toro's wave speeds in both directions (HLL_Toro: no Y-face
// slot reuse), Steger-Warming, or the contact-restoring HLLC_Toro; the
// reference's HLL (the HLL and HLLC keys) has no cut-cell form.

template <typename T, int NRM, int RIE>
__device__ __forceinline__ void ccm_solve(const T UL[4], const T UR[4], const GasConst<T> &K, T F[4])
{
    static_assert(RIE == SW || RIE == HLLCT || RIE == HLLT, "no cut-cell form of this solver");
    if constexpr (RIE == SW)
        sw_fast<T, NRM>(UL, UR, K, F);
    else if constexpr (RIE == HLLCT)
        hllc_toro<T, NRM>(UL, UR, K, F);
    else
        hll_plain<T, NRM>(UL, UR, K, F);
}

// One face of a cut-cell case, normal NRM (1: X, 2: Y), from the four cells
// across it.  first_order: a stencil cell is cut or solid, so the face takes
// the two cell averages (no slopes, no predictor); a reconstructed pair that
// is not physical also falls back to the cell averages (positivity_fallback).
template <typename T, int NRM, int SCH, int RIE, int LIM>
__device__ __forceinline__ void ccm_face(const T c0[4], const T c1[4], const T c2[4], const T c3[4],
                                         const GasConst<T> &K, T h2, bool first_order, T F[4])
{
    T UL[4], UR[4];
    if (first_order || SCH == GODUNOV)
    {
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            UL[k] = c1[k];
            UR[k] = c2[k];
        }
    }
    else
    {
        face_states_fast<T, SCH, LIM>(c0, c1, c2, c3, UL, UR);
        if (SCH == MHM)
            mhm_predict_fast<T, NRM>(UL, UR, K, h2);
        positivity_fallback(c1, c2, UL, UR); // every cut-cell solver: no face with p <= 0
    }
    ccm_solve<T, NRM, RIE>(UL, UR, K, F);
}

// Flux through a wall of outward unit normal (nx, ny) out of a cell of state
// U: the Riemann problem between U and its mirror image (normal velocity
// reversed), solved in the wall's frame.  Only its normal-momentum flux (the
// wall pressure p_w) is kept: W = (0, p_w nx, p_w ny, 0), so no mass, energy
// or tangential momentum crosses the wall whichever branch the solver takes.
template <typename T, int RIE>
__device__ __forceinline__ void ccm_wall_flux(const T U[4], T nx, T ny, const GasConst<T> &K, T W[4])
{
    const T mn = U[1] * nx + U[2] * ny, mt = -U[1] * ny + U[2] * nx;
    const T UL[4] = {U[0], mn, mt, U[3]};
    const T UR[4] = {U[0], -mn, mt, U[3]};
    T F[4];
    ccm_solve<T, 1, RIE>(UL, UR, K, F);
    W[0] = (T)0;
    W[1] = F[1] * nx;
    W[2] = F[1] * ny;
    W[3] = (T)0;
}

} // namespace ibtfo
