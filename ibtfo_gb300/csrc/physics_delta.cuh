// Face fluxes of the FP32 form in difference form, for the HLL_Toro key.
//
// The plain FP32 face solve rounds each flux to about 1e-7 of its size, and
// the update takes the difference of two such fluxes, which in smooth flow is
// a hundred to a thousand times smaller than either: each step then adds an
// error of about 1e-7 of the flux to every cell that is not in uniform flow.
// Over thousands of steps in the unsteady wake of a body this is the error
// that separates an FP32 run from its FP64 twin.  Here no full-size flux is
// ever formed.  A face between cells a (left / lower) and b stores
//   P = F_face - F(U_a)   and   Q = F_face - F(U_b),
// and cell i updates with  F_east - F_west = P_east - Q_west  (the same
// value in exact arithmetic).  Every quantity is built from differences of
// the compensated (hi, lo) state, which are accurate to FP32 rounding of the
// difference itself:
//   F(U_b) - F(U_a) and F(U_face) - F(U_cell)  by delta_flux (the product
//   rule on the primitive variables, below), and
//   HLL:  F_face - F(U_a) = w_L dF_L + w_R (dF + dF_R) + (S_L S_R / (S_R - S_L)) (U_R - U_L)
//   with w_L = S_R / (S_R - S_L), w_R = -S_L / (S_R - S_L), so that rounding
//   errors are relative to these small terms, not to F.  The wave speeds
//   (Toro's PVRS estimates, as hll_plain) multiply small quantities only and
//   are formed from the FP32 face states.
// The algorithm is HLL_Toro's (MUSCL / MHM / Godunov reconstruction with the
// limiter, the positivity fallback and the same HLL flux); only the order of
// evaluation differs.
#pragma once

#include "physics_fast.cuh"

namespace ibtfo {

// reciprocal density, velocities and pressure of a base state (FP32)
struct DeltaBase
{
    float ir, un, ut, p;
};

template <int NRM>
__device__ __forceinline__ DeltaBase delta_base(const float U[4], const GasConst<float> &K)
{
    DeltaBase b;
    b.ir = rcp_t(U[0]);
    b.un = U[NRM] * b.ir;
    b.ut = U[3 - NRM] * b.ir;
    b.p = K.gm1 * fmaf(-0.5f, fmaf(U[NRM], b.un, U[3 - NRM] * b.ut), U[3]);
    return b;
}

// the primitive variables of a state from its base (no second reciprocal)
__device__ __forceinline__ Prim<float> prim_of_base(const float U[4], const DeltaBase &b, const GasConst<float> &K)
{
    Prim<float> s;
    s.r = U[0];
    s.ir = b.ir;
    s.un = b.un;
    s.ut = b.ut;
    s.p = b.p;
    s.gi = K.g * b.ir;
    s.a = sqrt_t(s.gi * s.p);
    return s;
}

// physical() from the primitive variables: positive density and an internal
// energy p / (gamma - 1) above 1e-6 of E (NaN fails)
__device__ __forceinline__ bool physical_prim(float r, float p, float E, const GasConst<float> &K)
{
    return r > 0.0f && p * K.igm1 > 1e-6f * fabsf(E);
}

// dF = F(U_a + d) - F(U_a), normal direction NRM, from the base state U_a
// (FP32 values, velocities and pressure in `a`), the difference d and
// irb = 1 / (rho_a + d rho):
//   du_n = (d m_n - u_n d rho) / rho_b          (u = m / rho)
//   d(m_n u_n) = m_nb du_n + u_na d m_n,  d(m_t u_t) = m_tb du_t + u_ta d m_t
//   dp = (gamma - 1) (dE - (d(m_n u_n) + d(m_t u_t)) / 2)
//   dF = (d m_n, d(m_n u_n) + dp, m_tb du_n + u_na d m_t, (E_b + p_b) du_n + u_na (dE + dp))
// (components in state order; exact identities, so the rounding is relative
// to the differences).
template <int NRM>
__device__ __forceinline__ void delta_flux(const float Ua[4], const DeltaBase &a, const float d[4], float irb,
                                           const GasConst<float> &K, float dF[4])
{
    const float dun = (d[NRM] - a.un * d[0]) * irb;
    const float dut = (d[3 - NRM] - a.ut * d[0]) * irb;
    const float mnb = Ua[NRM] + d[NRM], mtb = Ua[3 - NRM] + d[3 - NRM];
    const float dnn = fmaf(mnb, dun, a.un * d[NRM]);
    const float dtt = fmaf(mtb, dut, a.ut * d[3 - NRM]);
    const float dp = K.gm1 * fmaf(-0.5f, dnn + dtt, d[3]);
    dF[0] = d[NRM];
    dF[NRM] = dnn + dp;
    dF[3 - NRM] = fmaf(mtb, dun, a.un * d[3 - NRM]);
    dF[3] = fmaf((Ua[3] + d[3]) + (a.p + dp), dun, a.un * (d[3] + dp));
}

// one face in difference form: cells c0 c1 | c2 c3 across it (hi and lo
// parts), normal NRM; P = F_face - F(c1), Q = F_face - F(c2).  hp = dt/(2h)
// for the MHM predictor.  The reciprocal densities of the cell and face
// states serve both the primitive variables and the flux differences, and
// the positivity tests read the primitive variables.
template <int SCH, int LIM, int NRM>
__device__ __forceinline__ void face_delta(const float h0[4], const float l0[4], const float h1[4],
                                           const float l1[4], const float h2[4], const float l2[4],
                                           const float h3[4], const float l3[4], const GasConst<float> &K,
                                           float hp, float P[4], float Q[4])
{
    float D1[4], dL[4], dR[4], UcL[4], UcR[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        // differences of the compensated states: hi parts first (exact for
        // neighbouring values), then the lo parts
        const float D0 = (h1[k] - h0[k]) + (l1[k] - l0[k]);
        D1[k] = (h2[k] - h1[k]) + (l2[k] - l1[k]);
        const float D2 = (h3[k] - h2[k]) + (l3[k] - l2[k]);
        if (SCH == GODUNOV)
            dL[k] = dR[k] = 0.0f;
        else if (LIM == VANLEER)
        {
            dL[k] = 0.5f * vanleer_t<float>(D0, h2[k] + l2[k], h1[k] + l1[k]);
            dR[k] = -0.5f * vanleer_t<float>(D2, h2[k] + l2[k], h1[k] + l1[k]);
        }
        else
        {
            dL[k] = 0.5f * minmod_t(D0, D1[k]);
            dR[k] = -0.5f * minmod_t(D2, D1[k]);
        }
        UcL[k] = h1[k] + l1[k];
        UcR[k] = h2[k] + l2[k];
    }
    const DeltaBase bL = delta_base<NRM>(UcL, K), bR = delta_base<NRM>(UcR, K);
    float dF[4], fL[4], fR[4];
    delta_flux<NRM>(UcL, bL, D1, bR.ir, K, dF);
    float UL[4], UR[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        UL[k] = h1[k] + (l1[k] + dL[k]);
        UR[k] = h2[k] + (l2[k] + dR[k]);
    }
    Prim<float> L, R;
    if (SCH == GODUNOV)
    {
        L = prim_of_base(UcL, bL, K);
        R = prim_of_base(UcR, bR, K);
#pragma unroll
        for (int k = 0; k < 4; k++)
            fL[k] = fR[k] = 0.0f;
    }
    else
    {
        if (SCH == MHM)
        {
            // U_L, U_R += (dt / 2h) (F(U_L) - F(U_R)), F(U_L) - F(U_R) = dF_L - dF - dF_R
            delta_flux<NRM>(UcL, bL, dL, rcp_t(UL[0]), K, fL);
            delta_flux<NRM>(UcR, bR, dR, rcp_t(UR[0]), K, fR);
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                const float m = hp * ((fL[k] - dF[k]) - fR[k]);
                dL[k] += m;
                dR[k] += m;
                UL[k] = h1[k] + (l1[k] + dL[k]);
                UR[k] = h2[k] + (l2[k] + dR[k]);
            }
        }
        L = prim_fast<float, NRM>(UL, K);
        R = prim_fast<float, NRM>(UR, K);
        if (physical_prim(UcL[0], bL.p, UcL[3], K) && physical_prim(UcR[0], bR.p, UcR[3], K) &&
            !(physical_prim(L.r, L.p, UL[3], K) && physical_prim(R.r, R.p, UR[3], K)))
        {
            // positivity fallback: the first-order pair (the two cell averages)
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                dL[k] = dR[k] = fL[k] = fR[k] = 0.0f;
                UL[k] = UcL[k];
                UR[k] = UcR[k];
            }
            L = prim_of_base(UcL, bL, K);
            R = prim_of_base(UcR, bR, K);
        }
        else
        {
            delta_flux<NRM>(UcL, bL, dL, L.ir, K, fL);
            delta_flux<NRM>(UcR, bR, dR, R.ir, K, fR);
        }
    }
    // Toro's PVRS wave-speed estimates from the face states (hll_plain)
    float p_star = 0.5f * (L.p + R.p) + 0.125f * (L.un - R.un) * ((L.r + R.r) * (L.a + R.a));
    p_star = p_star > 0.0f ? p_star : 0.0f;
    const float t = K.c1 * p_star;
    const float S_L = L.un - ((p_star > L.p) ? sqrt_t(L.gi * fmaf(K.c2, L.p, t)) : L.a);
    const float S_R = R.un + ((p_star > R.p) ? sqrt_t(R.gi * fmaf(K.c2, R.p, t)) : R.a);
    if (S_L >= 0.0f)
    {
        // F_face = F(U_L) = F(c1) + dF_L
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            P[k] = fL[k];
            Q[k] = fL[k] - dF[k];
        }
    }
    else if (S_R <= 0.0f)
    {
        // F_face = F(U_R) = F(c2) + dF_R
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            P[k] = dF[k] + fR[k];
            Q[k] = fR[k];
        }
    }
    else
    {
        const float inv = rcp_t(S_R - S_L);
        const float wr = -S_L * inv, wl = S_R * inv, c = S_L * S_R * inv;
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            const float dU = (D1[k] + dR[k]) - dL[k]; // U_R - U_L
            P[k] = fmaf(wl, fL[k], fmaf(wr, dF[k] + fR[k], c * dU));
            Q[k] = P[k] - dF[k];
        }
    }
}

} // namespace ibtfo
