/* CPU oracle for the IBTFO per-timestep update (FP64, plain C).
 *
 * TEST INFRASTRUCTURE ONLY -- see ibtfo_oracle.h.  Compiled with
 * -ffp-contract=off (and optionally -fopenmp, which parallelises the outer
 * row loops exactly where the reference's OpenACC gang loops are).
 *
 * Every routine restates one reference routine; the citation in front of each
 * names the reference file:line.  Loop ranges, the array-of-structures scratch
 * layout (so that slot aliasing behaves the same) and the left-to-right
 * evaluation order of every expression are kept, because the parity bar is
 * bit-for-bit agreement with the reference on the same inputs.
 */
#include "ibtfo_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct or_case
{
    int n_x, n_y, ng, M, N, nsch;
    double lo_x, lo_y, hi_x, hi_y, gamma, cfl;
    int scheme, riemann, limiter, boundary, gbc, time_advance;
    double *U_OLD, *U_NEW, *U_TMP, *XY, *SCH;
    double *U_RK; /* RK2: the state at the start of the step */
    double dt, now_t, mass_start, mass_now;
    int iter;
};

#define NSLOT 28 /* 7 slots x 4 equations, Src/Base/Euler/Advection/MUSCL/EQDefine.H:5-6 */
#define IX(i, j) ((long)c->M * (long)(j) + (long)(i))
#define U_(A, i, j, k) (A)[IX(i, j) * 4 + (k)]
#define T_(i, j, s, k) c->U_TMP[IX(i, j) * NSLOT + (s) * 4 + (k)]
#define XY_(i, j, col) c->XY[IX(i, j) * 6 + (col)]
#define SC_(i, j, col) c->SCH[IX(i, j) * c->nsch + (col)]
/* scratch slots, MUSCL/EQDefine.H:33-44 (F_OLD and G_OLD share slot 2, F_L/G_D 3,
 * F_R/G_U 4, U_L/U_D 5, U_R/U_U 6) */
enum { S_FOLD = 2, S_FL = 3, S_FR = 4, S_UL = 5, S_UR = 6 };

static double smax(double a, double b) { return (a < b) ? b : a; } /* std::max */

void or_set_threads(int n)
{
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

static int nsch_of(int boundary)
{
    switch (boundary)
    {
    case OR_IDW: return 8;           /* IDWBaseGFM/SchDefine.H:4 */
    case OR_LINEAR:
    case OR_RIEMANNGFM: return 4;    /* LinearBaseGFM/SchDefine.H:4 */
    case OR_BCGFM:
    case OR_HBCGFM: return 16;       /* BCGFM/SchDefine.H:4 */
    default: return 1;               /* Regular/SchDefine.H:1 */
    }
}

or_case *or_create(int n_x, int n_y, int ng, double lo_x, double lo_y, double hi_x, double hi_y,
                   double gamma, double cfl, int scheme, int riemann, int limiter, int boundary, int gbc)
{
    if (n_x < 2 || n_y < 2 || ng < 2)
        return NULL;
    or_case *c = (or_case *)calloc(1, sizeof(or_case));
    c->n_x = n_x; c->n_y = n_y; c->ng = ng;
    c->M = n_x + 2 * ng; c->N = n_y + 2 * ng;
    c->lo_x = lo_x; c->lo_y = lo_y; c->hi_x = hi_x; c->hi_y = hi_y;
    c->gamma = gamma; c->cfl = cfl;
    c->scheme = scheme; c->riemann = riemann; c->limiter = limiter;
    c->boundary = boundary; c->gbc = gbc;
    c->nsch = nsch_of(boundary);
    long cells = (long)c->M * c->N;
    c->U_OLD = (double *)calloc(cells * 4, sizeof(double));
    c->U_NEW = (double *)calloc(cells * 4, sizeof(double));
    c->U_TMP = (double *)calloc(cells * NSLOT, sizeof(double));
    c->XY = (double *)calloc(cells * 6, sizeof(double));
    c->SCH = (double *)calloc(cells * c->nsch, sizeof(double));
    if (!c->U_OLD || !c->U_NEW || !c->U_TMP || !c->XY || !c->SCH)
    {
        or_destroy(c);
        return NULL;
    }
    return c;
}

void or_destroy(or_case *c)
{
    if (!c)
        return;
    free(c->U_OLD); free(c->U_NEW); free(c->U_TMP); free(c->XY); free(c->SCH); free(c->U_RK);
    free(c);
}

int or_num_sch(const or_case *c) { return c->nsch; }

/* ---------------------------------------------------------------- limiters */

/* Src/Base/Slope_limiter/minmod/Slope_limiter.H:4 */
static double lim_minmod(double a, double b) { return ((a * b) > 0) ? ((a / b > 1) ? b : a) : 0; }

/* Src/Base/Slope_limiter/VanLeer/Slope_limiter.H:4.  The macro body contains
 * `* b /` with b unparenthesised; every call site passes b as the text
 * `P - Q`, so the expansion evaluates `(r*r + r) * P - Q / (r*r + 1)`. */
static double lim_vanleer(double a, double P, double Q)
{
    double b = P - Q;
    double r = (a + 1e-7) / (b + 1e-7);
    return (r > 0) ? ((r * r + r) * P - Q / (r * r + 1)) : 0;
}

/* value of `0.5 * limiter(am - a0, bp - bq)` */
static double half_slope(const or_case *c, double am_hi, double am_lo, double P, double Q)
{
    double a = am_hi - am_lo;
    if (c->limiter == OR_VANLEER)
        return 0.5 * lim_vanleer(a, P, Q);
    return 0.5 * lim_minmod(a, P - Q);
}

/* ------------------------------------------------ physical flux (Conserve2Flux) */

/* Src/Base/Common/Conserve2Flux.cpp:45-78 over all cells, slot src -> slot dst */
static void c2f_x(or_case *c, int src, int dst)
{
    const double g = c->gamma;
#pragma omp parallel for
    for (int j = 0; j < c->N; j++)
        for (int i = 0; i < c->M; i++)
        {
            double rho = T_(i, j, src, 0);
            double u = T_(i, j, src, 1) / rho;
            double v = T_(i, j, src, 2) / rho;
            double p = (g - 1) * (T_(i, j, src, 3) - 0.5 * rho * (u * u + v * v));
            T_(i, j, dst, 0) = rho * u;
            T_(i, j, dst, 1) = rho * u * u + p;
            T_(i, j, dst, 2) = rho * u * v;
            T_(i, j, dst, 3) = (T_(i, j, src, 3) + p) * u;
        }
}

/* Src/Base/Common/Conserve2Flux.cpp:80-113 */
static void c2f_y(or_case *c, int src, int dst)
{
    const double g = c->gamma;
#pragma omp parallel for
    for (int j = 0; j < c->N; j++)
        for (int i = 0; i < c->M; i++)
        {
            double rho = T_(i, j, src, 0);
            double u = T_(i, j, src, 1) / rho;
            double v = T_(i, j, src, 2) / rho;
            double p = (g - 1) * (T_(i, j, src, 3) - 0.5 * rho * (u * u + v * v));
            T_(i, j, dst, 0) = rho * v;
            T_(i, j, dst, 1) = rho * u * v;
            T_(i, j, dst, 2) = rho * v * v + p;
            T_(i, j, dst, 3) = (T_(i, j, src, 3) + p) * v;
        }
}

/* ------------------------------------------------------------ HLL (= HLLC) */

/* Src/Base/Euler/Riemann/HLL/Riemann_solver.cpp:106-174 (HLLC/Riemann_solver.cpp is identical) */
static void hll_x(or_case *c)
{
    const double g = c->gamma;
    c2f_x(c, S_UL, S_FL);
    c2f_x(c, S_UR, S_FR);
#pragma omp parallel for
    for (int j = 0; j < c->N; j++)
        for (int i = 0; i < c->M; i++)
        {
            double rho_L = T_(i, j, S_UL, 0);
            double rho_R = T_(i, j, S_UR, 0);
            double u_L = T_(i, j, S_UL, 1) / rho_L;
            double v_L = T_(i, j, S_UL, 2) / rho_L;
            double p_L = (g - 1) * (T_(i, j, S_UL, 3) - 0.5 * rho_L * (u_L * u_L + v_L * v_L));
            double u_R = T_(i, j, S_UR, 1) / rho_R;
            double v_R = T_(i, j, S_UR, 2) / rho_R;
            double p_R = (g - 1) * (T_(i, j, S_UR, 3) - 0.5 * rho_R * (u_R * u_R + v_R * v_R));
            double a_L = pow((g * p_L / rho_L), 0.5);
            double a_R = pow((g * p_R / rho_R), 0.5);
            double rho_bar = 0.5 * (rho_L + rho_R);
            double a_bar = 0.5 * (a_L + a_R);
            double p_star = 0.5 * (p_L + p_R) + 0.5 * (u_L - u_R) * (rho_bar * a_bar);
            double S_L = u_L - a_L * sqrt((g + 1) * p_star / 2 / g / p_L + (g - 1) / 2 / g);
            double S_R = u_R + a_R * sqrt((g + 1) * p_star / 2 / g / p_R + (g - 1) / 2 / g);
            for (int k = 0; k < 4; k++)
            {
                if (S_L >= 0)
                    T_(i, j, S_FOLD, k) = T_(i, j, S_FL, k);
                else if (S_R <= 0)
                    T_(i, j, S_FOLD, k) = T_(i, j, S_FR, k);
                else
                    T_(i, j, S_FOLD, k) = (S_R * T_(i, j, S_FL, k) - S_L * T_(i, j, S_FR, k) +
                                           S_R * S_L * (T_(i, j, S_UR, k) - T_(i, j, S_UL, k))) /
                                          (S_R - S_L);
            }
        }
}

/* Src/Base/Euler/Riemann/HLL/Riemann_solver.cpp:177-240.  When S_D >= 0 the
 * solver stores nothing (:224-227), so slot 2 keeps the X-face flux. */
static void hll_y(or_case *c)
{
    const double g = c->gamma;
    c2f_y(c, S_UL, S_FL); /* U_D -> G_D */
    c2f_y(c, S_UR, S_FR); /* U_U -> G_U */
#pragma omp parallel for
    for (int j = 0; j < c->N; j++)
        for (int i = 0; i < c->M; i++)
        {
            double rho_U = T_(i, j, S_UR, 0);
            double rho_D = T_(i, j, S_UL, 0);
            double u_U = T_(i, j, S_UR, 1) / rho_U;
            double v_U = T_(i, j, S_UR, 2) / rho_U;
            double p_U = (g - 1) * (T_(i, j, S_UR, 3) - 0.5 * rho_U * (u_U * u_U + v_U * v_U));
            double u_D = T_(i, j, S_UL, 1) / rho_D;
            double v_D = T_(i, j, S_UL, 2) / rho_D;
            double p_D = (g - 1) * (T_(i, j, S_UL, 3) - 0.5 * rho_D * (u_D * u_D + v_D * v_D));
            double a_U = pow((g * p_U / rho_U), 0.5);
            double a_D = pow((g * p_D / rho_D), 0.5);
            double rho_bar = 0.5 * (rho_U + rho_D);
            double a_bar = 0.5 * (a_U + a_D);
            double p_star = 0.5 * (p_U + p_D) + 0.5 * (v_D - v_U) * (rho_bar * a_bar);
            double S_D = v_D - a_D * sqrt((g + 1) * p_star / 2 / g / p_D + (g - 1) / 2 / g);
            double S_U = v_U + a_U * sqrt((g + 1) * p_star / 2 / g / p_U + (g - 1) / 2 / g);
            (void)u_U; (void)u_D;
            for (int k = 0; k < 4; k++)
            {
                if (S_D >= 0)
                {
                }
                else if (S_U <= 0)
                    T_(i, j, S_FOLD, k) = T_(i, j, S_FR, k);
                else
                    T_(i, j, S_FOLD, k) = (S_U * T_(i, j, S_FL, k) - S_D * T_(i, j, S_FR, k) +
                                           S_U * S_D * (T_(i, j, S_UR, k) - T_(i, j, S_UL, k))) /
                                          (S_U - S_D);
            }
        }
}

/* ---------------------------------------------------------------- PVRS */

#define SET4(s, a0, a1, a2, a3) \
    do { T_(i, j, s, 0) = (a0); T_(i, j, s, 1) = (a1); T_(i, j, s, 2) = (a2); T_(i, j, s, 3) = (a3); } while (0)

/* Src/Base/Euler/Riemann/PVRS/Riemann_solver.cpp:286-439, including the
 * reference's S_TL (uses p_star over p_R, :331) and fan-state (rho where u belongs,
 * :375-377) formulas. */
static void pvrs_x(or_case *c)
{
    const double g = c->gamma;
#pragma omp parallel for
    for (int j = 0; j < c->N; j++)
        for (int i = 0; i < c->M; i++)
        {
            double rho_L = T_(i, j, S_UL, 0);
            double rho_R = T_(i, j, S_UR, 0);
            double u_L = T_(i, j, S_UL, 1) / rho_L;
            double v_L = T_(i, j, S_UL, 2) / rho_L;
            double p_L = (g - 1) * (T_(i, j, S_UL, 3) - 0.5 * rho_L * (u_L * u_L + v_L * v_L));
            double u_R = T_(i, j, S_UR, 1) / rho_R;
            double v_R = T_(i, j, S_UR, 2) / rho_R;
            double p_R = (g - 1) * (T_(i, j, S_UR, 3) - 0.5 * rho_R * (u_R * u_R + v_R * v_R));
            double a_L = pow((g * p_L / rho_L), 0.5);
            double a_R = pow((g * p_R / rho_R), 0.5);
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
            const double E_L = T_(i, j, S_UL, 3), E_R = T_(i, j, S_UR, 3);
#define PV_LDIRECT SET4(S_FOLD, rho_L * u_L, rho_L * u_L * u_L + p_L, rho_L * u_L * v_L, (E_L + p_L) * u_L)
#define PV_LSTAR SET4(S_FOLD, rhoL_star * u_star, rhoL_star * u_star * u_star + p_star, rhoL_star * u_star * v_L, \
                      (g * p_star / (g - 1) + 0.5 * rhoL_star * (u_star * u_star + v_L * v_L)) * u_star)
#define PV_RDIRECT SET4(S_FOLD, rho_R * u_R, rho_R * u_R * u_R + p_R, rho_R * u_R * v_R, (E_R + p_R) * u_R)
#define PV_RSTAR SET4(S_FOLD, rhoR_star * u_star, rhoR_star * u_star * u_star + p_star, rhoR_star * u_star * v_R, \
                      (g * p_star / (g - 1) + 0.5 * rhoR_star * (u_star * u_star + v_R * v_R)) * u_star)
            if (u_star > 0)
            {
                if (p_star > p_L)
                {
                    if (S_L > 0) PV_LDIRECT; else PV_LSTAR;
                }
                else
                {
                    if (S_HL > 0) PV_LDIRECT;
                    else if (S_TL < 0) PV_LSTAR;
                    else
                    {
                        double rho_f = rho_L * pow(2 / (g + 1) + (g - 1) * (rho_L) / (g + 1) / a_L, 2 / (g - 1));
                        double u_f = 2 * (a_L + (g - 1) * u_L / 2) / (g + 1);
                        double p_f = p_L * pow((2 / (g + 1) + (g - 1) * (rho_L) / (g + 1) / a_L), 2 * g / (g - 1));
                        SET4(S_FOLD, rho_f * u_f, rho_f * u_f * u_f + p_f, rho_f * u_f * v_L,
                             (g * p_f / (g - 1) + 0.5 * rho_f * (u_f * u_f + v_L * v_L)) * u_f);
                    }
                }
            }
            else
            {
                if (p_star > p_R)
                {
                    if (S_R < 0) PV_RDIRECT; else PV_RSTAR;
                }
                else
                {
                    if (S_HR < 0) PV_RDIRECT;
                    else if (S_TR > 0) PV_RSTAR;
                    else
                    {
                        double rho_f = rho_R * pow(2 / (g + 1) + (g - 1) * (rho_R) / (g + 1) / a_R, 2 / (g - 1));
                        double u_f = 2 * (a_R + (g - 1) * u_R / 2) / (g + 1);
                        double p_f = p_R * pow((2 / (g + 1) + (g - 1) * (rho_R) / (g + 1) / a_R), 2 * g / (g - 1));
                        SET4(S_FOLD, rho_f * u_f, rho_f * u_f * u_f + p_f, rho_f * u_f * v_R,
                             (g * p_f / (g - 1) + 0.5 * rho_f * (u_f * u_f + v_R * v_R)) * u_f);
                    }
                }
            }
#undef PV_LDIRECT
#undef PV_LSTAR
#undef PV_RDIRECT
#undef PV_RSTAR
        }
}

/* Src/Base/Euler/Riemann/PVRS/Riemann_solver.cpp:441-593.  The branch at
 * :547-550 stores its energy flux at U_TMP[(M*j+i)*4+3] (state indexing
 * applied to the scratch array), leaving G_OLD(i,j,3) unchanged; that store is
 * kept as written.  With the serial row-major loop it lands in a cell that has
 * already been processed. */
static void pvrs_y(or_case *c)
{
    const double g = c->gamma;
    /* the stray store makes the loop order significant: keep it serial */
    for (int j = 0; j < c->N; j++)
        for (int i = 0; i < c->M; i++)
        {
            double rho_U = T_(i, j, S_UR, 0);
            double rho_D = T_(i, j, S_UL, 0);
            double u_U = T_(i, j, S_UR, 1) / rho_U;
            double v_U = T_(i, j, S_UR, 2) / rho_U;
            double p_U = (g - 1) * (T_(i, j, S_UR, 3) - 0.5 * rho_U * (u_U * u_U + v_U * v_U));
            double u_D = T_(i, j, S_UL, 1) / rho_D;
            double v_D = T_(i, j, S_UL, 2) / rho_D;
            double p_D = (g - 1) * (T_(i, j, S_UL, 3) - 0.5 * rho_D * (u_D * u_D + v_D * v_D));
            double a_U = pow((g * p_U / rho_U), 0.5);
            double a_D = pow((g * p_D / rho_D), 0.5);
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
            const double E_D = T_(i, j, S_UL, 3), E_U = T_(i, j, S_UR, 3);
#define PV_DDIRECT SET4(S_FOLD, rho_D * v_D, rho_D * u_D * v_D, rho_D * v_D * v_D + p_D, (E_D + p_D) * v_D)
#define PV_DSTAR SET4(S_FOLD, rhoD_star * v_star, rhoD_star * v_star * u_D, rhoD_star * v_star * v_star + p_star, \
                      (g * p_star / (g - 1) + 0.5 * rhoD_star * (v_star * v_star + u_D * u_D)) * v_star)
#define PV_USTAR SET4(S_FOLD, rhoU_star * v_star, rhoU_star * v_star * u_U, rhoU_star * v_star * v_star + p_star, \
                      (g * p_star / (g - 1) + 0.5 * rhoU_star * (v_star * v_star + u_U * u_U)) * v_star)
            if (v_star > 0)
            {
                if (p_star > p_D)
                {
                    if (S_D > 0) PV_DDIRECT; else PV_DSTAR;
                }
                else
                {
                    if (S_HD > 0) PV_DDIRECT;
                    else if (S_TD < 0) PV_DSTAR;
                    else
                    {
                        double rho_f = rho_D * pow(2 / (g + 1) + (g - 1) * (rho_D) / (g + 1) / a_D, 2 / (g - 1));
                        double v_f = 2 * (a_D + (g - 1) * v_D / 2) / (g + 1);
                        double p_f = p_D * pow((2 / (g + 1) + (g - 1) * (rho_D) / (g + 1) / a_D), 2 * g / (g - 1));
                        SET4(S_FOLD, rho_f * v_f, rho_f * v_f * u_D, rho_f * v_f * v_f + p_f,
                             (g * p_f / (g - 1) + 0.5 * rho_f * (v_f * v_f + u_D * u_D)) * v_f);
                    }
                }
            }
            else
            {
                if (p_star > p_U)
                {
                    if (S_U < 0)
                    {
                        T_(i, j, S_FOLD, 0) = rho_U * v_U;
                        T_(i, j, S_FOLD, 1) = rho_U * u_U * v_U;
                        T_(i, j, S_FOLD, 2) = rho_U * v_U * v_U + p_U;
                        c->U_TMP[IX(i, j) * 4 + 3] = (E_U + p_U) * v_U;
                    }
                    else PV_USTAR;
                }
                else
                {
                    if (S_HU < 0)
                        SET4(S_FOLD, rho_U * v_U, rho_U * u_U * v_U, rho_U * v_U * v_U + p_U, (E_U + p_U) * v_U);
                    else if (S_TU > 0) PV_USTAR;
                    else
                    {
                        double rho_f = rho_U * pow(2 / (g + 1) + (g - 1) * (rho_U) / (g + 1) / a_U, 2 / (g - 1));
                        double v_f = 2 * (a_U + (g - 1) * v_U / 2) / (g + 1);
                        double p_f = p_U * pow((2 / (g + 1) + (g - 1) * (rho_U) / (g + 1) / a_U), 2 * g / (g - 1));
                        SET4(S_FOLD, rho_f * v_f, rho_f * v_f * u_U, rho_f * v_f * v_f + p_f,
                             (g * p_f / (g - 1) + 0.5 * rho_f * (v_f * v_f + u_U * u_U)) * v_f);
                    }
                }
            }
#undef PV_DDIRECT
#undef PV_DSTAR
#undef PV_USTAR
        }
}

/* ------------------------------------------------------------ Steger-Warming */

/* one side's split flux, written as the reference's expressions; `n` is the
 * face-normal velocity, `t` the tangential one.  sign = +1 for the "+" part. */
#define SW_LAM(x, sgn) (0.5 * ((x) sgn sqrt((x) * (x) + delta * delta)))

/* Src/Base/Euler/Riemann/StegerWarming/Riemann_solver.cpp:151-238 */
static void sw_x(or_case *c)
{
    const double g = c->gamma;
#pragma omp parallel for
    for (int j = 0; j < c->N; j++)
        for (int i = 0; i < c->M; i++)
        {
            double rho_L = T_(i, j, S_UL, 0);
            double rho_R = T_(i, j, S_UR, 0);
            double u_L = T_(i, j, S_UL, 1) / rho_L;
            double v_L = T_(i, j, S_UL, 2) / rho_L;
            double p_L = (g - 1) * (T_(i, j, S_UL, 3) - 0.5 * rho_L * (u_L * u_L + v_L * v_L));
            double u_R = T_(i, j, S_UR, 1) / rho_R;
            double v_R = T_(i, j, S_UR, 2) / rho_R;
            double p_R = (g - 1) * (T_(i, j, S_UR, 3) - 0.5 * rho_R * (u_R * u_R + v_R * v_R));
            double a_L = pow((g * p_L / rho_L), 0.5);
            double a_R = pow((g * p_R / rho_R), 0.5);
            double e_L = p_L / (g - 1) / rho_L;
            double e_R = p_R / (g - 1) / rho_R;
            double h_L = e_L + u_L * u_L / 2 + v_L * v_L / 2 + p_L / rho_L;
            double h_R = e_R + u_R * u_R / 2 + v_R * v_R / 2 + p_R / rho_R;
            double delta = 1e-6;
            double l1Lp = SW_LAM(u_L, +), l3Lp = SW_LAM((u_L - a_L), +), l4Lp = SW_LAM((u_L + a_L), +);
            double l1Rn = SW_LAM(u_R, -), l3Rn = SW_LAM((u_R - a_R), -), l4Rn = SW_LAM((u_R + a_R), -);
            double f1p = rho_L * (2 * (g - 1) * l1Lp + l3Lp + l4Lp) / 2 / g;
            double f2p = rho_L * (2 * (g - 1) * u_L * l1Lp + (u_L - a_L) * l3Lp + (u_L + a_L) * l4Lp) / 2 / g;
            double f3p = rho_L * (2 * (g - 1) * v_L * l1Lp + l3Lp * v_L + l4Lp * v_L) / 2 / g;
            double f4p = rho_L * ((g - 1) * (u_L * u_L + v_L * v_L) * l1Lp + (h_L - a_L * u_L) * l3Lp + (h_L + a_L * u_L) * l4Lp) / 2 / g;
            double f1n = rho_R * (2 * (g - 1) * l1Rn + l3Rn + l4Rn) / 2 / g;
            double f2n = rho_R * (2 * (g - 1) * u_R * l1Rn + (u_R - a_R) * l3Rn + (u_R + a_R) * l4Rn) / 2 / g;
            double f3n = rho_R * (2 * (g - 1) * v_R * l1Rn + l3Rn * v_R + l4Rn * v_R) / 2 / g;
            double f4n = rho_R * ((g - 1) * (u_R * u_R + v_R * v_R) * l1Rn + (h_R - a_R * u_R) * l3Rn + (h_R + a_R * u_R) * l4Rn) / 2 / g;
            T_(i, j, S_FOLD, 0) = f1p + f1n;
            T_(i, j, S_FOLD, 1) = f2p + f2n;
            T_(i, j, S_FOLD, 2) = f3p + f3n;
            T_(i, j, S_FOLD, 3) = f4p + f4n;
        }
}

/* Src/Base/Euler/Riemann/StegerWarming/Riemann_solver.cpp:240-328 */
static void sw_y(or_case *c)
{
    const double g = c->gamma;
#pragma omp parallel for
    for (int j = 0; j < c->N; j++)
        for (int i = 0; i < c->M; i++)
        {
            double rho_U = T_(i, j, S_UR, 0);
            double rho_D = T_(i, j, S_UL, 0);
            double u_U = T_(i, j, S_UR, 1) / rho_U;
            double v_U = T_(i, j, S_UR, 2) / rho_U;
            double p_U = (g - 1) * (T_(i, j, S_UR, 3) - 0.5 * rho_U * (u_U * u_U + v_U * v_U));
            double u_D = T_(i, j, S_UL, 1) / rho_D;
            double v_D = T_(i, j, S_UL, 2) / rho_D;
            double p_D = (g - 1) * (T_(i, j, S_UL, 3) - 0.5 * rho_D * (u_D * u_D + v_D * v_D));
            double a_U = pow((g * p_U / rho_U), 0.5);
            double a_D = pow((g * p_D / rho_D), 0.5);
            double e_U = p_U / (g - 1) / rho_U;
            double e_D = p_D / (g - 1) / rho_D;
            double h_U = e_U + u_U * u_U / 2 + v_U * v_U / 2 + p_U / rho_U;
            double h_D = e_D + u_D * u_D / 2 + v_D * v_D / 2 + p_D / rho_D;
            double delta = 1e-6;
            double m1Dp = SW_LAM(v_D, +), m3Dp = SW_LAM((v_D - a_D), +), m4Dp = SW_LAM((v_D + a_D), +);
            double m1Un = SW_LAM(v_U, -), m3Un = SW_LAM((v_U - a_U), -), m4Un = SW_LAM((v_U + a_U), -);
            double g1p = rho_D * (2 * (g - 1) * m1Dp + m3Dp + m4Dp) / 2 / g;
            double g2p = rho_D * (2 * (g - 1) * u_D * m1Dp + m3Dp * u_D + m4Dp * u_D) / 2 / g;
            double g3p = rho_D * (2 * (g - 1) * v_D * m1Dp + (v_D - a_D) * m3Dp + (v_D + a_D) * m4Dp) / 2 / g;
            double g4p = rho_D * ((g - 1) * (u_D * u_D + v_D * v_D) * m1Dp + (h_D - a_D * v_D) * m3Dp + (h_D + a_D * v_D) * m4Dp) / 2 / g;
            double g1n = rho_U * (2 * (g - 1) * m1Un + m3Un + m4Un) / 2 / g;
            double g2n = rho_U * (2 * (g - 1) * u_U * m1Un + m3Un * u_U + m4Un * u_U) / 2 / g;
            double g3n = rho_U * (2 * (g - 1) * v_U * m1Un + (v_U - a_U) * m3Un + (v_U + a_U) * m4Un) / 2 / g;
            double g4n = rho_U * ((g - 1) * (u_U * u_U + v_U * v_U) * m1Un + (h_U - a_U * v_U) * m3Un + (h_U + a_U * v_U) * m4Un) / 2 / g;
            T_(i, j, S_FOLD, 0) = g1p + g1n;
            T_(i, j, S_FOLD, 1) = g2p + g2n;
            T_(i, j, S_FOLD, 2) = g3p + g3n;
            T_(i, j, S_FOLD, 3) = g4p + g4n;
        }
}

static void riemann_x(or_case *c)
{
    if (c->riemann == OR_PVRS) pvrs_x(c);
    else if (c->riemann == OR_SW) sw_x(c);
    else hll_x(c);
}

static void riemann_y(or_case *c)
{
    if (c->riemann == OR_PVRS) pvrs_y(c);
    else if (c->riemann == OR_SW) sw_y(c);
    else hll_y(c);
}

/* --------------------------------------------------------------- Advance */

/* MUSCL_Scheme.cpp:30-60, MHM_Scheme.cpp:28-59, Godunov_Scheme.cpp:30-56:
 * face states of the X sweep (U_L for i in [il0, M-1), U_R for i in [0, M-2)) */
static void recon_x(or_case *c)
{
    const int M = c->M, N = c->N;
    const double *U = c->U_OLD;
    const int il0 = (c->scheme == OR_MHM) ? c->ng - 1 : 1;
#pragma omp parallel for
    for (int j = 0; j < N; j++)
        for (int i = il0; i < M - 1; i++)
            for (int k = 0; k < 4; k++)
                T_(i, j, S_UL, k) = (c->scheme == OR_GODUNOV)
                                        ? U_(U, i, j, k)
                                        : U_(U, i, j, k) + half_slope(c, U_(U, i, j, k), U_(U, i - 1, j, k),
                                                                      U_(U, i + 1, j, k), U_(U, i, j, k));
#pragma omp parallel for
    for (int j = 0; j < N; j++)
        for (int i = 0; i < M - 2; i++)
            for (int k = 0; k < 4; k++)
                T_(i, j, S_UR, k) = (c->scheme == OR_GODUNOV)
                                        ? U_(U, i + 1, j, k)
                                        : U_(U, i + 1, j, k) - half_slope(c, U_(U, i + 2, j, k), U_(U, i + 1, j, k),
                                                                          U_(U, i + 1, j, k), U_(U, i, j, k));
}

/* MUSCL_Scheme.cpp:91-121 (same ranges in MHM and Godunov): U_D for rows
 * [ng-1, N-1), U_U for rows [0, N-2), all columns */
static void recon_y(or_case *c)
{
    const int M = c->M, N = c->N, ng = c->ng;
    const double *U = c->U_OLD;
#pragma omp parallel for
    for (int j = ng - 1; j < N - 1; j++)
        for (int i = 0; i < M; i++)
            for (int k = 0; k < 4; k++)
                T_(i, j, S_UL, k) = (c->scheme == OR_GODUNOV)
                                        ? U_(U, i, j, k)
                                        : U_(U, i, j, k) + half_slope(c, U_(U, i, j, k), U_(U, i, j - 1, k),
                                                                      U_(U, i, j + 1, k), U_(U, i, j, k));
#pragma omp parallel for
    for (int j = 0; j < N - 2; j++)
        for (int i = 0; i < M; i++)
            for (int k = 0; k < 4; k++)
                T_(i, j, S_UR, k) = (c->scheme == OR_GODUNOV)
                                        ? U_(U, i, j + 1, k)
                                        : U_(U, i, j + 1, k) - half_slope(c, U_(U, i, j + 2, k), U_(U, i, j + 1, k),
                                                                          U_(U, i, j + 1, k), U_(U, i, j, k));
}

/* MHM_Scheme.cpp:61-96 (X, h = dt/dx) and :148-183 (Y, h = dt/dy): half-step
 * predictor built from the two states of the same interface */
static void mhm_predict(or_case *c, int ydir, double dt, double h)
{
    const int M = c->M, N = c->N, ng = c->ng;
    if (ydir)
    {
        c2f_y(c, S_UL, S_FL);
        c2f_y(c, S_UR, S_FR);
    }
    else
    {
        c2f_x(c, S_UL, S_FL);
        c2f_x(c, S_UR, S_FR);
    }
    /* U_L (X: rows all, i in [ng-1, M-1)) / U_D (Y: rows [ng-1, N-1), all i) */
    const int j0 = ydir ? ng - 1 : 0, j1 = ydir ? N - 1 : N;
    const int i0 = ydir ? 0 : ng - 1, i1 = ydir ? M : M - 1;
#pragma omp parallel for
    for (int j = j0; j < j1; j++)
        for (int i = i0; i < i1; i++)
            for (int k = 0; k < 4; k++)
                T_(i, j, S_UL, k) = T_(i, j, S_UL, k) + 0.5 * (T_(i, j, S_FL, k) - T_(i, j, S_FR, k)) * dt / h;
    /* U_R (X: rows all, i in [0, M-2)) / U_U (Y: rows [0, N-2), all i) */
    const int k1 = ydir ? N - 2 : N, m1 = ydir ? M : M - 2;
#pragma omp parallel for
    for (int j = 0; j < k1; j++)
        for (int i = 0; i < m1; i++)
            for (int k = 0; k < 4; k++)
                T_(i, j, S_UR, k) = T_(i, j, S_UR, k) + 0.5 * (T_(i, j, S_FL, k) - T_(i, j, S_FR, k)) * dt / h;
}

/* Lax_Scheme.cpp:15-60: U_TMP = U_OLD and Conserve2Flux (Conserve2Flux.cpp:2-37)
 * over every cell, then the Lax-Friedrichs update of the fluid cells.  The
 * fluxes are kept in scratch slots 2 (F) and 3 (G), as in the Lax
 * scheme's own layout (Lax/EQDefine.H: U_TMP, U_TMPRK, F_OLD, G_OLD). */
static void lax_advance(or_case *c, double dt)
{
    const int M = c->M, N = c->N, ng = c->ng, n_x = c->n_x;
    const double g = c->gamma;
    const double dx = (c->hi_x - c->lo_x) / c->n_x;
    const double dy = (c->hi_y - c->lo_y) / c->n_y;
    const double *U = c->U_OLD;
    double *V = c->U_NEW;
#pragma omp parallel for
    for (int j = 0; j < N; j++)
        for (int i = 0; i < M; i++)
        {
            double rho = U_(U, i, j, 0);
            double u = U_(U, i, j, 1) / rho;
            double v = U_(U, i, j, 2) / rho;
            double p = (g - 1) * (U_(U, i, j, 3) - 0.5 * rho * (u * u + v * v));
            T_(i, j, 2, 0) = rho * u;
            T_(i, j, 2, 1) = rho * u * u + p;
            T_(i, j, 2, 2) = rho * u * v;
            T_(i, j, 2, 3) = (U_(U, i, j, 3) + p) * u;
            T_(i, j, 3, 0) = rho * v;
            T_(i, j, 3, 1) = rho * u * v;
            T_(i, j, 3, 2) = rho * v * v + p;
            T_(i, j, 3, 3) = (U_(U, i, j, 3) + p) * v;
        }
#pragma omp parallel for
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            for (int k = 0; k < 4; k++)
                if (XY_(i, j, 5) == 0)
                    U_(V, i, j, k) = 0.25 * (U_(U, i - 1, j, k) + U_(U, i + 1, j, k) + U_(U, i, j + 1, k) +
                                             U_(U, i, j - 1, k)) -
                                     0.5 * dt * (T_(i + 1, j, 2, k) - T_(i - 1, j, 2, k)) / dx -
                                     0.5 * dt * (T_(i, j + 1, 3, k) - T_(i, j - 1, 3, k)) / dy;
}

/* Advance: MUSCL_Scheme.cpp:6-152, MHM_Scheme.cpp:5-203, Godunov_Scheme.cpp:6-140,
 * Lax_Scheme.cpp:2-64 */
void or_advance(or_case *c, double dt)
{
    const int ng = c->ng, N = c->N, n_x = c->n_x;
    const double dx = (c->hi_x - c->lo_x) / c->n_x;
    const double dy = (c->hi_y - c->lo_y) / c->n_y;
    double *U = c->U_OLD, *V = c->U_NEW;
    if (c->scheme == OR_LAX)
    {
        lax_advance(c, dt);
        return;
    }

    recon_x(c);
    if (c->scheme == OR_MHM)
        mhm_predict(c, 0, dt, dx);
    riemann_x(c);
#pragma omp parallel for
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            for (int k = 0; k < 4; k++)
                if (XY_(i, j, 5) == 0)
                    U_(V, i, j, k) = U_(U, i, j, k) - dt * (T_(i, j, S_FOLD, k) - T_(i - 1, j, S_FOLD, k)) / dx;

    recon_y(c);
    if (c->scheme == OR_MHM)
        mhm_predict(c, 1, dt, dy);
    riemann_y(c);
#pragma omp parallel for
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            for (int k = 0; k < 4; k++)
                if (XY_(i, j, 5) == 0)
                    U_(V, i, j, k) = U_(V, i, j, k) - dt * (T_(i, j, S_FOLD, k) - T_(i, j - 1, S_FOLD, k)) / dy;
}

/* ---------------------------------------------------------------- CFL / mass */

/* Src/Base/Common/ComputeDt.cpp:4-51 */
double or_compute_dt(or_case *c)
{
    const int ng = c->ng, N = c->N, n_x = c->n_x;
    const double g = c->gamma;
    double a_max = 0.0, u_max = 0.0, v_max = 0.0;
    const double dx = (c->hi_x - c->lo_x) / c->n_x;
    const double *U = c->U_OLD;
#pragma omp parallel for reduction(max : a_max, u_max, v_max)
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            if (XY_(i, j, 5) < 1)
            {
                double rho = U_(U, i, j, 0);
                double u = U_(U, i, j, 1) / U_(U, i, j, 0);
                double v = U_(U, i, j, 2) / U_(U, i, j, 0);
                double p = (g - 1) * (U_(U, i, j, 3) - 0.5 * rho * (u * u + v * v));
                double a = pow((g * p / rho), 0.5);
                a_max = smax(a_max, a);
                u_max = smax(u_max, fabs(u));
                v_max = smax(v_max, fabs(v));
            }
    return c->cfl * dx / (a_max + smax(u_max, v_max));
}

/* Src/Utils/CaculateMass.cpp:5-42 (rows [0, N), fluid cells only) */
double or_mass(or_case *c)
{
    const int ng = c->ng, N = c->N, n_x = c->n_x;
    const double dx = (c->hi_x - c->lo_x) / c->n_x;
    const double dy = (c->hi_y - c->lo_y) / c->n_y;
    double mass = 0;
    const double *U = c->U_OLD;
#pragma omp parallel for reduction(+ : mass)
    for (int j = 0; j < N; j++)
        for (int i = ng; i < n_x + ng; i++)
            if (XY_(i, j, 5) < 0.5)
                mass += U_(U, i, j, 0) * dx * dy;
    return mass;
}

/* ---------------------------------------------------------------- geometry */

/* Src/Geometry/Psy_coord.cpp:5-39 (dy is Psy_L/N_x, as in the reference) */
static void psy_coord(or_case *c)
{
    const double Psy_L = c->hi_x - c->lo_x;
    const double dx = Psy_L / c->n_x;
    const double dy = Psy_L / c->n_x;
    double Li = -dx * c->ng + c->lo_x + dx / 2;
    double Hi = -dy * c->ng + c->lo_y + dy / 2;
    for (int j = 0; j < c->N; j++)
        for (int i = 0; i < c->M; i++)
        {
            XY_(i, j, 0) = Li + i * dx;
            XY_(i, j, 1) = Hi + j * dx;
        }
}

/* Src/Geometry/Level_Set.cpp:6-128, with phi supplied by the caller in place
 * of the per-case Level_Set_function plug-in */
static void level_set(or_case *c, const double *phi)
{
    const int M = c->M, N = c->N, ng = c->ng, n_x = c->n_x, n_y = c->n_y;
    for (long q = 0; q < (long)M * N; q++)
        c->XY[q * 6 + 2] = phi[q];
    for (int j = 1; j < N - 1; j++)
        for (int i = 1; i < M - 1; i++)
        {
            XY_(i, j, 3) = (XY_(i + 1, j, 2) - XY_(i - 1, j, 2)) / ((XY_(i + 1, j, 0) - XY_(i - 1, j, 0)));
            XY_(i, j, 4) = (XY_(i, j + 1, 2) - XY_(i, j - 1, 2)) / ((XY_(i, j + 1, 1) - XY_(i, j - 1, 1)));
        }
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            XY_(i, j, 5) = (XY_(i, j, 2) >= 0) ? 0 : 1;
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            if (XY_(i, j, 5) == 0)
                for (int k = 1; k < ng + 1; k++)
                {
                    XY_(i + k, j, 5) = 2 * XY_(i + k, j, 5);
                    XY_(i - k, j, 5) = 2 * XY_(i - k, j, 5);
                    XY_(i, j + k, 5) = 2 * XY_(i, j + k, 5);
                    XY_(i, j - k, 5) = 2 * XY_(i, j - k, 5);
                }
    for (int j = 0; j < N; j++)
        for (int i = 0; i < M; i++)
            if (XY_(i, j, 5) > 1)
                XY_(i, j, 5) = 2;
    for (int j = 0; j < N; j++)
        for (int i = 0; i < M; i++)
            if (i < ng || i >= n_x + ng || j < ng || j >= n_y + ng)
                XY_(i, j, 5) = 2;
}

/* Src/Geometry/Mirror_IDX.cpp:6-64: bracket search by linear scan, last match wins */
static void mirror_idx(or_case *c, int kp)
{
    const int M = c->M, N = c->N, ng = c->ng, n_x = c->n_x;
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            if (XY_(i, j, 5) > 1)
            {
                double xm = SC_(i, j, kp);
                for (int ii = 0; ii < M - 1; ii++)
                    if (xm < XY_(ii + 1, j, 0) && xm >= XY_(ii, j, 0))
                        SC_(i, j, kp + 2) = ii;
            }
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            if (XY_(i, j, 5) > 1)
            {
                double ym = SC_(i, j, kp + 1);
                for (int jj = 0; jj < N - 1; jj++)
                    if (ym < XY_(0, jj + 1, 1) && ym >= XY_(0, jj, 1))
                        SC_(i, j, kp + 3) = jj;
            }
}

/* inverse-distance weights of the four bracket corners around the probe point
 * stored at slots (kp, kp+1) with bracket (kp+2, kp+3), into slots wslot..+3.
 * IDWBaseGFM/GFM_Method.cpp:60-120 (corner test `type < 1`) and
 * BCGFM/BCGFM_Method.cpp:90-208 (corner test `type != 1`). */
static void idw_weights(or_case *c, int kp, int wslot, int ne_one)
{
    const int N = c->N, ng = c->ng, n_x = c->n_x;
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            if (XY_(i, j, 5) > 1)
            {
                int IDX = (int)SC_(i, j, kp + 2);
                int IDY = (int)SC_(i, j, kp + 3);
                const int ci[4] = {IDX, IDX, IDX + 1, IDX + 1};
                const int cj[4] = {IDY, IDY + 1, IDY + 1, IDY};
                double a[4] = {0, 0, 0, 0};
                for (int q = 0; q < 4; q++)
                {
                    double t = XY_(ci[q], cj[q], 5);
                    if (ne_one ? (t != 1) : (t < 1))
                    {
                        double d = sqrt((XY_(ci[q], cj[q], 0) - SC_(i, j, kp)) * (XY_(ci[q], cj[q], 0) - SC_(i, j, kp)) +
                                        (XY_(ci[q], cj[q], 1) - SC_(i, j, kp + 1)) * (XY_(ci[q], cj[q], 1) - SC_(i, j, kp + 1)));
                        a[q] = 1 / d;
                    }
                }
                for (int q = 0; q < 4; q++)
                    SC_(i, j, wslot + q) = a[q];
            }
}

/* Scheme_Index for each boundary variant:
 * IDWBaseGFM/GFM_Method.cpp:5-113, LinearBaseGFM/GFM_Method.cpp:5-47,
 * BCGFM/BCGFM_Method.cpp:7-210, HBCGFM/HBCGFM_Method.cpp (|phi| > delta switch) */
static void scheme_index(or_case *c)
{
    const int N = c->N, ng = c->ng, n_x = c->n_x;
    if (c->boundary == OR_REGULAR)
        return;
    if (c->boundary == OR_IDW || c->boundary == OR_LINEAR || c->boundary == OR_RIEMANNGFM)
    {
        for (int j = ng; j < N - ng; j++)
            for (int i = ng; i < n_x + ng; i++)
            {
                if (XY_(i, j, 5) > 1)
                {
                    SC_(i, j, 0) = XY_(i, j, 0) + 2 * XY_(i, j, 3) * fabs(XY_(i, j, 2));
                    SC_(i, j, 1) = XY_(i, j, 1) + 2 * XY_(i, j, 4) * fabs(XY_(i, j, 2));
                }
                else
                {
                    SC_(i, j, 0) = 0;
                    SC_(i, j, 1) = 0;
                }
            }
        mirror_idx(c, 0);
        if (c->boundary == OR_IDW)
            idw_weights(c, 0, 4, 0);
        return;
    }
    /* BCGFM / HBCGFM */
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
        {
            if (XY_(i, j, 5) > 1)
            {
                double dx = XY_(1, 1, 0) - XY_(0, 1, 0);
                double dy = XY_(1, 2, 1) - XY_(1, 1, 1);
                double delta = sqrt(dx * dx + dy * dy) / 2;
                double ap = fabs(XY_(i, j, 2));
                if (c->boundary == OR_HBCGFM && ap > delta)
                {
                    SC_(i, j, 0) = XY_(i, j, 0) + XY_(i, j, 3) * (2 * ap);
                    SC_(i, j, 1) = XY_(i, j, 1) + XY_(i, j, 4) * (2 * ap);
                    SC_(i, j, 8) = XY_(i, j, 0) + XY_(i, j, 3) * (2 * ap);
                    SC_(i, j, 9) = XY_(i, j, 1) + XY_(i, j, 4) * (2 * ap);
                }
                else
                {
                    SC_(i, j, 0) = XY_(i, j, 0) + XY_(i, j, 3) * (ap + delta);
                    SC_(i, j, 1) = XY_(i, j, 1) + XY_(i, j, 4) * (ap + delta);
                    SC_(i, j, 8) = XY_(i, j, 0) + XY_(i, j, 3) * (ap + 2 * delta);
                    SC_(i, j, 9) = XY_(i, j, 1) + XY_(i, j, 4) * (ap + 2 * delta);
                }
            }
            else
            {
                SC_(i, j, 0) = 0;
                SC_(i, j, 1) = 0;
                SC_(i, j, 8) = 0;
                SC_(i, j, 9) = 0;
            }
        }
    mirror_idx(c, 0);
    mirror_idx(c, 8);
    idw_weights(c, 0, 4, 1);
    idw_weights(c, 8, 12, 1);
}

void or_setup_geometry(or_case *c, const double *phi)
{
    psy_coord(c);
    level_set(c, phi);
    scheme_index(c);
}

/* --------------------------------------------------------------- boundaries */

/* primitive variables of U_NEW at (i, j), as every GFM fill computes them */
static void prim(const or_case *c, int i, int j, double *rho, double *u, double *v, double *p)
{
    const double g = c->gamma;
    const double *V = c->U_NEW;
    *rho = U_(V, i, j, 0);
    *u = U_(V, i, j, 1) / *rho;
    *v = U_(V, i, j, 2) / *rho;
    *p = (g - 1) * (U_(V, i, j, 3) - 0.5 * *rho * (*u * *u + *v * *v));
}

/* conserved ghost value from primitives after reflecting u_n, IDWBaseGFM/GFM_Bound.cpp:219-228 */
static void store_reflected(or_case *c, int i, int j, double rho_w, double u_w, double v_w, double p_w)
{
    const double g = c->gamma;
    double n_x = XY_(i, j, 3), n_y = XY_(i, j, 4);
    double u_n = u_w * n_x + v_w * n_y;
    double u_t = u_w * n_y - v_w * n_x;
    u_n = -u_n;
    u_w = u_n * n_x + u_t * n_y;
    v_w = u_n * n_y - u_t * n_x;
    double *U = c->U_OLD;
    U_(U, i, j, 0) = rho_w;
    U_(U, i, j, 1) = rho_w * u_w;
    U_(U, i, j, 2) = rho_w * v_w;
    U_(U, i, j, 3) = p_w / (g - 1) + 0.5 * rho_w * (u_w * u_w + v_w * v_w);
}

/* IDW average at the bracket (IDX, IDY) with weights a[0..3] (corner order
 * (IDX,IDY), (IDX,IDY+1), (IDX+1,IDY+1), (IDX+1,IDY)), GFM_Bound.cpp:195-217 */
static void idw_average(const or_case *c, int IDX, int IDY, const double *a, double *w)
{
    double r[4], u[4], v[4], p[4];
    prim(c, IDX, IDY, &r[0], &u[0], &v[0], &p[0]);
    prim(c, IDX, IDY + 1, &r[1], &u[1], &v[1], &p[1]);
    prim(c, IDX + 1, IDY + 1, &r[2], &u[2], &v[2], &p[2]);
    prim(c, IDX + 1, IDY, &r[3], &u[3], &v[3], &p[3]);
    double s = a[0] + a[1] + a[2] + a[3];
    w[0] = (a[0] * r[0] + a[1] * r[1] + a[2] * r[2] + a[3] * r[3]) / s;
    w[1] = (a[0] * u[0] + a[1] * u[1] + a[2] * u[2] + a[3] * u[3]) / s;
    w[2] = (a[0] * v[0] + a[1] * v[1] + a[2] * v[2] + a[3] * v[3]) / s;
    w[3] = (a[0] * p[0] + a[1] * p[1] + a[2] * p[2] + a[3] * p[3]) / s;
}

/* LinearBaseGFM/GFM_Bound.cpp:58-575: one corner picked by the fluid pattern
 * of the four bracket corners and by x_d (the reference computes y_d from x
 * coordinates too, :100-101).  Returns the corner number 1..4, or 0 when no
 * corner is fluid (the ghost value then stays all-zero primitives). */
static int linear_pick(double t1, double t2, double t3, double t4, int xbig, int ybig)
{
    const int f1 = t1 < 1, f2 = t2 < 1, f3 = t3 < 1, f4 = t4 < 1;
    if (f1 && f4 && f2 && f3) return ybig ? (xbig ? 3 : 2) : (xbig ? 4 : 1); /* case 1 */
    if (!f1 && f4 && f2 && f3) return ybig ? (xbig ? 3 : 2) : 4;             /* case 2 */
    if (f1 && !f4 && f2 && f3) return ybig ? (xbig ? 3 : 2) : 1;             /* case 3 */
    if (f1 && f4 && !f2 && f3) return ybig ? 3 : (xbig ? 4 : 1);             /* case 4 */
    if (f1 && f4 && f2 && !f3) return ybig ? 2 : (xbig ? 4 : 1);             /* case 5 */
    if (f1 && f4 && !f2 && !f3) return xbig ? 4 : 1;                         /* case 6 */
    if (!f1 && !f4 && f2 && f3) return xbig ? 3 : 2;                         /* case 7 */
    if (f1 && !f4 && f2 && !f3) return ybig ? 2 : 1;                         /* case 8 */
    if (!f1 && f4 && !f2 && f3) return ybig ? 3 : 4;                         /* case 9 */
    if (f1 && !f4 && !f2 && f3) return ybig ? 3 : 1;                         /* case 10 */
    if (!f1 && f4 && f2 && !f3) return ybig ? 2 : 4;                         /* case 11 */
    if (f1 && !f4 && !f2 && !f3) return 1;                                   /* case 12 */
    if (!f1 && !f4 && f2 && !f3) return 2;                                   /* case 13 */
    if (!f1 && !f4 && !f2 && f3) return 3;                                   /* case 14 */
    if (!f1 && f4 && !f2 && !f3) return 4;                                   /* case 15 */
    return 0;
}

/* Boundary for each variant: Regular/RegularBound.cpp:6-36,
 * IDWBaseGFM/GFM_Bound.cpp:5-148, LinearBaseGFM/GFM_Bound.cpp:5-627,
 * BCGFM/BCGFM_Bound.cpp:6-240, HBCGFM/HBCGFM_Bound.cpp */
void or_boundary(or_case *c)
{
    const int M = c->M, N = c->N, ng = c->ng, n_x = c->n_x;
    double *U = c->U_OLD, *V = c->U_NEW;
    if (c->boundary == OR_REGULAR)
    {
        for (int j = ng; j < N - ng; j++)
            for (int i = ng; i < n_x + ng; i++)
                for (int k = 0; k < 4; k++)
                    U_(U, i, j, k) = U_(V, i, j, k);
        return;
    }
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            for (int k = 0; k < 4; k++)
                if (XY_(i, j, 5) == 0)
                    U_(U, i, j, k) = U_(V, i, j, k);
    memcpy(V, U, sizeof(double) * 4 * (size_t)M * N);

    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
        {
            if (!(XY_(i, j, 5) > 1))
                continue;
            if (c->boundary == OR_IDW)
            {
                double a[4] = {SC_(i, j, 4), SC_(i, j, 5), SC_(i, j, 6), SC_(i, j, 7)}, w[4];
                idw_average(c, (int)SC_(i, j, 2), (int)SC_(i, j, 3), a, w);
                store_reflected(c, i, j, w[0], w[1], w[2], w[3]);
            }
            else if (c->boundary == OR_LINEAR || c->boundary == OR_RIEMANNGFM)
            {
                int IDX = (int)SC_(i, j, 2), IDY = (int)SC_(i, j, 3);
                double dx = XY_(1, 1, 0) - XY_(0, 1, 0);
                double dy = XY_(1, 2, 1) - XY_(1, 1, 1);
                double r[5] = {0}, u[5] = {0}, v[5] = {0}, p[5] = {0};
                prim(c, IDX, IDY, &r[1], &u[1], &v[1], &p[1]);
                prim(c, IDX, IDY + 1, &r[2], &u[2], &v[2], &p[2]);
                prim(c, IDX + 1, IDY + 1, &r[3], &u[3], &v[3], &p[3]);
                prim(c, IDX + 1, IDY, &r[4], &u[4], &v[4], &p[4]);
                double x_d = SC_(i, j, 0) - XY_(IDX, IDY, 0);
                double y_d = SC_(i, j, 0) - XY_(IDX, IDY, 0);
                int q = linear_pick(XY_(IDX, IDY, 5), XY_(IDX, IDY + 1, 5), XY_(IDX + 1, IDY + 1, 5),
                                    XY_(IDX + 1, IDY, 5), x_d > dx / 2, y_d > dy / 2);
                store_reflected(c, i, j, r[q], u[q], v[q], p[q]);
            }
            else
            {
                const double g = c->gamma;
                double dx = XY_(1, 1, 0) - XY_(0, 1, 0);
                double dy = XY_(1, 2, 1) - XY_(1, 1, 1);
                double delta = sqrt(dx * dx + dy * dy) / 2;
                double R_E = (c->boundary == OR_HBCGFM) ? 1.0 * delta : delta;
                double R_G = fabs(XY_(i, j, 2));
                double n_x = XY_(i, j, 3), n_y = XY_(i, j, 4);
                double ai[4] = {SC_(i, j, 4), SC_(i, j, 5), SC_(i, j, 6), SC_(i, j, 7)}, wi[4];
                double ae[4] = {SC_(i, j, 12), SC_(i, j, 13), SC_(i, j, 14), SC_(i, j, 15)}, we[4];
                idw_average(c, (int)SC_(i, j, 2), (int)SC_(i, j, 3), ai, wi);
                double u_n_i = wi[1] * n_x + wi[2] * n_y;
                double u_t_i = wi[1] * n_y - wi[2] * n_x;
                idw_average(c, (int)SC_(i, j, 10), (int)SC_(i, j, 11), ae, we);
                double u_n_e = we[1] * n_x + we[2] * n_y;
                double u_t_e = we[1] * n_y - we[2] * n_x;
                double rho_m, p_m, u_t_m, u_n_m;
                if (c->boundary == OR_HBCGFM && fabs(XY_(i, j, 2)) > delta)
                {
                    rho_m = wi[0];
                    p_m = wi[3];
                    u_t_m = u_t_i;
                    u_n_m = -u_n_i;
                }
                else
                {
                    rho_m = (wi[0] * ((delta + R_E) * (delta + R_E) - R_G * R_G) - we[0] * (delta * delta - R_G * R_G)) / (R_E * R_E + 2 * delta * R_E);
                    p_m = (wi[3] * ((delta + R_E) * (delta + R_E) - R_G * R_G) - we[3] * (delta * delta - R_G * R_G)) / (R_E * R_E + 2 * delta * R_E);
                    u_t_m = (u_t_i * ((delta + R_E) * (delta + R_E) - R_G * R_G) - u_t_e * (delta * delta - R_G * R_G)) / (R_E * R_E + 2 * delta * R_E);
                    u_n_m = -(u_n_i * ((delta + R_E) * (delta + R_E) - R_G * R_G) - u_n_e * (delta * delta - R_G * R_G)) / (R_E * R_E + 2 * delta * R_E);
                }
                double u_m = u_n_m * n_x + u_t_m * n_y;
                double v_m = u_n_m * n_y - u_t_m * n_x;
                U_(U, i, j, 0) = rho_m;
                U_(U, i, j, 1) = rho_m * u_m;
                U_(U, i, j, 2) = rho_m * v_m;
                U_(U, i, j, 3) = p_m / (g - 1) + 0.5 * rho_m * (u_m * u_m + v_m * v_m);
            }
        }
}

/* Global_Boundary.  Walls: Test/Sod/Global_Boudary.cpp:9-77 (identical in
 * Test/InclineSod and Test/Vortex): ghost rows from interior rows 2ng-1 and
 * N_y+ng-1 of U_NEW, then rho*v mirrored, then ghost columns from U_NEW
 * columns ng and N_x+ng-1 over every row.  Periodic: the harness plug-in
 * (oracle/harness/gb_periodic.cpp), which the reference does not have. */
void or_global_boundary(or_case *c)
{
    const int N = c->N, ng = c->ng, n_x = c->n_x, n_y = c->n_y;
    double *U = c->U_OLD, *V = c->U_NEW;
    if (c->gbc == OR_GB_PERIODIC)
    {
        for (int j = 0; j < N; j++)
            for (int i = ng; i < n_x + ng; i++)
                for (int k = 0; k < 4; k++)
                {
                    if (j < ng)
                        U_(U, i, j, k) = U_(V, i, j + n_y, k);
                    if (j >= n_y + ng)
                        U_(U, i, j, k) = U_(V, i, j - n_y, k);
                }
        for (int j = 0; j < N; j++)
            for (int i = 0; i < ng; i++)
                for (int k = 0; k < 4; k++)
                {
                    U_(U, i, j, k) = U_(U, i + n_x, j, k);
                    U_(U, n_x + ng + i, j, k) = U_(U, ng + i, j, k);
                }
        return;
    }
    for (int j = 0; j < N; j++)
        for (int i = ng; i < n_x + ng; i++)
            for (int k = 0; k < 4; k++)
            {
                if (j < ng)
                    U_(U, i, j, k) = U_(V, i, 2 * ng - 1, k);
                if (j >= n_y + ng)
                    U_(U, i, j, k) = U_(V, i, n_y + ng - 1, k);
            }
    for (int j = 0; j < N; j++)
        for (int i = ng; i < n_x + ng; i++)
        {
            if (j < ng)
                U_(U, i, j, 2) = -U_(V, i, 2 * ng - j - 1, 2);
            if (j >= n_y + ng)
                U_(U, i, j, 2) = -U_(V, i, 2 * (n_y + ng) - 1 - j, 2);
        }
    for (int j = 0; j < N; j++)
        for (int i = 0; i < ng; i++)
            for (int k = 0; k < 4; k++)
            {
                U_(U, i, j, k) = U_(V, ng, j, k);
                U_(U, n_x + ng + i, j, k) = U_(V, n_x + ng - 1, j, k);
            }
}

/* ---------------------------------------------------------------- driver */

void or_set_initial_state(or_case *c, const double *u0)
{
    long n = (long)c->M * c->N * 4;
    memcpy(c->U_OLD, u0, sizeof(double) * n);
    memcpy(c->U_NEW, u0, sizeof(double) * n);
    or_boundary(c);
    c->dt = or_compute_dt(c);
    c->mass_start = c->mass_now = or_mass(c);
    c->now_t = 0.0;
    c->iter = 0;
}

void or_set_time_advance(or_case *c, int time_advance) { c->time_advance = time_advance; }

/* Time = RK2 (Src/Base/TimeAdvance/RK2/RK2.cpp:12-48 names the stages: Advance,
 * Boundary, Global_Boundary, Advance, then U_NEW = 0.5 (U_OLD + U_TMPRK) on
 * fluid cells and U_NEW = U_OLD elsewhere).  That file does not compile
 * (its signatures lack ndevices/device), its second Advance stores U_TMPRK
 * with the state's stride (4 per cell) while the average reads it with the
 * scratch stride, and by the time of the average Boundary has overwritten
 * U_OLD with the first stage.  This restates the two-stage method the file
 * describes, Heun's method: U1 = U0 + dt L(U0) with its ghost and edge
 * fills, U_NEW = 0.5 (U0 + (U1 + dt L(U1))) on fluid cells (U1 elsewhere),
 * both stages with the dt computed before the step. */
static void rk2_advance(or_case *c, double dt)
{
    const int ng = c->ng, N = c->N, n_x = c->n_x;
    const long n = (long)c->M * c->N * 4;
    if (!c->U_RK)
        c->U_RK = (double *)malloc(sizeof(double) * n);
    memcpy(c->U_RK, c->U_OLD, sizeof(double) * n);
    or_advance(c, dt);
    or_boundary(c);
    or_global_boundary(c);
    or_advance(c, dt);
    double *U = c->U_OLD, *V = c->U_NEW, *U0 = c->U_RK;
#pragma omp parallel for
    for (int j = ng; j < N - ng; j++)
        for (int i = ng; i < n_x + ng; i++)
            for (int k = 0; k < 4; k++)
            {
                if (XY_(i, j, 5) == 0)
                    U_(V, i, j, k) = 0.5 * (U_(U0, i, j, k) + U_(V, i, j, k));
                else
                    U_(V, i, j, k) = U_(U, i, j, k);
            }
}

/* time loop, Test/Sod/Sod.cpp:123-181: the dt applied in a step is the one
 * computed before it, and now_t advances by the dt computed after it (:176) */
int or_run(or_case *c, int nsteps, double t_end, int max_iter, double *dts, double *masses)
{
    int done = 0;
    while (c->now_t < t_end && c->iter < max_iter && done < nsteps)
    {
        if (c->time_advance == OR_RK2)
            rk2_advance(c, c->dt);
        else
            or_advance(c, c->dt);
        or_boundary(c);
        or_global_boundary(c);
        c->dt = or_compute_dt(c);
        c->mass_now = or_mass(c);
        c->now_t = c->now_t + c->dt;
        c->iter++;
        if (dts)
            dts[done] = c->dt;
        if (masses)
            masses[done] = c->mass_now;
        done++;
    }
    return done;
}

long or_array_len(const or_case *c, int which)
{
    long cells = (long)c->M * c->N;
    switch (which)
    {
    case 0:
    case 1: return cells * 4;
    case 2: return cells * 6;
    case 3: return cells * c->nsch;
    case 4: return cells * NSLOT;
    default: return 0;
    }
}

static double *arr(const or_case *c, int which)
{
    switch (which)
    {
    case 0: return c->U_OLD;
    case 1: return c->U_NEW;
    case 2: return c->XY;
    case 3: return c->SCH;
    case 4: return c->U_TMP;
    default: return NULL;
    }
}

void or_get(const or_case *c, int which, double *dst)
{
    long n = or_array_len(c, which);
    if (n)
        memcpy(dst, arr(c, which), sizeof(double) * n);
}

void or_put(or_case *c, int which, const double *src)
{
    long n = or_array_len(c, which);
    if (n)
        memcpy(arr(c, which), src, sizeof(double) * n);
}

void or_scalars(const or_case *c, double *out4)
{
    out4[0] = c->dt;
    out4[1] = c->now_t;
    out4[2] = c->mass_start;
    out4[3] = c->mass_now;
}

int or_iter(const or_case *c) { return c->iter; }
