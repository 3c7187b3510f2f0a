/* CPU restatement of the library's cut-cell method (boundary key CCM) in
 * plain FP64 C -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * The reference has no cut-cell method, so there is nothing of the
 * reference's to pin this to ("parity unpinned"): it restates the
 * algorithm the library documents -- corner level set as the mean of the
 * four cells around a corner, face apertures from linear crossings, volume
 * fractions from the fluid polygon, first-order faces next to the body, the
 * mirrored-state wall flux, the FP64 cut-cell update, conservative mixing of
 * cells with volume fraction below 0.5, the domain-edge pass -- serially,
 * from its definitions, so that the GPU kernels can be checked against an
 * independent evaluation.  Checks of the algorithm itself (conservation,
 * free-stream preservation, volume of a body) are in tests/test_ccm_cpu.py.
 *
 * Layout: structure-of-arrays planes U[k][j*M + i], two buffers, ng ghost
 * layers, as the library's planes (without its row padding). */
#include <math.h>
#include <stdlib.h>
#include <string.h>

enum { T_FLUID = 0, T_SOLID = 1, T_GHOST = 2, T_CUT = 3 };
enum { S_MUSCL = 0, S_MHM = 1, S_GODUNOV = 2 };
enum { R_SW = 3, R_HLLCT = 4, R_HLLT = 5 }; /* the library's solver keys */

typedef struct
{
    int n_x, n_y, ng, M, N;
    double lo_x, lo_y, hi_x, hi_y, dx, dy, Li, Hi, gamma, cfl, t_end;
    int scheme, riemann, limiter, periodic, max_iter;
    double gm1, c1, c2;
    double *U[2][4];
    double *alpha, *ax, *ay;
    unsigned char *type;
    /* mixing */
    int nex;
    long *ex_s, *ex_t;
    double *ex_w;
    double *E;
    int npart;
    long *part_o;
    double *part_inv;
    int *part_first, *part_count, *links;
    /* loop */
    int cur, iter;
    double dt, now_t, mass, mass_start;
} ccm_case;

#define IDX(c, i, j) ((long)(j) * (c)->M + (i))

static int interior(const ccm_case *c, int i, int j)
{
    return i >= c->ng && i < c->ng + c->n_x && j >= c->ng && j < c->ng + c->n_y;
}
static int updated(unsigned char t) { return t == T_FLUID || t == T_CUT; }

ccm_case *ccm_create(int n_x, int n_y, int ng, double lo_x, double lo_y, double hi_x, double hi_y, double gamma,
                     double cfl, double t_end, int scheme, int riemann, int limiter, int periodic)
{
    ccm_case *c = (ccm_case *)calloc(1, sizeof(ccm_case));
    c->n_x = n_x;
    c->n_y = n_y;
    c->ng = ng;
    c->M = n_x + 2 * ng;
    c->N = n_y + 2 * ng;
    c->lo_x = lo_x;
    c->lo_y = lo_y;
    c->hi_x = hi_x;
    c->hi_y = hi_y;
    c->dx = (hi_x - lo_x) / n_x;
    c->dy = (hi_y - lo_y) / n_y;
    c->Li = -c->dx * ng + lo_x + c->dx / 2; /* coordinates with dy := dx, as the reference's Psy_coord */
    c->Hi = -c->dx * ng + lo_y + c->dx / 2;
    c->gamma = gamma;
    c->cfl = cfl;
    c->t_end = t_end;
    c->scheme = scheme;
    c->riemann = riemann;
    c->limiter = limiter;
    c->periodic = periodic;
    c->max_iter = 2147483647;
    c->gm1 = gamma - 1;
    c->c1 = (gamma + 1) / (2 * gamma);
    c->c2 = (gamma - 1) / (2 * gamma);
    long cells = (long)c->M * c->N;
    for (int b = 0; b < 2; b++)
        for (int k = 0; k < 4; k++)
            c->U[b][k] = (double *)calloc(cells, sizeof(double));
    c->alpha = (double *)calloc(cells, sizeof(double));
    c->ax = (double *)calloc(cells, sizeof(double));
    c->ay = (double *)calloc(cells, sizeof(double));
    c->type = (unsigned char *)calloc(cells, 1);
    return c;
}

static void free_mix(ccm_case *c)
{
    free(c->ex_s);
    free(c->ex_t);
    free(c->ex_w);
    free(c->E);
    free(c->part_o);
    free(c->part_inv);
    free(c->part_first);
    free(c->part_count);
    free(c->links);
    c->ex_s = c->ex_t = c->part_o = NULL;
    c->ex_w = c->E = c->part_inv = NULL;
    c->part_first = c->part_count = c->links = NULL;
    c->nex = c->npart = 0;
}

void ccm_destroy(ccm_case *c)
{
    if (!c)
        return;
    for (int b = 0; b < 2; b++)
        for (int k = 0; k < 4; k++)
            free(c->U[b][k]);
    free(c->alpha);
    free(c->ax);
    free(c->ay);
    free(c->type);
    free_mix(c);
    free(c);
}

/* ------------------------------------------------------------------ geometry */

static double face_aperture(double a, double b)
{
    int fa = a >= 0.0, fb = b >= 0.0;
    if (fa && fb)
        return 1.0;
    if (!fa && !fb)
        return 0.0;
    double t = a / (a - b);
    return fa ? t : 1.0 - t;
}

static double cell_fraction(const double v[4])
{
    const double px[4] = {0.0, 1.0, 1.0, 0.0}, py[4] = {0.0, 0.0, 1.0, 1.0};
    double qx[8], qy[8];
    int n = 0;
    for (int k = 0; k < 4; k++)
    {
        int k1 = (k + 1) & 3;
        if (v[k] >= 0.0)
        {
            qx[n] = px[k];
            qy[n] = py[k];
            n++;
        }
        if ((v[k] >= 0.0) != (v[k1] >= 0.0))
        {
            double t = v[k] / (v[k] - v[k1]);
            qx[n] = px[k] + t * (px[k1] - px[k]);
            qy[n] = py[k] + t * (py[k1] - py[k]);
            n++;
        }
    }
    double a2 = 0.0;
    for (int k = 0; k < n; k++)
    {
        int k1 = (k + 1 == n) ? 0 : k + 1;
        a2 += qx[k] * qy[k1] - qx[k1] * qy[k];
    }
    return 0.5 * a2;
}

static double corner(const ccm_case *c, const double *phi, int a, int b)
{
    long o = IDX(c, a, b);
    return 0.25 * (phi[o] + phi[o + 1] + phi[o + c->M] + phi[o + c->M + 1]);
}

/* exchanges of one small cell, in the order x, y, diagonal target */
static int small_exchanges(const ccm_case *c, int i, int j, long t[3], double w[3])
{
    long o = IDX(c, i, j);
    double as = c->alpha[o];
    for (int k = 0; k < 3; k++)
    {
        t[k] = -1;
        w[k] = 0.0;
    }
    double nLx = (c->ax[o - 1] - c->ax[o]) * c->dy, nLy = (c->ay[o - c->M] - c->ay[o]) * c->dx;
    double L = sqrt(nLx * nLx + nLy * nLy);
    if (!(L > 0.0))
        return 0;
    double nx = nLx / L, ny = nLy / L;
    int sx = (nx > 0.0) ? -1 : 1, sy = (ny > 0.0) ? -1 : 1;
    int ti[3] = {i + sx, i, i + sx}, tj[3] = {j, j + sy, j + sy};
    double beta0[3] = {nx * nx, ny * ny, fabs(nx * ny)};
    double beta[3], bsum = 0.0;
    for (int k = 0; k < 3; k++)
    {
        int ok = interior(c, ti[k], tj[k]) && updated(c->type[IDX(c, ti[k], tj[k])]) && beta0[k] > 0.0;
        beta[k] = ok ? beta0[k] : 0.0;
        bsum += beta[k];
    }
    if (!(bsum > 0.0))
        return 0;
    for (int k = 0; k < 3; k++)
    {
        if (beta[k] == 0.0)
            continue;
        long ot = IDX(c, ti[k], tj[k]);
        double at = c->alpha[ot];
        t[k] = ot;
        w[k] = (beta[k] / bsum) * (as * at / (as + at));
    }
    return 1;
}

/* geometry from the cell-centred level set (M*N doubles, phi >= 0 fluid) */
void ccm_setup(ccm_case *c, const double *phi)
{
    const int M = c->M, N = c->N;
    for (int j = 0; j < N; j++)
        for (int i = 0; i < M; i++)
        {
            long o = IDX(c, i, j);
            if (i < 1 || j < 1 || i >= M - 1 || j >= N - 1)
            {
                c->alpha[o] = 1.0;
                c->ax[o] = 1.0;
                c->ay[o] = 1.0;
                c->type[o] = T_GHOST;
                continue;
            }
            double sw = corner(c, phi, i - 1, j - 1), se = corner(c, phi, i, j - 1), ne = corner(c, phi, i, j),
                   nw = corner(c, phi, i - 1, j);
            c->ax[o] = face_aperture(se, ne);
            c->ay[o] = face_aperture(nw, ne);
            if (!interior(c, i, j))
            {
                c->alpha[o] = 1.0;
                c->type[o] = T_GHOST;
                continue;
            }
            double v[4] = {sw, se, ne, nw};
            int all_in = sw >= 0.0 && se >= 0.0 && ne >= 0.0 && nw >= 0.0;
            int all_out = sw < 0.0 && se < 0.0 && ne < 0.0 && nw < 0.0;
            double al = all_in ? 1.0 : (all_out ? 0.0 : cell_fraction(v));
            unsigned char t = all_in ? T_FLUID : T_CUT;
            if (all_out || al < 1e-10)
            {
                t = T_SOLID;
                al = 0.0;
            }
            c->alpha[o] = al;
            c->type[o] = t;
        }
    for (int j = 0; j < N - 1; j++)
        for (int i = 0; i < M - 1; i++)
        {
            long o = IDX(c, i, j);
            if (c->type[o] == T_SOLID || c->type[o + 1] == T_SOLID)
                c->ax[o] = 0.0;
            if (c->type[o] == T_SOLID || c->type[o + M] == T_SOLID)
                c->ay[o] = 0.0;
        }
    /* mixing lists: small cells row by row, then each participant's links in
     * exchange order (small side before target side) */
    free_mix(c);
    int cap = 16, nex = 0;
    c->ex_s = (long *)malloc(cap * sizeof(long));
    c->ex_t = (long *)malloc(cap * sizeof(long));
    c->ex_w = (double *)malloc(cap * sizeof(double));
    for (int j = c->ng; j < c->ng + c->n_y; j++)
        for (int i = c->ng; i < c->ng + c->n_x; i++)
        {
            long o = IDX(c, i, j);
            if (!(c->type[o] == T_CUT && c->alpha[o] < 0.5))
                continue;
            long t[3];
            double w[3];
            small_exchanges(c, i, j, t, w);
            for (int k = 0; k < 3; k++)
            {
                if (t[k] < 0)
                    continue;
                if (nex == cap)
                {
                    cap *= 2;
                    c->ex_s = (long *)realloc(c->ex_s, cap * sizeof(long));
                    c->ex_t = (long *)realloc(c->ex_t, cap * sizeof(long));
                    c->ex_w = (double *)realloc(c->ex_w, cap * sizeof(double));
                }
                c->ex_s[nex] = o;
                c->ex_t[nex] = t[k];
                c->ex_w[nex] = w[k];
                nex++;
            }
        }
    c->nex = nex;
    c->E = (double *)calloc(4 * (size_t)(nex > 0 ? nex : 1), sizeof(double));
    /* participants: cells in increasing offset; links in increasing exchange id */
    long cells = (long)M * N;
    int *nlink = (int *)calloc(cells, sizeof(int));
    for (int k = 0; k < nex; k++)
    {
        nlink[c->ex_s[k]]++;
        nlink[c->ex_t[k]]++;
    }
    int npart = 0;
    for (long o = 0; o < cells; o++)
        npart += nlink[o] > 0;
    c->npart = npart;
    c->part_o = (long *)malloc((npart + 1) * sizeof(long));
    c->part_inv = (double *)malloc((npart + 1) * sizeof(double));
    c->part_first = (int *)malloc((npart + 1) * sizeof(int));
    c->part_count = (int *)malloc((npart + 1) * sizeof(int));
    c->links = (int *)malloc((2 * nex + 1) * sizeof(int));
    int p = 0, l = 0;
    for (long o = 0; o < cells; o++)
    {
        if (!nlink[o])
            continue;
        c->part_o[p] = o;
        c->part_inv[p] = 1.0 / c->alpha[o];
        c->part_first[p] = l;
        for (int k = 0; k < nex; k++)
        {
            if (c->ex_s[k] == o)
                c->links[l++] = 2 * k;
            else if (c->ex_t[k] == o)
                c->links[l++] = 2 * k + 1;
        }
        c->part_count[p] = l - c->part_first[p];
        p++;
    }
    free(nlink);
}

/* ------------------------------------------------------------------ physics */

typedef struct
{
    double r, ir, un, ut, p, a;
} prim_t;

static prim_t prim(const double U[4], int nrm, const ccm_case *c)
{
    prim_t s;
    s.r = U[0];
    s.ir = 1.0 / U[0];
    s.un = U[nrm] * s.ir;
    s.ut = U[3 - nrm] * s.ir;
    s.p = c->gm1 * (U[3] - 0.5 * s.r * (s.un * s.un + s.ut * s.ut));
    s.a = sqrt(c->gamma * s.p * s.ir);
    return s;
}

static void flux(const double U[4], const prim_t *s, int nrm, double F[4])
{
    double m = s->r * s->un;
    F[0] = m;
    F[nrm] = m * s->un + s->p;
    F[3 - nrm] = m * s->ut;
    F[3] = (U[3] + s->p) * s->un;
}

static void hll_plain(const double UL[4], const double UR[4], int nrm, const ccm_case *c, double F[4])
{
    prim_t L = prim(UL, nrm, c), R = prim(UR, nrm, c);
    double ps = 0.5 * (L.p + R.p) + 0.125 * (L.un - R.un) * ((L.r + R.r) * (L.a + R.a));
    ps = ps > 0 ? ps : 0;
    double t = c->c1 * ps;
    double qL = (ps > L.p) ? sqrt(t / L.p + c->c2) : 1.0;
    double qR = (ps > R.p) ? sqrt(t / R.p + c->c2) : 1.0;
    double SL = L.un - L.a * qL;
    double SR = R.un + R.a * qR;
    double FL[4], FR[4];
    flux(UL, &L, nrm, FL);
    flux(UR, &R, nrm, FR);
    for (int k = 0; k < 4; k++)
    {
        if (SL >= 0)
            F[k] = FL[k];
        else if (SR <= 0)
            F[k] = FR[k];
        else
            F[k] = (SR * FL[k] - SL * FR[k] + SR * SL * (UR[k] - UL[k])) / (SR - SL);
    }
}

static void sw_split(const double U[4], int nrm, double sign, const ccm_case *c, double F[4])
{
    prim_t s = prim(U, nrm, c);
    const double d2 = 1e-12;
#define LAM(x) (0.5 * ((x) + sign * sqrt((x) * (x) + d2)))
    double l1 = LAM(s.un), l3 = LAM(s.un - s.a), l4 = LAM(s.un + s.a);
#undef LAM
    double h = s.p / c->gm1 * s.ir + 0.5 * (s.un * s.un + s.ut * s.ut) + s.p * s.ir;
    double w = s.r / (2 * c->gamma);
    F[0] = w * (2 * c->gm1 * l1 + l3 + l4);
    F[nrm] = w * (2 * c->gm1 * s.un * l1 + (s.un - s.a) * l3 + (s.un + s.a) * l4);
    F[3 - nrm] = w * s.ut * (2 * c->gm1 * l1 + l3 + l4);
    F[3] = w * (c->gm1 * (s.un * s.un + s.ut * s.ut) * l1 + (h - s.a * s.un) * l3 + (h + s.a * s.un) * l4);
}

static void hllc_toro(const double UL[4], const double UR[4], int nrm, const ccm_case *c, double F[4])
{
    prim_t L = prim(UL, nrm, c), R = prim(UR, nrm, c);
    double ps = 0.5 * (L.p + R.p) + 0.125 * (L.un - R.un) * ((L.r + R.r) * (L.a + R.a));
    ps = ps > 0 ? ps : 0;
    double t = c->c1 * ps;
    double qL = (ps > L.p) ? sqrt(t / L.p + c->c2) : 1.0;
    double qR = (ps > R.p) ? sqrt(t / R.p + c->c2) : 1.0;
    double SL = L.un - L.a * qL, SR = R.un + R.a * qR;
    double FL[4], FR[4];
    flux(UL, &L, nrm, FL);
    flux(UR, &R, nrm, FR);
    if (SL >= 0)
    {
        memcpy(F, FL, sizeof FL);
        return;
    }
    if (SR <= 0)
    {
        memcpy(F, FR, sizeof FR);
        return;
    }
    double mL = L.r * (SL - L.un), mR = R.r * (SR - R.un);
    double Ss = (R.p - L.p + L.un * mL - R.un * mR) / (mL - mR);
    int left = Ss >= 0;
    const prim_t *s = left ? &L : &R;
    const double *U = left ? UL : UR;
    const double *Fk = left ? FL : FR;
    double S = left ? SL : SR, m = left ? mL : mR;
    double fac = m / (S - Ss);
    double Us[4];
    Us[0] = fac;
    Us[nrm] = fac * Ss;
    Us[3 - nrm] = fac * s->ut;
    Us[3] = fac * (U[3] * s->ir + (Ss - s->un) * (Ss + s->p / m));
    for (int k = 0; k < 4; k++)
        F[k] = Fk[k] + S * (Us[k] - U[k]);
}

static void solve(const double UL[4], const double UR[4], int nrm, const ccm_case *c, double F[4])
{
    if (c->riemann == R_SW)
    {
        double Fp[4], Fm[4];
        sw_split(UL, nrm, 1.0, c, Fp);
        sw_split(UR, nrm, -1.0, c, Fm);
        for (int k = 0; k < 4; k++)
            F[k] = Fp[k] + Fm[k];
    }
    else if (c->riemann == R_HLLCT)
        hllc_toro(UL, UR, nrm, c, F);
    else /* R_HLLT */
        hll_plain(UL, UR, nrm, c, F);
}

static double minmod(double a, double b)
{
    if (!(a * b > 0))
        return 0.0;
    return fabs(a) > fabs(b) ? b : a;
}

/* the reference's VanLeer macro as it expands (Slope_limiter/VanLeer) */
static double vanleer(double a, double P, double Q)
{
    double b = P - Q;
    double r = (a + 1e-7) / (b + 1e-7);
    return (r > 0) ? ((r * r + r) * P - Q / (r * r + 1)) : 0.0;
}

static double internal_energy(const double U[4])
{
    double ir = 1.0 / U[0];
    double u = U[1] * ir, v = U[2] * ir;
    return U[3] - 0.5 * U[0] * (u * u + v * v);
}

static int physical(const double U[4]) { return U[0] > 0 && internal_energy(U) > 1e-6 * fabs(U[3]); }

static void face(const ccm_case *c, const double c0[4], const double c1[4], const double c2[4], const double c3[4],
                 int nrm, int first_order, double h2, double F[4])
{
    double UL[4], UR[4];
    if (first_order || c->scheme == S_GODUNOV)
    {
        memcpy(UL, c1, sizeof UL);
        memcpy(UR, c2, sizeof UR);
    }
    else
    {
        for (int k = 0; k < 4; k++)
        {
            if (c->limiter == 1)
            {
                UL[k] = c1[k] + 0.5 * vanleer(c1[k] - c0[k], c2[k], c1[k]);
                UR[k] = c2[k] - 0.5 * vanleer(c3[k] - c2[k], c2[k], c1[k]);
            }
            else
            {
                double dm = c1[k] - c0[k], d0 = c2[k] - c1[k], dp = c3[k] - c2[k];
                UL[k] = c1[k] + 0.5 * minmod(dm, d0);
                UR[k] = c2[k] - 0.5 * minmod(dp, d0);
            }
        }
        if (c->scheme == S_MHM)
        {
            double FL[4], FR[4];
            prim_t L = prim(UL, nrm, c), R = prim(UR, nrm, c);
            flux(UL, &L, nrm, FL);
            flux(UR, &R, nrm, FR);
            for (int k = 0; k < 4; k++)
            {
                double d = h2 * (FL[k] - FR[k]);
                UL[k] += d;
                UR[k] += d;
            }
        }
        if (physical(c1) && physical(c2) && !(physical(UL) && physical(UR)))
        {
            memcpy(UL, c1, sizeof UL);
            memcpy(UR, c2, sizeof UR);
        }
    }
    solve(UL, UR, nrm, c, F);
}

static void wall_flux(const ccm_case *c, const double U[4], double nx, double ny, double W[4])
{
    double mn = U[1] * nx + U[2] * ny, mt = -U[1] * ny + U[2] * nx;
    double UL[4] = {U[0], mn, mt, U[3]}, UR[4] = {U[0], -mn, mt, U[3]};
    double F[4];
    solve(UL, UR, 1, c, F);
    W[0] = 0.0;
    W[1] = F[1] * nx;
    W[2] = F[1] * ny;
    W[3] = 0.0;
}

static void pressure_floor(double v[4])
{
    if (!(v[0] > 0))
        return;
    double f = 1e-5 * fabs(v[3]);
    double e = internal_energy(v);
    if (e < f)
        v[3] = (v[3] - e) + f;
}

/* ------------------------------------------------------------------ step */

static void load(const ccm_case *c, int b, long o, double u[4])
{
    for (int k = 0; k < 4; k++)
        u[k] = c->U[b][k][o];
}

static int low_order(unsigned char t) { return t == T_SOLID || t == T_CUT; }

/* the face flux at (i+1/2, j) (nrm 1) or (i, j+1/2) (nrm 2) from buffer b */
static void face_at(const ccm_case *c, int b, int i, int j, int nrm, double h2, double F[4])
{
    int di = (nrm == 1), dj = (nrm == 2);
    double s[4][4];
    int lo = 0;
    for (int q = 0; q < 4; q++)
    {
        int ii = i + (q - 1) * di, jj = j + (q - 1) * dj;
        long o = IDX(c, ii, jj);
        load(c, b, o, s[q]);
        lo |= low_order(c->type[o]);
    }
    face(c, s[0], s[1], s[2], s[3], nrm, lo, h2, F);
}

static double face_term(double A, double F) { return (A > 0.0) ? A * F : 0.0; }

/* ComputeDt / mass statistics of one cell of the new state */
typedef struct
{
    double amax, umax, vmax, mass;
} stats_t;

static void stats_full(const ccm_case *c, const double v[4], stats_t *st)
{
    double ir = 1.0 / v[0];
    double u = v[1] * ir, w = v[2] * ir;
    double p = c->gm1 * (v[3] - 0.5 * v[0] * (u * u + w * w));
    double x = c->gamma * p * ir;
    double a = (x == 0.0) ? 0.0 : sqrt(x);
    st->amax = fmax(st->amax, a);
    st->umax = fmax(st->umax, fabs(u));
    st->vmax = fmax(st->vmax, fabs(w));
    st->mass += v[0] * (c->dx * c->dy);
}

static void ring_fill(ccm_case *c, int next)
{
    const int ng = c->ng, n_x = c->n_x, n_y = c->n_y, N = c->N;
    const int prev = next ^ 1;
#define S_(i, j, k) ((interior(c, i, j) && updated(c->type[IDX(c, i, j)])) ? c->U[next][k][IDX(c, i, j)] \
                                                                              : c->U[prev][k][IDX(c, i, j)])
    /* rows */
    for (int r = 0; r < 2 * ng; r++)
        for (int ii = 0; ii < n_x; ii++)
        {
            int i = ng + ii, j = (r < ng) ? r : n_y + r;
            long o = IDX(c, i, j);
            double out[4];
            if (c->periodic)
            {
                int sj = (j < ng) ? j + n_y : j - n_y;
                for (int k = 0; k < 4; k++)
                    out[k] = S_(i, sj, k);
            }
            else
            {
                int bottom = j < ng;
                int src = bottom ? 2 * ng - 1 : n_y + ng - 1;
                int mir = bottom ? 2 * ng - j - 1 : 2 * (n_y + ng) - 1 - j;
                out[0] = S_(i, src, 0);
                out[1] = S_(i, src, 1);
                out[2] = -S_(i, mir, 2);
                out[3] = S_(i, src, 3);
            }
            for (int k = 0; k < 4; k++)
                c->U[next][k][o] = out[k];
        }
    /* columns (all rows, corners included) */
    for (int cc = 0; cc < 2 * ng; cc++)
        for (int j = 0; j < N; j++)
        {
            int i = (cc < ng) ? cc : n_x + cc;
            long o = IDX(c, i, j);
            double out[4];
            if (c->periodic)
            {
                int si = (i < ng) ? i + n_x : i - n_x, sj = j;
                if (j < ng)
                    sj = j + n_y;
                else if (j >= n_y + ng)
                    sj = j - n_y;
                int src_interior_row = sj >= ng && sj < ng + n_y;
                for (int k = 0; k < 4; k++)
                    out[k] = (!src_interior_row || sj != j) ? S_(si, sj, k) : c->U[next][k][IDX(c, si, sj)];
            }
            else
            {
                int si = (i < ng) ? ng : n_x + ng - 1;
                for (int k = 0; k < 4; k++)
                    out[k] = S_(si, j, k);
            }
            for (int k = 0; k < 4; k++)
                c->U[next][k][o] = out[k];
        }
#undef S_
}

static void finish_stats(ccm_case *c, const stats_t *st, int set_start)
{
    c->dt = c->cfl * c->dx / (st->amax + ((st->umax < st->vmax) ? st->vmax : st->umax));
    c->mass = st->mass;
    if (set_start)
        c->mass_start = st->mass;
}

/* initial state (array of structures, M*N*4), then the initial dt and mass */
void ccm_set_state(ccm_case *c, const double *u0)
{
    long cells = (long)c->M * c->N;
    for (int b = 0; b < 2; b++)
        for (int k = 0; k < 4; k++)
            for (long o = 0; o < cells; o++)
                c->U[b][k][o] = u0[o * 4 + k];
    c->cur = 1;
    c->iter = 0;
    c->now_t = 0.0;
    stats_t st = {0, 0, 0, 0};
    for (int j = c->ng; j < c->ng + c->n_y; j++)
        for (int i = c->ng; i < c->ng + c->n_x; i++)
        {
            long o = IDX(c, i, j);
            double v[4];
            load(c, c->cur, o, v);
            if (c->type[o] == T_FLUID || c->type[o] == T_CUT)
            {
                /* the library's initial reduction (ComputeDt.cpp:38-45 and
                 * CaculateMass.cpp:36 as written); cut cells weighted by alpha */
                double u = v[1] / v[0], w = v[2] / v[0];
                double p = (c->gamma - 1) * (v[3] - 0.5 * v[0] * (u * u + w * w));
                double x = c->gamma * p / v[0];
                double a = (x == 0.0) ? 0.0 : sqrt(x);
                double m = v[0] * c->dx * c->dy;
                st.mass += (c->type[o] == T_CUT) ? c->alpha[o] * m : m;
                if (c->type[o] == T_FLUID || c->alpha[o] >= 0.5)
                {
                    st.amax = fmax(st.amax, a);
                    st.umax = fmax(st.umax, fabs(u));
                    st.vmax = fmax(st.vmax, fabs(w));
                }
            }
        }
    finish_stats(c, &st, 1);
}

static void step(ccm_case *c)
{
    if (!(c->now_t < c->t_end && c->iter < c->max_iter))
        return;
    const int cur = c->cur, nxt = cur ^ 1;
    const double dt = c->dt;
    const double lx = dt * (1.0 / c->dx), ly = dt * (1.0 / c->dy);
    const double hx2 = 0.5 * lx, hy2 = 0.5 * ly;
    stats_t st = {0, 0, 0, 0};
    for (int j = c->ng; j < c->ng + c->n_y; j++)
        for (int i = c->ng; i < c->ng + c->n_x; i++)
        {
            long o = IDX(c, i, j);
            unsigned char t = c->type[o];
            if (!updated(t))
                continue;
            double Fw[4], Fe[4], Gs[4], Gn[4], u0[4], v[4];
            face_at(c, cur, i - 1, j, 1, hx2, Fw);
            face_at(c, cur, i, j, 1, hx2, Fe);
            face_at(c, cur, i, j - 1, 2, hy2, Gs);
            face_at(c, cur, i, j, 2, hy2, Gn);
            load(c, cur, o, u0);
            if (t == T_FLUID)
            {
                for (int k = 0; k < 4; k++)
                {
                    double x = u0[k] - lx * (Fe[k] - Fw[k]);
                    v[k] = x - ly * (Gn[k] - Gs[k]);
                }
                if (c->riemann == R_HLLCT || c->riemann == R_HLLT)
                    pressure_floor(v);
                stats_full(c, v, &st);
            }
            else
            {
                double al = c->alpha[o];
                double aw = c->ax[o - 1], ae = c->ax[o], as = c->ay[o - c->M], an = c->ay[o];
                double nLx = (aw - ae) * c->dy, nLy = (as - an) * c->dx;
                double L = sqrt(nLx * nLx + nLy * nLy);
                double W[4] = {0, 0, 0, 0};
                if (L > 0.0)
                    wall_flux(c, u0, nLx / L, nLy / L, W);
                double lxd = dt / c->dx, lyd = dt / c->dy, lw = dt / (c->dx * c->dy) * L;
                for (int k = 0; k < 4; k++)
                {
                    double fx = face_term(ae, Fe[k]) - face_term(aw, Fw[k]);
                    double gy = face_term(an, Gn[k]) - face_term(as, Gs[k]);
                    v[k] = (al * u0[k] - lxd * fx - lyd * gy - lw * W[k]) / al;
                }
                if ((c->riemann == R_HLLCT || c->riemann == R_HLLT) && al >= 0.5)
                    pressure_floor(v);
                st.mass += al * v[0] * (c->dx * c->dy);
                if (al >= 0.5)
                {
                    double ir = 1.0 / v[0];
                    double uu = v[1] * ir, ww = v[2] * ir;
                    double p = (c->gamma - 1.0) * (v[3] - 0.5 * v[0] * (uu * uu + ww * ww));
                    st.amax = fmax(st.amax, sqrt(c->gamma * p * ir));
                    st.umax = fmax(st.umax, fabs(uu));
                    st.vmax = fmax(st.vmax, fabs(ww));
                }
            }
            for (int k = 0; k < 4; k++)
                c->U[nxt][k][o] = v[k];
        }
    /* small-cell mixing on the new state */
    for (int k = 0; k < c->nex; k++)
        for (int q = 0; q < 4; q++)
            c->E[4 * k + q] = c->ex_w[k] * (c->U[nxt][q][c->ex_t[k]] - c->U[nxt][q][c->ex_s[k]]);
    for (int p = 0; p < c->npart; p++)
        for (int q = 0; q < 4; q++)
        {
            double d = 0.0;
            for (int l = 0; l < c->part_count[p]; l++)
            {
                int x = c->links[c->part_first[p] + l];
                double e = c->E[4 * (x >> 1) + q];
                d += (x & 1) ? -e : e;
            }
            long o = c->part_o[p];
            c->U[nxt][q][o] = c->U[nxt][q][o] + d * c->part_inv[p];
        }
    ring_fill(c, nxt);
    finish_stats(c, &st, 0);
    c->now_t = c->now_t + c->dt;
    c->iter++;
    c->cur = nxt;
}

/* up to nsteps iterations of the loop; returns how many ran, dt and mass of each */
int ccm_run(ccm_case *c, int nsteps, double *dts, double *masses)
{
    int n = 0;
    for (int s = 0; s < nsteps; s++)
    {
        if (!(c->now_t < c->t_end && c->iter < c->max_iter))
            break;
        double dt = c->dt;
        step(c);
        if (dts)
            dts[n] = dt;
        if (masses)
            masses[n] = c->mass;
        n++;
    }
    return n;
}

void ccm_get_state(const ccm_case *c, double *u)
{
    long cells = (long)c->M * c->N;
    for (long o = 0; o < cells; o++)
        for (int k = 0; k < 4; k++)
            u[o * 4 + k] = c->U[c->cur][k][o];
}

void ccm_get_geometry(const ccm_case *c, double *alpha, double *ax, double *ay, unsigned char *type)
{
    long cells = (long)c->M * c->N;
    memcpy(alpha, c->alpha, cells * sizeof(double));
    memcpy(ax, c->ax, cells * sizeof(double));
    memcpy(ay, c->ay, cells * sizeof(double));
    memcpy(type, c->type, cells);
}

/* dt, now_t, mass, mass_start, iter, number of exchanges */
void ccm_scalars(const ccm_case *c, double *out)
{
    out[0] = c->dt;
    out[1] = c->now_t;
    out[2] = c->mass;
    out[3] = c->mass_start;
    out[4] = c->iter;
    out[5] = c->nex;
}
