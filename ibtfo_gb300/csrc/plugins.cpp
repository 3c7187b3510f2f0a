// Case plug-ins: the level set and the initial state of named problems.
//
// The reference defines a problem by three per-case files compiled into its
// driver: Level_Set_function (phi), Initialize (conserved state) and
// Global_Boundary (Src/Geometry/Level_Set_function.H:13-19,
// Src/Base/Common/Initialize.H:12-23).  Here a problem is a name plus the
// .inp parameters; the library evaluates phi and the initial state on the
// host in the reference layouts.  Three problems restate the reference's own
// test plug-ins (Test/Sod, Test/InclineSod, Test/Vortex) with the same
// expressions; the others are the benchmark workloads.
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/ibtfo.h"

namespace ibtfo {
void set_last_error(const char *msg);
}

namespace {

struct Grid
{
    int n_x, n_y, ng, M, N;
    double lo_x, lo_y, hi_x, hi_y, dx, Li, Hi;
    explicit Grid(const ibtfo_config &c)
    {
        n_x = c.n_x;
        n_y = c.n_y;
        ng = c.num_ghost_cell;
        M = n_x + 2 * ng;
        N = n_y + 2 * ng;
        lo_x = c.lo_x;
        lo_y = c.lo_y;
        hi_x = c.hi_x;
        hi_y = c.hi_y;
        dx = (hi_x - lo_x) / n_x;      // Psy_coord.cpp:29-30 (dy := dx)
        Li = -dx * ng + lo_x + dx / 2; // Psy_coord.cpp:33-34
        Hi = -dx * ng + lo_y + dx / 2;
    }
    double x(int i) const { return Li + i * dx; }
    double y(int j) const { return Hi + j * dx; }
};

double param(const ibtfo_inp *p, const char *key, double def)
{
    double v = def;
    if (p)
        ibtfo_inp_get(p, key, def, &v);
    return v;
}

void put_state(double *u, double rho, double uu, double vv, double pp, double gamma)
{
    u[0] = rho;
    u[1] = rho * uu;
    u[2] = rho * vv;
    u[3] = pp / (gamma - 1) + 0.5 * rho * (uu * uu + vv * vv);
}

// Test/InclineSod/Level_Set_function.cpp:8-21
double line_dist(double x, double y, double k, double b, int dir)
{
    if (y > k * x + b)
        return dir * std::abs(k * x - y + b) / std::pow(1 + k * k, 0.5);
    return -dir * std::abs(k * x - y + b) / std::pow(1 + k * k, 0.5);
}

struct Sides
{
    double rL, uL, vL, pL, rR, uR, vR, pR;
    explicit Sides(const ibtfo_inp *p)
    {
        rL = param(p, "rho_L", 1);
        uL = param(p, "u_L", 0);
        vL = param(p, "v_L", 0);
        pL = param(p, "p_L", 1);
        rR = param(p, "rho_R", 0.125);
        uR = param(p, "u_R", 0);
        vR = param(p, "v_R", 0);
        pR = param(p, "p_R", 0.1);
    }
};

const double kPi = 3.14159265358979323846;

} // namespace

extern "C" {

ibtfo_status ibtfo_case_phi(const char *name, const ibtfo_inp *p, const ibtfo_config *cfg, double *phi)
{
    if (!name || !cfg || !phi)
    {
        ibtfo::set_last_error("ibtfo_case_phi: null argument");
        return IBTFO_EINVAL;
    }
    const Grid g(*cfg);
    const std::string n(name);
    for (int j = 0; j < g.N; j++)
        for (int i = 0; i < g.M; i++)
        {
            const double x = g.x(i), y = g.y(j);
            double v;
            if (n == "sod_ref" || n == "sod_x" || n == "isentropic_vortex")
                v = 1; // Test/Sod/Level_Set_function.cpp:27 (no body)
            else if (n == "incline_ref")
            {
                // Test/InclineSod/Level_Set_function.cpp:34-50
                double angle = 3.1415926535 * param(p, "angle", 30) / 180;
                double Axisd = param(p, "AxisD", 0.4);
                double AxisD = Axisd / std::cos(angle);
                double phi1 = line_dist(x, y, std::tan(angle), 0.05, 1);
                double phi2 = line_dist(x, y, std::tan(angle), AxisD, -1);
                v = (phi1 < phi2) ? phi1 : phi2;
            }
            else if (n == "vortex_ref")
            {
                // Test/Vortex/Level_Set_function.cpp:16-41
                const double rvortex = 0.40;
                double rl0 = param(p, "f0", 0) * rvortex;
                double rl1 = param(p, "f1", 1) * rvortex;
                double r = std::sqrt((x - 0.50) * (x - 0.50) + (y - 0.50) * (y - 0.50));
                double phi1 = rl1 - r, phi2 = r - rl0;
                v = (phi1 < phi2) ? phi1 : phi2;
            }
            else if (n == "channel")
            {
                // two walls parallel to an axis through the domain centre
                double th = param(p, "angle", 30.0) * (kPi / 180.0);
                double w = param(p, "width", 0.25);
                double xc = param(p, "x_c", 0.5 * (g.lo_x + g.hi_x)), yc = param(p, "y_c", 0.5 * (g.lo_y + g.hi_y));
                double s = (x - xc) * (-std::sin(th)) + (y - yc) * std::cos(th);
                double a = s + 0.5 * w, b = 0.5 * w - s;
                v = (a < b) ? a : b;
            }
            else
            {
                ibtfo::set_last_error(("unknown case '" + n + "'").c_str());
                return IBTFO_EINVAL;
            }
            phi[(size_t)g.M * j + i] = v;
        }
    return IBTFO_OK;
}

ibtfo_status ibtfo_case_init(const char *name, const ibtfo_inp *p, const ibtfo_config *cfg, const double *xycoord,
                             double *u0)
{
    if (!name || !cfg || !xycoord || !u0)
    {
        ibtfo::set_last_error("ibtfo_case_init: null argument");
        return IBTFO_EINVAL;
    }
    const Grid g(*cfg);
    const std::string n(name);
    const double gamma = cfg->gamma;
    const Sides s(p);
    for (int j = 0; j < g.N; j++)
        for (int i = 0; i < g.M; i++)
        {
            const size_t c = (size_t)g.M * j + i;
            const double x = xycoord[c * 6 + 0], y = xycoord[c * 6 + 1], type = xycoord[c * 6 + 5];
            double *u = u0 + c * 4;
            const bool open = (type < 0.5 || type > 1.5); // fluid or ghost
            if (n == "sod_ref")
            {
                // Test/Sod/Initialize.cpp:41-56 (split on the row index)
                if (j < (g.n_x + 2 * g.ng) / 2)
                    put_state(u, s.rL, s.uL, s.vL, s.pL, gamma);
                else
                    put_state(u, s.rR, s.uR, s.vR, s.pR, gamma);
            }
            else if (n == "sod_x")
            {
                if (x < param(p, "x0", 0.5))
                    put_state(u, s.rL, s.uL, s.vL, s.pL, gamma);
                else
                    put_state(u, s.rR, s.uR, s.vR, s.pR, gamma);
            }
            else if (n == "incline_ref")
            {
                // Test/InclineSod/Initialize.cpp:43-67
                const double angle = 3.1415926535 * param(p, "angle", 30) / 180;
                if (open)
                {
                    if (y < -(1 / std::tan(angle)) * x + 0.5 * (1 / std::tan(angle)) + 0.5)
                        put_state(u, s.rL, s.uL, s.vL, s.pL, gamma);
                    else
                        put_state(u, s.rR, s.uR, s.vR, s.pR, gamma);
                }
                else
                {
                    u[0] = -1;
                    u[1] = 0;
                    u[2] = 0;
                    u[3] = -1;
                }
            }
            else if (n == "channel")
            {
                double th = param(p, "angle", 30.0) * (kPi / 180.0);
                double xc = param(p, "x_c", 0.5 * (g.lo_x + g.hi_x)), yc = param(p, "y_c", 0.5 * (g.lo_y + g.hi_y));
                double a = (x - xc) * std::cos(th) + (y - yc) * std::sin(th);
                if (!open)
                {
                    u[0] = -1;
                    u[1] = 0;
                    u[2] = 0;
                    u[3] = -1;
                }
                else if (a < 0)
                    put_state(u, s.rL, s.uL, s.vL, s.pL, gamma);
                else
                    put_state(u, s.rR, s.uR, s.vR, s.pR, gamma);
            }
            else if (n == "vortex_ref")
            {
                // Test/Vortex/Initialize.cpp:20-92 (rotating vortex in a circular wall)
                const double fa = param(p, "fa", 0);
                const double rho0 = 1.0, p0 = 2.0, xlc = 0.50, ylc = 0.50, rvortex = 0.40, pi = M_PI;
                const double ua = fa * rvortex * pi;
                double ur = 0, pp = 0, uu = 0, vv = 0;
                u[0] = rho0;
                u[1] = rho0 * uu;
                u[2] = rho0 * vv;
                u[3] = (p0 + 2.0 * rho0 * ua * ua * pp) / (gamma - 1) + 0.5 * rho0 * (uu * uu + vv * vv);
                if (open)
                {
                    double r = std::pow((x - xlc) * (x - xlc) + (y - ylc) * (y - ylc), 0.5);
                    double ph = std::atan((y - ylc) / (x - xlc));
                    if (x - xlc < 0.0)
                        ph = ph + pi;
                    if (r < rvortex)
                    {
                        if (r < rvortex / 2.0)
                        {
                            ur = ua * 2.0 * r / rvortex;
                            pp = (r / rvortex) * (r / rvortex) + 1.0 - 2.0 * std::log(2.0);
                        }
                        else
                        {
                            ur = ua * 2.0 * (1.0 - r / rvortex);
                            pp = (r / rvortex) * (r / rvortex) + 3.0 - 4.0 * r / rvortex + 2.0 * std::log(r / rvortex);
                        }
                        uu = -std::sin(ph) * ur;
                        vv = std::cos(ph) * ur;
                    }
                    u[0] = rho0;
                    u[1] = rho0 * uu;
                    u[2] = rho0 * vv;
                    u[3] = (p0 + 2.0 * rho0 * ua * ua * pp) / (gamma - 1) + 0.5 * rho0 * (uu * uu + vv * vv);
                }
            }
            else if (n == "isentropic_vortex")
            {
                // uniform (1, u_inf, v_inf, 1) stream plus an isentropic vortex of strength beta
                const double beta = param(p, "beta", 5.0), xc = param(p, "x_c", 5.0), yc = param(p, "y_c", 5.0);
                const double uinf = param(p, "u_inf", 1.0), vinf = param(p, "v_inf", 1.0);
                const double Lx = g.hi_x - g.lo_x, Ly = g.hi_y - g.lo_y;
                double ddx = std::fmod(x - xc + 0.5 * Lx, Lx), ddy = std::fmod(y - yc + 0.5 * Ly, Ly);
                if (ddx < 0)
                    ddx += Lx;
                if (ddy < 0)
                    ddy += Ly;
                ddx -= 0.5 * Lx;
                ddy -= 0.5 * Ly;
                const double r2 = ddx * ddx + ddy * ddy;
                const double f = std::exp(0.5 * (1.0 - r2));
                const double du = -beta / (2 * kPi) * ddy * f, dv = beta / (2 * kPi) * ddx * f;
                const double T = 1.0 - (gamma - 1.0) * beta * beta / (8.0 * gamma * kPi * kPi) * std::exp(1.0 - r2);
                const double rho = std::pow(T, 1.0 / (gamma - 1.0));
                put_state(u, rho, uinf + du, vinf + dv, rho * T, gamma);
            }
            else
            {
                ibtfo::set_last_error(("unknown case '" + n + "'").c_str());
                return IBTFO_EINVAL;
            }
        }
    return IBTFO_OK;
}

} // extern "C"
