// Reference-signature entry points (include/ibtfo_ref.h) over the C ABI.
//
// The reference's drivers call free functions over host arrays that OpenACC
// mirrors on the device (Test/InclineSod/InclineSod.cpp:77-189).  Here the
// mirror is a present table: the XYCOORD pointer of the first geometry call
// names a case, its U_OLD pointer is bound at the first state call, and every
// later call with those pointers works on the resident device state.
#include <cstdio>
#include <cstring>
#include <iterator>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ibtfo.h"
#include "../../include/ibtfo_ref.h"
#include "internal.h"

namespace {

struct Entry
{
    ibtfo_case *cs = nullptr;
    ibtfo_config cfg{};
    double *xy = nullptr, *u_old = nullptr, *u_new = nullptr;
    bool state = false;   // U_OLD has been sent to the GPU
    bool cfl_set = false; // ComputeDt has supplied the CFL number
};

std::mutex g_mu;
std::map<const double *, Entry *> g_by_xy, g_by_u;
int g_slots[6] = {IBTFO_SCHEME_MUSCL, IBTFO_RIEMANN_HLL, IBTFO_LIMITER_MINMOD, IBTFO_BOUNDARY_REGULAR,
                  IBTFO_GLOBAL_WALLS, IBTFO_PRECISION_FP64};
thread_local int g_status = IBTFO_OK;

int set_status(int s, const char *msg = nullptr)
{
    g_status = s;
    if (msg)
        ibtfo::set_last_error(msg);
    return s;
}

bool one_device(int ndevices, int device)
{
    if (ndevices != 1 || device != 0)
    {
        set_status(IBTFO_EINVAL, "the GB300 library runs one case on one device (ndevices = 1, device = 0)");
        return false;
    }
    return true;
}

Entry *by_xy(const double *xy)
{
    auto it = g_by_xy.find(xy);
    if (it == g_by_xy.end())
    {
        set_status(IBTFO_ESTATE, "XYCOORD not set up: call Psy_coord and Level_Set first");
        return nullptr;
    }
    return it->second;
}

Entry *by_u(const double *u)
{
    auto it = g_by_u.find(u);
    if (it == g_by_u.end())
    {
        set_status(IBTFO_ESTATE, "U_OLD is not bound to a case: call Boundary or TimeAdvance with its XYCOORD first");
        return nullptr;
    }
    return it->second;
}

// sends U_OLD (== U_NEW after Initialize) and applies the initial Boundary
int bind_state(Entry *e, double *U_OLD, double *U_NEW, double gamma)
{
    int s = ibtfo::case_set_gas(e->cs, gamma, e->cfl_set ? ibtfo::case_cfl(e->cs) : e->cfg.cfl_number);
    if (s != IBTFO_OK)
        return set_status(s);
    s = ibtfo_set_state(e->cs, U_OLD);
    if (s != IBTFO_OK)
        return set_status(s);
    e->state = true;
    e->u_old = U_OLD;
    e->u_new = U_NEW;
    g_by_u[U_OLD] = e;
    if (U_NEW)
        g_by_u[U_NEW] = e;
    return set_status(IBTFO_OK);
}

} // namespace

extern "C" {

void ibtfo_ref_configure(int scheme, int riemann, int limiter, int boundary, int global_boundary, int precision)
{
    std::lock_guard<std::mutex> lock(g_mu);
    const int v[6] = {scheme, riemann, limiter, boundary, global_boundary, precision};
    memcpy(g_slots, v, sizeof v);
    set_status(IBTFO_OK);
}

int ibtfo_ref_status(void) { return g_status; }

void ibtfo_ref_Psy_coord(double lo_x, double lo_y, double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell,
                         double *XYCOORD, int ndevices, int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!one_device(ndevices, device) || !XYCOORD)
        return;
    Entry *&e = g_by_xy[XYCOORD];
    if (!e)
        e = new Entry();
    e->xy = XYCOORD;
    ibtfo_config &c = e->cfg;
    c.n_x = N_x;
    c.n_y = N_y;
    c.num_ghost_cell = num_ghost_cell;
    c.lo_x = lo_x;
    c.lo_y = lo_y;
    c.hi_x = lo_x + Psy_L;
    c.hi_y = lo_y + Psy_H;
    c.gamma = 1.4;      // replaced by the first call that carries gamma
    c.cfl_number = 0.5; // replaced by ComputeDt
    c.psy_time = 1e300;
    c.max_iter = 2147483647;
    c.scheme = g_slots[0];
    c.riemann = g_slots[1];
    c.limiter = g_slots[2];
    c.boundary = g_slots[3];
    c.global_boundary = g_slots[4];
    c.precision = g_slots[5];
    // Psy_coord.cpp:29-44 (dy := dx, as in the reference)
    const int M = N_x + 2 * num_ghost_cell, N = N_y + 2 * num_ghost_cell;
    const double dx = Psy_L / N_x;
    const double dy = Psy_L / N_x;
    const double Li = -dx * num_ghost_cell + lo_x + dx / 2;
    const double Hi = -dy * num_ghost_cell + lo_y + dy / 2;
    for (int j = 0; j < N; j++)
        for (int i = 0; i < M; i++)
        {
            XYCOORD[((size_t)M * j + i) * 6 + 0] = Li + i * dx;
            XYCOORD[((size_t)M * j + i) * 6 + 1] = Hi + j * dx;
        }
    set_status(IBTFO_OK);
}

void ibtfo_ref_Level_Set(int N_x, int N_y, int num_ghost_cell, double *XYCOORD, int ndevices, int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!one_device(ndevices, device))
        return;
    Entry *e = by_xy(XYCOORD);
    if (!e)
        return;
    if (e->cfg.n_x != N_x || e->cfg.n_y != N_y || e->cfg.num_ghost_cell != num_ghost_cell)
    {
        set_status(IBTFO_EINVAL, "grid differs from the Psy_coord call");
        return;
    }
    if (!e->cs && set_status(ibtfo_create(&e->cfg, &e->cs)) != IBTFO_OK)
        return;
    const size_t cells = (size_t)(N_x + 2 * num_ghost_cell) * (N_y + 2 * num_ghost_cell);
    std::vector<double> phi(cells), xy(cells * 6);
    for (size_t q = 0; q < cells; q++)
        phi[q] = XYCOORD[q * 6 + 2];
    if (set_status(ibtfo_setup_geometry(e->cs, phi.data())) != IBTFO_OK ||
        set_status(ibtfo_get_geometry(e->cs, xy.data())) != IBTFO_OK)
        return;
    for (size_t q = 0; q < cells; q++)
        for (int k = 3; k < 6; k++)
            XYCOORD[q * 6 + k] = xy[q * 6 + k];
    e->state = false;
}

void ibtfo_ref_Scheme_Index(int N_x, int N_y, int num_ghost_cell, double *XYCOORD, double *SCHEME_IDX, int ndevices,
                            int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!one_device(ndevices, device))
        return;
    Entry *e = by_xy(XYCOORD);
    if (!e || !e->cs)
    {
        set_status(IBTFO_ESTATE, "Scheme_Index before Level_Set");
        return;
    }
    (void)N_x;
    (void)N_y;
    (void)num_ghost_cell;
    // the image points, brackets and weights were computed with the geometry
    set_status(ibtfo_get_scheme_index(e->cs, SCHEME_IDX));
}

void ibtfo_ref_Advance(double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell, double gamma, double dt,
                       double *U_OLD, double *U_TMP, double *U_NEW, double *XYCOORD, int ndevices, int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    (void)Psy_L;
    (void)Psy_H;
    (void)N_x;
    (void)N_y;
    (void)num_ghost_cell;
    (void)U_TMP;
    if (!one_device(ndevices, device))
        return;
    Entry *e = by_xy(XYCOORD);
    if (!e || !e->cs)
    {
        set_status(IBTFO_ESTATE, "TimeAdvance before Level_Set");
        return;
    }
    if (!e->state && bind_state(e, U_OLD, U_NEW, gamma) != IBTFO_OK)
        return;
    if (U_NEW && !e->u_new)
    {
        e->u_new = U_NEW;
        g_by_u[U_NEW] = e;
    }
    if (set_status(ibtfo::case_set_gas(e->cs, gamma, ibtfo::case_cfl(e->cs))) != IBTFO_OK)
        return;
    // the reference applies the dt it is given (Sod.cpp:154)
    if (set_status(ibtfo::case_set_dt(e->cs, dt)) != IBTFO_OK)
        return;
    set_status(ibtfo::case_sweep_unguarded(e->cs));
}

void ibtfo_ref_TimeAdvance(double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell, double gamma, double dt,
                           double *U_OLD, double *U_TMP, double *U_NEW, double *XYCOORD, double *SCHEME_IDX,
                           int ndevices, int device)
{
    // Src/Base/TimeAdvance/SingleStep/SingleStep.cpp:20
    (void)SCHEME_IDX;
    ibtfo_ref_Advance(Psy_L, Psy_H, N_x, N_y, num_ghost_cell, gamma, dt, U_OLD, U_TMP, U_NEW, XYCOORD, ndevices,
                      device);
}

void ibtfo_ref_Boundary(int N_x, int N_y, int num_ghost_cell, double gamma, double *U_OLD, double *U_NEW,
                        double *XYCOORD, double *SCHEME_IDX, int ndevices, int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    (void)N_x;
    (void)N_y;
    (void)num_ghost_cell;
    (void)SCHEME_IDX;
    if (!one_device(ndevices, device))
        return;
    Entry *e = by_xy(XYCOORD);
    if (!e || !e->cs)
    {
        set_status(IBTFO_ESTATE, "Boundary before Level_Set");
        return;
    }
    if (!e->state)
    {
        // the initial Boundary (InclineSod.cpp:105): send the state and fill the ghost cells
        bind_state(e, U_OLD, U_NEW, gamma);
        return;
    }
    set_status(ibtfo::case_fill(e->cs, 1, 0));
}

void ibtfo_ref_Global_Boundary(int N_x, int N_y, int num_ghost_cell, double gamma, double *U_OLD, double *U_NEW,
                               int ndevices, int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    (void)N_x;
    (void)N_y;
    (void)num_ghost_cell;
    (void)gamma;
    (void)U_NEW;
    if (!one_device(ndevices, device))
        return;
    Entry *e = by_u(U_OLD);
    if (!e)
        return;
    set_status(ibtfo::case_fill(e->cs, 0, 1));
}

void ibtfo_ref_ComputeDt(double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell, double gamma,
                         double CFL_number, double *U_OLD, double *XYCOORD, double *TMP_DT, int ndevices, int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    (void)Psy_L;
    (void)Psy_H;
    (void)N_x;
    (void)N_y;
    (void)num_ghost_cell;
    if (!one_device(ndevices, device))
        return;
    Entry *e = by_xy(XYCOORD);
    if (!e || !e->cs)
    {
        set_status(IBTFO_ESTATE, "ComputeDt before Level_Set");
        return;
    }
    if (!e->state && bind_state(e, U_OLD, nullptr, gamma) != IBTFO_OK)
        return;
    const bool changed = !e->cfl_set || ibtfo::case_cfl(e->cs) != CFL_number || ibtfo::case_gamma(e->cs) != gamma;
    if (set_status(ibtfo::case_set_gas(e->cs, gamma, CFL_number)) != IBTFO_OK)
        return;
    e->cfl_set = true;
    // the sweep already reduced the current state with these constants;
    // otherwise reduce it now
    if (changed && set_status(ibtfo::case_reduce_current(e->cs)) != IBTFO_OK)
        return;
    ibtfo_progress p;
    if (set_status(ibtfo_get_progress(e->cs, &p)) != IBTFO_OK)
        return;
    TMP_DT[device] = p.dt;
}

void ibtfo_ref_CaculateMass(double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell, double *U_OLD,
                            double *XYCOORD, double *MASS_DEVICE, int ndevices, int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    (void)Psy_L;
    (void)Psy_H;
    (void)N_x;
    (void)N_y;
    (void)num_ghost_cell;
    if (!one_device(ndevices, device))
        return;
    Entry *e = by_xy(XYCOORD);
    if (!e || !e->cs)
    {
        set_status(IBTFO_ESTATE, "CaculateMass before Level_Set");
        return;
    }
    if (!e->state && bind_state(e, U_OLD, nullptr, ibtfo::case_gamma(e->cs)) != IBTFO_OK)
        return;
    ibtfo_progress p;
    if (set_status(ibtfo_get_progress(e->cs, &p)) != IBTFO_OK)
        return;
    MASS_DEVICE[device] = p.mass;
}

void ibtfo_ref_WriteData(double lo_x, double lo_y, double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell,
                         int iter, double now_t, double gamma, double *U_OLD, double *XYCOORD, int ndevices,
                         int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    (void)lo_x;
    (void)lo_y;
    (void)Psy_L;
    (void)Psy_H;
    (void)N_x;
    (void)N_y;
    (void)num_ghost_cell;
    if (!one_device(ndevices, device))
        return;
    Entry *e = by_xy(XYCOORD);
    if (!e || !e->cs)
    {
        set_status(IBTFO_ESTATE, "WriteData before Level_Set");
        return;
    }
    if (!e->state && bind_state(e, U_OLD, nullptr, gamma) != IBTFO_OK)
        return;
    // WriteData.cpp:20-27
    FILE *visit = fopen("result.visit", "a");
    if (!visit)
    {
        set_status(IBTFO_EINVAL, "cannot open result.visit");
        return;
    }
    if (iter == 0 && device == 0)
        fprintf(visit, "!NBLOCKS %d\n", ndevices);
    const std::string name = "dat_" + std::to_string(device) + "_" + std::to_string(iter) + ".vtk";
    fprintf(visit, "%s\n", name.c_str());
    fclose(visit);
    set_status(ibtfo::case_write_vtk_at(e->cs, name.c_str(), now_t));
}

void ibtfo_ref_update_self(double *U)
{
    std::lock_guard<std::mutex> lock(g_mu);
    Entry *e = by_u(U);
    if (!e)
        return;
    if (U == e->u_old)
        set_status(ibtfo_get_state(e->cs, U, nullptr));
    else
        set_status(ibtfo_get_state(e->cs, nullptr, U));
}

void ibtfo_ref_update_device(double *U)
{
    std::lock_guard<std::mutex> lock(g_mu);
    Entry *e = by_u(U);
    if (!e)
        return;
    if (U != e->u_old)
    {
        set_status(IBTFO_EINVAL, "only U_OLD can be sent to the GPU");
        return;
    }
    set_status(ibtfo_put_state(e->cs, U));
}

void ibtfo_ref_release(double *XYCOORD)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_by_xy.find(XYCOORD);
    if (it == g_by_xy.end())
        return;
    Entry *e = it->second;
    for (auto u = g_by_u.begin(); u != g_by_u.end();)
        u = (u->second == e) ? g_by_u.erase(u) : std::next(u);
    g_by_xy.erase(it);
    ibtfo_destroy(e->cs);
    delete e;
    set_status(IBTFO_OK);
}

} // extern "C"
