// ibtfo_forward.cpp -- the reference solver's entry points, forwarded to the
// GB300 library, for a reference driver (Test/<case>/<Case>.cpp) that links
// this file in place of the Src/ solver files its Makefile slots select.
//
// Compile it with the driver's own include paths (the reference's Src/
// headers are included below, so the compiler checks every signature against
// the declaration the driver calls) and with the slot keys as macros, e.g.
//   -DIBTFO_SCHEME=IBTFO_SCHEME_MUSCL -DIBTFO_RIEMANN=IBTFO_RIEMANN_HLLC
//   -DIBTFO_LIMITER=IBTFO_LIMITER_MINMOD -DIBTFO_BOUNDARY=IBTFO_BOUNDARY_IDW_GFM
// (the Makefile variables Scheme / Riemann / Limiter / Boundary of
// Test/InclineSod/Makefile:1-4), then link against libibtfo_gb300.so.
//
// What replaces what (the driver's calls, Test/InclineSod/InclineSod.cpp:97-186):
//   Psy_coord, Level_Set, Scheme_Index     Src/Geometry/*.cpp, Src/BoundaryCondition/<Boundary>/*_Method.cpp
//   TimeAdvance (Advance inside)           Src/Base/TimeAdvance/<Time>, Src/Base/Euler/Advection/<Scheme>
//   Boundary, Global_Boundary              Src/BoundaryCondition/<Boundary>, the test's Global_Boudary.cpp
//   ComputeDt, CaculateMass, WriteData     Src/Base/Common/ComputeDt.cpp, Src/Utils/{CaculateMass,WriteData}.cpp
// The case's own plug-ins stay: Initialize and Level_Set_function (phi on the
// host), and the .inp reader (Src/Utils/ParamReader.cpp).  The Global_Boundary
// forwarded here is the walls variant every reference test defines
// (reflective y walls, transmissive x edges); drop the test's
// Global_Boudary.cpp from the link.
#include "Boundary.H"
#include "CaculateMass.H"
#include "ComputeDt.H"
#include "Level_Set.H"
#include "Level_Set_function.H"
#include "Psy_coord.H"
#include "Scheme_Index.H"
#include "TimeAdvance.H"
#include "WriteData.H"

#include "ibtfo_ref.h"

#ifndef IBTFO_SCHEME
#define IBTFO_SCHEME IBTFO_SCHEME_MUSCL
#endif
#ifndef IBTFO_RIEMANN
#define IBTFO_RIEMANN IBTFO_RIEMANN_HLLC
#endif
#ifndef IBTFO_LIMITER
#define IBTFO_LIMITER IBTFO_LIMITER_MINMOD
#endif
#ifndef IBTFO_BOUNDARY
#define IBTFO_BOUNDARY IBTFO_BOUNDARY_IDW_GFM
#endif
#ifndef IBTFO_PRECISION
#define IBTFO_PRECISION IBTFO_PRECISION_FP64
#endif

// slot selection before main() runs, as the Makefile fixes it at link time
static const int ibtfo_slots_configured =
    (ibtfo_ref_configure(IBTFO_SCHEME, IBTFO_RIEMANN, IBTFO_LIMITER, IBTFO_BOUNDARY, IBTFO_GLOBAL_WALLS,
                         IBTFO_PRECISION),
     0);

void Psy_coord(const double lo_x, const double lo_y, const double Psy_L, const double Psy_H, const int N_x,
               const int N_y, const int num_ghost_cell, double *XYCOORD, const int ndevices, const int device)
{
    ibtfo_ref_Psy_coord(lo_x, lo_y, Psy_L, Psy_H, N_x, N_y, num_ghost_cell, XYCOORD, ndevices, device);
}

void Level_Set(char *filename, const int N_x, const int N_y, const int num_ghost_cell, double *XYCOORD,
               const int ndevices, const int device)
{
    // phi from the case's plug-in on the host, then normals and cell types on the GPU
    Level_Set_function(filename, N_x, N_y, num_ghost_cell, XYCOORD, ndevices, device);
    ibtfo_ref_Level_Set(N_x, N_y, num_ghost_cell, XYCOORD, ndevices, device);
}

void Scheme_Index(const int N_x, const int N_y, const int num_ghost_cell, double *XYCOORD, double *GFM_Index,
                  const int ndevices, const int device)
{
    ibtfo_ref_Scheme_Index(N_x, N_y, num_ghost_cell, XYCOORD, GFM_Index, ndevices, device);
}

void TimeAdvance(const double Psy_L, const double Psy_H, const int N_x, const int N_y, const int num_ghost_cell,
                 const double gamma, double dt, double *U_OLD, double *U_TMP, double *U_NEW, double *XYCOORD,
                 double *SCHEME_IDX, const int ndevices, const int device)
{
    ibtfo_ref_TimeAdvance(Psy_L, Psy_H, N_x, N_y, num_ghost_cell, gamma, dt, U_OLD, U_TMP, U_NEW, XYCOORD,
                          SCHEME_IDX, ndevices, device);
}

void Boundary(const int N_x, const int N_y, const int num_ghost_cell, const double gamma, double *U_OLD,
              double *U_NEW, double *XYCOORD, double *SCHEME_IDX, const int ndevices, const int device)
{
    ibtfo_ref_Boundary(N_x, N_y, num_ghost_cell, gamma, U_OLD, U_NEW, XYCOORD, SCHEME_IDX, ndevices, device);
}

void Global_Boundary(const int N_x, const int N_y, const int num_ghost_cell, const double gamma, double *U_OLD,
                     double *U_NEW, const int ndevices, const int device)
{
    ibtfo_ref_Global_Boundary(N_x, N_y, num_ghost_cell, gamma, U_OLD, U_NEW, ndevices, device);
}

void ComputeDt(const double Psy_L, const double Psy_H, const int N_x, const int N_y, const int num_ghost_cell,
               const double gamma, const double CFL_number, double *U_OLD, double *XYCOORD, double *TMP_DT,
               const int ndevices, const int device)
{
    ibtfo_ref_ComputeDt(Psy_L, Psy_H, N_x, N_y, num_ghost_cell, gamma, CFL_number, U_OLD, XYCOORD, TMP_DT, ndevices,
                        device);
}

void CaculateMass(const double Psy_L, const double Psy_H, const int N_x, const int N_y, const int num_ghost_cell,
                  double *U_OLD, double *XYCOORD, double *MASS_DEVICE, const int ndevices, const int device)
{
    ibtfo_ref_CaculateMass(Psy_L, Psy_H, N_x, N_y, num_ghost_cell, U_OLD, XYCOORD, MASS_DEVICE, ndevices, device);
}

void WriteData(const double lo_x, const double lo_y, const double Psy_L, const double Psy_H, const int N_x,
               const int N_y, const int num_ghost_cell, const int iter, const double now_t, const double gamma,
               double *U_OLD, double *XYCOORD, const int ndevices, const int device)
{
    ibtfo_ref_WriteData(lo_x, lo_y, Psy_L, Psy_H, N_x, N_y, num_ghost_cell, iter, now_t, gamma, U_OLD, XYCOORD,
                        ndevices, device);
}
