/* ibtfo_ref.h -- the reference's solver entry points, with their argument
 * lists, over host arrays, backed by the GB300 library.
 *
 * A reference driver (Test/<case>/<Case>.cpp) links these through one-line
 * C++ forwarding functions (ibtfo_gb300/forward/ibtfo_forward.cpp) in place
 * of the Src/ files of its Makefile slots.  Each function takes the same arguments as the reference
 * function it replaces (file:line below); the trailing (ndevices, device)
 * pair is accepted and must describe one device.
 *
 * Host arrays are keyed like OpenACC's present table: the XYCOORD pointer
 * identifies a case, and the U_OLD pointer is bound to it at its first
 * TimeAdvance/Boundary call.  The state stays on the GPU between calls:
 * ibtfo_ref_update_self copies U_OLD / U_NEW back to the host arrays (the
 * reference's `acc update self`), ibtfo_ref_update_device sends a host U_OLD
 * that the caller changed.  Geometry results (XYCOORD normals and types,
 * SCHEME_IDX) are written to the host arrays at once, because the
 * reference's plug-ins read them on the host.
 *
 * The reference functions return void; the status of the last call of the
 * calling thread is available from ibtfo_ref_status() and
 * ibtfo_last_error().
 */
#ifndef IBTFO_REF_H
#define IBTFO_REF_H

#include "ibtfo.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Slot selection for cases created afterwards (the Makefile variables
 * Scheme / Riemann / Limiter / Boundary of Test/Sod/Makefile:1-7, plus the
 * global boundary and precision keys of include/ibtfo.h). */
void ibtfo_ref_configure(int scheme, int riemann, int limiter, int boundary, int global_boundary, int precision);
int ibtfo_ref_status(void);

/* Src/Geometry/Psy_coord.H:11-20 */
void ibtfo_ref_Psy_coord(double lo_x, double lo_y, double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell,
                         double *XYCOORD, int ndevices, int device);
/* Src/Geometry/Level_Set.H:12-18, after the case's Level_Set_function has put
 * phi in XYCOORD[..*6+2]; fills n_x, n_y and the cell type. */
void ibtfo_ref_Level_Set(int N_x, int N_y, int num_ghost_cell, double *XYCOORD, int ndevices, int device);
/* Src/BoundaryCondition/Scheme_Index.H:13-19 */
void ibtfo_ref_Scheme_Index(int N_x, int N_y, int num_ghost_cell, double *XYCOORD, double *SCHEME_IDX, int ndevices,
                            int device);
/* Src/Base/TimeAdvance/TimeAdvance.H:33-46 and Src/Base/Euler/Advection/Advance.H:14-26
 * (U_TMP is not used: the scratch lives on the GPU) */
void ibtfo_ref_TimeAdvance(double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell, double gamma, double dt,
                           double *U_OLD, double *U_TMP, double *U_NEW, double *XYCOORD, double *SCHEME_IDX,
                           int ndevices, int device);
void ibtfo_ref_Advance(double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell, double gamma, double dt,
                       double *U_OLD, double *U_TMP, double *U_NEW, double *XYCOORD, int ndevices, int device);
/* Src/BoundaryCondition/Boundary.H:11-20 (the first call on a case, before
 * any TimeAdvance, is the initial Boundary and sends U_OLD to the GPU) */
void ibtfo_ref_Boundary(int N_x, int N_y, int num_ghost_cell, double gamma, double *U_OLD, double *U_NEW,
                        double *XYCOORD, double *SCHEME_IDX, int ndevices, int device);
/* Src/BoundaryCondition/Boundary.H:22-29 */
void ibtfo_ref_Global_Boundary(int N_x, int N_y, int num_ghost_cell, double gamma, double *U_OLD, double *U_NEW,
                               int ndevices, int device);
/* Src/Base/Common/ComputeDt.H:12-23 (writes TMP_DT[device]) */
void ibtfo_ref_ComputeDt(double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell, double gamma,
                         double CFL_number, double *U_OLD, double *XYCOORD, double *TMP_DT, int ndevices, int device);
/* Src/Utils/CaculateMass.H (writes MASS_DEVICE[device]; the state is not
 * copied back -- use ibtfo_ref_update_self for that) */
void ibtfo_ref_CaculateMass(double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell, double *U_OLD,
                            double *XYCOORD, double *MASS_DEVICE, int ndevices, int device);

/* Src/Utils/WriteData.H (WriteData.cpp:5-247): appends dat_<device>_<iter>.vtk
 * to result.visit (with the "!NBLOCKS 1" line at iter 0) and writes that file
 * in the reference's ASCII layout from the resident state; U_OLD is not
 * copied back. */
void ibtfo_ref_WriteData(double lo_x, double lo_y, double Psy_L, double Psy_H, int N_x, int N_y, int num_ghost_cell,
                         int iter, double now_t, double gamma, double *U_OLD, double *XYCOORD, int ndevices,
                         int device);

/* `acc update self` / `acc update device` of a registered U_OLD or U_NEW */
void ibtfo_ref_update_self(double *U);
void ibtfo_ref_update_device(double *U);
/* releases the case keyed by XYCOORD (the driver's `acc exit data`) */
void ibtfo_ref_release(double *XYCOORD);

#ifdef __cplusplus
}
#endif
#endif
