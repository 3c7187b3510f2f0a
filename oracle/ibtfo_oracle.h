/* CPU oracle for the IBTFO per-timestep update: a plain-C, FP64 restatement
 * of the reference algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library; the product path
 * (ibtfo_gb300/ and its CUDA kernels) never calls it.
 *
 * The restatement keeps the reference's array-of-structures layout, its loop
 * ranges and its expression evaluation order so that, compiled with
 * -ffp-contract=off, it reproduces the reference bit for bit (pinned against
 * the reference's own sources in tests/test_oracle_golden.py).  Each function
 * in ibtfo_oracle.c cites the reference file:line it restates.
 *
 * Layout (reference Src/Base/Euler/Advection/MUSCL/EQDefine.H:4-44,
 * Src/Geometry/CoordDefine.H:4-7), with M = N_x + 2 ng, N = N_y + 2 ng:
 *   U[(M*j + i)*4 + k]            conserved state (rho, rho u, rho v, E)
 *   U_TMP[(M*j + i)*28 + 4*s + k] scratch slot s in 0..6
 *   XY[(M*j + i)*6 + c]           c = x, y, phi, n_x, n_y, cell type
 *   SCH[(M*j + i)*num_sch + c]    per-cell boundary data, num_sch per variant
 */
#ifndef IBTFO_ORACLE_H
#define IBTFO_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

enum { OR_MUSCL = 0, OR_MHM = 1, OR_GODUNOV = 2, OR_LAX = 3 };
enum { OR_SINGLESTEP = 0, OR_RK2 = 1 };
enum { OR_HLL = 0, OR_HLLC = 1, OR_PVRS = 2, OR_SW = 3 };
enum { OR_MINMOD = 0, OR_VANLEER = 1 };
enum { OR_REGULAR = 0, OR_IDW = 1, OR_LINEAR = 2, OR_RIEMANNGFM = 3, OR_BCGFM = 4, OR_HBCGFM = 5 };
enum { OR_GB_WALLS = 0, OR_GB_PERIODIC = 1 };

typedef struct or_case or_case;

or_case *or_create(int n_x, int n_y, int ng, double lo_x, double lo_y, double hi_x, double hi_y,
                   double gamma, double cfl, int scheme, int riemann, int limiter, int boundary, int gbc);
void or_destroy(or_case *c);
/* Time = SingleStep (default) or RK2 (two-stage, see or_run) */
void or_set_time_advance(or_case *c, int time_advance);
void or_set_threads(int n);
int or_num_sch(const or_case *c);

/* Psy_coord + Level_Set (phi supplied, M*N values) + Scheme_Index (GFM variants). */
void or_setup_geometry(or_case *c, const double *phi);
/* Initialize (U_OLD = U_NEW = u0), the initial Boundary call, the first
 * ComputeDt and CaculateMass (reference Test/InclineSod/InclineSod.cpp:103-128). */
void or_set_initial_state(or_case *c, const double *u0);
/* Runs the reference time loop for at most nsteps iterations (also stopping at
 * now_t >= t_end or iter >= max_iter).  dts/masses (may be NULL) receive one
 * value per completed step.  Returns the number of steps taken. */
int or_run(or_case *c, int nsteps, double t_end, int max_iter, double *dts, double *masses);

/* Single stages, for unit-level parity tests. */
void or_advance(or_case *c, double dt);
void or_boundary(or_case *c);
void or_global_boundary(or_case *c);
double or_compute_dt(or_case *c);
double or_mass(or_case *c);

/* Accessors.  which: 0 U_OLD, 1 U_NEW, 2 XYCOORD, 3 SCHEME_IDX, 4 U_TMP */
long or_array_len(const or_case *c, int which);
void or_get(const or_case *c, int which, double *dst);
void or_put(or_case *c, int which, const double *src);
void or_scalars(const or_case *c, double *out4); /* dt, now_t, mass_start, mass_now */
int or_iter(const or_case *c);

#ifdef __cplusplus
}
#endif
#endif
