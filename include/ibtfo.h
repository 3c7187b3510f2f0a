/* ibtfo.h -- C ABI of the GB300 (sm_103a) IBTFO per-timestep solver.
 *
 * One `ibtfo_case` is one 2D compressible-Euler problem resident on one GPU:
 * the reference's Src/Base + Src/BoundaryCondition + Src/Geometry hot path
 * (Advance, Riemann solvers, limiters, ghost-fluid Boundary,
 * Global_Boundary, ComputeDt, CaculateMass, Level_Set/Scheme_Index set-up)
 * behind plain pointers and sizes.  All host arrays use the reference's
 * array-of-structures layout with M = N_x + 2*num_ghost_cell columns and
 * N = N_y + 2*num_ghost_cell rows:
 *   state     U[(M*j + i)*4 + k]   k = rho, rho*u, rho*v, E   (EQDefine.H:31)
 *   geometry  XY[(M*j + i)*6 + c]  c = x, y, phi, n_x, n_y, type (CoordDefine.H:7)
 *   level set PHI[M*j + i]
 * Host pointers are only read or written during the call that receives them.
 * Functions return IBTFO_OK or an error code; ibtfo_last_error() describes
 * the last failure of the calling thread.
 */
#ifndef IBTFO_H
#define IBTFO_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IBTFO_ABI_VERSION 1

typedef enum ibtfo_status {
    IBTFO_OK = 0,
    IBTFO_EINVAL = 1,   /* bad argument or configuration */
    IBTFO_ENOMEM = 2,   /* device or pinned-host allocation failed */
    IBTFO_ENAN = 3,     /* the state holds NaN (reported by ibtfo_run when asked to stop on NaN) */
    IBTFO_ETIMEOUT = 4, /* a bounded wait gave up */
    IBTFO_ECUDA = 5,    /* a CUDA runtime call failed */
    IBTFO_ESTATE = 6    /* call out of order (e.g. stepping before ibtfo_set_state) */
} ibtfo_status;

/* selection keys: the reference Makefile slots Scheme / Riemann / Limiter /
 * Boundary (Test/Sod/Makefile:1-7) and the per-case Global_Boundary plug-in */
/* LAX: the reference's Lax-Friedrichs scheme (Lax/Lax_Scheme.cpp; no Riemann
 * solver or limiter), FP64 precisions, not with cut cells or in batches */
enum { IBTFO_SCHEME_MUSCL = 0, IBTFO_SCHEME_MHM = 1, IBTFO_SCHEME_GODUNOV = 2, IBTFO_SCHEME_LAX = 3 };
/* the reference's Time slot (Test/Sod/Makefile:5).  RK2: Heun's two-stage
 * method, U1 = U0 + dt L(U0) with its Boundary and Global_Boundary passes,
 * then 0.5 (U0 + U1 + dt L(U1)) on fluid cells, both stages with the dt of
 * the step (the two-stage method Src/Base/TimeAdvance/RK2/RK2.cpp describes;
 * that file itself does not compile); in the FP32 form the average is taken
 * on the (hi, lo) pairs.  Not with cut cells; a batch runs one Time key
 * for all its cases. */
enum { IBTFO_TIME_SINGLESTEP = 0, IBTFO_TIME_RK2 = 1 };
/* HLLC is the reference's HLLC directory, whose solver is HLL (including the
 * Y-face slot reuse); HLLC_TORO is a contact-restoring HLLC with no
 * reference counterpart, with two positivity safeguards: a face whose
 * reconstructed state has rho <= 0 or an internal energy below 1e-6 of E
 * takes the first-order pair (the two cell averages), and an updated fluid
 * cell whose internal energy falls below 1e-5 of E has E raised to
 * E_kin + 1e-5 E.  HLL_TORO (no reference counterpart) is the reference's
 * HLL flux with Toro's wave-speed estimates (p* clamped at 0, q_K = 1 where
 * p* <= p_K, so no square root of a negative number behind a strong
 * shock), no Y-face slot reuse, and the same two safeguards; like every HLL
 * flux it does not suffer the carbuncle / odd-even decoupling of
 * contact-restoring solvers at strong grid-aligned shocks.  The cut-cell
 * method (IBTFO_BOUNDARY_CCM) runs HLL_TORO, STEGER_WARMING and HLLC_TORO;
 * the reference's HLL (the HLL and HLLC keys) and PVRS have no cut-cell
 * form, and ibtfo_create rejects them there (IBTFO_EINVAL). */
enum {
    IBTFO_RIEMANN_HLL = 0,
    IBTFO_RIEMANN_HLLC = 1,
    IBTFO_RIEMANN_PVRS = 2,
    IBTFO_RIEMANN_STEGER_WARMING = 3,
    IBTFO_RIEMANN_HLLC_TORO = 4,
    IBTFO_RIEMANN_HLL_TORO = 5
};
enum { IBTFO_LIMITER_MINMOD = 0, IBTFO_LIMITER_VANLEER = 1 };
enum {
    IBTFO_BOUNDARY_REGULAR = 0,
    IBTFO_BOUNDARY_IDW_GFM = 1,     /* IDWBaseGFM */
    IBTFO_BOUNDARY_LINEAR_GFM = 2,  /* LinearBaseGFM */
    IBTFO_BOUNDARY_RIEMANN_GFM = 3, /* RiemannBaseGFM (same algorithm as LinearBaseGFM) */
    IBTFO_BOUNDARY_BCGFM = 4,
    IBTFO_BOUNDARY_HBCGFM = 5,
    /* Cartesian cut cells, no reference counterpart: face apertures and
     * volume fractions from the level set, a wall flux from the mirrored-state
     * Riemann problem, first-order faces next to the body, and conservative
     * mixing of cut cells with volume fraction below 0.5 with their
     * neighbours (FP64 for the geometry, the cut-cell update and the
     * mixing); solvers HLL_TORO, Steger-Warming, HLLC_TORO; both FP64
     * precision keys run the same FP64 arithmetic */
    IBTFO_BOUNDARY_CCM = 6
};
enum { IBTFO_GLOBAL_WALLS = 0, IBTFO_GLOBAL_PERIODIC = 1 };
/* arithmetic of the step: FP64 evaluating the reference's expressions in
 * their order (bit-for-bit with the reference except where the library
 * pow(x, 0.5) and sqrt differ in the last bit); FP64 with shared
 * reciprocals and fused multiply-adds (rounding-level differences, well
 * inside a 1e-12 relative bar); or the precision form: FP32 face
 * reconstruction, Riemann solves and fluxes with the state held as FP32
 * (hi, lo) pairs updated by an error-free sum, FP64 for the mass sum, dt and
 * the ghost-fluid fill (HLL/HLLC and Steger-Warming) */
enum { IBTFO_PRECISION_FP64 = 0, IBTFO_PRECISION_FP64_FAST = 1, IBTFO_PRECISION_FP32_COMPENSATED = 2 };

/* Case parameters: the numeric .inp keys the reference driver reads
 * (Test/Sod/Sod.cpp:34-48) plus the slot selections. */
typedef struct ibtfo_config {
    int n_x, n_y, num_ghost_cell; /* num_ghost_cell >= 2 */
    double lo_x, lo_y, hi_x, hi_y;
    double gamma, cfl_number, psy_time;
    int max_iter;
    int scheme, riemann, limiter, boundary, global_boundary;
    int precision;    /* IBTFO_PRECISION_* */
    int time_advance; /* IBTFO_TIME_* */
    int reserved[6];  /* zero */
} ibtfo_config;

/* The reference time-loop scalars after the last completed step. */
typedef struct ibtfo_progress {
    int iter;       /* completed steps */
    int status;     /* bit 0: a fluid cell held NaN after some step (sticky); bit 1: a
                       sweep tile's staging copy missed its bounded wait (sticky; the
                       calls that report progress then return IBTFO_ETIMEOUT) */
    int nan_cells;  /* fluid cells with a NaN component after the latest step */
    int reserved;
    double now_t;   /* loop time, advanced by the dt computed after each step (Sod.cpp:176) */
    double dt;      /* dt the next step applies (ComputeDt of the current state) */
    double mass;    /* CaculateMass of the current state */
    double mass_start;
} ibtfo_progress;

typedef struct ibtfo_case ibtfo_case;

int ibtfo_abi_version(void);
const char *ibtfo_last_error(void);
/* kernels launched by this library since load (graph replays counted per node) */
long long ibtfo_launch_count(void);

/* Creates a case on the current CUDA device.  Allocates the device state
 * (two structure-of-arrays buffers, geometry, reduction scratch). */
ibtfo_status ibtfo_create(const ibtfo_config *cfg, ibtfo_case **out);
ibtfo_status ibtfo_destroy(ibtfo_case *c);
/* Issue all work of this case on `stream` (a cudaStream_t); NULL selects the
 * case's own stream. */
ibtfo_status ibtfo_set_stream(ibtfo_case *c, void *stream);

/* Psy_coord + Level_Set + Scheme_Index (Src/Geometry/Psy_coord.cpp:5-39,
 * Level_Set.cpp:6-128, the Scheme_Index of each Src/BoundaryCondition variant) from the
 * level set phi (M*N doubles). */
ibtfo_status ibtfo_setup_geometry(ibtfo_case *c, const double *phi);
/* XYCOORD in the reference layout (M*N*6 doubles). */
ibtfo_status ibtfo_get_geometry(ibtfo_case *c, double *xycoord);
/* SCHEME_IDX in the reference layout of the selected boundary variant
 * (num_sch = 1, 4, 8 or 16 doubles per cell; see ibtfo_num_sch). */
int ibtfo_num_sch(const ibtfo_case *c);
ibtfo_status ibtfo_get_scheme_index(ibtfo_case *c, double *scheme_idx);
/* number of ghost-fluid cells found by the set-up */
int ibtfo_num_ghost_cells(const ibtfo_case *c);
/* Cut-cell cases (IBTFO_BOUNDARY_CCM; no reference counterpart): volume
 * fraction of each cell, aperture of its X face (i+1/2, j) and of its Y face
 * (i, j+1/2), each M*N doubles (cell types are in ibtfo_get_geometry: 0
 * fluid, 1 solid, 2 domain ring, 3 cut). */
ibtfo_status ibtfo_get_cut_cells(ibtfo_case *c, double *alpha, double *ax, double *ay);

/* Initial state (M*N*4 doubles): Initialize sets U_OLD = U_NEW = u0, then the
 * initial Boundary call, ComputeDt and CaculateMass
 * (Test/InclineSod/InclineSod.cpp:103-128).  Resets the loop accounting. */
ibtfo_status ibtfo_set_state(ibtfo_case *c, const double *u0);
/* Current U_OLD and U_NEW in the reference layout; either pointer may be NULL.
 * Waits for queued work. */
ibtfo_status ibtfo_get_state(ibtfo_case *c, double *u_old, double *u_new);

/* ---------------------------------------------------------------- device-side set-up
 *
 * No counterparts in the reference, which builds phi and the initial state
 * on the host (Test/InclineSod/Level_Set_function.cpp:8-52,
 * Test/PNGGeo/Level_Set.cpp:31-142 and each test's Initialize.cpp).  These build
 * them on the GPU, so a case of millions of cells is set up without a host
 * array or a host-to-device copy. */
enum { IBTFO_BODY_CIRCLE = 0, IBTFO_BODY_ELLIPSE = 1 };
typedef struct ibtfo_body {
    int kind;          /* IBTFO_BODY_* */
    int reserved;
    double xc, yc;     /* centre */
    double a, b;       /* circle: radius a; ellipse: semi-axes a (along theta) and b */
    double theta;      /* ellipse orientation, radians */
} ibtfo_body;

/* ibtfo_setup_geometry with phi = the signed distance to the union of the
 * bodies (positive in the fluid outside them; exact within 16 cells of an
 * outline, a lower bound of the right sign farther out).  n = 0: no body. */
ibtfo_status ibtfo_setup_bodies(ibtfo_case *c, const ibtfo_body *bodies, int n);
/* ibtfo_set_state with primitive states (rho, u, v, p) `left` for
 * x < x_split and `right` elsewhere; solid cells hold rho = -1, E = -1 as the
 * reference's Initialize writes them. */
ibtfo_status ibtfo_init_x_split(ibtfo_case *c, double x_split, const double left[4], const double right[4]);
/* Primitive state behind a normal shock moving in +x at Mach `mach` into the
 * primitive state `pre` (Rankine-Hugoniot). */
ibtfo_status ibtfo_post_shock_state(double mach, double gamma, const double pre[4], double post[4]);
/* Free phi and the normals once the geometry is set up (ibtfo_get_geometry
 * and ibtfo_setup_geometry then return IBTFO_ESTATE). */
ibtfo_status ibtfo_release_geometry(ibtfo_case *c);
/* Interior density of the current state, n_y rows of n_x doubles; wait = 0
 * queues the copy on the case's stream and returns (use pinned memory). */
ibtfo_status ibtfo_get_density(ibtfo_case *c, double *out, int wait);
/* Device bytes a case of this configuration holds: `resident` while it runs
 * (after ibtfo_release_geometry, without the host-transfer staging that
 * ibtfo_set_state / ibtfo_get_state allocate on first use), `setup` at the
 * peak of its set-up. */
ibtfo_status ibtfo_case_bytes(const ibtfo_config *cfg, long long *resident, long long *setup);

/* Replaces U_OLD (the current state, M*N*4 doubles) without touching the
 * loop accounting, dt or U_NEW: the host-buffer round trip of a caller that
 * keeps its own copy of the state between steps. */
ibtfo_status ibtfo_put_state(ibtfo_case *c, const double *u_old);
/* One time-loop iteration on host arrays: u_in (M*N*4 doubles) replaces the
 * current state as ibtfo_put_state does, the step runs as ibtfo_step does,
 * and the new U_OLD is written to u_out (which may be u_in); waits for the
 * result and fills `p` (may be NULL).  The transfers go in row chunks on two
 * copy streams, overlapped with the layout conversion and the sweep (rows of
 * the sweep start once their stencil is on the device): from page-locked
 * host memory the copies run concurrently with the kernels.
 * In place (u_out == u_in) a step copies back only the cells it can change,
 * and from the second call on the same array (with no ibtfo_set_state,
 * ibtfo_put_state, ibtfo_init_x_split or ibtfo_load_checkpoint in between)
 * copies in only the cells it reads: the fluid cells with two cells around
 * them, the ghost cells and the domain edge (PVRS solvers: every row).  The
 * result in the array is the same; the device copy of the cells no step
 * reads (solid cells away from the fluid) keeps the values the array held
 * at the first call. */
ibtfo_status ibtfo_step_host(ibtfo_case *c, const double *u_in, double *u_out, ibtfo_progress *p);
/* Bytes one ibtfo_step_host call moves each way (in place: a call after the
 * first on the same array).  In place only the cells a step can change go
 * back: the interior rows of the columns holding fluid cells, plus the ghost
 * cells and the domain ring. */
ibtfo_status ibtfo_step_host_bytes(const ibtfo_case *c, int in_place, long long *h2d, long long *d2h);

/* Queues `nsteps` iterations of the reference loop body (Sod.cpp:154-177:
 * TimeAdvance, Boundary, Global_Boundary, ComputeDt, CaculateMass,
 * now_t += dt) without waiting.  An iteration whose loop condition
 * (now_t < psy_time && iter < max_iter) is false when it reaches the GPU does
 * nothing. */
ibtfo_status ibtfo_advance(ibtfo_case *c, int nsteps);
/* The two launches of one guarded iteration, for callers that time or
 * capture them separately: the fused sweep (Advance + ComputeDt +
 * CaculateMass + loop accounting) and the boundary pass (ghost-fluid
 * Boundary + Global_Boundary).  ibtfo_advance(c, 1) == sweep then boundary.
 * Time = RK2: the "sweep" is the first stage, its boundary pass and the
 * second stage. */
ibtfo_status ibtfo_enqueue_sweep(ibtfo_case *c);
ibtfo_status ibtfo_enqueue_boundary(ibtfo_case *c);
/* One iteration regardless of the loop condition; waits and reports. */
ibtfo_status ibtfo_step(ibtfo_case *c, ibtfo_progress *p);
/* Runs the loop to completion (now_t >= psy_time or iter >= max_iter).
 * stop_on_nan != 0 returns IBTFO_ENAN as soon as a NaN appears. */
ibtfo_status ibtfo_run(ibtfo_case *c, int stop_on_nan, ibtfo_progress *p);
/* Waits for queued work and reports the loop scalars. */
ibtfo_status ibtfo_get_progress(ibtfo_case *c, ibtfo_progress *p);
ibtfo_status ibtfo_synchronize(ibtfo_case *c);

/* .inp files, read as the reference's ParamReader reads them
 * (Src/Utils/ParamReader.cpp:14-68: '#' lines skipped, spaces removed, the
 * first [+-]?(\d*\.\d+|\d+) after '=' converted with atof), plus string
 * values for the solver-slot keys. */
typedef struct ibtfo_inp ibtfo_inp;
ibtfo_status ibtfo_inp_open(const char *path, ibtfo_inp **out);
ibtfo_status ibtfo_inp_parse(const char *text, ibtfo_inp **out);
void ibtfo_inp_close(ibtfo_inp *p);
/* value of `key`, or `def` when absent (Params::get, ParamReader.H:47-55);
 * returns 1 if the key is present */
int ibtfo_inp_get(const ibtfo_inp *p, const char *key, double def, double *value);
int ibtfo_inp_get_string(const ibtfo_inp *p, const char *key, char *buf, int size);
/* numeric keys with the reference drivers' defaults (Test/Sod/Sod.cpp:34-48)
 * and the slot keys Scheme (MUSCL|MHM|Godunov), Riemann (HLL|HLLC|PVRS|
 * StegerWarming|HLLC_Toro), Limiter (minmod|VanLeer), Boundary (Regular|IDWBaseGFM|
 * LinearBaseGFM|RiemannBaseGFM|BCGFM|HBCGFM), Global_Boundary (Walls|
 * Periodic), Precision (FP64|FP64_FAST|FP32_COMPENSATED) */
ibtfo_status ibtfo_config_from_inp(const ibtfo_inp *p, ibtfo_config *cfg);

/* Case plug-ins (the reference's per-case Level_Set_function and Initialize
 * files): sod_ref (Test/Sod), incline_ref (Test/InclineSod), vortex_ref
 * (Test/Vortex), sod_x, channel, isentropic_vortex; parameters from `p`
 * (may be NULL for defaults).  phi: M*N doubles.  init: M*N*4 doubles from
 * XYCOORD (coordinates and cell types, as Initialize reads them). */
ibtfo_status ibtfo_case_phi(const char *name, const ibtfo_inp *p, const ibtfo_config *cfg, double *phi);
ibtfo_status ibtfo_case_init(const char *name, const ibtfo_inp *p, const ibtfo_config *cfg, const double *xycoord,
                             double *u0);

/* CFL time step and fluid mass of a device-resident state, allocating
 * nothing.  No counterpart in the reference: it serves callers that cannot
 * call cudaMalloc -- code running inside a framework that owns all device
 * memory through its own pool, or that must not let an allocation
 * synchronise the device between its kernels -- and that already hold the
 * state on the GPU.
 *   d_u      four planes (rho, rho u, rho v, E), `plane` doubles apart, rows
 *            `pitch` doubles long (pitch >= N_x + 2 ng), index j*pitch + i
 *   d_type   cell types (0 fluid, 1 solid, 2 ghost), uint8, same pitch
 *   d_out    two doubles on the device: dt = CFL dx / (max a + max(max|u|,
 *            max|v|)) and mass = sum rho dx dy, both over fluid interior cells
 * The work is queued on `stream` (a cudaStream_t, NULL for the default
 * stream) and the call returns without waiting.  Scratch is a fixed array
 * inside the library (512 KiB per GPU, held by every GPU that loads the
 * library until the process exits), so grids above 65536 tiles of 32 x 8
 * interior cells (e.g. 4096 x 4096) are rejected with IBTFO_EINVAL.  The
 * first call on a device looks up that array's device address (every call
 * looks it up; the first may load the library's code onto that device): make
 * that first call before any stream capture.  Every call shares the one array
 * and it keeps the last call's contents: calls that overlap on the GPU (other
 * streams, other threads) race and give wrong results.  NaN is not reported:
 * a NaN density in a fluid cell makes the mass NaN, and NaN in the other
 * components drops out of the maxima (ibtfo_get_progress of a case counts
 * NaN cells). */
ibtfo_status ibtfo_dt_mass_noalloc(const double *d_u, long long plane, int pitch, const unsigned char *d_type,
                                   int n_x, int n_y, int num_ghost_cell, double lo_x, double lo_y, double hi_x,
                                   double hi_y, double gamma, double cfl_number, double *d_out, void *stream);

/* ---------------------------------------------------------------- batches
 *
 * No counterpart in the reference: its drivers (Test/Sod/Sod.cpp:108-181)
 * advance one case per process.  A batch steps many cases of uneven grid
 * sizes together: one persistent sweep kernel over a shared tile table, one
 * boundary pass over all cases, each step captured in a CUDA graph.  Every
 * case keeps its own dt, loop time and loop condition (t_end, max_iter);
 * cases whose loop has ended are skipped.  A case advances in a batch bit for
 * bit as it does alone (same kernels), and with the 32 x 8 tile shape its
 * mass sum is bitwise identical too.
 *
 * Cases join with ibtfo_batch_add (after ibtfo_set_state) and leave with
 * ibtfo_batch_remove; in between, the batch alone steps them (do not call
 * ibtfo_advance/ibtfo_step on a case in a batch; ibtfo_get_state and
 * ibtfo_get_progress remain valid after ibtfo_batch_synchronize).  All
 * cases of a batch share the kernel variant (scheme, Riemann solver,
 * limiter, precision); grid size, geometry, boundary method, domain
 * boundaries, gamma, CFL, t_end and max_iter are per case.  Batches run the
 * fp64_fast and FP32 compensated precisions. */
typedef struct ibtfo_batch ibtfo_batch;

enum { IBTFO_TILE_32x8 = 0, IBTFO_TILE_32x16 = 1, IBTFO_TILE_64x8 = 2 };

typedef struct ibtfo_batch_config {
    int scheme, riemann, limiter, precision; /* the kernel variant of every case */
    int tile_shape;   /* IBTFO_TILE_*: interior cells per CTA (256 threads) */
    int ctas_per_sm;  /* resident CTAs per SM of the persistent sweep (0: the occupancy limit) */
    int graph_steps;  /* steps per captured graph (0: 16) */
    int time_advance; /* IBTFO_TIME_* of every case: RK2 steps are two sweeps, each followed by
                         the boundary pass */
    int reserved[4];
} ibtfo_batch_config;

typedef struct ibtfo_batch_tiling {
    int tile_shape, ctas_per_sm, max_ctas_per_sm, grid; /* grid = SMs x ctas_per_sm */
    long long tiles;    /* tiles in the table */
    double ms_per_step; /* autotuner timing (0 elsewhere) */
    int reserved[4];
} ibtfo_batch_tiling;

ibtfo_status ibtfo_batch_create(const ibtfo_batch_config *cfg, ibtfo_batch **out);
ibtfo_status ibtfo_batch_destroy(ibtfo_batch *b); /* does not destroy the cases */
ibtfo_status ibtfo_batch_set_stream(ibtfo_batch *b, void *stream);
/* add a case (state set, same kernel variant); *slot receives its slot */
ibtfo_status ibtfo_batch_add(ibtfo_batch *b, ibtfo_case *c, int *slot);
/* take a case out; returns without waiting: the case's own stream (its
 * transfers, ibtfo_destroy) is ordered after the steps already queued */
ibtfo_status ibtfo_batch_remove(ibtfo_batch *b, int slot);
int ibtfo_batch_size(const ibtfo_batch *b);      /* cases in the batch */
int ibtfo_batch_num_slots(const ibtfo_batch *b); /* highest used slot + 1 */
ibtfo_case *ibtfo_batch_case(const ibtfo_batch *b, int slot);
/* queue nsteps steps of every case (graph launches of graph_steps, then
 * single steps); returns without waiting */
ibtfo_status ibtfo_batch_advance(ibtfo_batch *b, int nsteps);
/* progress of every slot: enqueue a snapshot after the queued steps, then
 * read it (wait != 0 blocks; wait == 0 returns IBTFO_ETIMEOUT while the
 * snapshot is not ready).  active[k] = the case's loop condition still holds. */
ibtfo_status ibtfo_batch_progress_enqueue(ibtfo_batch *b);
ibtfo_status ibtfo_batch_progress_read(ibtfo_batch *b, ibtfo_progress *out, int *active, int n, int wait);
ibtfo_status ibtfo_batch_progress(ibtfo_batch *b, ibtfo_progress *out, int *active, int n);
ibtfo_status ibtfo_batch_synchronize(ibtfo_batch *b);
ibtfo_status ibtfo_batch_set_tiling(ibtfo_batch *b, int tile_shape, int ctas_per_sm);
ibtfo_status ibtfo_batch_get_tiling(const ibtfo_batch *b, ibtfo_batch_tiling *t);
/* time every tile shape x resident-CTA count on `steps` real steps of the
 * current cases and keep the fastest (the state is the same under every
 * tiling, so the trial steps are ordinary steps) */
ibtfo_status ibtfo_batch_autotune(ibtfo_batch *b, int steps, ibtfo_batch_tiling *best, ibtfo_batch_tiling *trials,
                                  int max_trials, int *n_trials);

/* ---------------------------------------------------------------- serving
 *
 * No counterpart in the reference.  A server accepts solves as requests,
 * admits them in arrival order while its device-memory budget and
 * active-case limit allow, steps all admitted cases together in one batch
 * (continuous batching: requests that arrive while others run join between
 * chunks of steps), and retires each case when its own loop ends.  Each
 * request is one case set up on the GPU: bodies (ibtfo_setup_bodies) and a
 * two-state initial condition split at x = x_split (ibtfo_init_x_split; a
 * shock with ibtfo_post_shock_state).  Results carry the final loop scalars,
 * the times of arrival, admission and completion on the server clock, and,
 * when requested, the final density. */
typedef struct ibtfo_server ibtfo_server;

#define IBTFO_MAX_BODIES 8

typedef struct ibtfo_server_config {
    int scheme, riemann, limiter, precision; /* kernel variant of every case */
    long long memory_budget; /* device bytes for cases (0: 80% of the free memory at creation) */
    int max_active;          /* cases stepped at once (0: no limit) */
    int chunk_steps;         /* steps per scheduling round (0: 32) */
    int tile_shape;          /* IBTFO_TILE_*, or -1: autotune once 4 cases are active */
    int ctas_per_sm;         /* 0: the occupancy limit */
    int time_advance;        /* IBTFO_TIME_* of every case */
    int reserved[5];
} ibtfo_server_config;

typedef struct ibtfo_request {
    long long id;
    double arrival;          /* seconds on the server clock; admitted no earlier */
    int n_x, n_y;
    double lo_x, lo_y, hi_x, hi_y;
    double gamma, cfl_number, t_end;
    int max_iter;            /* 0: no limit */
    int boundary, global_boundary;
    int n_bodies;
    ibtfo_body bodies[IBTFO_MAX_BODIES];
    double x_split;
    double left[4], right[4]; /* primitive (rho, u, v, p) */
    double *density_out;     /* optional, n_x*n_y doubles (pinned for an asynchronous copy) */
    int reserved[8];
} ibtfo_request;

typedef struct ibtfo_result {
    long long id;
    int status;              /* IBTFO_OK, or the error that failed the request */
    int iter, nan_cells, reserved;
    double now_t, mass, mass_start;
    double arrival, admitted, finished; /* server clock, seconds */
} ibtfo_result;

typedef struct ibtfo_server_stats {
    long long submitted, admitted, completed, failed;
    int pending, active, retiring, peak_active;
    long long bytes_in_use, peak_bytes, memory_budget;
    long long chunks, steps;
    int tile_shape, ctas_per_sm;
    int reserved[6];
} ibtfo_server_stats;

ibtfo_status ibtfo_server_create(const ibtfo_server_config *cfg, ibtfo_server **out);
ibtfo_status ibtfo_server_destroy(ibtfo_server *s);
/* thread-safe; requests are kept in arrival order */
ibtfo_status ibtfo_server_submit(ibtfo_server *s, const ibtfo_request *r);
/* sets the server clock to zero (the first pump does it otherwise) */
ibtfo_status ibtfo_server_start(ibtfo_server *s);
double ibtfo_server_clock(const ibtfo_server *s);
/* one scheduling round; *busy = 1 while requests are pending, active or retiring */
ibtfo_status ibtfo_server_pump(ibtfo_server *s, int *busy);
/* pump until no work is left (IBTFO_ETIMEOUT after max_seconds > 0) */
ibtfo_status ibtfo_server_run(ibtfo_server *s, double max_seconds);
/* move up to `max` completed results into `out`; returns how many (thread-safe) */
int ibtfo_server_poll(ibtfo_server *s, ibtfo_result *out, int max);
ibtfo_status ibtfo_server_stats_get(ibtfo_server *s, ibtfo_server_stats *out);

/* ---------------------------------------------------------------- output
 *
 * VTK file of the current state in the layout of the reference's WriteData
 * (Src/Utils/WriteData.cpp:5-247): legacy structured points over the
 * interior cells, fields density / x-vel / y-vel / pressure (non-fluid cells
 * -1 and -100, density floored at 1e-6), the time as field data; binary = 0
 * writes the reference's ASCII "%f" values, 1 big-endian floats. */
ibtfo_status ibtfo_write_vtk(ibtfo_case *c, const char *path, int binary);
/* The same file written off the step path: the fields of the current state
 * are derived into a device snapshot in order with the case's steps, then
 * copied to pinned host memory on a second stream and written by a host
 * thread while the case keeps stepping.  One write is in flight per case;
 * the next call (or ibtfo_output_wait) waits for it and reports a failure of
 * it (IBTFO_EINVAL, the reason in ibtfo_last_error). */
ibtfo_status ibtfo_write_vtk_async(ibtfo_case *c, const char *path, int binary);
ibtfo_status ibtfo_output_wait(ibtfo_case *c);
/* Checkpoint (no reference counterpart): configuration, loop scalars and the
 * current state buffer as the device holds it (plus, for Regular
 * boundaries, the initial state and the corner sources), in native byte
 * order.  ibtfo_load_checkpoint restores it into a case created with the
 * same configuration (psy_time and max_iter may differ) whose geometry is
 * set up; stepping then continues bit for bit as the saved run would. */
ibtfo_status ibtfo_save_checkpoint(ibtfo_case *c, const char *path);
ibtfo_status ibtfo_load_checkpoint(ibtfo_case *c, const char *path);

/* IBTFO_OK when every operation queued on the case's stream has finished,
 * IBTFO_ETIMEOUT while some are pending (does not wait) */
ibtfo_status ibtfo_query(ibtfo_case *c);

/* Page-locked host memory for fast transfers (cudaHostAlloc / cudaFreeHost). */
ibtfo_status ibtfo_host_alloc(size_t bytes, void **p);
ibtfo_status ibtfo_host_free(void *p);

/* ---------------------------------------------------------------- measurement
 *
 * No reference counterpart.  FP64 pipe rate of the current GPU: a kernel of
 * independent DFMA chains (8 per thread, 8 CTAs of 256 threads per SM,
 * `iters` FMAs per chain) timed with CUDA events after one warm-up launch.
 * *inst_per_s = FP64 thread instructions per second (flops = twice that);
 * *seconds (may be NULL) = the timed launch.  The plain FP64 sweep is bound
 * by this rate, not by HBM bandwidth. */
ibtfo_status ibtfo_fp64_pipe_rate(int iters, double *inst_per_s, double *seconds);
/* y[i] = f(x[i]) on the GPU for n host values (copies in and out), for
 * error-bound tests of the arithmetic the fast precisions use: their
 * reciprocal and square root (Newton-Raphson refinements of the hardware
 * estimates; the FP32 ones take x and return the result as float) and,
 * for comparison, CUDA's IEEE division and square root. */
enum {
    IBTFO_MATH_RCP_F64 = 0,     /* fp64_fast 1/x */
    IBTFO_MATH_SQRT_F64 = 1,    /* fp64_fast sqrt(x) */
    IBTFO_MATH_RCP_F32 = 2,     /* FP32 form 1/x */
    IBTFO_MATH_SQRT_F32 = 3,    /* FP32 form sqrt(x) */
    IBTFO_MATH_DIV_F64 = 4,     /* 1.0 / x, IEEE double division */
    IBTFO_MATH_LIBSQRT_F64 = 5, /* sqrt(x), CUDA's double square root */
    IBTFO_MATH_DIV_F32 = 6,     /* 1.0f / x, IEEE float division */
    IBTFO_MATH_LIBSQRT_F32 = 7  /* sqrtf(x), CUDA's float square root */
};
ibtfo_status ibtfo_fast_math_eval(int fn, const double *x, double *y, int n);

#ifdef __cplusplus
}
#endif
#endif
