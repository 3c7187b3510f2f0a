// Internal data structures shared by the CUDA translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda.h> // CUtensorMap (the tensor maps are encoded through the runtime's driver entry point)
#include <cuda_runtime.h>
#include <string>
#include <vector>

namespace ibtfo {

enum Boundary { BC_REGULAR = 0, BC_IDW = 1, BC_LINEAR = 2, BC_RIEMANNGFM = 3, BC_BCGFM = 4, BC_HBCGFM = 5, BC_CCM = 6 };

// cell types: 0 fluid, 1 solid, 2 ghost-fluid ghost or domain ring; cut-cell
// cases (BC_CCM) also have 3: a cell the body outline crosses
enum { CELL_FLUID = 0, CELL_SOLID = 1, CELL_GHOST = 2, CELL_CUT = 3 };
// cells whose state a sweep advances
__host__ __device__ __forceinline__ bool updated_cell(uint8_t t) { return t == CELL_FLUID || t == CELL_CUT; }
enum GlobalBC { GB_WALLS = 0, GB_PERIODIC = 1 };

// Per-case scalars that live in device memory so that consecutive steps run
// without a host round trip: the dt to apply next, the reference's loop
// accounting (now_t, iter), the ping-pong selector and the reduction state.
struct DevState
{
    double dt;         // dt applied by the next step (ComputeDt of the current state)
    double now_t;      // reference loop time, advanced by the dt computed after each step
    double mass;       // CaculateMass of the current state
    double mass_start; // CaculateMass of the initial state
    unsigned long long amax_bits, umax_bits, vmax_bits; // running maxima (non-negative doubles)
    int iter;          // completed steps
    int cur;           // buffer holding the current state
    int fill_pending;  // a step completed and its boundary pass has not run yet
    int nan_cells;     // fluid cells with a NaN component after the latest step (or reduction)
    int nan_step;      // running count of the launch in progress
    unsigned int ticket;       // blocks finished in the current reduction launch
    int status;                // bit flags, see STATUS_*
    int step_cur;              // ibtfo_step_host: the buffer that held the state when its step began
    double last_amax, last_umax, last_vmax; // maxima behind the latest dt
};

enum { STATUS_NAN = 1, STATUS_STALL = 2 }; // STALL: a bounded wait of a kernel gave up

// One ghost-fluid cell (interior cell of type 2) with everything its fill
// needs, computed once at set-up (reference Scheme_Index).
struct GhostRec
{
    int i, j;
    int idx, idy;   // bracket of the image point (lower-left corner)
    int idx2, idy2; // bracket of the extra point (BCGFM/HBCGFM)
    int pick;       // LinearBaseGFM: chosen corner 1..4, 0 if none is fluid
    int hmirror;    // HBCGFM: |phi| > delta (pure mirror)
    int snext;      // bit c (c + 4): corner c of the image (extra) bracket is an
                    // updated interior cell, read from the new state
    double xm, ym;  // image point
    double xm2, ym2; // extra point
    double w[4];    // inverse-distance weights, corners (idx,idy),(idx,idy+1),(idx+1,idy+1),(idx+1,idy)
    double w2[4];   // extra-point weights
    double nx, ny;  // unnormalised level-set gradient
    double rg;      // |phi|
    double delta;   // half cell diagonal (BCGFM/HBCGFM)
};

// Geometry of the padded grid.  Arrays are structure-of-arrays planes with a
// row pitch (elements) that keeps every row 256-byte aligned.
struct GridDesc
{
    int n_x, n_y, ng, M, N, pitch;
    long long plane; // elements per plane
    double dx, dy;   // update spacings: Psy_L/N_x and Psy_H/N_y
    double Li, Hi;   // coordinate of cell (0,0) centre: x_i = Li + i*dx, y_j = Hi + j*dx
    double gamma, cfl;
    int f32;         // state stored as float (hi, lo) pairs: planes 0-3 hi, 4-7 lo
    // gas constants precomputed on the host (no per-thread divisions):
    // gamma - 1, (gamma+1)/(2 gamma), (gamma-1)/(2 gamma), and their FP32 copies
    double gm1, c1, c2, igm1, ig2; // ..., 1/(gamma - 1), 1/(2 gamma)
    float gf, gm1f, c1f, c2f, igm1f, ig2f;
    // 1/dx, 1/dy, dx*dy and FP32 copies of the reciprocals
    double idx, idy, dxdy;
    float idxf, idyf;
};

// One conserved component of one cell of a state buffer, as a double.  FP64
// states hold four double planes; FP32 compensated states hold eight float
// planes with the same byte size (hi then lo), value = hi + lo.
__device__ __forceinline__ double state_ld(const double *b, int k, long long o, const GridDesc &g)
{
    if (g.f32)
    {
        const float *f = reinterpret_cast<const float *>(b);
        return (double)f[k * g.plane + o] + (double)f[(4 + k) * g.plane + o];
    }
    return b[k * g.plane + o];
}

__device__ __forceinline__ void state_st(double *b, int k, long long o, double v, const GridDesc &g)
{
    if (g.f32)
    {
        float *f = reinterpret_cast<float *>(b);
        const float hi = (float)v;
        f[k * g.plane + o] = hi;
        f[(4 + k) * g.plane + o] = (float)(v - (double)hi);
        return;
    }
    b[k * g.plane + o] = v;
}

struct SweepArgs
{
    GridDesc g;
    double *buf0, *buf1;     // two state buffers, 4 planes each
    const uint8_t *type;     // cell type plane (uint8, same pitch)
    DevState *st;
    double *partial;         // one mass partial per block
    const unsigned *tiles;   // active tiles (bx | by << 16): tiles holding at least one fluid cell
    double t_end;
    int max_iter;
    int guard;               // apply the reference loop condition before stepping
    int stage;               // 0: one step; Time = RK2: 1 the first stage, 2 the second stage and average
    int tile0;               // a step split over several launches: first tile of this launch
    int nblocks;             // ... and the tiles of the whole step (0: one launch, its grid)
    int tma;                 // stage tiles with the tensor maps below (else element-wise loads)
    CUtensorMap tmap[2];     // buf0 / buf1 as (column, row, plane) tensors, box = tile + halo, 4 planes
};

struct FillArgs
{
    GridDesc g;
    double *buf0, *buf1;
    const uint8_t *type;
    DevState *st;
    const GhostRec *ghosts;
    int nghost;
    int bc;          // Boundary variant
    int gb;          // GlobalBC
    int do_ghosts;   // run the ghost-fluid fill
    int do_ring;     // run the domain-edge (Global_Boundary) pass
    int init_mode;   // initial Boundary call: fill without requiring a completed step
    const double *ring_ic; // Regular: initial values feeding the corner columns [2][2*ng][4]
    int pre_flip;    // a step in flight: its output buffer is the one st->step_cur does not name
    int ghost0;      // the ghost records this launch fills start here
};

struct ReduceArgs
{
    GridDesc g;
    const double *u;       // state planes to reduce
    const uint8_t *type;
    DevState *st;
    double *partial;
    int set_start;         // also store mass as mass_start
    const double *alpha;   // cut-cell volume fractions (BC_CCM), else null
};

// ---------------------------------------------------------------- cut cells
//
// Geometry of a cut-cell case (per cell, FP64): volume fraction alpha (fluid
// area / cell area), aperture ax of the X face (i+1/2, j) and ay of the Y face
// (i, j+1/2) (fluid length / face length).  Small cut cells (alpha < 0.5)
// exchange conserved quantities with up to three neighbours after each
// sweep; the exchanges and their participants are compact lists built once.
struct CcmArgs
{
    SweepArgs s;
    const double *alpha, *ax, *ay;
};

struct MixExchange   // E = w (U[t] - U[s]); alpha_s U_s += E, alpha_t U_t -= E
{
    long long s, t;  // cell offsets (j * pitch + i)
    double w;        // beta alpha_s alpha_t / (alpha_s + alpha_t)
};

struct MixParticipant
{
    long long o;     // cell offset
    double inv_alpha;
    int first, count; // its links (exchange index, sign) in the link list
};

struct MixArgs
{
    GridDesc g;
    double *buf0, *buf1;
    DevState *st;
    const MixExchange *ex;
    int nex;
    const MixParticipant *part;
    int npart;
    const int *links; // exchange index * 2 + (1 for the target side)
    double *e;        // exchange values, 4 per exchange
};

typedef void (*CcmLaunch)(const CcmArgs &, dim3 grid, dim3 block, cudaStream_t s);
CcmLaunch ccm_launcher(int scheme, int riemann, int limiter, int precision);
void launch_mix(const MixArgs &a, cudaStream_t s);
// geometry of a cut-cell case from the cell-centred level set: alpha, ax, ay,
// the cell types, and the mixing lists (device arrays allocated here with
// stream-ordered allocation); 0, 2 (allocation) or 5 (CUDA error)
int ccm_setup(const GridDesc &g, const double *d_phi, double *d_alpha, double *d_ax, double *d_ay, uint8_t *d_type,
              MixExchange **d_ex, int *nex, MixParticipant **d_part, int *npart, int **d_links, double **d_e,
              cudaStream_t s);

typedef void (*SweepLaunch)(const SweepArgs &, dim3 grid, dim3 block, cudaStream_t s);

// sweep tile (interior cells per CTA)
constexpr int TILE_X = 32;
constexpr int TILE_Y = 8;
// Rows of the fp64_fast sweep's tiles (not with the PVRS solvers, whose 158
// registers leave room for one 32x8 tile per SM at most): a 32x16 tile solves
// 2.16 faces per cell where a 32x8 tile solves 2.28, and stages 1.41 cells
// per cell, not 1.69.  Every sweep CTA has TILE_X x TILE_Y threads.
constexpr int FAST_TILE_Y = 16;

// A tile-list entry: the tile's column index in bits 0-15, its row index in
// bits 16-30, and TILE_INTERIOR when every cell of the tile and of the
// one-cell ring around it is an interior fluid cell (the sweep then solves
// every face without looking at cell types).
constexpr unsigned TILE_INTERIOR = 0x80000000u;
__host__ __device__ __forceinline__ int tile_ix(unsigned t) { return (int)(t & 0xFFFFu); }
__host__ __device__ __forceinline__ int tile_jy(unsigned t) { return (int)((t >> 16) & 0x7FFFu); }

// the sweep of a configuration over TILE_X x ty tiles (capi.cu)
SweepLaunch sweep_launcher(int scheme, int riemann, int limiter, int precision, int ty);
void launch_fill(const FillArgs &a, cudaStream_t s);
// ghost records [g0, g1) of a step in flight (FillArgs.pre_flip)
void launch_fill_ghosts(const FillArgs &a, int g0, int g1, cudaStream_t s);
void launch_reduce(const ReduceArgs &a, int nblocks_max, cudaStream_t s);
void launch_aos_to_soa(const double *aos, double *soa, const GridDesc &g, cudaStream_t s);
void launch_soa_to_aos(const double *soa, double *aos, const GridDesc &g, cudaStream_t s);
// rows [r0, r1) of the current state buffer (picked on the device by st->cur)
void launch_cur_to_aos_rows(const double *b0, const double *b1, const DevState *st, double *aos, const GridDesc &g,
                            int r0, int r1, cudaStream_t s);
// up to five boxes of array rows [r0, r1) x columns [c0, c1) of one transfer chunk
struct HostBoxes
{
    int n;
    int r0[5], r1[5], c0[5], c1[5];
};
// the boxes from the host-layout array into the current state buffer (and,
// with `both`, into the other buffer too); `first` records st->cur as the
// step's input buffer (st->step_cur)
void launch_aos_to_cur_boxes(const double *aos, double *b0, double *b1, const DevState *st, const GridDesc &g,
                             const HostBoxes &bx, bool first, bool both, cudaStream_t s);
// rows [r0, r1), columns [c0, c1) of a step in flight: fluid and ghost-fluid
// cells from the step's output buffer (the ghost cells of these rows are
// filled by then), the rest from its input (st->step_cur).  `aos` (here and
// below) is a device buffer or a page-locked host array the device writes.
void launch_snapshot_to_aos_rows(const double *b0, const double *b1, const DevState *st, const uint8_t *type,
                                 double *aos, const GridDesc &g, int r0, int r1, int c0, int c1, cudaStream_t s);
// the domain ring of the current buffer into the host-layout array
void launch_ring_to_aos(const double *b0, const double *b1, const DevState *st, double *aos, const GridDesc &g,
                        cudaStream_t s);


// ---------------------------------------------------------------- batches
//
// A batch steps many cases (each with its own grid, geometry, dt and loop
// accounting) with one persistent sweep kernel over a shared tile table and
// one fill kernel per boundary phase.  The kernels take the address of a
// BatchHeader whose device copy the host rewrites (stream-ordered) when
// cases join or leave, so a captured graph of steps stays valid.

// one case of a batch
struct BatchCase
{
    SweepArgs s;  // buffers, cell types, device state, this case's mass partials, t_end, max_iter
    FillArgs f;   // ghost list and domain-edge pass
    int ntiles;   // tiles of this case in the table (the case's block count)
    int slot;
};

// tile table entry: x = tile (bx | by << 16), y = index of the tile within
// its case, z = batch slot
typedef uint4 BatchTile;

struct BatchHeader
{
    const BatchCase *cases;   // indexed by slot
    const BatchTile *tiles;
    const int2 *fill[2];      // (slot, block of the case's fill pass) per boundary phase
    int ntiles;
    int nfill[2];
    int nslots;
};

// progress of one slot, gathered for the host after a chunk of steps
struct BatchProgress
{
    double now_t, dt, mass, mass_start;
    int iter, status, nan_cells, active;
};

// tile shapes of the batched sweep (cells per CTA; 256 threads)
enum BatchShape { SHAPE_32x8 = 0, SHAPE_32x16 = 1, SHAPE_64x8 = 2, SHAPE_COUNT = 3 };
constexpr int shape_tx(int shape) { return shape == SHAPE_64x8 ? 64 : 32; }
constexpr int shape_ty(int shape) { return shape == SHAPE_32x16 ? 16 : 8; }
constexpr int BATCH_THREADS = 256;
// threads of a boundary-pass block: the ghost fill is FP64-heavy and its
// records are few (about one per wall cell), so small blocks spread them
// over every SM
constexpr int FILL_THREADS = 64;
// lanes that fill one ghost record together (one bracket corner each)
constexpr int GHOST_LANES = 4;
constexpr int ghost_blocks(long long n) { return (int)((n * GHOST_LANES + FILL_THREADS - 1) / FILL_THREADS); }

struct BatchKernel
{
    // stage: 0 a whole step; Time = RK2: 1 the first stage, 2 the second
    void (*launch)(const BatchHeader *h, int grid, cudaStream_t s, int stage);
    int (*prepare)(); // sets the shared-memory limit, returns resident CTAs per SM (0 on failure)
};
// precision: 1 = fp64_fast, 2 = FP32 compensated (strict FP64 runs one case per launch)
BatchKernel batch_kernel(int scheme, int riemann, int limiter, int precision, int shape);
void launch_batch_fill(const BatchHeader *h, int phase, int grid, cudaStream_t s);
void launch_batch_progress(const BatchHeader *h, int nslots_max, BatchProgress *out, cudaStream_t s);

// device-side case set-up (bodies.cu); ibtfo_body is declared in ibtfo.h
}
struct ibtfo_body;
namespace ibtfo {
void launch_bodies_phi(const GridDesc &g, const ibtfo_body *d_bodies, int n, double *phi, cudaStream_t s);
void launch_x_split_init(const GridDesc &g, const uint8_t *type, double x_split, const double L[4],
                         const double R[4], double *buf, double *ring_ic, cudaStream_t s);
void launch_density(const GridDesc &g, const double *b0, const double *b1, const DevState *st, double *out,
                    cudaStream_t s);
// output.cu
void launch_vtk_fields(const GridDesc &g, const double *b0, const double *b1, const DevState *st,
                       const uint8_t *type, float *out, double *now_t, cudaStream_t s);
int write_vtk_file(const char *path, const GridDesc &g, double lo_x, double lo_y, double Psy_L, double Psy_H,
                   double now_t, const float *fields, int binary);
struct VtkWriter;
VtkWriter *vtk_writer_create(int device, const GridDesc &g, cudaStream_t s);
int vtk_writer_submit(VtkWriter *w, const GridDesc &g, const double *b0, const double *b1, const DevState *st,
                      const uint8_t *type, cudaStream_t s, const char *path, int binary, double lo_x, double lo_y,
                      double Psy_L, double Psy_H, std::string *why);
int vtk_writer_wait(VtkWriter *w, std::string *why);
void vtk_writer_destroy(VtkWriter *w, cudaStream_t s);

// geometry set-up (geometry.cu)
// the tiles of TILE_X x ty cells holding fluid cells, on the device and (host_list) on the host
int active_tiles(const GridDesc &g, const uint8_t *d_type, int ty, unsigned **d_tiles, int *ntiles, cudaStream_t s,
                 std::vector<unsigned> *host_list = nullptr, bool row_order = false);
// host list of the tx x ty tiles holding at least one fluid cell (bx | by << 16,
// with TILE_INTERIOR where it applies): 32x16 tiles longest first unless
// row_order, others in row order;
// 0, or 2 (allocation) / 5 (CUDA error)
int active_tile_list(const GridDesc &g, const uint8_t *d_type, int tx, int ty, std::vector<unsigned> &list,
                     cudaStream_t s, bool row_order = false);
int setup_geometry(const GridDesc &g, int bc, const double *d_phi, double *d_nx, double *d_ny, uint8_t *d_type,
                   GhostRec **d_ghosts, int *nghost, cudaStream_t s);

// kernel launch counter (every launch made by the library)
void count_launch(int n = 1);

} // namespace ibtfo

// operations on a case used by the reference-signature entry points
struct ibtfo_case;
namespace ibtfo {
int case_set_gas(ibtfo_case *c, double gamma, double cfl);       // 0 or an ibtfo_status
int case_set_dt(ibtfo_case *c, double dt);
int case_sweep_unguarded(ibtfo_case *c);
int case_fill(ibtfo_case *c, int ghosts, int ring);
int case_reduce_current(ibtfo_case *c);
double case_cfl(const ibtfo_case *c);
// batch view of a case: its sweep/fill arguments and the arguments of the batch kernel variant
int case_batch_view(ibtfo_case *c, SweepArgs *s, FillArgs *f, int *scheme, int *riemann, int *limiter,
                    int *precision, int *has_state);
cudaStream_t case_stream(const ibtfo_case *c);
int case_time_advance(const ibtfo_case *c);
int case_write_vtk_at(ibtfo_case *c, const char *path, double now_t); // ASCII, TIME field = now_t
int case_device(const ibtfo_case *c);
double case_gamma(const ibtfo_case *c);
void set_last_error(const char *msg);

} // namespace ibtfo
