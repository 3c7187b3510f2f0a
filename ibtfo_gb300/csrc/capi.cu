// C ABI (include/ibtfo.h): case lifetime, host transfers, step orchestration.
//
// A step is two launches on the case's stream: the fused sweep (which also
// produces the next dt, the mass and the loop accounting in device memory)
// and the boundary pass.  Because dt and the loop condition live on the
// device, ibtfo_advance queues any number of steps without a host round trip;
// chunks of steps are captured once into a CUDA graph and replayed.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ibtfo.h"
#include "internal.h"
#include "physics.cuh"

namespace ibtfo {
SweepLaunch sweep_launcher_muscl(int riemann, int limiter);
SweepLaunch sweep_launcher_mhm(int riemann, int limiter);
SweepLaunch sweep_launcher_godunov(int riemann, int limiter);
SweepLaunch sweep_launcher_muscl_fast(int riemann, int limiter, int ty);
SweepLaunch sweep_launcher_mhm_fast(int riemann, int limiter, int ty);
SweepLaunch sweep_launcher_godunov_fast(int riemann, int limiter, int ty);
SweepLaunch sweep_launcher_muscl_f32(int riemann, int limiter, int ty);
SweepLaunch sweep_launcher_mhm_f32(int riemann, int limiter, int ty);
SweepLaunch sweep_launcher_godunov_f32(int riemann, int limiter, int ty);
SweepLaunch sweep_launcher_lax();

// the sweep of a case's configuration over TILE_X x ty tiles (ty = TILE_Y,
// or FAST_TILE_Y for the fp64_fast sweeps without PVRS and the FP32 sweeps)
SweepLaunch sweep_launcher(int scheme, int riemann, int limiter, int precision, int ty)
{
    const int r = (riemann == HLLC) ? HLL : riemann; // HLLC/Riemann_solver.cpp is HLL
    const bool fast = (precision == IBTFO_PRECISION_FP64_FAST);
    if (scheme == LAX)
        return sweep_launcher_lax(); // strict FP64 for both FP64 keys
    if (precision == IBTFO_PRECISION_FP32_COMPENSATED)
    {
        switch (scheme)
        {
        case MHM: return sweep_launcher_mhm_f32(r, limiter, ty);
        case GODUNOV: return sweep_launcher_godunov_f32(r, limiter, ty);
        default: return sweep_launcher_muscl_f32(r, limiter, ty);
        }
    }
    switch (scheme)
    {
    case MHM: return fast ? sweep_launcher_mhm_fast(r, limiter, ty) : sweep_launcher_mhm(r, limiter);
    case GODUNOV: return fast ? sweep_launcher_godunov_fast(r, limiter, ty) : sweep_launcher_godunov(r, limiter);
    default: return fast ? sweep_launcher_muscl_fast(r, limiter, ty) : sweep_launcher_muscl(r, limiter);
    }
}

static std::atomic<long long> g_launches{0};
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
} // namespace ibtfo

using namespace ibtfo;

static thread_local std::string g_err;

static ibtfo_status fail(ibtfo_status s, const std::string &msg)
{
    g_err = msg;
    return s;
}

static ibtfo_status cuda_fail(cudaError_t e, const char *what)
{
    return fail(IBTFO_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace ibtfo {
void set_last_error(const char *msg) { g_err = msg; }
} // namespace ibtfo

#define CK(call)                                      \
    do                                                \
    {                                                 \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess)                        \
            return cuda_fail(e_, #call);              \
    } while (0)

static void set_derived_constants(GridDesc &g)
{
    g.gm1 = g.gamma - 1;
    g.c1 = (g.gamma + 1) / (2 * g.gamma);
    g.c2 = (g.gamma - 1) / (2 * g.gamma);
    g.gf = (float)g.gamma;
    g.gm1f = (float)g.gm1;
    g.c1f = (float)g.c1;
    g.c2f = (float)g.c2;
    g.igm1 = 1.0 / g.gm1;
    g.ig2 = 1.0 / (2 * g.gamma);
    g.igm1f = (float)g.igm1;
    g.ig2f = (float)g.ig2;
    g.idx = 1.0 / g.dx;
    g.idy = 1.0 / g.dy;
    g.dxdy = g.dx * g.dy;
    g.idxf = (float)g.idx;
    g.idyf = (float)g.idy;
}

static constexpr int NBANDS = 8; // row bands of ibtfo_step_host
static constexpr int NSW = 4;    // streams the bands' sweeps alternate on
static constexpr int NFIN = 4;   // streams the bands' finishing work alternates on

struct ibtfo_case
{
    ibtfo_config cfg;
    GridDesc g;
    int device = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    double *buf[2] = {nullptr, nullptr};
    double *ic = nullptr;      // Regular: initial state (U_NEW's never-written cells)
    double *staging = nullptr; // M*N*4 doubles, array-of-structures transfers
    double *phi = nullptr, *nx = nullptr, *ny = nullptr;
    uint8_t *type = nullptr;
    GhostRec *ghosts = nullptr;
    int nghost = 0;
    DevState *st = nullptr;
    double *partial = nullptr;
    double *ring_ic = nullptr; // [2][2*ng][4]
    int tma = 0;                // tensor maps of buf[0], buf[1] below are valid
    CUtensorMap tmap[2];        // boxes of TILE_X x tile_y cells and their halo
    unsigned *tiles = nullptr;  // active sweep tiles (TILE_X x tile_y)
    int ntiles = 0;
    // the same tiles in row order: the row bands of the host-array step
    unsigned *band_list = nullptr;
    int nband_list = 0;
    // cut cells (BC_CCM): volume fractions, apertures, small-cell mixing lists
    double *alpha = nullptr, *ax = nullptr, *ay = nullptr;
    MixExchange *mix_ex = nullptr;
    MixParticipant *mix_part = nullptr;
    int *mix_links = nullptr;
    double *mix_e = nullptr;
    int nex = 0, npart = 0;
    CcmLaunch ccm = nullptr;
    int nblocks = 0;
    bool geometry = false, state = false;
    SweepLaunch sweep = nullptr;
    int tile_y = TILE_Y; // rows of the sweep's tiles (TILE_X columns)
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    long long graph_launches = 0; // kernel launches in one replay of the graph
    VtkWriter *vtk = nullptr;     // asynchronous VTK output, created on first use
    // ibtfo_step_host: row bands of the pipelined host-buffer step
    std::vector<int> band_rows;   // NBANDS + 1 array-row offsets of the host-to-device chunks
    std::vector<int> out_rows;    // NBANDS + 1 array-row offsets of the device-to-host chunks
    std::vector<int> band_tiles;  // NBANDS + 1 offsets into the active-tile list
    std::vector<int> fluid_cols;  // 2 NBANDS: columns [c0, c1) holding the fluid cells of each band
    std::vector<HostBoxes> in_boxes; // NBANDS: the cells of each chunk an in-place step reads
    // the host array of the last in-place ibtfo_step_host: the cells outside
    // in_boxes hold in both state buffers what they hold there
    const double *mirror_in = nullptr;
    std::vector<int> band_ghosts; // NBANDS + 1 offsets into the ghost list (rows of each band)
    std::vector<int> ghost_ready; // NBANDS: the last band whose fluid cells the band's ghost fills read
    // copies (h2d, d2h), band sweeps (sw), and at the highest priority the
    // short kernels the bands wait on: conversions in (conv) and each band's
    // ghost fill and conversion out (fin), whose blocks then take the next
    // free SM slot ahead of the sweeps' pending tiles
    cudaStream_t h2d = nullptr, d2h = nullptr, sw[NSW] = {}, fin[NFIN] = {}, conv = nullptr;
    cudaEvent_t ev_in[NBANDS] = {}, ev_conv[NBANDS] = {}, ev_out[NBANDS] = {}, ev_swept[NBANDS] = {},
                ev_sw[NSW] = {}, ev_fin[NFIN] = {}, ev_done = nullptr, ev_cv = nullptr;
    // the banded step captured as a CUDA graph for one pair of page-locked host arrays
    cudaGraphExec_t host_graph = nullptr;
    const double *host_graph_in = nullptr;
    double *host_graph_out = nullptr;
    long long host_graph_launches = 0;
};

// the streams of ibtfo_step_host besides the case's own
static std::array<cudaStream_t, 3 + NSW + NFIN> helper_streams(const ibtfo_case *c)
{
    std::array<cudaStream_t, 3 + NSW + NFIN> a;
    a[0] = c->h2d, a[1] = c->d2h, a[2] = c->conv;
    for (int q = 0; q < NSW; q++)
        a[3 + q] = c->sw[q];
    for (int q = 0; q < NFIN; q++)
        a[3 + NSW + q] = c->fin[q];
    return a;
}

// graphs embed the case's kernel arguments and buffers: dropped whenever those change
static void drop_graphs(ibtfo_case *c)
{
    if (c->graph)
    {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
        c->graph_steps = 0;
    }
    if (c->host_graph)
    {
        cudaGraphExecDestroy(c->host_graph);
        c->host_graph = nullptr;
        c->host_graph_in = nullptr;
        c->host_graph_out = nullptr;
    }
}

// Row bands of ibtfo_step_host.  Band k sweeps the active tiles whose tile
// row lies in [k*nty/NB, (k+1)*nty/NB); its transfer chunk ends at the last
// array row that band's stencil reads (two rows above its tiles), so band k
// can start once chunks 0..k are on the device.
static void make_bands(ibtfo_case *c, const std::vector<unsigned> &tiles)
{
    const GridDesc &g = c->g;
    const int nty = (g.n_y + c->tile_y - 1) / c->tile_y;
    c->band_rows.assign(NBANDS + 1, 0);
    c->out_rows.assign(NBANDS + 1, 0);
    c->band_tiles.assign(NBANDS + 1, 0);
    c->fluid_cols.assign(2 * NBANDS, 0);
    size_t t = 0;
    for (int k = 1; k <= NBANDS; k++)
    {
        // the first and the last band half as tall as the others: the
        // pipeline waits for the first chunk alone and drains the last one alone
        const int tb = (k == NBANDS) ? nty : (int)((long long)(2 * k - 1) * nty / (2 * NBANDS - 2));
        c->band_rows[k] = (k == NBANDS) ? g.N : std::min(g.N, g.ng + tb * c->tile_y + 2);
        c->out_rows[k] = (k == NBANDS) ? g.N : std::min(g.N, g.ng + tb * c->tile_y);
        while (t < tiles.size() && tile_jy(tiles[t]) < tb)
            t++;
        c->band_tiles[k] = (k == NBANDS) ? (int)tiles.size() : (int)t;
    }
    // the columns of each band's active tiles (tiles without fluid cells are not listed)
    for (int k = 0; k < NBANDS; k++)
    {
        int lo = g.M, hi = 0;
        for (int q = c->band_tiles[k]; q < c->band_tiles[k + 1]; q++)
        {
            const int tx = tile_ix(tiles[q]);
            lo = std::min(lo, g.ng + tx * TILE_X);
            hi = std::max(hi, std::min(g.ng + g.n_x, g.ng + (tx + 1) * TILE_X));
        }
        c->fluid_cols[2 * k] = lo < hi ? lo : 0;
        c->fluid_cols[2 * k + 1] = lo < hi ? hi : 0;
    }
}

// Ghost records by band: the records of each band's rows (the list is in
// row order), the last band whose fluid cells their fills read (the image
// and extra points' bracket rows), and the columns they add to the band's
// copy box.
static void make_ghost_bands(ibtfo_case *c, const std::vector<GhostRec> &gl)
{
    const GridDesc &g = c->g;
    auto band_of_row = [&](int j) {
        int k = 0;
        while (k + 1 < NBANDS && j >= c->out_rows[k + 1])
            k++;
        return k;
    };
    c->band_ghosts.assign(NBANDS + 1, (int)gl.size());
    c->ghost_ready.assign(NBANDS, 0);
    size_t t = 0;
    for (int k = 0; k < NBANDS; k++)
    {
        c->band_ghosts[k] = (int)t;
        int ready = k;
        while (t < gl.size() && gl[t].j < c->out_rows[k + 1])
        {
            const GhostRec &r = gl[t];
            ready = std::max(ready, band_of_row(std::min(g.N - 1, r.idy + 1)));
            if (c->cfg.boundary == IBTFO_BOUNDARY_BCGFM || c->cfg.boundary == IBTFO_BOUNDARY_HBCGFM)
                ready = std::max(ready, band_of_row(std::min(g.N - 1, r.idy2 + 1)));
            int &lo = c->fluid_cols[2 * k], &hi = c->fluid_cols[2 * k + 1];
            if (lo >= hi)
                lo = r.i, hi = r.i + 1;
            else
                lo = std::min(lo, r.i), hi = std::max(hi, r.i + 1);
            t++;
        }
        c->ghost_ready[k] = ready;
    }
    c->band_ghosts[NBANDS] = (int)gl.size();
}

// Copy-in boxes of an in-place ibtfo_step_host, per transfer chunk: the
// cells some part of the step reads or copies back.  Those are the staged
// box of every active tile (the tile and two cells around it: the widest
// reconstruction stencil), the band's copy-back columns (fluid and ghost
// cells, whose rows' other cells go back from the input), and the domain
// edge: 2 ng rows and columns at each side, the ring and the cells its fill
// copies.  Per chunk: whole edge rows, and over the other rows the union of
// their columns with the two edge strips (at most five boxes).  Solid cells
// away from the fluid and the edge are neither read nor written by a step.
static void make_in_boxes(ibtfo_case *c, const std::vector<unsigned> &tiles)
{
    const GridDesc &g = c->g;
    std::vector<int> lo(g.N, g.M), hi(g.N, 0);
    auto add = [&](int j0, int j1, int i0, int i1) {
        j0 = std::max(j0, 0);
        j1 = std::min(j1, g.N);
        i0 = std::max(i0, 0);
        i1 = std::min(i1, g.M);
        if (i0 >= i1)
            return;
        for (int j = j0; j < j1; j++)
        {
            lo[j] = std::min(lo[j], i0);
            hi[j] = std::max(hi[j], i1);
        }
    };
    const int halo = std::max(2, g.ng);
    for (unsigned t : tiles)
    {
        const int i0 = g.ng + tile_ix(t) * TILE_X, j0 = g.ng + tile_jy(t) * c->tile_y;
        add(j0 - halo, j0 + c->tile_y + halo, i0 - halo, i0 + TILE_X + halo);
    }
    for (int k = 0; k < NBANDS; k++)
        add(std::max(c->out_rows[k], g.ng), std::min(c->out_rows[k + 1], g.ng + g.n_y), c->fluid_cols[2 * k],
            c->fluid_cols[2 * k + 1]);
    const int e = 2 * g.ng, bottom = std::max(e, g.N - e);
    c->in_boxes.assign(NBANDS, HostBoxes{});
    for (int k = 0; k < NBANDS; k++)
    {
        HostBoxes &b = c->in_boxes[k];
        auto push = [&](int r0, int r1, int c0, int c1) {
            if (r1 > r0 && c1 > c0)
            {
                b.r0[b.n] = r0, b.r1[b.n] = r1, b.c0[b.n] = c0, b.c1[b.n] = c1;
                b.n++;
            }
        };
        const int r0 = c->band_rows[k], r1 = c->band_rows[k + 1];
        push(r0, std::min(r1, e), 0, g.M);
        const int a = std::max(r0, e), z = std::min(r1, bottom);
        if (a < z)
        {
            int clo = g.M, chi = 0;
            for (int j = a; j < z; j++)
                if (lo[j] < hi[j])
                    clo = std::min(clo, lo[j]), chi = std::max(chi, hi[j]);
            // [0, e), [clo, chi), [M - e, M) in column order, overlaps merged
            int iv[3][2] = {{0, e}, {clo, chi}, {g.M - e, g.M}};
            int n = 0, m[3][2];
            for (auto &v : iv)
            {
                if (v[0] >= v[1])
                    continue;
                if (n && v[0] <= m[n - 1][1])
                    m[n - 1][1] = std::max(m[n - 1][1], v[1]);
                else
                    m[n][0] = v[0], m[n][1] = v[1], n++;
            }
            for (int q = 0; q < n; q++)
                push(a, z, m[q][0], m[q][1]);
        }
        push(std::max(r0, bottom), r1, 0, g.M);
    }
}

// The device-side address of a page-locked host array the kernels can write
// directly, or null (pageable memory, or no mapping).
static double *device_view(double *host)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? static_cast<double *>(at.devicePointer) : nullptr;
}

// The domain ring of the current state into u_out: converted to the host
// layout on stream ks and copied on cs (two runs of whole rows and two
// strided runs of the side columns), or, with zc (u_out's device view),
// written into the host array by the conversion kernel itself, after the row
// copies queued on the second copy stream when those cover the ring (full
// rows back: their ring cells are stale).
static ibtfo_status ring_to_host(ibtfo_case *c, double *u_out, cudaStream_t ks, cudaStream_t cs, double *zc,
                                 bool after_rows)
{
    const GridDesc &g = c->g;
    const size_t row = sizeof(double) * 4 * (size_t)g.M, cell = sizeof(double) * 4;
    if (zc)
    {
        if (after_rows)
        {
            CK(cudaEventRecord(c->ev_done, c->d2h));
            CK(cudaStreamWaitEvent(ks, c->ev_done, 0));
        }
        launch_ring_to_aos(c->buf[0], c->buf[1], c->st, zc, g, ks);
        return IBTFO_OK;
    }
    launch_ring_to_aos(c->buf[0], c->buf[1], c->st, c->staging, g, ks);
    if (cs != ks)
    {
        CK(cudaEventRecord(c->ev_done, ks));
        CK(cudaStreamWaitEvent(cs, c->ev_done, 0));
    }
    const size_t top = (size_t)(g.ng + g.n_y) * g.M * 4, side = (size_t)g.ng * g.M * 4;
    CK(cudaMemcpyAsync(u_out, c->staging, row * g.ng, cudaMemcpyDeviceToHost, cs));
    CK(cudaMemcpyAsync(u_out + top, c->staging + top, row * g.ng, cudaMemcpyDeviceToHost, cs));
    CK(cudaMemcpy2DAsync(u_out + side, row, c->staging + side, row, cell * g.ng, g.n_y, cudaMemcpyDeviceToHost, cs));
    const size_t right = side + (size_t)(g.ng + g.n_x) * 4;
    CK(cudaMemcpy2DAsync(u_out + right, row, c->staging + right, row, cell * g.ng, g.n_y, cudaMemcpyDeviceToHost,
                         cs));
    return IBTFO_OK;
}

// Tensor maps of the two state buffers for the sweeps' bulk tensor copies:
// (column, row, plane) with the row pitch and plane stride of the buffers,
// box = a 32x8 tile plus its two-cell halo over the four planes (FP64, or
// the FP32 form's hi planes).  A box starts at column i0 - 2 = 32 k + ng - 2,
// so the copies need ng == 2 for their 16-byte start alignment; other
// ghost widths keep the element-wise staging.  0 when not available.
static int make_state_tmaps(ibtfo_case *c)
{
    const GridDesc &g = c->g;
    if (g.ng != 2)
        return 0;
    typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                     const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                     CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeTiled encode = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<EncodeTiled>(fn);
        cudaGetLastError();
    });
    if (!encode)
        return 0;
    const bool f32 = g.f32 != 0;
    const cuuint64_t elem = f32 ? sizeof(float) : sizeof(double);
    // FP32 form: all eight planes (hi 0-3, lo 4-7); a box covers four of them
    const cuuint64_t dims[3] = {(cuuint64_t)g.M, (cuuint64_t)g.N, (cuuint64_t)(f32 ? 8 : 4)};
    const cuuint64_t strides[2] = {(cuuint64_t)g.pitch * elem, (cuuint64_t)g.plane * elem};
    const cuuint32_t estr[3] = {1, 1, 1};
    const cuuint32_t box[3] = {TILE_X + 4, (cuuint32_t)c->tile_y + 4, 4};
    for (int b = 0; b < 2; b++)
        if (encode(&c->tmap[b], f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, c->buf[b],
                   dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return 0;
    return 1;
}

// Case buffers come from the device's stream-ordered pool; freed memory stays
// in the pool (no release threshold) so that cases created and destroyed
// while others run reuse it without device-wide synchronisation.
static void retain_pool_memory(int device)
{
    static std::mutex mu;
    static std::vector<int> done;
    std::lock_guard<std::mutex> lk(mu);
    for (int d : done)
        if (d == device)
            return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess)
    {
        uint64_t thr = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    done.push_back(device);
}

extern "C" {
static ibtfo_status geometry_from_phi(ibtfo_case *c);
static ibtfo_status finish_initial_state(ibtfo_case *c);
}

// the array-of-structures staging buffer of host transfers, allocated on first use
static cudaError_t ensure_staging(ibtfo_case *c)
{
    if (c->staging)
        return cudaSuccess;
    const size_t cells = (size_t)c->g.M * c->g.N;
    return cudaMallocAsync(&c->staging, sizeof(double) * 4 * cells, c->stream);
}

static int nsch_of(int bc)
{
    switch (bc)
    {
    case BC_IDW: return 8;
    case BC_LINEAR:
    case BC_RIEMANNGFM: return 4;
    case BC_BCGFM:
    case BC_HBCGFM: return 16;
    default: return 1;
    }
}

extern "C" {

int ibtfo_abi_version(void) { return IBTFO_ABI_VERSION; }
const char *ibtfo_last_error(void) { return g_err.c_str(); }
long long ibtfo_launch_count(void) { return g_launches.load(); }

ibtfo_status ibtfo_destroy(ibtfo_case *c)
{
    if (!c)
        return IBTFO_OK;
    cudaSetDevice(c->device);
    if (c->stream)
        cudaStreamSynchronize(c->stream);
    drop_graphs(c);
    vtk_writer_destroy(c->vtk, c->own ? c->own : c->stream);
    for (cudaStream_t s : helper_streams(c))
        if (s)
        {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    for (int k = 0; k < NBANDS; k++)
        for (cudaEvent_t e : {c->ev_in[k], c->ev_conv[k], c->ev_out[k], c->ev_swept[k]})
            if (e)
                cudaEventDestroy(e);
    for (cudaEvent_t e : c->ev_sw)
        if (e)
            cudaEventDestroy(e);
    for (cudaEvent_t e : c->ev_fin)
        if (e)
            cudaEventDestroy(e);
    for (cudaEvent_t e : {c->ev_done, c->ev_cv})
        if (e)
            cudaEventDestroy(e);
    // stream-ordered frees: the memory returns to the device pool without a
    // device-wide synchronisation (other cases keep running)
    cudaStream_t fs = c->own ? c->own : c->stream;
    void *bufs[] = {c->buf[0], c->buf[1], c->ic, c->staging, c->phi, c->nx, c->ny, c->type, c->ghosts,
                    c->st, c->partial, c->ring_ic, c->tiles, c->band_list, c->alpha, c->ax, c->ay, c->mix_ex, c->mix_part,
                    c->mix_links, c->mix_e};
    for (void *p : bufs)
        if (p)
            cudaFreeAsync(p, fs);
    if (c->own)
    {
        cudaStreamSynchronize(c->own);
        cudaStreamDestroy(c->own);
    }
    delete c;
    return IBTFO_OK;
}

ibtfo_status ibtfo_create(const ibtfo_config *cfg, ibtfo_case **out)
{
    if (!cfg || !out)
        return fail(IBTFO_EINVAL, "null argument");
    *out = nullptr;
    const ibtfo_config &k = *cfg;
    if (k.n_x < 2 || k.n_y < 2 || k.num_ghost_cell < 2 || k.num_ghost_cell > 64)
        return fail(IBTFO_EINVAL, "need n_x, n_y >= 2 and 2 <= num_ghost_cell <= 64");
    if (k.n_x > 262144 || k.n_y > 262144 || (long long)(k.n_x + 2 * k.num_ghost_cell) * (k.n_y + 2 * k.num_ghost_cell) > (1LL << 31))
        return fail(IBTFO_EINVAL, "grid too large (n_x, n_y <= 262144 and at most 2^31 cells)");
    if (!(k.hi_x > k.lo_x) || !(k.hi_y > k.lo_y) || !(k.gamma > 1.0) || !(k.cfl_number > 0.0))
        return fail(IBTFO_EINVAL, "need hi > lo, gamma > 1, cfl_number > 0");
    if (k.scheme < 0 || k.scheme > 3 || k.riemann < 0 || k.riemann > 5 || k.limiter < 0 || k.limiter > 1 ||
        k.boundary < 0 || k.boundary > 6 || k.global_boundary < 0 || k.global_boundary > 1 || k.precision < 0 ||
        k.precision > 2 || k.time_advance < 0 || k.time_advance > 1)
        return fail(IBTFO_EINVAL, "unknown scheme/riemann/limiter/boundary/global_boundary/precision/time key");
    if (k.scheme == IBTFO_SCHEME_LAX &&
        (k.precision == IBTFO_PRECISION_FP32_COMPENSATED || k.boundary == IBTFO_BOUNDARY_CCM))
        return fail(IBTFO_EINVAL, "Scheme = Lax runs in the FP64 precisions without cut cells");
    if (k.time_advance == IBTFO_TIME_RK2 && k.boundary == IBTFO_BOUNDARY_CCM)
        return fail(IBTFO_EINVAL, "Time = RK2 runs without cut cells");
    if (k.precision == IBTFO_PRECISION_FP32_COMPENSATED && k.riemann == IBTFO_RIEMANN_PVRS)
        return fail(IBTFO_EINVAL, "PVRS is available in the FP64 precisions only");
    if (k.boundary == IBTFO_BOUNDARY_CCM && k.riemann != IBTFO_RIEMANN_HLL_TORO &&
        k.riemann != IBTFO_RIEMANN_STEGER_WARMING && k.riemann != IBTFO_RIEMANN_HLLC_TORO)
        return fail(IBTFO_EINVAL, "the cut-cell method runs HLL_Toro, StegerWarming or HLLC_Toro (the reference's "
                                  "HLL and PVRS have no cut-cell form)");
    if (k.global_boundary == IBTFO_GLOBAL_PERIODIC && (k.n_x < k.num_ghost_cell || k.n_y < k.num_ghost_cell))
        return fail(IBTFO_EINVAL, "periodic boundaries need n_x, n_y >= num_ghost_cell");

    ibtfo_case *c = new ibtfo_case();
    c->cfg = k;
    cudaGetDevice(&c->device);
    GridDesc &g = c->g;
    g.n_x = k.n_x;
    g.n_y = k.n_y;
    g.ng = k.num_ghost_cell;
    g.M = k.n_x + 2 * g.ng;
    g.N = k.n_y + 2 * g.ng;
    g.pitch = (g.M + 31) / 32 * 32;
    g.plane = (long long)g.pitch * g.N;
    const double Psy_L = k.hi_x - k.lo_x, Psy_H = k.hi_y - k.lo_y;
    g.dx = Psy_L / k.n_x; // MUSCL_Scheme.cpp:20 and Psy_coord.cpp:29
    g.dy = Psy_H / k.n_y; // MUSCL_Scheme.cpp:21
    g.Li = -g.dx * g.ng + k.lo_x + g.dx / 2; // Psy_coord.cpp:33-34 (dy := dx there)
    g.Hi = -g.dx * g.ng + k.lo_y + g.dx / 2;
    g.gamma = k.gamma;
    g.cfl = k.cfl_number;
    g.f32 = (k.precision == IBTFO_PRECISION_FP32_COMPENSATED) ? 1 : 0;
    set_derived_constants(g);
    c->nblocks = ((k.n_x + TILE_X - 1) / TILE_X) * ((k.n_y + TILE_Y - 1) / TILE_Y);
    // rows per tile: the fp64_fast and FP32 sweeps and the FP32 cut-cell sweep
    // run 32 x FAST_TILE_Y tiles, except with PVRS; Lax, the strict form and
    // the FP64 cut-cell sweeps 32x8 (ccm_tile_rows in csrc/ccm_impl.cuh)
    const bool ccm = k.boundary == IBTFO_BOUNDARY_CCM;
    const bool f32 = k.precision == IBTFO_PRECISION_FP32_COMPENSATED;
    c->tile_y = ((k.precision == IBTFO_PRECISION_FP64_FAST && !ccm) || f32) && k.scheme != IBTFO_SCHEME_LAX &&
                        k.riemann != IBTFO_RIEMANN_PVRS
                    ? FAST_TILE_Y
                    : TILE_Y;
    c->sweep = sweep_launcher(k.scheme, k.riemann, k.limiter, k.precision, c->tile_y);
    if (k.boundary == IBTFO_BOUNDARY_CCM)
        c->ccm = ccm_launcher(k.scheme, k.riemann, k.limiter, k.precision);

    const size_t plane_bytes = sizeof(double) * (size_t)g.plane;
    retain_pool_memory(c->device);
    cudaError_t e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
    auto A = [&](void **p, size_t bytes) {
        if (e == cudaSuccess)
            e = cudaMallocAsync(p, bytes, c->own);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(*p, 0, bytes, c->own);
    };
    A((void **)&c->buf[0], 4 * plane_bytes);
    A((void **)&c->buf[1], 4 * plane_bytes);
    if (k.boundary == IBTFO_BOUNDARY_REGULAR)
        A((void **)&c->ic, 4 * plane_bytes);
    A((void **)&c->phi, plane_bytes);
    A((void **)&c->nx, plane_bytes);
    A((void **)&c->ny, plane_bytes);
    A((void **)&c->type, (size_t)g.plane);
    A((void **)&c->st, sizeof(DevState));
    A((void **)&c->partial, sizeof(double) * (size_t)c->nblocks);
    A((void **)&c->ring_ic, sizeof(double) * 2 * 2 * g.ng * 4);
    if (k.boundary == IBTFO_BOUNDARY_CCM)
    {
        A((void **)&c->alpha, plane_bytes);
        A((void **)&c->ax, plane_bytes);
        A((void **)&c->ay, plane_bytes);
    }
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->own);
    if (e != cudaSuccess)
    {
        ibtfo_status s = (e == cudaErrorMemoryAllocation) ? fail(IBTFO_ENOMEM, "device allocation failed")
                                                          : cuda_fail(e, "ibtfo_create");
        cudaGetLastError();
        ibtfo_destroy(c);
        return s;
    }
    c->stream = c->own;
    c->tma = make_state_tmaps(c);
    *out = c;
    return IBTFO_OK;
}

ibtfo_status ibtfo_set_stream(ibtfo_case *c, void *stream)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null case");
    cudaSetDevice(c->device);
    CK(cudaStreamSynchronize(c->stream));
    c->stream = stream ? (cudaStream_t)stream : c->own;
    drop_graphs(c);
    return IBTFO_OK;
}

int ibtfo_num_sch(const ibtfo_case *c) { return c ? nsch_of(c->cfg.boundary) : 0; }
int ibtfo_num_ghost_cells(const ibtfo_case *c) { return c ? c->nghost : 0; }

ibtfo_status ibtfo_setup_geometry(ibtfo_case *c, const double *phi)
{
    if (!c || !phi)
        return fail(IBTFO_EINVAL, "null argument");
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    if (!c->phi)
        return fail(IBTFO_ESTATE, "the geometry arrays were released (ibtfo_release_geometry)");
    CK(cudaMemcpy2DAsync(c->phi, sizeof(double) * g.pitch, phi, sizeof(double) * g.M, sizeof(double) * g.M, g.N,
                         cudaMemcpyHostToDevice, c->stream));
    return geometry_from_phi(c);
}

// normals, cell types, ghost list and tiles from the level set in c->phi
static ibtfo_status geometry_from_phi(ibtfo_case *c)
{
    const GridDesc &g = c->g;
    if (c->ghosts)
    {
        cudaFreeAsync(c->ghosts, c->stream);
        c->ghosts = nullptr;
        c->nghost = 0;
    }
    int rc;
    if (c->cfg.boundary == IBTFO_BOUNDARY_CCM)
    {
        void *old[] = {c->mix_ex, c->mix_part, c->mix_links, c->mix_e};
        for (void *p : old)
            if (p)
                cudaFreeAsync(p, c->stream);
        c->mix_ex = nullptr;
        c->mix_part = nullptr;
        c->mix_links = nullptr;
        c->mix_e = nullptr;
        rc = ccm_setup(g, c->phi, c->alpha, c->ax, c->ay, c->type, &c->mix_ex, &c->nex, &c->mix_part, &c->npart,
                       &c->mix_links, &c->mix_e, c->stream);
    }
    else
        rc = setup_geometry(g, c->cfg.boundary, c->phi, c->nx, c->ny, c->type, &c->ghosts, &c->nghost, c->stream);
    std::vector<unsigned> tile_list;
    if (rc == 0)
        rc = active_tiles(g, c->type, c->tile_y, &c->band_list, &c->nband_list, c->stream, &tile_list, true);
    if (rc == 0)
        rc = active_tiles(g, c->type, c->tile_y, &c->tiles, &c->ntiles, c->stream);
    if (rc == 0)
    {
        make_bands(c, tile_list);
        std::vector<GhostRec> gl(c->nghost);
        if (c->nghost && (cudaMemcpyAsync(gl.data(), c->ghosts, sizeof(GhostRec) * c->nghost, cudaMemcpyDeviceToHost,
                                          c->stream) != cudaSuccess ||
                          cudaStreamSynchronize(c->stream) != cudaSuccess))
            rc = 5;
        make_ghost_bands(c, gl);
        make_in_boxes(c, tile_list);
        c->mirror_in = nullptr;
    }
    if (rc == 2)
        return fail(IBTFO_ENOMEM, "geometry allocation failed");
    if (rc != 0)
        return cuda_fail(cudaGetLastError(), "geometry set-up");
    drop_graphs(c);
    CK(cudaStreamSynchronize(c->stream));
    c->geometry = true;
    c->state = false;
    return IBTFO_OK;
}

ibtfo_status ibtfo_get_geometry(ibtfo_case *c, double *xy)
{
    if (!c || !xy)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->geometry)
        return fail(IBTFO_ESTATE, "ibtfo_setup_geometry has not run");
    if (!c->phi)
        return fail(IBTFO_ESTATE, "the geometry arrays were released (ibtfo_release_geometry)");
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    std::vector<double> phi((size_t)g.plane), nx((size_t)g.plane), ny((size_t)g.plane);
    std::vector<uint8_t> t((size_t)g.plane);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(phi.data(), c->phi, sizeof(double) * g.plane, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(nx.data(), c->nx, sizeof(double) * g.plane, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ny.data(), c->ny, sizeof(double) * g.plane, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(t.data(), c->type, (size_t)g.plane, cudaMemcpyDeviceToHost));
    for (int j = 0; j < g.N; j++)
        for (int i = 0; i < g.M; i++)
        {
            size_t o = (size_t)j * g.pitch + i;
            double *r = xy + ((size_t)g.M * j + i) * 6;
            r[0] = g.Li + i * g.dx; // Psy_coord.cpp:42-43
            r[1] = g.Hi + j * g.dx;
            r[2] = phi[o];
            r[3] = nx[o];
            r[4] = ny[o];
            r[5] = (double)t[o];
        }
    return IBTFO_OK;
}

ibtfo_status ibtfo_get_cut_cells(ibtfo_case *c, double *alpha, double *ax, double *ay)
{
    if (!c || !alpha || !ax || !ay)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->alpha)
        return fail(IBTFO_EINVAL, "not a cut-cell case");
    if (!c->geometry)
        return fail(IBTFO_ESTATE, "ibtfo_setup_geometry has not run");
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    CK(cudaStreamSynchronize(c->stream));
    double *dst[3] = {alpha, ax, ay};
    const double *src[3] = {c->alpha, c->ax, c->ay};
    for (int k = 0; k < 3; k++)
        CK(cudaMemcpy2D(dst[k], sizeof(double) * g.M, src[k], sizeof(double) * g.pitch, sizeof(double) * g.M, g.N,
                        cudaMemcpyDeviceToHost));
    return IBTFO_OK;
}

ibtfo_status ibtfo_get_scheme_index(ibtfo_case *c, double *sch)
{
    if (!c || !sch)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->geometry)
        return fail(IBTFO_ESTATE, "ibtfo_setup_geometry has not run");
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    const int ns = nsch_of(c->cfg.boundary);
    memset(sch, 0, sizeof(double) * (size_t)g.M * g.N * ns);
    if (c->nghost == 0)
        return IBTFO_OK;
    std::vector<GhostRec> gl(c->nghost);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(gl.data(), c->ghosts, sizeof(GhostRec) * c->nghost, cudaMemcpyDeviceToHost));
    for (const GhostRec &r : gl)
    {
        double *s = sch + ((size_t)g.M * r.j + r.i) * ns;
        s[0] = r.xm;
        s[1] = r.ym;
        s[2] = r.idx;
        s[3] = r.idy;
        if (ns >= 8)
            for (int q = 0; q < 4; q++)
                s[4 + q] = r.w[q];
        if (ns == 16)
        {
            s[8] = r.xm2;
            s[9] = r.ym2;
            s[10] = r.idx2;
            s[11] = r.idy2;
            for (int q = 0; q < 4; q++)
                s[12 + q] = r.w2[q];
        }
    }
    return IBTFO_OK;
}

static FillArgs fill_args(ibtfo_case *c)
{
    FillArgs a{};
    a.g = c->g;
    a.buf0 = c->buf[0];
    a.buf1 = c->buf[1];
    a.type = c->type;
    a.st = c->st;
    a.ghosts = c->ghosts;
    a.nghost = c->nghost;
    a.bc = c->cfg.boundary;
    a.gb = c->cfg.global_boundary;
    a.ring_ic = c->ring_ic;
    return a;
}

static SweepArgs sweep_args(ibtfo_case *c, int guard)
{
    SweepArgs a{};
    a.tma = c->tma;
    a.tmap[0] = c->tmap[0];
    a.tmap[1] = c->tmap[1];
    a.g = c->g;
    a.buf0 = c->buf[0];
    a.buf1 = c->buf[1];
    a.type = c->type;
    a.st = c->st;
    a.partial = c->partial;
    a.tiles = c->tiles;
    a.t_end = c->cfg.psy_time;
    a.max_iter = c->cfg.max_iter;
    a.guard = guard;
    return a;
}

// the boundary pass after a sweep (ghost fill + domain edges)
static void enqueue_boundary(ibtfo_case *c)
{
    FillArgs f = fill_args(c);
    const bool gfm = c->cfg.boundary != IBTFO_BOUNDARY_REGULAR;
    if (gfm && c->cfg.global_boundary == IBTFO_GLOBAL_PERIODIC)
    {
        // periodic columns copy filled interior cells: fill first, edges second
        f.do_ghosts = 1;
        f.do_ring = 0;
        launch_fill(f, c->stream);
        f.do_ghosts = 0;
        f.do_ring = 1;
        launch_fill(f, c->stream);
    }
    else
    {
        f.do_ghosts = gfm ? 1 : 0;
        f.do_ring = 1;
        launch_fill(f, c->stream);
    }
}

// TimeAdvance: the sweep (and, for cut cells, the small-cell mixing after it)
static void enqueue_advance(ibtfo_case *c, int guard)
{
    if (c->ccm)
    {
        CcmArgs a{};
        a.s = sweep_args(c, guard);
        a.alpha = c->alpha;
        a.ax = c->ax;
        a.ay = c->ay;
        c->ccm(a, dim3(c->ntiles), dim3(TILE_X * TILE_Y), c->stream); // cut-cell cases: 32x8 tiles
        count_launch();
        MixArgs m{};
        m.g = c->g;
        m.buf0 = c->buf[0];
        m.buf1 = c->buf[1];
        m.st = c->st;
        m.ex = c->mix_ex;
        m.nex = c->nex;
        m.part = c->mix_part;
        m.npart = c->npart;
        m.links = c->mix_links;
        m.e = c->mix_e;
        launch_mix(m, c->stream);
        return;
    }
    c->sweep(sweep_args(c, guard), dim3(c->ntiles), dim3(TILE_X * TILE_Y), c->stream);
    count_launch();
}

// the sweep part of one iteration: Time = RK2, the first stage and its
// Boundary + Global_Boundary, then the second stage with the average (the
// loop accounting happens there); else the single sweep
static void enqueue_sweeps(ibtfo_case *c, int guard)
{
    if (c->cfg.time_advance == IBTFO_TIME_RK2)
    {
        SweepArgs a = sweep_args(c, guard);
        a.stage = 1;
        c->sweep(a, dim3(c->ntiles), dim3(TILE_X * TILE_Y), c->stream);
        count_launch();
        enqueue_boundary(c);
        a.stage = 2;
        c->sweep(a, dim3(c->ntiles), dim3(TILE_X * TILE_Y), c->stream);
        count_launch();
        return;
    }
    enqueue_advance(c, guard);
}

static void enqueue_step(ibtfo_case *c, int guard)
{
    enqueue_sweeps(c, guard);
    enqueue_boundary(c);
}

ibtfo_status ibtfo_set_state(ibtfo_case *c, const double *u0)
{
    if (!c || !u0)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->geometry)
        return fail(IBTFO_ESTATE, "ibtfo_setup_geometry must run before ibtfo_set_state");
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    const size_t cells = (size_t)g.M * g.N;
    CK(ensure_staging(c));
    CK(cudaMemcpyAsync(c->staging, u0, sizeof(double) * 4 * cells, cudaMemcpyHostToDevice, c->stream));
    launch_aos_to_soa(c->staging, c->buf[0], g, c->stream);
    // initial values at the corner-column sources (columns ng and N_x+ng-1, ghost rows)
    std::vector<double> ring(2 * 2 * g.ng * 4);
    for (int side = 0; side < 2; side++)
        for (int rr = 0; rr < 2 * g.ng; rr++)
        {
            int i = side ? g.n_x + g.ng - 1 : g.ng;
            int j = (rr < g.ng) ? rr : g.n_y + rr;
            for (int k = 0; k < 4; k++)
                ring[(side * 2 * g.ng + rr) * 4 + k] = u0[((size_t)g.M * j + i) * 4 + k];
        }
    CK(cudaMemcpyAsync(c->ring_ic, ring.data(), sizeof(double) * ring.size(), cudaMemcpyHostToDevice, c->stream));
    return finish_initial_state(c);
}

// buffer 0 holds the initial state and ring_ic its corner-column sources:
// mirror it into buffer 1 (and the Regular initial copy), run the initial
// Boundary call and the initial ComputeDt / CaculateMass (InclineSod.cpp:105-120)
static ibtfo_status finish_initial_state(ibtfo_case *c)
{
    c->mirror_in = nullptr;
    const GridDesc &g = c->g;
    CK(cudaMemcpyAsync(c->buf[1], c->buf[0], sizeof(double) * 4 * (size_t)g.plane, cudaMemcpyDeviceToDevice,
                       c->stream));
    if (c->ic)
        CK(cudaMemcpyAsync(c->ic, c->buf[0], sizeof(double) * 4 * (size_t)g.plane, cudaMemcpyDeviceToDevice,
                           c->stream));
    DevState s{};
    const bool gfm = c->cfg.boundary != IBTFO_BOUNDARY_REGULAR;
    s.cur = gfm ? 1 : 0; // the initial Boundary call writes the ghost cells into buffer 1
    CK(cudaMemcpyAsync(c->st, &s, sizeof(DevState), cudaMemcpyHostToDevice, c->stream));
    if (gfm)
    {
        FillArgs f = fill_args(c);
        f.do_ghosts = 1;
        f.do_ring = 0;
        f.init_mode = 1;
        launch_fill(f, c->stream);
    }
    ReduceArgs r{};
    r.g = g;
    r.u = c->buf[s.cur];
    r.type = c->type;
    r.st = c->st;
    r.partial = c->partial;
    r.set_start = 1;
    r.alpha = c->alpha;
    launch_reduce(r, c->nblocks, c->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    c->state = true;
    return IBTFO_OK;
}

ibtfo_status ibtfo_put_state(ibtfo_case *c, const double *u)
{
    if (!c || !u)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state: call ibtfo_set_state first");
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    DevState s;
    CK(cudaMemcpyAsync(&s, c->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CK(ensure_staging(c));
    CK(cudaMemcpyAsync(c->staging, u, sizeof(double) * 4 * (size_t)g.M * g.N, cudaMemcpyHostToDevice, c->stream));
    // both buffers: a step leaves solid cells as they are (the reference copies
    // U_NEW into U_OLD for fluid cells only, IDWBaseGFM/GFM_Bound.cpp:24-35)
    launch_aos_to_soa(c->staging, c->buf[s.cur], g, c->stream);
    launch_aos_to_soa(c->staging, c->buf[s.cur ^ 1], g, c->stream);
    c->mirror_in = nullptr;
    CK(cudaGetLastError());
    return IBTFO_OK;
}

// A page-locked record per host thread for the loop state read back after
// every step (a pageable destination goes through a staging buffer of the
// driver); allocated once, portable across devices, never freed, so that
// creating and destroying cases still never synchronises the device.  Null
// when page-locked memory is not available.
static DevState *progress_record()
{
    thread_local DevState *rec = nullptr;
    thread_local bool tried = false;
    if (!tried)
    {
        tried = true;
        void *p = nullptr;
        if (cudaHostAlloc(&p, sizeof(DevState), cudaHostAllocPortable) == cudaSuccess)
            rec = static_cast<DevState *>(p);
        else
            cudaGetLastError();
    }
    return rec;
}

ibtfo_status ibtfo_get_progress(ibtfo_case *c, ibtfo_progress *p)
{
    if (!c || !p)
        return fail(IBTFO_EINVAL, "null argument");
    cudaSetDevice(c->device);
    DevState s;
    DevState *rec = progress_record();
    CK(cudaMemcpyAsync(rec ? rec : &s, c->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (rec)
        s = *rec;
    p->iter = s.iter;
    p->status = s.status;
    p->nan_cells = s.nan_cells;
    p->reserved = 0;
    p->now_t = s.now_t;
    p->dt = s.dt;
    p->mass = s.mass;
    p->mass_start = s.mass_start;
    if (s.status & STATUS_STALL)
        return fail(IBTFO_ETIMEOUT, "a tile's staging copy missed its bounded wait: the state of the steps since is "
                                    "not trusted");
    return IBTFO_OK;
}

ibtfo_status ibtfo_setup_bodies(ibtfo_case *c, const ibtfo_body *bodies, int n)
{
    if (!c || n < 0 || (n > 0 && !bodies))
        return fail(IBTFO_EINVAL, "null case, or bodies missing");
    if (!c->phi)
        return fail(IBTFO_ESTATE, "the geometry arrays were released (ibtfo_release_geometry)");
    for (int k = 0; k < n; k++)
    {
        const ibtfo_body &b = bodies[k];
        if ((b.kind != IBTFO_BODY_CIRCLE && b.kind != IBTFO_BODY_ELLIPSE) || !(b.a > 0) ||
            (b.kind == IBTFO_BODY_ELLIPSE && !(b.b > 0)))
            return fail(IBTFO_EINVAL, "body " + std::to_string(k) + ": unknown kind or non-positive semi-axis");
    }
    cudaSetDevice(c->device);
    ibtfo_body *d = nullptr;
    if (n > 0)
    {
        CK(cudaMallocAsync(&d, sizeof(ibtfo_body) * n, c->stream));
        CK(cudaMemcpyAsync(d, bodies, sizeof(ibtfo_body) * n, cudaMemcpyHostToDevice, c->stream));
    }
    launch_bodies_phi(c->g, d, n, c->phi, c->stream);
    if (d)
        cudaFreeAsync(d, c->stream);
    CK(cudaGetLastError());
    return geometry_from_phi(c);
}

ibtfo_status ibtfo_init_x_split(ibtfo_case *c, double x_split, const double left[4], const double right[4])
{
    if (!c || !left || !right)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->geometry)
        return fail(IBTFO_ESTATE, "the geometry must be set up before the initial state");
    cudaSetDevice(c->device);
    const double g1 = c->g.gamma - 1;
    double L[4], R[4];
    const double *P[2] = {left, right};
    double *Q[2] = {L, R};
    for (int k = 0; k < 2; k++) // conserved (rho, rho u, rho v, E) as Test/Sod/Initialize.cpp:45-48
    {
        const double rho = P[k][0], u = P[k][1], v = P[k][2], p = P[k][3];
        Q[k][0] = rho;
        Q[k][1] = rho * u;
        Q[k][2] = rho * v;
        Q[k][3] = p / g1 + 0.5 * rho * (u * u + v * v);
    }
    launch_x_split_init(c->g, c->type, x_split, L, R, c->buf[0], c->ring_ic, c->stream);
    CK(cudaGetLastError());
    return finish_initial_state(c);
}

ibtfo_status ibtfo_post_shock_state(double mach, double gamma, const double pre[4], double post[4])
{
    if (!pre || !post || !(mach >= 1.0) || !(gamma > 1.0) || !(pre[0] > 0) || !(pre[3] > 0))
        return fail(IBTFO_EINVAL, "need mach >= 1, gamma > 1, positive pre-shock density and pressure");
    // normal shock moving in +x into the state `pre` (Rankine-Hugoniot jump conditions)
    const double a1 = std::sqrt(gamma * pre[3] / pre[0]), m2 = mach * mach;
    post[0] = pre[0] * (gamma + 1) * m2 / ((gamma - 1) * m2 + 2);
    post[1] = pre[1] + 2 * a1 / (gamma + 1) * (mach - 1 / mach);
    post[2] = pre[2];
    post[3] = pre[3] * (2 * gamma * m2 - (gamma - 1)) / (gamma + 1);
    return IBTFO_OK;
}

ibtfo_status ibtfo_release_geometry(ibtfo_case *c)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null case");
    cudaSetDevice(c->device);
    for (double **p : {&c->phi, &c->nx, &c->ny})
    {
        if (*p)
            cudaFreeAsync(*p, c->stream);
        *p = nullptr;
    }
    CK(cudaGetLastError());
    return IBTFO_OK;
}

ibtfo_status ibtfo_get_density(ibtfo_case *c, double *out, int wait)
{
    if (!c || !out)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state");
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    const size_t n = (size_t)g.n_x * g.n_y;
    double *d = nullptr;
    CK(cudaMallocAsync(&d, sizeof(double) * n, c->stream));
    launch_density(g, c->buf[0], c->buf[1], c->st, d, c->stream);
    CK(cudaMemcpyAsync(out, d, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    cudaFreeAsync(d, c->stream);
    if (wait)
        CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    return IBTFO_OK;
}

ibtfo_status ibtfo_case_bytes(const ibtfo_config *k, long long *resident, long long *setup)
{
    if (!k || !resident || !setup)
        return fail(IBTFO_EINVAL, "null argument");
    if (k->n_x < 2 || k->n_y < 2 || k->num_ghost_cell < 2)
        return fail(IBTFO_EINVAL, "bad grid");
    const long long M = k->n_x + 2LL * k->num_ghost_cell, N = k->n_y + 2LL * k->num_ghost_cell;
    const long long pitch = (M + 31) / 32 * 32, plane = pitch * N;
    const long long nblocks = ((k->n_x + TILE_X - 1) / TILE_X) * (long long)((k->n_y + TILE_Y - 1) / TILE_Y);
    long long r = 2 * 4 * 8 * plane;                      // two state buffers
    if (k->boundary == IBTFO_BOUNDARY_REGULAR)
        r += 4 * 8 * plane;                               // Regular: initial state
    if (k->boundary == IBTFO_BOUNDARY_CCM)
        r += 3 * 8 * plane;                               // cut cells: alpha and the two apertures
    r += plane + (long long)sizeof(DevState) + 8 * nblocks + 4 * nblocks + 2 * 2 * k->num_ghost_cell * 4 * 8;
    // ghost records: at most every interior cell next to the outline, bounded
    // here by two layers around the domain perimeter per unit of perimeter
    if (k->boundary != IBTFO_BOUNDARY_REGULAR)
        r += (long long)sizeof(GhostRec) * 4 * (M + N) * k->num_ghost_cell;
    *resident = r;
    *setup = r + 3 * 8 * plane; // plus phi, n_x, n_y until ibtfo_release_geometry
    return IBTFO_OK;
}

// ---------------------------------------------------------------- output

// the VTK file of the current state; the TIME field is the state's loop time
// unless `time` is given (the reference's WriteData takes it from its caller)
static ibtfo_status write_vtk(ibtfo_case *c, const char *path, int binary, const double *time);

ibtfo_status ibtfo_write_vtk(ibtfo_case *c, const char *path, int binary) { return write_vtk(c, path, binary, nullptr); }

static ibtfo_status write_vtk(ibtfo_case *c, const char *path, int binary, const double *time)
{
    if (!c || !path)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state");
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    const size_t n = (size_t)g.n_x * g.n_y;
    float *d = nullptr;
    CK(cudaMallocAsync(&d, sizeof(float) * 4 * n, c->stream));
    launch_vtk_fields(g, c->buf[0], c->buf[1], c->st, c->type, d, nullptr, c->stream);
    std::vector<float> h(4 * n);
    DevState s;
    CK(cudaMemcpyAsync(h.data(), d, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&s, c->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
    cudaFreeAsync(d, c->stream);
    CK(cudaStreamSynchronize(c->stream));
    const ibtfo_config &k = c->cfg;
    if (write_vtk_file(path, g, k.lo_x, k.lo_y, k.hi_x - k.lo_x, k.hi_y - k.lo_y, time ? *time : s.now_t, h.data(),
                       binary))
        return fail(IBTFO_EINVAL, std::string("cannot write ") + path);
    return IBTFO_OK;
}

ibtfo_status ibtfo_write_vtk_async(ibtfo_case *c, const char *path, int binary)
{
    if (!c || !path)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state");
    cudaSetDevice(c->device);
    if (!c->vtk && !(c->vtk = vtk_writer_create(c->device, c->g, c->stream)))
        return fail(IBTFO_ENOMEM, "VTK snapshot buffers");
    const ibtfo_config &k = c->cfg;
    std::string why;
    if (vtk_writer_submit(c->vtk, c->g, c->buf[0], c->buf[1], c->st, c->type, c->stream, path, binary, k.lo_x,
                          k.lo_y, k.hi_x - k.lo_x, k.hi_y - k.lo_y, &why))
        return fail(IBTFO_EINVAL, why);
    return IBTFO_OK;
}

ibtfo_status ibtfo_output_wait(ibtfo_case *c)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null argument");
    std::string why;
    if (c->vtk && vtk_writer_wait(c->vtk, &why))
        return fail(IBTFO_EINVAL, why);
    return IBTFO_OK;
}

static const char CK_MAGIC[8] = {'I', 'B', 'T', 'F', 'O', 'C', 'K', '1'};

struct CheckpointHeader
{
    char magic[8];
    int32_t version, header_bytes;
    ibtfo_config cfg;
    double dt, now_t, mass, mass_start;
    int32_t iter, status, nan_cells, has_ic;
};

ibtfo_status ibtfo_save_checkpoint(ibtfo_case *c, const char *path)
{
    if (!c || !path)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state");
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    const size_t cells = (size_t)g.M * g.N;
    DevState s;
    CK(cudaMemcpyAsync(&s, c->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CheckpointHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, CK_MAGIC, 8);
    h.version = 1;
    h.header_bytes = (int32_t)sizeof(h);
    h.cfg = c->cfg;
    h.dt = s.dt;
    h.now_t = s.now_t;
    h.mass = s.mass;
    h.mass_start = s.mass_start;
    h.iter = s.iter;
    h.status = s.status;
    h.nan_cells = s.nan_cells;
    h.has_ic = c->ic ? 1 : 0;
    // the device buffers as they are (structure-of-arrays planes with the
    // row pitch; in the FP32 form the float (hi, lo) planes): exact in both
    // precisions
    const size_t bytes = sizeof(double) * 4 * (size_t)g.plane;
    std::vector<unsigned char> raw(bytes);
    FILE *f = fopen(path, "wb");
    if (!f)
        return fail(IBTFO_EINVAL, std::string("cannot write ") + path);
    bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
    const double *planes[2] = {c->buf[s.cur], c->ic};
    for (int b = 0; b < 1 + h.has_ic && ok; b++)
    {
        cudaError_t e = cudaMemcpyAsync(raw.data(), planes[b], bytes, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess)
        {
            fclose(f);
            return cuda_fail(e, "checkpoint read-back");
        }
        ok = fwrite(raw.data(), 1, bytes, f) == bytes;
    }
    if (ok && h.has_ic)
    {
        // the corner-column sources of the Regular domain edges, as the case holds them
        std::vector<double> ring(2 * 2 * g.ng * 4);
        cudaError_t e = cudaMemcpyAsync(ring.data(), c->ring_ic, sizeof(double) * ring.size(),
                                        cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        ok = e == cudaSuccess && fwrite(ring.data(), sizeof(double), ring.size(), f) == ring.size();
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? IBTFO_OK : fail(IBTFO_EINVAL, std::string("cannot write ") + path);
}

ibtfo_status ibtfo_load_checkpoint(ibtfo_case *c, const char *path)
{
    if (!c || !path)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->geometry)
        return fail(IBTFO_ESTATE, "set up the geometry before loading a checkpoint");
    FILE *f = fopen(path, "rb");
    if (!f)
        return fail(IBTFO_EINVAL, std::string("cannot read ") + path);
    CheckpointHeader h;
    if (fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, CK_MAGIC, 8) != 0 || h.version != 1 ||
        h.header_bytes != (int32_t)sizeof(h))
    {
        fclose(f);
        return fail(IBTFO_EINVAL, std::string(path) + " is not a checkpoint of this library");
    }
    // everything but the loop's end (psy_time, max_iter) must match
    ibtfo_config a = h.cfg, b = c->cfg;
    a.psy_time = b.psy_time = 0.0;
    a.max_iter = b.max_iter = 0;
    if (std::memcmp(&a, &b, sizeof(a)) != 0 || h.has_ic != (c->ic ? 1 : 0))
    {
        fclose(f);
        return fail(IBTFO_EINVAL, "the checkpoint's configuration differs from the case's");
    }
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    const size_t bytes = sizeof(double) * 4 * (size_t)g.plane;
    std::vector<unsigned char> u(bytes), ic;
    std::vector<double> ring(2 * 2 * g.ng * 4);
    bool ok = fread(u.data(), 1, bytes, f) == bytes;
    if (ok && h.has_ic)
    {
        ic.resize(bytes);
        ok = fread(ic.data(), 1, bytes, f) == bytes &&
             fread(ring.data(), sizeof(double), ring.size(), f) == ring.size();
    }
    fclose(f);
    if (!ok)
        return fail(IBTFO_EINVAL, std::string(path) + " is truncated");
    CK(cudaMemcpyAsync(c->buf[0], u.data(), bytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->buf[1], u.data(), bytes, cudaMemcpyHostToDevice, c->stream));
    c->mirror_in = nullptr;
    if (h.has_ic)
    {
        CK(cudaMemcpyAsync(c->ic, ic.data(), bytes, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(c->ring_ic, ring.data(), sizeof(double) * ring.size(), cudaMemcpyHostToDevice,
                           c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    DevState s{};
    s.dt = h.dt;
    s.now_t = h.now_t;
    s.mass = h.mass;
    s.mass_start = h.mass_start;
    s.iter = h.iter;
    s.status = h.status;
    s.nan_cells = h.nan_cells;
    s.cur = 0;
    CK(cudaMemcpyAsync(c->st, &s, sizeof(DevState), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->state = true;
    return IBTFO_OK;
}

ibtfo_status ibtfo_query(ibtfo_case *c)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null case");
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamQuery(c->stream);
    if (e == cudaErrorNotReady)
        return IBTFO_ETIMEOUT;
    CK(e);
    return IBTFO_OK;
}

ibtfo_status ibtfo_synchronize(ibtfo_case *c)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null case");
    cudaSetDevice(c->device);
    CK(cudaStreamSynchronize(c->stream));
    return IBTFO_OK;
}

// U_NEW of the reference: the snapshot the boundary routines read (interior
// fluid cells from the current buffer, other interior cells from the
// previous one; edge ring from the previous buffer, or from the initial state
// for Regular, whose U_NEW ring is never written)
__global__ void export_unew_kernel(GridDesc g, const double *cur, const double *prev, const double *ring_src,
                                   const uint8_t *type, double *aos)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)g.M * g.N)
        return;
    int j = (int)(q / g.M), i = (int)(q - (long long)j * g.M);
    long long o = (long long)j * g.pitch + i;
    bool in = i >= g.ng && i < g.ng + g.n_x && j >= g.ng && j < g.ng + g.n_y;
    const double *b = in ? (updated_cell(type[o]) ? cur : prev) : ring_src;
    for (int k = 0; k < 4; k++)
        aos[q * 4 + k] = state_ld(b, k, o, g);
}

ibtfo_status ibtfo_get_state(ibtfo_case *c, double *u_old, double *u_new)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null case");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state: call ibtfo_set_state first");
    cudaSetDevice(c->device);
    const GridDesc &g = c->g;
    const size_t cells = (size_t)g.M * g.N;
    DevState s;
    CK(ensure_staging(c));
    CK(cudaMemcpyAsync(&s, c->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (u_old)
    {
        launch_soa_to_aos(c->buf[s.cur], c->staging, g, c->stream);
        CK(cudaMemcpyAsync(u_old, c->staging, sizeof(double) * 4 * cells, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    if (u_new)
    {
        const double *cur = c->buf[s.cur], *prev = c->buf[s.cur ^ 1];
        const double *ring = c->ic ? c->ic : prev;
        export_unew_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, c->stream>>>(g, cur, prev, ring, c->type,
                                                                                 c->staging);
        count_launch();
        CK(cudaMemcpyAsync(u_new, c->staging, sizeof(double) * 4 * cells, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    CK(cudaGetLastError());
    return IBTFO_OK;
}

static const int GRAPH_STEPS = 16;

static ibtfo_status build_graph(ibtfo_case *c)
{
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    long long before = g_launches.load();
    for (int s = 0; s < GRAPH_STEPS; s++)
        enqueue_step(c, 1);
    c->graph_launches = g_launches.load() - before;
    g_launches.store(before); // captured launches are counted when replayed
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (e != cudaSuccess)
        return cuda_fail(e, "graph capture");
    e = cudaGraphInstantiate(&c->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return cuda_fail(e, "graph instantiate");
    c->graph_steps = GRAPH_STEPS;
    return IBTFO_OK;
}

ibtfo_status ibtfo_advance(ibtfo_case *c, int nsteps)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null case");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state: call ibtfo_set_state first");
    if (nsteps < 0)
        return fail(IBTFO_EINVAL, "nsteps < 0");
    cudaSetDevice(c->device);
    int left = nsteps;
    if (left >= GRAPH_STEPS)
    {
        if (!c->graph)
        {
            ibtfo_status s = build_graph(c);
            if (s != IBTFO_OK)
                return s;
        }
        while (left >= GRAPH_STEPS)
        {
            CK(cudaGraphLaunch(c->graph, c->stream));
            count_launch((int)c->graph_launches);
            left -= GRAPH_STEPS;
        }
    }
    for (; left > 0; left--)
        enqueue_step(c, 1);
    CK(cudaGetLastError());
    return IBTFO_OK;
}

ibtfo_status ibtfo_enqueue_sweep(ibtfo_case *c)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null case");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state: call ibtfo_set_state first");
    cudaSetDevice(c->device);
    enqueue_sweeps(c, 1);
    CK(cudaGetLastError());
    return IBTFO_OK;
}

ibtfo_status ibtfo_enqueue_boundary(ibtfo_case *c)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null case");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state: call ibtfo_set_state first");
    cudaSetDevice(c->device);
    enqueue_boundary(c);
    CK(cudaGetLastError());
    return IBTFO_OK;
}

ibtfo_status ibtfo_step(ibtfo_case *c, ibtfo_progress *p)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null case");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state: call ibtfo_set_state first");
    cudaSetDevice(c->device);
    enqueue_step(c, 0);
    CK(cudaGetLastError());
    if (p)
        return ibtfo_get_progress(c, p);
    CK(cudaStreamSynchronize(c->stream));
    return IBTFO_OK;
}

// streams and events of ibtfo_step_host, created on first use
static cudaError_t ensure_pipeline(ibtfo_case *c)
{
    cudaError_t e = cudaSuccess;
    if (!c->ev_done)
    {
        int least = 0, greatest = 0;
        e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
        for (cudaStream_t *s : {&c->h2d, &c->d2h})
            if (e == cudaSuccess)
                e = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaStreamCreateWithPriority(&c->conv, cudaStreamNonBlocking, greatest);
        for (cudaStream_t &s : c->fin)
            if (e == cudaSuccess)
                e = cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, greatest);
        for (cudaStream_t &s : c->sw)
            if (e == cudaSuccess)
                e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        for (int k = 0; k < NBANDS && e == cudaSuccess; k++)
            for (cudaEvent_t *v : {&c->ev_in[k], &c->ev_conv[k], &c->ev_out[k], &c->ev_swept[k]})
                if (e == cudaSuccess)
                    e = cudaEventCreateWithFlags(v, cudaEventDisableTiming);
        for (cudaEvent_t &v : c->ev_sw)
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(&v, cudaEventDisableTiming);
        for (cudaEvent_t &v : c->ev_fin)
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(&v, cudaEventDisableTiming);
        for (cudaEvent_t *v : {&c->ev_cv, &c->ev_done})
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(v, cudaEventDisableTiming);
    }
    return e;
}

// The cells of transfer chunk k an ibtfo_step_host copies in: every row, or
// (boxes) the in-place copy-in boxes.  They go into both state buffers: a
// step leaves solid cells as they are (the reference copies U_NEW into U_OLD
// for fluid cells only, e.g. IDWBaseGFM/GFM_Bound.cpp:24-35), which with two
// alternating buffers needs them in both.
static HostBoxes chunk_boxes(const ibtfo_case *c, int k, bool boxes)
{
    if (boxes)
        return c->in_boxes[k];
    HostBoxes b{};
    if (c->band_rows[k + 1] > c->band_rows[k])
    {
        b.n = 1;
        b.r0[0] = c->band_rows[k], b.r1[0] = c->band_rows[k + 1], b.c0[0] = 0, b.c1[0] = c->g.M;
    }
    return b;
}

// The step when the banded pipeline does not apply (cut cells, RK2): the
// whole state in, the step, the whole state out, still in row chunks.
static ibtfo_status step_host_plain(ibtfo_case *c, const double *u_in, double *u_out)
{
    const GridDesc &g = c->g;
    const size_t row = sizeof(double) * 4 * (size_t)g.M;
    for (int k = 0; k < NBANDS; k++)
    {
        const int r0 = c->band_rows[k], r1 = c->band_rows[k + 1];
        if (r1 > r0)
            CK(cudaMemcpyAsync(c->staging + (size_t)r0 * 4 * g.M, u_in + (size_t)r0 * 4 * g.M, row * (r1 - r0),
                               cudaMemcpyHostToDevice, c->h2d));
        CK(cudaEventRecord(c->ev_in[k], c->h2d));
        CK(cudaStreamWaitEvent(c->stream, c->ev_in[k], 0));
        launch_aos_to_cur_boxes(c->staging, c->buf[0], c->buf[1], c->st, g, chunk_boxes(c, k, false), k == 0, true,
                                c->stream);
    }
    enqueue_step(c, 0);
    for (int k = 0; k < NBANDS; k++)
    {
        const int r0 = c->band_rows[k], r1 = c->band_rows[k + 1];
        launch_cur_to_aos_rows(c->buf[0], c->buf[1], c->st, c->staging, g, r0, r1, c->stream);
        CK(cudaEventRecord(c->ev_out[k], c->stream));
        CK(cudaStreamWaitEvent(c->d2h, c->ev_out[k], 0));
        if (r1 > r0)
            CK(cudaMemcpyAsync(u_out + (size_t)r0 * 4 * g.M, c->staging + (size_t)r0 * 4 * g.M, row * (r1 - r0),
                               cudaMemcpyDeviceToHost, c->d2h));
    }
    CK(cudaEventRecord(c->ev_done, c->d2h));
    CK(cudaStreamWaitEvent(c->stream, c->ev_done, 0));
    return IBTFO_OK;
}

// The banded pipeline.  Row chunk k goes host -> device on one copy stream;
// a conversion stream converts it into the current state buffer; band k of the
// sweep (the tiles of its tile rows, which read array rows up to the end of
// chunk k) runs on one of NSW sweep streams, so that consecutive bands
// overlap on the SMs.  One of NFIN finishing streams then fills the ghost
// cells of band k's rows (once every band their image points read has been
// swept), converts the band's rows back (fluid and ghost cells from the
// step's output, other cells from its input) and hands them to the second
// copy stream, while later bands compute (the copy engines move them at the
// link's rate without holding SMs the sweeps need; kernels writing the host
// array across the link would hold their SM slots for as long).  The domain
// edges are filled and go back by two row copies and two strided column
// copies, or to a page-locked u_out by the conversion kernel itself (a few
// hundred KB; the strided copies move 2-cell pieces row by row): in place between
// walls (they read swept cells and the step's input only) as soon as every
// band is swept, beside the bands' finishing work; otherwise after it
// (periodic edges copy interior cells, ghost cells included, and full-row
// copies back cover the edges).
// The chunks partition the rows and band k writes back only rows below the
// start of chunk k + 1, which it has read; the ring goes back after every
// chunk has landed: so u_out may be u_in.  In place (u_out == u_in) the host array already holds every cell the step
// leaves alone (solid cells are never written), so each band copies back
// only its interior rows over the columns of its fluid and ghost cells, and
// (boxes) copies in only the cells some part of the step reads.
static ibtfo_status step_host_banded(ibtfo_case *c, const double *u_in, double *u_out, bool boxes)
{
    const GridDesc &g = c->g;
    const size_t row = sizeof(double) * 4 * (size_t)g.M, cell = sizeof(double) * 4;
    const bool inplace = (u_out == u_in);
    double *zc = device_view(u_out);
    for (int k = 0; k < NBANDS; k++)
    {
        const HostBoxes b = chunk_boxes(c, k, boxes);
        for (int q = 0; q < b.n; q++)
        {
            const size_t o = ((size_t)b.r0[q] * g.M + b.c0[q]) * 4;
            if (b.c0[q] == 0 && b.c1[q] == g.M)
                CK(cudaMemcpyAsync(c->staging + o, u_in + o, row * (b.r1[q] - b.r0[q]), cudaMemcpyHostToDevice,
                                   c->h2d));
            else
                CK(cudaMemcpy2DAsync(c->staging + o, row, u_in + o, row, cell * (b.c1[q] - b.c0[q]),
                                     (size_t)(b.r1[q] - b.r0[q]), cudaMemcpyHostToDevice, c->h2d));
        }
        CK(cudaEventRecord(c->ev_in[k], c->h2d));
    }
    // the bands sweep the case's tiles, in row order
    SweepArgs a = sweep_args(c, 0);
    a.tiles = c->band_list;
    a.nblocks = c->nband_list;
    FillArgs f = fill_args(c);
    const bool gfm = c->cfg.boundary != IBTFO_BOUNDARY_REGULAR;
    auto finish = [&](int k) -> ibtfo_status {
        // band k's ghost cells, its rows back to the host layout, and their copy
        cudaStream_t fs = c->fin[k % NFIN];
        for (int b = 0; b <= c->ghost_ready[k]; b++)
            CK(cudaStreamWaitEvent(fs, c->ev_swept[b], 0));
        if (gfm)
            launch_fill_ghosts(f, c->band_ghosts[k], c->band_ghosts[k + 1], fs);
        int o0 = c->out_rows[k], o1 = c->out_rows[k + 1], x0 = 0, x1 = g.M;
        if (inplace)
        {
            o0 = std::max(o0, g.ng);
            o1 = std::min(o1, g.ng + g.n_y);
            x0 = c->fluid_cols[2 * k];
            x1 = c->fluid_cols[2 * k + 1];
        }
        launch_snapshot_to_aos_rows(c->buf[0], c->buf[1], c->st, c->type, c->staging, g, o0, o1, x0, x1, fs);
        CK(cudaEventRecord(c->ev_out[k], fs));
        CK(cudaStreamWaitEvent(c->d2h, c->ev_out[k], 0));
        if (o1 > o0 && x1 > x0)
            CK(cudaMemcpy2DAsync(u_out + ((size_t)o0 * g.M + x0) * 4, row, c->staging + ((size_t)o0 * g.M + x0) * 4,
                                 row, sizeof(double) * 4 * (size_t)(x1 - x0), (size_t)(o1 - o0),
                                 cudaMemcpyDeviceToHost, c->d2h));
        return IBTFO_OK;
    };
    int next = 0; // the next band to finish
    for (int k = 0; k < NBANDS; k++)
    {
        CK(cudaStreamWaitEvent(c->conv, c->ev_in[k], 0));
        launch_aos_to_cur_boxes(c->staging, c->buf[0], c->buf[1], c->st, g, chunk_boxes(c, k, boxes), k == 0, true,
                                c->conv);
        CK(cudaEventRecord(c->ev_conv[k], c->conv));
        cudaStream_t s = c->sw[k % NSW];
        CK(cudaStreamWaitEvent(s, c->ev_conv[k], 0));
        const int t0 = c->band_tiles[k], t1 = c->band_tiles[k + 1];
        if (t1 > t0)
        {
            a.tile0 = t0;
            c->sweep(a, dim3(t1 - t0), dim3(TILE_X * TILE_Y), s);
            count_launch();
        }
        CK(cudaEventRecord(c->ev_swept[k], s));
        for (; next < NBANDS && c->ghost_ready[next] <= k; next++)
        {
            ibtfo_status st = finish(next);
            if (st != IBTFO_OK)
                return st;
        }
    }
    for (; next < NBANDS; next++)
    {
        ibtfo_status st = finish(next);
        if (st != IBTFO_OK)
            return st;
    }
    const bool early_ring = inplace && c->cfg.global_boundary != IBTFO_GLOBAL_PERIODIC;
    // the ring's kernels and copies: the conversion stream (idle once the
    // last chunk is in) or, after everything else, the case's stream
    cudaStream_t rk = early_ring ? c->conv : c->stream, rc = early_ring ? c->conv : c->d2h;
    for (int q = 0; q < NSW; q++)
    {
        CK(cudaEventRecord(c->ev_sw[q], c->sw[q]));
        CK(cudaStreamWaitEvent(rk, c->ev_sw[q], 0));
    }
    auto join_finishing = [&]() -> ibtfo_status {
        for (int q = 0; q < NFIN; q++)
        {
            CK(cudaEventRecord(c->ev_fin[q], c->fin[q]));
            CK(cudaStreamWaitEvent(c->stream, c->ev_fin[q], 0));
        }
        return IBTFO_OK;
    };
    if (!early_ring)
    {
        ibtfo_status js = join_finishing();
        if (js != IBTFO_OK)
            return js;
        CK(cudaEventRecord(c->ev_cv, c->conv));
        CK(cudaStreamWaitEvent(c->stream, c->ev_cv, 0));
    }
    f.do_ghosts = 0;
    f.do_ring = 1;
    launch_fill(f, rk);
    ibtfo_status rs = ring_to_host(c, u_out, rk, rc, zc, !inplace);
    if (rs != IBTFO_OK)
        return rs;
    if (early_ring)
    {
        ibtfo_status js = join_finishing();
        if (js != IBTFO_OK)
            return js;
        CK(cudaEventRecord(c->ev_cv, c->conv));
        CK(cudaStreamWaitEvent(c->stream, c->ev_cv, 0));
    }
    CK(cudaEventRecord(c->ev_done, c->d2h));
    CK(cudaStreamWaitEvent(c->stream, c->ev_done, 0));
    return IBTFO_OK;
}

// The PVRS solvers read, for a Y face, the state of cell 7 c + 2 (the
// reference's stray scratch store): anywhere in the array, so their in-place
// steps copy every row in.
static bool boxes_apply(const ibtfo_case *c) { return c->cfg.riemann != IBTFO_RIEMANN_PVRS; }

ibtfo_status ibtfo_step_host_bytes(const ibtfo_case *c, int in_place, long long *h2d, long long *d2h)
{
    if (!c || !h2d || !d2h)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->geometry)
        return fail(IBTFO_ESTATE, "ibtfo_setup_geometry has not run");
    const GridDesc &g = c->g;
    const long long cell = sizeof(double) * 4;
    *h2d = cell * g.M * g.N;
    const bool banded = !c->ccm && c->cfg.time_advance == IBTFO_TIME_SINGLESTEP;
    if (banded && in_place && boxes_apply(c))
    {
        *h2d = 0;
        for (int k = 0; k < NBANDS; k++)
        {
            const HostBoxes &b = c->in_boxes[k];
            for (int q = 0; q < b.n; q++)
                *h2d += cell * (long long)(b.r1[q] - b.r0[q]) * (b.c1[q] - b.c0[q]);
        }
    }
    long long out = cell * g.M * g.N;
    if (banded)
    {
        out = cell * (2LL * g.ng * g.M + 2LL * g.ng * g.n_y); // the domain ring
        for (int k = 0; k < NBANDS; k++)
        {
            if (!in_place)
            {
                out += cell * (long long)(c->out_rows[k + 1] - c->out_rows[k]) * g.M;
                continue;
            }
            const int o0 = std::max(c->out_rows[k], g.ng), o1 = std::min(c->out_rows[k + 1], g.ng + g.n_y);
            if (o1 > o0)
                out += cell * (long long)(o1 - o0) * (c->fluid_cols[2 * k + 1] - c->fluid_cols[2 * k]);
        }
    }
    *d2h = out + (long long)sizeof(DevState); // the loop state read for the progress
    return IBTFO_OK;
}

ibtfo_status ibtfo_step_host(ibtfo_case *c, const double *u_in, double *u_out, ibtfo_progress *p)
{
    if (!c || !u_in || !u_out)
        return fail(IBTFO_EINVAL, "null argument");
    if (!c->state)
        return fail(IBTFO_ESTATE, "no state: call ibtfo_set_state first");
    cudaSetDevice(c->device);
    CK(ensure_staging(c));
    CK(ensure_pipeline(c));
    const bool banded = !c->ccm && c->cfg.time_advance == IBTFO_TIME_SINGLESTEP;
    // page-locked arrays: the banded step replays as one CUDA graph (captured
    // for this pair of arrays; about 100 stream operations in one launch)
    bool graph = false;
    if (banded)
    {
        cudaPointerAttributes ai, ao;
        graph = cudaPointerGetAttributes(&ai, u_in) == cudaSuccess && ai.type == cudaMemoryTypeHost &&
                cudaPointerGetAttributes(&ao, u_out) == cudaSuccess && ao.type == cudaMemoryTypeHost;
        cudaGetLastError();
    }
    ibtfo_status st = IBTFO_OK;
    bool boxes = false;
    if (banded && u_in == u_out && boxes_apply(c))
    {
        if (c->mirror_in != u_in)
        {
            // the first in-place step on this array since the device state was
            // last written from elsewhere: every row in, so that the cells
            // later steps do not copy agree with the array
            CK(cudaEventRecord(c->ev_done, c->stream));
            for (cudaStream_t s : helper_streams(c))
                CK(cudaStreamWaitEvent(s, c->ev_done, 0));
            st = step_host_banded(c, u_in, u_out, false);
            if (st != IBTFO_OK)
                return st;
            CK(cudaGetLastError());
            c->mirror_in = u_in;
            ibtfo_progress q;
            return ibtfo_get_progress(c, p ? p : &q);
        }
        boxes = true;
    }
    if (graph && (c->host_graph_in != u_in || c->host_graph_out != u_out || !c->host_graph))
    {
        if (c->host_graph)
            cudaGraphExecDestroy(c->host_graph);
        c->host_graph = nullptr;
        cudaGraph_t gr;
        long long before = g_launches.load();
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        cudaEventRecord(c->ev_done, c->stream);
        for (cudaStream_t s : helper_streams(c))
            cudaStreamWaitEvent(s, c->ev_done, 0);
        st = step_host_banded(c, u_in, u_out, boxes);
        c->host_graph_launches = g_launches.load() - before;
        g_launches.store(before); // counted when replayed
        cudaError_t e = cudaStreamEndCapture(c->stream, &gr);
        if (st != IBTFO_OK)
            return st;
        if (e != cudaSuccess)
            return cuda_fail(e, "capturing the host step");
        // kernel nodes keep the priorities of the streams they were captured from
        e = cudaGraphInstantiate(&c->host_graph, gr, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess)
            return cuda_fail(e, "instantiating the host step");
        c->host_graph_in = u_in;
        c->host_graph_out = u_out;
    }
    if (graph)
    {
        CK(cudaGraphLaunch(c->host_graph, c->stream));
        count_launch((int)c->host_graph_launches);
    }
    else
    {
        // every helper stream starts after what is already queued on the case's stream
        CK(cudaEventRecord(c->ev_done, c->stream));
        for (cudaStream_t s : helper_streams(c))
            CK(cudaStreamWaitEvent(s, c->ev_done, 0));
        st = banded ? step_host_banded(c, u_in, u_out, boxes) : step_host_plain(c, u_in, u_out);
        if (st != IBTFO_OK)
            return st;
    }
    CK(cudaGetLastError());
    ibtfo_progress q;
    return ibtfo_get_progress(c, p ? p : &q); // waits for the copies
}

ibtfo_status ibtfo_run(ibtfo_case *c, int stop_on_nan, ibtfo_progress *p)
{
    if (!c)
        return fail(IBTFO_EINVAL, "null case");
    ibtfo_progress q;
    ibtfo_status s = ibtfo_get_progress(c, &q);
    if (s != IBTFO_OK)
        return s;
    while (q.now_t < c->cfg.psy_time && q.iter < c->cfg.max_iter)
    {
        // queue about as many steps as the current dt says are left (extra ones do nothing)
        double left = (c->cfg.psy_time - q.now_t) / q.dt;
        int n = (std::isfinite(left) && left > 0) ? (int)std::min(left + 1.0, 4096.0) : 4096;
        n = std::min(n, c->cfg.max_iter - q.iter);
        n = std::max(n, 1);
        if (stop_on_nan)
            n = std::min(n, 64);
        s = ibtfo_advance(c, n);
        if (s != IBTFO_OK)
            return s;
        s = ibtfo_get_progress(c, &q);
        if (s != IBTFO_OK)
            return s;
        if (stop_on_nan && (q.status & STATUS_NAN))
        {
            if (p)
                *p = q;
            return fail(IBTFO_ENAN, "NaN in the state");
        }
    }
    if (p)
        *p = q;
    return IBTFO_OK;
}

ibtfo_status ibtfo_host_alloc(size_t bytes, void **p)
{
    if (!p)
        return fail(IBTFO_EINVAL, "null argument");
    cudaError_t e = cudaHostAlloc(p, bytes, cudaHostAllocDefault);
    if (e != cudaSuccess)
    {
        *p = nullptr;
        return fail(IBTFO_ENOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    }
    return IBTFO_OK;
}

ibtfo_status ibtfo_host_free(void *p)
{
    if (p)
        cudaFreeHost(p);
    return IBTFO_OK;
}

} // extern "C"

// ---------------------------------------------------------------- internal
namespace ibtfo {

static void drop_graph(ibtfo_case *c) { drop_graphs(c); }

int case_set_gas(ibtfo_case *c, double gamma, double cfl)
{
    if (!(gamma > 1.0) || !(cfl > 0.0))
        return fail(IBTFO_EINVAL, "need gamma > 1 and cfl > 0");
    if (c->g.gamma != gamma || c->g.cfl != cfl)
    {
        cudaSetDevice(c->device);
        cudaStreamSynchronize(c->stream);
        c->g.gamma = c->cfg.gamma = gamma;
        c->g.cfl = c->cfg.cfl_number = cfl;
        set_derived_constants(c->g);
        drop_graph(c);
    }
    return IBTFO_OK;
}

double case_cfl(const ibtfo_case *c) { return c->g.cfl; }
double case_gamma(const ibtfo_case *c) { return c->g.gamma; }

int case_batch_view(ibtfo_case *c, SweepArgs *sa, FillArgs *fa, int *scheme, int *riemann, int *limiter,
                    int *precision, int *has_state)
{
    *sa = sweep_args(c, 1);
    *fa = fill_args(c);
    *scheme = c->cfg.scheme;
    *riemann = c->cfg.riemann;
    *limiter = c->cfg.limiter;
    *precision = c->cfg.precision;
    *has_state = c->state ? 1 : 0;
    return 0;
}

cudaStream_t case_stream(const ibtfo_case *c) { return c->stream; }
int case_write_vtk_at(ibtfo_case *c, const char *path, double now_t) { return write_vtk(c, path, 0, &now_t); }
int case_time_advance(const ibtfo_case *c) { return c->cfg.time_advance; }
int case_device(const ibtfo_case *c) { return c->device; }

int case_set_dt(ibtfo_case *c, double dt)
{
    cudaSetDevice(c->device);
    CK(cudaMemcpyAsync(&c->st->dt, &dt, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream)); // dt lives on this stack frame
    return IBTFO_OK;
}

int case_sweep_unguarded(ibtfo_case *c)
{
    cudaSetDevice(c->device);
    enqueue_advance(c, 0);
    count_launch();
    CK(cudaGetLastError());
    return IBTFO_OK;
}

int case_fill(ibtfo_case *c, int ghosts, int ring)
{
    cudaSetDevice(c->device);
    FillArgs f = fill_args(c);
    f.do_ghosts = (ghosts && c->cfg.boundary != IBTFO_BOUNDARY_REGULAR) ? 1 : 0;
    f.do_ring = ring ? 1 : 0;
    launch_fill(f, c->stream);
    CK(cudaGetLastError());
    return IBTFO_OK;
}

int case_reduce_current(ibtfo_case *c)
{
    cudaSetDevice(c->device);
    DevState s;
    CK(cudaMemcpyAsync(&s, c->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    ReduceArgs r{};
    r.g = c->g;
    r.u = c->buf[s.cur];
    r.type = c->type;
    r.st = c->st;
    r.partial = c->partial;
    r.set_start = 0;
    r.alpha = c->alpha;
    launch_reduce(r, c->nblocks, c->stream);
    CK(cudaGetLastError());
    return IBTFO_OK;
}

} // namespace ibtfo

