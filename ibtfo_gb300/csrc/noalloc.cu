// CFL time step and fluid mass of a device-resident state, for callers that
// cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not
// wanted -- inside a memory-pool-owning framework that forbids stray
// allocations, in a process that has handed all device memory to its own
// allocator, or between other work that must not be serialised by an
// allocation (cudaMalloc/cudaFree can synchronise the device).  Such a caller
// already owns the state arrays and only wants the reduction.
//
// The reduction is the library's reduce_kernel (ComputeDt + CaculateMass of
// one state).  Its scratch -- the per-block mass partials and the reduction
// state (running maxima, finishing-block ticket, results) -- lives in the
// file-scope array below instead of allocated memory.  The array is part of
// the loaded library: every GPU that loads the library holds it until the
// process exits.
#include "../../include/ibtfo.h"
#include "internal.h"

namespace ibtfo {
void set_last_error(const char *msg);
}

namespace {
constexpr int kStateSlots = 16;        // doubles reserved for the DevState (128 bytes)
constexpr int kMaxTiles = 65536;       // 32x8-cell tiles: at most 16,777,216 interior cells
static_assert(sizeof(ibtfo::DevState) <= kStateSlots * sizeof(double), "DevState slot too small");
} // namespace

// 512 KiB + 128 B per device
static __device__ __align__(256) double g_noalloc_scratch[kStateSlots + kMaxTiles];

// Device address of the scratch array on the current device.  Looked up on
// every call (a cheap runtime query, so a call after cudaDeviceReset or in a
// new primary context gets the current address); the first lookup on a device
// may load the library's module there, which is why the first call on a
// device should come before any stream capture.
static cudaError_t noalloc_scratch(double **out)
{
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e == cudaSuccess)
        *out = static_cast<double *>(p);
    return e;
}

__global__ void noalloc_out_kernel(const ibtfo::DevState *st, double *out)
{
    out[0] = st->dt;
    out[1] = st->mass;
}

extern "C" ibtfo_status ibtfo_dt_mass_noalloc(const double *d_u, long long plane, int pitch,
                                              const unsigned char *d_type, int n_x, int n_y, int num_ghost_cell,
                                              double lo_x, double lo_y, double hi_x, double hi_y, double gamma,
                                              double cfl_number, double *d_out, void *stream)
{
    using namespace ibtfo;
    if (!d_u || !d_type || !d_out)
    {
        set_last_error("ibtfo_dt_mass_noalloc: null pointer");
        return IBTFO_EINVAL;
    }
    const int M = n_x + 2 * num_ghost_cell, N = n_y + 2 * num_ghost_cell;
    if (n_x < 1 || n_y < 1 || num_ghost_cell < 0 || pitch < M || plane < (long long)pitch * N ||
        !(hi_x > lo_x) || !(hi_y > lo_y))
    {
        set_last_error("ibtfo_dt_mass_noalloc: need n_x, n_y >= 1, num_ghost_cell >= 0, pitch >= N_x + 2 ng, "
                     "plane >= pitch * (N_y + 2 ng), hi > lo");
        return IBTFO_EINVAL;
    }
    const long long tx = (n_x + TILE_X - 1) / TILE_X, ty = (n_y + TILE_Y - 1) / TILE_Y;
    if (tx * ty > kMaxTiles || ty > 65535)
    {
        set_last_error("ibtfo_dt_mass_noalloc: grid too large for the fixed scratch (at most 65536 tiles of "
                     "32 x 8 interior cells, e.g. 4096 x 4096)");
        return IBTFO_EINVAL;
    }
    double *scratch = nullptr;
    cudaError_t e = noalloc_scratch(&scratch);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DevState *st = reinterpret_cast<DevState *>(scratch);
    // the maxima and the finishing-block ticket must start at zero; the
    // partials are written before they are read
    if (e == cudaSuccess)
        e = cudaMemsetAsync(st, 0, sizeof(DevState), s);
    if (e != cudaSuccess)
    {
        set_last_error(cudaGetErrorString(e));
        return IBTFO_ECUDA;
    }
    ReduceArgs r{};
    r.g.n_x = n_x;
    r.g.n_y = n_y;
    r.g.ng = num_ghost_cell;
    r.g.M = M;
    r.g.N = N;
    r.g.pitch = pitch;
    r.g.plane = plane;
    r.g.dx = (hi_x - lo_x) / n_x; // ComputeDt.cpp:26
    r.g.dy = (hi_y - lo_y) / n_y; // CaculateMass.cpp:25
    r.g.gamma = gamma;
    r.g.cfl = cfl_number;
    r.u = d_u;
    r.type = d_type;
    r.st = st;
    r.partial = scratch + kStateSlots;
    r.set_start = 0;
    launch_reduce(r, (int)(tx * ty), s);
    noalloc_out_kernel<<<1, 1, 0, s>>>(st, d_out);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess)
    {
        set_last_error(cudaGetErrorString(e));
        return IBTFO_ECUDA;
    }
    return IBTFO_OK;
}
