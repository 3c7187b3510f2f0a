// Per-step boundary pass (ghost-fluid fill over the compacted ghost list and
// the domain-edge layers), the stand-alone CFL/mass reduction, and the
// array-of-structures <-> structure-of-arrays conversion used at the host
// boundary.
//
// State-buffer semantics.  The reference keeps U_OLD and U_NEW and, each
// step, copies U_NEW into U_OLD and (ghost-fluid variants) snapshots U_OLD
// into U_NEW before filling ghost cells (IDWBaseGFM/GFM_Bound.cpp:23-50);
// Global_Boundary then reads U_NEW (Test/Sod/Global_Boudary.cpp:23-75).
// Here the two buffers ping-pong: after a sweep, `next` holds the new fluid
// values and `prev` the previous state, so the reference's snapshot S is
//   S(i,j) = type(i,j) == 0 (or a cut cell) ? next(i,j) : prev(i,j)   (interior cells)
//   S(ring) = prev(ring)            ghost-fluid variants (snapshot of U_OLD)
//   S(ring) = initial values        Regular (U_NEW's ring is never written)
// and this pass writes next's ghost cells and ring from S.
#include "internal.h"
#include "physics.cuh"
#include "sweep_impl.cuh"

namespace ibtfo {

// The buffers of the state after the step (`next`, which the pass writes)
// and before it (`prev`).  The reference's U_NEW at an updated interior cell
// is next's value there, elsewhere prev's (the snapshot rule above); which
// one a read takes is a static property of the geometry, resolved before the
// pass reads the device state that names the buffers, so that the loads of a
// record, of its cell types and of that state do not wait on one another.
struct View
{
    const double *next, *prev;
    GridDesc g;
    __device__ __forceinline__ double S(long long o, int k, bool from_next) const
    {
        return state_ld(from_next ? next : prev, k, o, g);
    }
};

// primitives of S at (i, j), as GFM_Bound.cpp:197-212 computes them
__device__ __forceinline__ void prim(const View &v, int i, int j, bool from_next, double g, double &rho, double &u,
                                     double &w, double &p)
{
    const long long o = (long long)j * v.g.pitch + i;
    rho = v.S(o, 0, from_next);
    u = v.S(o, 1, from_next) / rho;
    w = v.S(o, 2, from_next) / rho;
    p = (g - 1) * (v.S(o, 3, from_next) - 0.5 * rho * (u * u + w * w));
}

// A ghost record is filled by GHOST_LANES consecutive lanes of one warp
// (a quad): lane c computes the primitives of bracket corner c and the
// weighted average of primitive c, and stores conserved component c.  Every
// value is the expression, in the order, that one thread computing all of
// them evaluates; the quad shortens the chain of dependent loads and FP64
// divides that bounds the pass (about one ghost record per wall cell).
struct Quad
{
    unsigned mask; // the quad's lanes in the warp
    int c;         // this lane's corner / component, 0..3
    __device__ __forceinline__ double get(double x, int src) const { return __shfl_sync(mask, x, src, GHOST_LANES); }
};

__device__ __forceinline__ double pick4(int c, double x0, double x1, double x2, double x3)
{
    return c == 0 ? x0 : c == 1 ? x1 : c == 2 ? x2 : x3;
}

// inverse-distance average of the four bracket corners (idx,idy),
// (idx,idy+1), (idx+1,idy+1), (idx+1,idy), GFM_Bound.cpp:214-217; every lane
// of the quad receives all four averages.  nxt: bit c set when corner c is
// read from the new state.
__device__ __forceinline__ void idw_average(const View &v, const Quad &q, int idx, int idy, int nxt, const double *a,
                                            double g, double w[4])
{
    double r, u, vv, p;
    prim(v, idx + (q.c >= 2), idy + (q.c == 1 || q.c == 2), (nxt >> q.c) & 1, g, r, u, vv, p);
    double x[4]; // primitive q.c of corners 0..3
#pragma unroll
    for (int s = 0; s < 4; s++)
    {
        const double rs = q.get(r, s), us = q.get(u, s), vs = q.get(vv, s), ps = q.get(p, s);
        x[s] = pick4(q.c, rs, us, vs, ps);
    }
    const double sum = a[0] + a[1] + a[2] + a[3];
    const double mine = (a[0] * x[0] + a[1] * x[1] + a[2] * x[2] + a[3] * x[3]) / sum;
#pragma unroll
    for (int k = 0; k < 4; k++)
        w[k] = q.get(mine, k);
}

// conserved component q.c of (rho, u, v, p) stored at o
__device__ __forceinline__ void store_conserved(double *dst, long long o, const GridDesc &gd, const Quad &q, double g,
                                                double rho, double u, double v, double p)
{
    state_st(dst, q.c, o, pick4(q.c, rho, rho * u, rho * v, p / (g - 1) + 0.5 * rho * (u * u + v * v)), gd);
}

// reflect the normal velocity and store conserved values, GFM_Bound.cpp:219-228
__device__ __forceinline__ void store_reflected(double *dst, long long o, const GridDesc &gd, const Quad &q, double g,
                                                double nx, double ny, double rho_w, double u_w, double v_w,
                                                double p_w)
{
    double u_n = u_w * nx + v_w * ny;
    double u_t = u_w * ny - v_w * nx;
    u_n = -u_n;
    u_w = u_n * nx + u_t * ny;
    v_w = u_n * ny - u_t * nx;
    store_conserved(dst, o, gd, q, g, rho_w, u_w, v_w, p_w);
}

__device__ void fill_ghost(const FillArgs &a, const View &v, double *dst, const GhostRec &h, const Quad &q)
{
    const double g = a.g.gamma;
    const long long o = (long long)h.j * a.g.pitch + h.i;
    if (a.bc == BC_IDW)
    {
        double w[4];
        idw_average(v, q, h.idx, h.idy, h.snext, h.w, g, w);
        store_reflected(dst, o, a.g, q, g, h.nx, h.ny, w[0], w[1], w[2], w[3]);
    }
    else if (a.bc == BC_LINEAR || a.bc == BC_RIEMANNGFM)
    {
        // LinearBaseGFM/GFM_Bound.cpp:83-575: one corner's primitives (zeros
        // if none is fluid); pick p is bracket corner p - 1
        double rho = 0, u = 0, w = 0, p = 0;
        if (h.pick > 0)
        {
            const int ci = (h.pick == 1 || h.pick == 2) ? h.idx : h.idx + 1;
            const int cj = (h.pick == 1 || h.pick == 4) ? h.idy : h.idy + 1;
            prim(v, ci, cj, (h.snext >> (h.pick - 1)) & 1, g, rho, u, w, p);
        }
        store_reflected(dst, o, a.g, q, g, h.nx, h.ny, rho, u, w, p);
    }
    else
    {
        // BCGFM/BCGFM_Bound.cpp:89-175 and HBCGFM_Bound.cpp (pure mirror when |phi| > delta)
        double wi[4], we[4];
        idw_average(v, q, h.idx, h.idy, h.snext, h.w, g, wi);
        idw_average(v, q, h.idx2, h.idy2, h.snext >> 4, h.w2, g, we);
        const double nx = h.nx, ny = h.ny, delta = h.delta, R_E = h.delta, R_G = h.rg;
        double u_n_i = wi[1] * nx + wi[2] * ny;
        double u_t_i = wi[1] * ny - wi[2] * nx;
        double u_n_e = we[1] * nx + we[2] * ny;
        double u_t_e = we[1] * ny - we[2] * nx;
        double rho_m, p_m, u_t_m, u_n_m;
        if (a.bc == BC_HBCGFM && h.hmirror)
        {
            rho_m = wi[0];
            p_m = wi[3];
            u_t_m = u_t_i;
            u_n_m = -u_n_i;
        }
        else
        {
            rho_m = (wi[0] * ((delta + R_E) * (delta + R_E) - R_G * R_G) - we[0] * (delta * delta - R_G * R_G)) / (R_E * R_E + 2 * delta * R_E);
            p_m = (wi[3] * ((delta + R_E) * (delta + R_E) - R_G * R_G) - we[3] * (delta * delta - R_G * R_G)) / (R_E * R_E + 2 * delta * R_E);
            u_t_m = (u_t_i * ((delta + R_E) * (delta + R_E) - R_G * R_G) - u_t_e * (delta * delta - R_G * R_G)) / (R_E * R_E + 2 * delta * R_E);
            u_n_m = -(u_n_i * ((delta + R_E) * (delta + R_E) - R_G * R_G) - u_n_e * (delta * delta - R_G * R_G)) / (R_E * R_E + 2 * delta * R_E);
        }
        double u_m = u_n_m * nx + u_t_m * ny;
        double v_m = u_n_m * ny - u_t_m * nx;
        store_conserved(dst, o, a.g, q, g, rho_m, u_m, v_m, p_m);
    }
}

// What one domain-edge cell copies: Global_Boundary, transmissive x /
// reflective y (Test/Sod/Global_Boudary.cpp:23-75), or the periodic harness
// plug-in; the cells enumerate row ghosts then column ghosts.
struct RingPlan
{
    long long o;      // the edge cell
    long long s0, s1; // sources: s0 every component (a wall row: all but v), s1 a wall row's mirrored v
    bool n0, n1;      // the source is read from the new state
    int kind;         // RING_COPY, RING_WALL_ROW, RING_INITIAL
    int ic;           // RING_INITIAL: the row of the initial ring values
    bool raw;         // periodic FP32 form: the (hi, lo) pair copied as it is
};
enum { RING_COPY = 0, RING_WALL_ROW = 1, RING_INITIAL = 2 };

__device__ __forceinline__ RingPlan ring_plan(const FillArgs &a, long long q)
{
    const GridDesc &g = a.g;
    const int ng = g.ng, n_x = g.n_x, n_y = g.n_y, N = g.N, pitch = g.pitch;
    auto interior = [&](int i, int j) { return i >= ng && i < ng + n_x && j >= ng && j < ng + n_y; };
    // S of (i, j) from the new state: an updated interior cell
    auto from_next = [&](int i, int j) {
        return interior(i, j) && updated_cell(a.type[(long long)j * pitch + i]);
    };
    const long long nrow = 2LL * ng * n_x;
    int i, j;
    bool row;
    if (q < nrow)
    {
        row = true;
        int r = (int)(q / n_x);
        i = ng + (int)(q - (long long)r * n_x);
        j = (r < ng) ? r : n_y + r; // r in [0, 2ng): bottom rows then top rows
    }
    else
    {
        row = false;
        long long qq = q - nrow;
        int c = (int)(qq / N);
        j = (int)(qq - (long long)c * N);
        i = (c < ng) ? c : n_x + c;
    }
    RingPlan p{};
    p.o = (long long)j * pitch + i;
    p.kind = RING_COPY;
    if (a.gb == GB_PERIODIC)
    {
        // rows from the opposite interior rows of S; columns from the opposite
        // columns of the updated state (corners from the diagonal)
        int si = i, sj = j;
        if (!row)
            si = (i < ng) ? i + n_x : i - n_x;
        if (j < ng)
            sj = j + n_y;
        else if (j >= n_y + ng)
            sj = j - n_y;
        const bool src_interior_row = (sj >= ng && sj < ng + n_y);
        p.s0 = (long long)sj * pitch + si;
        // an interior row's column ghosts copy the new state after the fill
        p.n0 = (row || !src_interior_row || (sj != j)) ? from_next(si, sj) : true;
        // a round trip through FP64 re-splits a pair whose lo is exactly half an ulp
        p.raw = g.f32;
    }
    else if (row)
    {
        const bool bottom = j < ng;
        const int src = bottom ? 2 * ng - 1 : n_y + ng - 1;
        const int mir = bottom ? 2 * ng - j - 1 : 2 * (n_y + ng) - 1 - j;
        p.kind = RING_WALL_ROW;
        p.s0 = (long long)src * pitch + i;
        p.s1 = (long long)mir * pitch + i;
        p.n0 = from_next(i, src);
        p.n1 = from_next(i, mir);
    }
    else
    {
        const int si = (i < ng) ? ng : n_x + ng - 1;
        const bool ghost_row = (j < ng || j >= n_y + ng);
        if (ghost_row && a.bc == BC_REGULAR)
        {
            const int side = (i < ng) ? 0 : 1;
            const int rr = (j < ng) ? j : j - n_y; // [0, 2ng)
            p.kind = RING_INITIAL;
            p.ic = side * 2 * ng + rr;
        }
        else
        {
            p.s0 = (long long)j * pitch + si;
            p.n0 = from_next(si, j);
        }
    }
    return p;
}

__device__ __forceinline__ void ring_apply(const FillArgs &a, const View &v, double *dst, const RingPlan &p)
{
    if (p.raw)
    {
        const float *sf = reinterpret_cast<const float *>(p.n0 ? v.next : v.prev);
        float *df = reinterpret_cast<float *>(dst);
        for (int k = 0; k < 8; k++)
            df[k * a.g.plane + p.o] = sf[k * a.g.plane + p.s0];
        return;
    }
    double out[4];
    if (p.kind == RING_INITIAL)
    {
        for (int k = 0; k < 4; k++)
            out[k] = a.ring_ic[p.ic * 4 + k];
    }
    else
    {
        for (int k = 0; k < 4; k++)
            out[k] = v.S(p.s0, k, p.n0);
        if (p.kind == RING_WALL_ROW)
            out[2] = -v.S(p.s1, 2, p.n1);
    }
    for (int k = 0; k < 4; k++)
        state_st(dst, k, p.o, out[k], a.g);
}

// the state buffer the pass writes; run: the pass has work (a step completed,
// the initial fill, or a step in flight)
__device__ __forceinline__ int fill_cur(const FillArgs &a, bool &run)
{
    const DevState *st = a.st;
    if (a.pre_flip)
    {
        run = true;
        return st->step_cur ^ 1; // the buffer the step in flight writes
    }
    run = a.init_mode || st->fill_pending;
    return st->cur;
}

// one FILL_THREADS block of a case's boundary pass: blocks [0, gblocks) fill
// the ghost list, the rest the domain edges.  What a cell reads is settled
// (record, types) before the device state names the buffers.
__device__ __forceinline__ void fill_block(const FillArgs &a, int vb, int do_ghosts, int do_ring)
{
    const int gblocks = do_ghosts ? ghost_blocks(a.nghost - a.ghost0) : 0;
    bool run;
    if (vb < gblocks)
    {
        static_assert(FILL_THREADS % GHOST_LANES == 0 && 32 % GHOST_LANES == 0, "a quad sits in one warp");
        const int t = a.ghost0 + (vb * FILL_THREADS + (int)threadIdx.x) / GHOST_LANES;
        if (t >= a.nghost) // the quad's lanes share t: all four fill or none
            return;
        const GhostRec h = a.ghosts[t];
        const int cur = fill_cur(a, run);
        if (!run)
            return;
        const int lane = (int)(threadIdx.x & 31);
        const Quad q{((1u << GHOST_LANES) - 1) << (lane & ~(GHOST_LANES - 1)), lane & (GHOST_LANES - 1)};
        const View v{cur ? a.buf1 : a.buf0, cur ? a.buf0 : a.buf1, a.g};
        fill_ghost(a, v, cur ? a.buf1 : a.buf0, h, q);
        return;
    }
    if (!do_ring)
        return;
    const long long q = (long long)(vb - gblocks) * FILL_THREADS + threadIdx.x;
    const long long nring = 2LL * a.g.ng * a.g.n_x + 2LL * a.g.ng * a.g.N;
    if (q >= nring)
        return;
    const RingPlan p = ring_plan(a, q);
    const int cur = fill_cur(a, run);
    if (!run)
        return;
    const View v{cur ? a.buf1 : a.buf0, cur ? a.buf0 : a.buf1, a.g};
    ring_apply(a, v, cur ? a.buf1 : a.buf0, p);
}

__global__ void __launch_bounds__(FILL_THREADS) fill_kernel(const FillArgs a)
{
    fill_block(a, blockIdx.x, a.do_ghosts, a.do_ring);
}

void launch_fill_ghosts(const FillArgs &a, int g0, int g1, cudaStream_t s)
{
    if (g1 <= g0)
        return;
    FillArgs b = a;
    b.pre_flip = 1;
    b.ghost0 = g0;
    b.nghost = g1; // records [ghost0, nghost)
    b.do_ghosts = 1;
    b.do_ring = 0;
    fill_kernel<<<ghost_blocks(g1 - g0), FILL_THREADS, 0, s>>>(b);
    count_launch();
}

void launch_fill(const FillArgs &a, cudaStream_t s)
{
    int gblocks = a.do_ghosts ? ghost_blocks(a.nghost) : 0;
    long long nring = 2LL * a.g.ng * a.g.n_x + 2LL * a.g.ng * a.g.N;
    int rblocks = a.do_ring ? (int)((nring + FILL_THREADS - 1) / FILL_THREADS) : 0;
    if (gblocks + rblocks == 0)
        return;
    fill_kernel<<<gblocks + rblocks, FILL_THREADS, 0, s>>>(a);
    count_launch();
}

// Boundary pass of every case of a batch, phase 0 or 1.  Phase 0: ghost
// list (ghost-fluid variants) and domain edges; phase 1: the domain edges of
// periodic ghost-fluid cases, which copy interior cells filled in phase 0.
// The (slot, block) table lists only blocks with work; persistent CTAs walk it.
__global__ void __launch_bounds__(FILL_THREADS) batch_fill_kernel(const BatchHeader *__restrict__ h, int phase)
{
    const int n = h->nfill[phase];
    const int2 *tab = h->fill[phase];
    for (int b = blockIdx.x; b < n; b += gridDim.x)
    {
        const int2 e = tab[b];
        const FillArgs &a = h->cases[e.x].f;
        const bool gfm = a.bc != BC_REGULAR;
        const bool split = gfm && a.gb == GB_PERIODIC;
        if (phase == 0)
            fill_block(a, e.y, gfm ? 1 : 0, split ? 0 : 1);
        else
            fill_block(a, e.y, 0, 1);
    }
}

void launch_batch_fill(const BatchHeader *h, int phase, int grid, cudaStream_t s)
{
    batch_fill_kernel<<<grid, FILL_THREADS, 0, s>>>(h, phase);
    count_launch();
}

// per-slot progress for the host (one thread per slot)
__global__ void batch_progress_kernel(const BatchHeader *__restrict__ h, BatchProgress *out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= h->nslots)
        return;
    const BatchCase &c = h->cases[k];
    BatchProgress p{};
    if (c.s.st)
    {
        const DevState *st = c.s.st;
        p.now_t = st->now_t;
        p.dt = st->dt;
        p.mass = st->mass;
        p.mass_start = st->mass_start;
        p.iter = st->iter;
        p.status = st->status;
        p.nan_cells = st->nan_cells;
        p.active = (st->now_t < c.s.t_end && st->iter < c.s.max_iter) ? 1 : 0;
    }
    out[k] = p;
}

void launch_batch_progress(const BatchHeader *h, int nslots_max, BatchProgress *out, cudaStream_t s)
{
    batch_progress_kernel<<<(nslots_max + 127) / 128, 128, 0, s>>>(h, out);
    count_launch();
}

// ---------------------------------------------------------------- reduction

// ComputeDt (Src/Base/Common/ComputeDt.cpp:4-51) and CaculateMass
// (Src/Utils/CaculateMass.cpp:5-42) of one state, without stepping.
__global__ void __launch_bounds__(TILE_X *TILE_Y) reduce_kernel(const ReduceArgs a)
{
    const GridDesc &g = a.g;
    const int i = g.ng + blockIdx.x * TILE_X + (threadIdx.x % TILE_X);
    const int j = g.ng + blockIdx.y * TILE_Y + (threadIdx.x / TILE_X);
    CellStats cs;
    if (i < g.ng + g.n_x && j < g.ng + g.n_y)
    {
        long long o = (long long)j * g.pitch + i;
        if (a.type[o] == CELL_FLUID)
        {
            double v[4];
            for (int k = 0; k < 4; k++)
                v[k] = state_ld(a.u, k, o, g);
            cell_stats(v, g.gamma, g.dx, g.dy, cs);
        }
        else if (a.type[o] == CELL_CUT && a.alpha)
        {
            // a cut cell: mass alpha rho; the CFL maxima only where alpha >= 0.5
            // (smaller cells are mixed with their neighbours)
            double v[4];
            for (int k = 0; k < 4; k++)
                v[k] = state_ld(a.u, k, o, g);
            CellStats c1;
            cell_stats(v, g.gamma, g.dx, g.dy, c1);
            cs.mass += a.alpha[o] * c1.mass;
            cs.nans += c1.nans;
            if (a.alpha[o] >= 0.5)
            {
                cs.a2max = fmax(cs.a2max, c1.a2max);
                cs.umax = fmax(cs.umax, c1.umax);
                cs.vmax = fmax(cs.vmax, c1.vmax);
            }
        }
    }
    block_reduce_finalize<TILE_X * TILE_Y>(cs, a.st, a.partial, g, false, a.set_start, gridDim.x * gridDim.y,
                                           blockIdx.y * gridDim.x + blockIdx.x);
}

void launch_reduce(const ReduceArgs &a, int, cudaStream_t s)
{
    dim3 grid((a.g.n_x + TILE_X - 1) / TILE_X, (a.g.n_y + TILE_Y - 1) / TILE_Y);
    reduce_kernel<<<grid, TILE_X * TILE_Y, 0, s>>>(a);
    count_launch();
}

// ---------------------------------------------------------------- layouts

__global__ void aos_to_soa_kernel(const double *__restrict__ aos, double *__restrict__ soa, GridDesc g)
{
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)g.M * g.N)
        return;
    int j = (int)(c / g.M), i = (int)(c - (long long)j * g.M);
    long long o = (long long)j * g.pitch + i;
    for (int k = 0; k < 4; k++)
        state_st(soa, k, o, aos[c * 4 + k], g);
}

__global__ void soa_to_aos_kernel(const double *__restrict__ soa, double *__restrict__ aos, GridDesc g)
{
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)g.M * g.N)
        return;
    int j = (int)(c / g.M), i = (int)(c - (long long)j * g.M);
    long long o = (long long)j * g.pitch + i;
    for (int k = 0; k < 4; k++)
        aos[c * 4 + k] = state_ld(soa, k, o, g);
}

void launch_aos_to_soa(const double *aos, double *soa, const GridDesc &g, cudaStream_t s)
{
    long long n = (long long)g.M * g.N;
    aos_to_soa_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(aos, soa, g);
    count_launch();
}

void launch_soa_to_aos(const double *soa, double *aos, const GridDesc &g, cudaStream_t s)
{
    long long n = (long long)g.M * g.N;
    soa_to_aos_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(soa, aos, g);
    count_launch();
}

// the same conversions over rows [r0, r1), with the current buffer taken from
// the device state when the kernel runs (so a step queued before it counts)
struct BoxArgs
{
    HostBoxes bx;
    long long start[6]; // cells before each box
};

__global__ void aos_to_cur_boxes_kernel(const double *__restrict__ aos, double *b0, double *b1, DevState *st,
                                        GridDesc g, const BoxArgs a, int first, int both)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (first && q == 0)
        st->step_cur = st->cur; // read by the snapshot conversions of this step
    if (q >= a.start[a.bx.n])
        return;
    int b = 0;
    while (q >= a.start[b + 1])
        b++;
    const int w = a.bx.c1[b] - a.bx.c0[b];
    const long long r = q - a.start[b];
    const int j = a.bx.r0[b] + (int)(r / w), i = a.bx.c0[b] + (int)(r % w);
    const long long c = (long long)j * g.M + i, o = (long long)j * g.pitch + i;
    double *soa = st->cur ? b1 : b0;
    double *other = st->cur ? b0 : b1;
    for (int k = 0; k < 4; k++)
    {
        const double v = aos[c * 4 + k];
        state_st(soa, k, o, v, g);
        if (both)
            state_st(other, k, o, v, g);
    }
}

void launch_aos_to_cur_boxes(const double *aos, double *b0, double *b1, const DevState *st, const GridDesc &g,
                             const HostBoxes &bx, bool first, bool both, cudaStream_t s)
{
    BoxArgs a;
    a.bx = bx;
    a.start[0] = 0;
    for (int b = 0; b < bx.n; b++)
        a.start[b + 1] = a.start[b] + (long long)(bx.r1[b] - bx.r0[b]) * (bx.c1[b] - bx.c0[b]);
    const long long n = a.start[bx.n];
    if (n <= 0)
        return;
    aos_to_cur_boxes_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(aos, b0, b1, const_cast<DevState *>(st), g,
                                                                        a, first ? 1 : 0, both ? 1 : 0);
    count_launch();
}

__global__ void cur_rows_to_aos_kernel(const double *b0, const double *b1, const DevState *__restrict__ st,
                                       double *__restrict__ aos, GridDesc g, int r0, int r1)
{
    long long c = (long long)r0 * g.M + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)r1 * g.M)
        return;
    const double *soa = st->cur ? b1 : b0;
    int j = (int)(c / g.M), i = (int)(c - (long long)j * g.M);
    long long o = (long long)j * g.pitch + i;
    for (int k = 0; k < 4; k++)
        aos[c * 4 + k] = state_ld(soa, k, o, g);
}

// one cell of a host-layout array: two 16-byte stores where the array allows
// (page-locked host memory written over the host link moves in whole sectors)
__device__ __forceinline__ void store_aos_cell(double *aos, long long c, const double v[4])
{
    double *p = aos + c * 4;
    if ((reinterpret_cast<uintptr_t>(aos) & 15) == 0)
    {
        reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
    }
    else
        for (int k = 0; k < 4; k++)
            p[k] = v[k];
}

__global__ void snapshot_rows_to_aos_kernel(const double *b0, const double *b1, const DevState *__restrict__ st,
                                            const uint8_t *__restrict__ type, double *__restrict__ aos, GridDesc g,
                                            int r0, int r1, int c0, int c1)
{
    const int w = c1 - c0;
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)(r1 - r0) * w)
        return;
    const int cur = st->step_cur;
    int j = r0 + (int)(q / w), i = c0 + (int)(q % w);
    long long c = (long long)j * g.M + i;
    long long o = (long long)j * g.pitch + i;
    const bool out = type[o] == CELL_FLUID ||
                     (type[o] == CELL_GHOST && i >= g.ng && i < g.ng + g.n_x && j >= g.ng && j < g.ng + g.n_y);
    const double *src = out ? (cur ? b0 : b1) : (cur ? b1 : b0);
    double v[4];
    for (int k = 0; k < 4; k++)
        v[k] = state_ld(src, k, o, g);
    store_aos_cell(aos, c, v);
}

void launch_snapshot_to_aos_rows(const double *b0, const double *b1, const DevState *st, const uint8_t *type,
                                 double *aos, const GridDesc &g, int r0, int r1, int c0, int c1, cudaStream_t s)
{
    long long n = (long long)(r1 - r0) * (c1 - c0);
    if (r1 <= r0 || c1 <= c0)
        return;
    snapshot_rows_to_aos_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b0, b1, st, type, aos, g, r0, r1, c0,
                                                                           c1);
    count_launch();
}

// the domain ring (rows below and above the interior, then the columns left
// and right of it) from the current buffer into the host-layout array
__global__ void ring_to_aos_kernel(const double *b0, const double *b1, const DevState *__restrict__ st,
                                   double *__restrict__ aos, GridDesc g)
{
    const long long nrow = 2LL * g.ng * g.M, ncol = 2LL * g.ng * g.n_y;
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrow + ncol)
        return;
    int i, j;
    if (q < nrow)
    {
        const int r = (int)(q / g.M);
        i = (int)(q - (long long)r * g.M);
        j = (r < g.ng) ? r : g.n_y + r;
    }
    else
    {
        const long long qq = q - nrow;
        const int r = (int)(qq / (2 * g.ng)), s = (int)(qq - (long long)r * 2 * g.ng);
        j = g.ng + r;
        i = (s < g.ng) ? s : g.n_x + s;
    }
    const double *src = st->cur ? b1 : b0;
    const long long o = (long long)j * g.pitch + i, c = (long long)j * g.M + i;
    double v[4];
    for (int k = 0; k < 4; k++)
        v[k] = state_ld(src, k, o, g);
    store_aos_cell(aos, c, v);
}

void launch_ring_to_aos(const double *b0, const double *b1, const DevState *st, double *aos, const GridDesc &g,
                        cudaStream_t s)
{
    const long long n = 2LL * g.ng * g.M + 2LL * g.ng * g.n_y;
    ring_to_aos_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b0, b1, st, aos, g);
    count_launch();
}


void launch_cur_to_aos_rows(const double *b0, const double *b1, const DevState *st, double *aos, const GridDesc &g,
                            int r0, int r1, cudaStream_t s)
{
    long long n = (long long)(r1 - r0) * g.M;
    if (n <= 0)
        return;
    cur_rows_to_aos_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b0, b1, st, aos, g, r0, r1);
    count_launch();
}

} // namespace ibtfo
