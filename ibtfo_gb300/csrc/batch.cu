// Batches: many cases of uneven grid sizes stepped together.
//
// No counterpart in the reference (its drivers, e.g. Test/Sod/Sod.cpp:108-181,
// advance one case per process).  Cases keep their own buffers, geometry,
// device state (dt, now_t, iter) and loop condition; the batch owns one tile
// table over all of them and, per step, launches
//   1. the persistent sweep (resident CTAs walk the tile table;
//      batch_impl.cuh), which also computes each case's next dt,
//   2. the boundary pass of every case (batch_fill_kernel, phase 0), and
//   3. phase 1 (domain edges of periodic ghost-fluid cases) when a case needs it,
// captured as a CUDA graph of `graph_steps` steps.  The kernels read the
// tables through a fixed device header, so cases join and leave between
// graph launches without a new capture: the host rewrites the tables with
// stream-ordered copies from double-buffered pinned staging.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ibtfo.h"
#include "internal.h"
#include "physics.cuh"

namespace ibtfo {

BatchKernel batch_kernel_muscl_fast(int, int, int);
BatchKernel batch_kernel_mhm_fast(int, int, int);
BatchKernel batch_kernel_godunov_fast(int, int, int);
BatchKernel batch_kernel_muscl_f32(int, int, int);
BatchKernel batch_kernel_mhm_f32(int, int, int);
BatchKernel batch_kernel_godunov_f32(int, int, int);

BatchKernel batch_kernel(int scheme, int riemann, int limiter, int precision, int shape)
{
    if (precision == 1)
    {
        switch (scheme)
        {
        case MHM: return batch_kernel_mhm_fast(riemann, limiter, shape);
        case GODUNOV: return batch_kernel_godunov_fast(riemann, limiter, shape);
        default: return batch_kernel_muscl_fast(riemann, limiter, shape);
        }
    }
    if (precision == 2)
    {
        switch (scheme)
        {
        case MHM: return batch_kernel_mhm_f32(riemann, limiter, shape);
        case GODUNOV: return batch_kernel_godunov_f32(riemann, limiter, shape);
        default: return batch_kernel_muscl_f32(riemann, limiter, shape);
        }
    }
    return {nullptr, nullptr};
}

} // namespace ibtfo

using namespace ibtfo;

namespace {

// device arrays of a batch, grown by doubling (stream-ordered)
template <typename T>
struct DevArray
{
    T *p = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t n, cudaStream_t s)
    {
        if (n <= cap)
            return cudaSuccess;
        size_t c = std::max<size_t>(n, std::max<size_t>(64, cap * 2));
        T *q = nullptr;
        cudaError_t e = cudaMallocAsync(&q, sizeof(T) * c, s);
        if (e != cudaSuccess)
            return e;
        if (p)
            cudaFreeAsync(p, s);
        p = q;
        cap = c;
        return cudaSuccess;
    }
    void release(cudaStream_t s)
    {
        if (p)
            cudaFreeAsync(p, s);
        p = nullptr;
        cap = 0;
    }
};

// pinned staging of one table upload
struct Staging
{
    unsigned char *p = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr; // the copies out of this staging have run
    bool pending = false;
};

struct Slot
{
    ibtfo_case *c = nullptr;
    std::vector<unsigned> tiles; // active tiles of the batch's tile shape
    int fill_blocks[2] = {0, 0};
};

} // namespace

struct ibtfo_batch
{
    ibtfo_batch_config cfg;
    int device = 0;
    int sms = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    BatchKernel kern{nullptr, nullptr};
    int occupancy = 0; // resident sweep CTAs per SM for the current shape
    int grid_sweep = 0, grid_fill = 0;
    std::vector<Slot> slots;
    bool dirty = true;
    bool need_phase1 = false;
    // device tables
    BatchHeader *d_hdr = nullptr;
    DevArray<BatchCase> d_cases;
    DevArray<BatchTile> d_tiles;
    DevArray<int2> d_fill[2];
    DevArray<double> d_partial;
    DevArray<BatchProgress> d_prog;
    Staging stage[2];
    int next_stage = 0;
    BatchProgress *h_prog = nullptr;
    int h_prog_cap = 0;
    cudaEvent_t prog_done = nullptr;
    int prog_n = 0;
    cudaGraphExec_t graph = nullptr;
    bool graph_phase1 = false;
};

namespace {

ibtfo_status bfail(ibtfo_status s, const std::string &m)
{
    set_last_error(m.c_str());
    return s;
}

ibtfo_status bcuda(cudaError_t e, const char *what)
{
    cudaGetLastError();
    return bfail(e == cudaErrorMemoryAllocation ? IBTFO_ENOMEM : IBTFO_ECUDA,
                 std::string(what) + ": " + cudaGetErrorString(e));
}

#define BCK(call)                                  \
    do                                             \
    {                                              \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess)                     \
            return bcuda(e_, #call);               \
    } while (0)

void drop_graph(ibtfo_batch *b)
{
    if (b->graph)
        cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
}

int fill_blocks(const FillArgs &f, int phase)
{
    const bool gfm = f.bc != BC_REGULAR;
    const bool split = gfm && f.gb == GB_PERIODIC;
    const long long nring = 2LL * f.g.ng * f.g.n_x + 2LL * f.g.ng * f.g.N;
    const int rblocks = (int)((nring + FILL_THREADS - 1) / FILL_THREADS);
    const int gblocks = ghost_blocks(f.nghost);
    if (phase == 0)
        return (gfm ? gblocks : 0) + (split ? 0 : rblocks);
    return split ? rblocks : 0;
}

ibtfo_status set_shape(ibtfo_batch *b, int shape, int ctas)
{
    BatchKernel k = batch_kernel(b->cfg.scheme, b->cfg.riemann, b->cfg.limiter, b->cfg.precision, shape);
    if (!k.launch)
        return bfail(IBTFO_EINVAL, "no batched kernel for this scheme/riemann/limiter/precision");
    const int occ = k.prepare();
    if (occ <= 0)
        return bcuda(cudaGetLastError(), "batched sweep occupancy");
    b->kern = k;
    b->occupancy = occ;
    b->cfg.tile_shape = shape;
    b->cfg.ctas_per_sm = (ctas <= 0 || ctas > occ) ? occ : ctas;
    b->grid_sweep = b->sms * b->cfg.ctas_per_sm;
    drop_graph(b);
    b->dirty = true;
    // tile lists of the new shape
    for (Slot &s : b->slots)
    {
        if (!s.c)
            continue;
        SweepArgs sa;
        FillArgs fa;
        int sch, rie, lim, prec, has;
        case_batch_view(s.c, &sa, &fa, &sch, &rie, &lim, &prec, &has);
        int rc = active_tile_list(sa.g, sa.type, shape_tx(shape), shape_ty(shape), s.tiles, case_stream(s.c));
        if (rc)
            return rc == 2 ? bfail(IBTFO_ENOMEM, "tile list") : bcuda(cudaGetLastError(), "tile list");
    }
    return IBTFO_OK;
}

// rebuild the tables on the host and copy them to the device (stream-ordered)
ibtfo_status upload(ibtfo_batch *b)
{
    const int nslots = (int)b->slots.size();
    std::vector<BatchCase> cases(nslots);
    std::vector<BatchTile> tiles;
    std::vector<int2> fill[2];
    std::vector<long long> poff(nslots, 0);
    long long ptot = 0;
    b->need_phase1 = false;
    for (int k = 0; k < nslots; k++)
    {
        Slot &s = b->slots[k];
        BatchCase &bc = cases[k];
        std::memset(&bc, 0, sizeof(bc));
        bc.slot = k;
        if (!s.c)
            continue;
        int sch, rie, lim, prec, has;
        case_batch_view(s.c, &bc.s, &bc.f, &sch, &rie, &lim, &prec, &has);
        bc.f.init_mode = 0;
        bc.ntiles = (int)s.tiles.size();
        poff[k] = ptot;
        ptot += bc.ntiles;
        for (int t = 0; t < bc.ntiles; t++)
            tiles.push_back(make_uint4(s.tiles[t], (unsigned)t, (unsigned)k, 0u));
        for (int ph = 0; ph < 2; ph++)
        {
            s.fill_blocks[ph] = fill_blocks(bc.f, ph);
            for (int v = 0; v < s.fill_blocks[ph]; v++)
                fill[ph].push_back(make_int2(k, v));
        }
        if (s.fill_blocks[1])
            b->need_phase1 = true;
    }
    cudaStream_t st = b->stream;
    BCK(b->d_cases.reserve(std::max(1, nslots), st));
    BCK(b->d_tiles.reserve(std::max<size_t>(1, tiles.size()), st));
    BCK(b->d_fill[0].reserve(std::max<size_t>(1, fill[0].size()), st));
    BCK(b->d_fill[1].reserve(std::max<size_t>(1, fill[1].size()), st));
    BCK(b->d_partial.reserve(std::max<long long>(1, ptot), st));
    BCK(b->d_prog.reserve(std::max(1, nslots), st));
    for (int k = 0; k < nslots; k++)
        if (b->slots[k].c)
            cases[k].s.partial = b->d_partial.p + poff[k];

    BatchHeader h{};
    h.cases = b->d_cases.p;
    h.tiles = b->d_tiles.p;
    h.fill[0] = b->d_fill[0].p;
    h.fill[1] = b->d_fill[1].p;
    h.ntiles = (int)tiles.size();
    h.nfill[0] = (int)fill[0].size();
    h.nfill[1] = (int)fill[1].size();
    h.nslots = nslots;

    // pinned staging (double-buffered: wait for the upload two rebuilds ago)
    const size_t a0 = sizeof(BatchHeader), a1 = sizeof(BatchCase) * cases.size(),
                 a2 = sizeof(BatchTile) * tiles.size(), a3 = sizeof(int2) * fill[0].size(),
                 a4 = sizeof(int2) * fill[1].size();
    auto align = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t need = align(a0) + align(a1) + align(a2) + align(a3) + align(a4);
    Staging &sg = b->stage[b->next_stage];
    b->next_stage ^= 1;
    if (sg.pending)
    {
        BCK(cudaEventSynchronize(sg.done));
        sg.pending = false;
    }
    if (sg.cap < need)
    {
        if (sg.p)
            cudaFreeHost(sg.p);
        sg.p = nullptr;
        sg.cap = 0;
        BCK(cudaMallocHost(&sg.p, need * 2));
        sg.cap = need * 2;
    }
    unsigned char *q = sg.p;
    auto put = [&](void *dst, const void *src, size_t n) -> cudaError_t {
        if (!n)
            return cudaSuccess;
        std::memcpy(q, src, n);
        cudaError_t e = cudaMemcpyAsync(dst, q, n, cudaMemcpyHostToDevice, st);
        q += align(n);
        return e;
    };
    BCK(put(b->d_cases.p, cases.data(), a1));
    BCK(put(b->d_tiles.p, tiles.data(), a2));
    BCK(put(b->d_fill[0].p, fill[0].data(), a3));
    BCK(put(b->d_fill[1].p, fill[1].data(), a4));
    BCK(put(b->d_hdr, &h, a0));
    BCK(cudaEventRecord(sg.done, st));
    sg.pending = true;
    b->dirty = false;
    if (b->graph && b->graph_phase1 != b->need_phase1)
        drop_graph(b);
    return IBTFO_OK;
}

// kernel launches of one step
int launches_per_step(const ibtfo_batch *b)
{
    return (b->cfg.time_advance == IBTFO_TIME_RK2 ? 2 : 1) * (b->need_phase1 ? 3 : 2);
}

void enqueue_steps(ibtfo_batch *b, int n)
{
    // Time = RK2: the first stage and its boundary pass, then the second
    // stage (which does the loop accounting) and its boundary pass, as the
    // one-case step does
    const bool rk2 = b->cfg.time_advance == IBTFO_TIME_RK2;
    for (int s = 0; s < n; s++)
        for (int stage = rk2 ? 1 : 0; stage <= (rk2 ? 2 : 0); stage++)
        {
            b->kern.launch(b->d_hdr, b->grid_sweep, b->stream, stage);
            count_launch();
            launch_batch_fill(b->d_hdr, 0, b->grid_fill, b->stream);
            if (b->need_phase1)
                launch_batch_fill(b->d_hdr, 1, b->grid_fill, b->stream);
        }
}

ibtfo_status build_graph(ibtfo_batch *b)
{
    cudaGraph_t g;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = ibtfo_launch_count();
    enqueue_steps(b, b->cfg.graph_steps);
    count_launch((int)(before - ibtfo_launch_count())); // replays are counted instead
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess)
        return bcuda(e, "batch graph capture");
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
        return bcuda(e, "batch graph instantiate");
    b->graph_phase1 = b->need_phase1;
    return IBTFO_OK;
}

} // namespace

extern "C" {

ibtfo_status ibtfo_batch_create(const ibtfo_batch_config *cfg, ibtfo_batch **out)
{
    if (!cfg || !out)
        return bfail(IBTFO_EINVAL, "null argument");
    *out = nullptr;
    const ibtfo_batch_config &k = *cfg;
    if (k.precision != IBTFO_PRECISION_FP64_FAST && k.precision != IBTFO_PRECISION_FP32_COMPENSATED)
        return bfail(IBTFO_EINVAL, "batches run the fp64_fast or FP32 compensated precision");
    if (k.scheme < 0 || k.scheme > 2 || k.riemann < 0 || k.riemann > 5 || k.limiter < 0 || k.limiter > 1)
        return bfail(IBTFO_EINVAL, "unknown scheme/riemann/limiter key (batches run MUSCL, MHM or Godunov)");
    if (k.tile_shape < 0 || k.tile_shape >= SHAPE_COUNT || k.ctas_per_sm < 0 || k.graph_steps < 0)
        return bfail(IBTFO_EINVAL, "bad tile_shape / ctas_per_sm / graph_steps");
    if (k.time_advance < 0 || k.time_advance > 1)
        return bfail(IBTFO_EINVAL, "unknown time_advance key");
    ibtfo_batch *b = new ibtfo_batch();
    b->cfg = k;
    if (b->cfg.graph_steps == 0)
        b->cfg.graph_steps = 16;
    cudaGetDevice(&b->device);
    cudaError_t e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMalloc(&b->d_hdr, sizeof(BatchHeader));
    if (e == cudaSuccess)
        e = cudaMemset(b->d_hdr, 0, sizeof(BatchHeader));
    for (int i = 0; i < 2 && e == cudaSuccess; i++)
        e = cudaEventCreateWithFlags(&b->stage[i].done, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&b->prog_done, cudaEventDisableTiming);
    if (e != cudaSuccess)
    {
        ibtfo_status s = bcuda(e, "ibtfo_batch_create");
        ibtfo_batch_destroy(b);
        return s;
    }
    b->stream = b->own;
    b->grid_fill = b->sms * 8;
    ibtfo_status s = set_shape(b, k.tile_shape, k.ctas_per_sm);
    if (s != IBTFO_OK)
    {
        ibtfo_batch_destroy(b);
        return s;
    }
    *out = b;
    return IBTFO_OK;
}

ibtfo_status ibtfo_batch_destroy(ibtfo_batch *b)
{
    if (!b)
        return IBTFO_OK;
    cudaSetDevice(b->device);
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    drop_graph(b);
    cudaStream_t s = b->own ? b->own : b->stream;
    b->d_cases.release(s);
    b->d_tiles.release(s);
    b->d_fill[0].release(s);
    b->d_fill[1].release(s);
    b->d_partial.release(s);
    b->d_prog.release(s);
    if (s)
        cudaStreamSynchronize(s);
    cudaFree(b->d_hdr);
    for (auto &sg : b->stage)
    {
        if (sg.p)
            cudaFreeHost(sg.p);
        if (sg.done)
            cudaEventDestroy(sg.done);
    }
    if (b->h_prog)
        cudaFreeHost(b->h_prog);
    if (b->prog_done)
        cudaEventDestroy(b->prog_done);
    if (b->own)
        cudaStreamDestroy(b->own);
    delete b;
    return IBTFO_OK;
}

ibtfo_status ibtfo_batch_set_stream(ibtfo_batch *b, void *stream)
{
    if (!b)
        return bfail(IBTFO_EINVAL, "null batch");
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->stream));
    b->stream = stream ? (cudaStream_t)stream : b->own;
    drop_graph(b);
    return IBTFO_OK;
}

ibtfo_status ibtfo_batch_add(ibtfo_batch *b, ibtfo_case *c, int *slot)
{
    if (!b || !c)
        return bfail(IBTFO_EINVAL, "null argument");
    if (case_device(c) != b->device)
        return bfail(IBTFO_EINVAL, "the case lives on another device");
    SweepArgs sa;
    FillArgs fa;
    int sch, rie, lim, prec, has;
    case_batch_view(c, &sa, &fa, &sch, &rie, &lim, &prec, &has);
    if (!has)
        return bfail(IBTFO_ESTATE, "no state: call ibtfo_set_state before adding the case");
    if (fa.bc == BC_CCM)
        return bfail(IBTFO_EINVAL, "cut-cell cases run one per launch (their mixing step is not batched)");
    if (case_time_advance(c) != b->cfg.time_advance)
        return bfail(IBTFO_EINVAL, "the case's Time key differs from the batch's");
    const int r0 = (rie == IBTFO_RIEMANN_HLLC) ? IBTFO_RIEMANN_HLL : rie;
    const int r1 = (b->cfg.riemann == IBTFO_RIEMANN_HLLC) ? IBTFO_RIEMANN_HLL : b->cfg.riemann;
    if (sch != b->cfg.scheme || r0 != r1 || lim != b->cfg.limiter || prec != b->cfg.precision)
        return bfail(IBTFO_EINVAL, "the case's scheme/riemann/limiter/precision differ from the batch's");
    for (const Slot &s : b->slots)
        if (s.c == c)
            return bfail(IBTFO_EINVAL, "the case is already in the batch");
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(case_stream(c)));
    Slot s;
    s.c = c;
    int rc = active_tile_list(sa.g, sa.type, shape_tx(b->cfg.tile_shape), shape_ty(b->cfg.tile_shape), s.tiles,
                              case_stream(c));
    if (rc)
        return rc == 2 ? bfail(IBTFO_ENOMEM, "tile list") : bcuda(cudaGetLastError(), "tile list");
    int k = 0;
    while (k < (int)b->slots.size() && b->slots[k].c)
        k++;
    if (k == (int)b->slots.size())
        b->slots.push_back(std::move(s));
    else
        b->slots[k] = std::move(s);
    b->dirty = true;
    if (slot)
        *slot = k;
    return IBTFO_OK;
}

ibtfo_status ibtfo_batch_remove(ibtfo_batch *b, int slot)
{
    if (!b || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].c)
        return bfail(IBTFO_EINVAL, "no case in that slot");
    cudaSetDevice(b->device);
    // steps already enqueued on the batch stream still read the case: order
    // the case's own stream (its transfers, its destruction) after them,
    // without blocking the host
    cudaEvent_t ev;
    BCK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, b->stream);
    if (e == cudaSuccess)
        e = cudaStreamWaitEvent(case_stream(b->slots[slot].c), ev, 0);
    cudaEventDestroy(ev);
    BCK(e);
    b->slots[slot] = Slot();
    while (!b->slots.empty() && !b->slots.back().c)
        b->slots.pop_back();
    b->dirty = true;
    return IBTFO_OK;
}

int ibtfo_batch_size(const ibtfo_batch *b)
{
    if (!b)
        return 0;
    int n = 0;
    for (const Slot &s : b->slots)
        n += s.c ? 1 : 0;
    return n;
}

int ibtfo_batch_num_slots(const ibtfo_batch *b) { return b ? (int)b->slots.size() : 0; }

ibtfo_case *ibtfo_batch_case(const ibtfo_batch *b, int slot)
{
    if (!b || slot < 0 || slot >= (int)b->slots.size())
        return nullptr;
    return b->slots[slot].c;
}

ibtfo_status ibtfo_batch_advance(ibtfo_batch *b, int nsteps)
{
    if (!b)
        return bfail(IBTFO_EINVAL, "null batch");
    if (nsteps < 0)
        return bfail(IBTFO_EINVAL, "nsteps < 0");
    cudaSetDevice(b->device);
    if (b->dirty)
    {
        ibtfo_status s = upload(b);
        if (s != IBTFO_OK)
            return s;
    }
    int left = nsteps;
    const int per_step = launches_per_step(b);
    if (left >= b->cfg.graph_steps)
    {
        if (!b->graph)
        {
            ibtfo_status s = build_graph(b);
            if (s != IBTFO_OK)
                return s;
        }
        while (left >= b->cfg.graph_steps)
        {
            BCK(cudaGraphLaunch(b->graph, b->stream));
            count_launch(b->cfg.graph_steps * per_step);
            left -= b->cfg.graph_steps;
        }
    }
    enqueue_steps(b, left);
    BCK(cudaGetLastError());
    return IBTFO_OK;
}

ibtfo_status ibtfo_batch_progress_enqueue(ibtfo_batch *b)
{
    if (!b)
        return bfail(IBTFO_EINVAL, "null batch");
    cudaSetDevice(b->device);
    if (b->dirty)
    {
        ibtfo_status s = upload(b);
        if (s != IBTFO_OK)
            return s;
    }
    const int n = (int)b->slots.size();
    if (n > b->h_prog_cap)
    {
        if (b->prog_n)
            BCK(cudaEventSynchronize(b->prog_done));
        if (b->h_prog)
            cudaFreeHost(b->h_prog);
        b->h_prog = nullptr;
        b->h_prog_cap = 0;
        BCK(cudaMallocHost(&b->h_prog, sizeof(BatchProgress) * (size_t)std::max(64, 2 * n)));
        b->h_prog_cap = std::max(64, 2 * n);
    }
    b->prog_n = n;
    if (n)
    {
        launch_batch_progress(b->d_hdr, n, b->d_prog.p, b->stream);
        BCK(cudaMemcpyAsync(b->h_prog, b->d_prog.p, sizeof(BatchProgress) * n, cudaMemcpyDeviceToHost, b->stream));
    }
    BCK(cudaEventRecord(b->prog_done, b->stream));
    return IBTFO_OK;
}

ibtfo_status ibtfo_batch_progress_read(ibtfo_batch *b, ibtfo_progress *out, int *active, int n, int wait)
{
    if (!b || (n > 0 && !out))
        return bfail(IBTFO_EINVAL, "null argument");
    cudaSetDevice(b->device);
    if (!wait)
    {
        cudaError_t q = cudaEventQuery(b->prog_done);
        if (q == cudaErrorNotReady)
            return bfail(IBTFO_ETIMEOUT, "progress not ready");
        BCK(q);
    }
    else
        BCK(cudaEventSynchronize(b->prog_done));
    for (int k = 0; k < n; k++)
    {
        ibtfo_progress &p = out[k];
        std::memset(&p, 0, sizeof(p));
        if (k >= b->prog_n)
        {
            if (active)
                active[k] = 0;
            continue;
        }
        const BatchProgress &q = b->h_prog[k];
        p.iter = q.iter;
        p.status = q.status;
        p.nan_cells = q.nan_cells;
        p.now_t = q.now_t;
        p.dt = q.dt;
        p.mass = q.mass;
        p.mass_start = q.mass_start;
        if (active)
            active[k] = q.active;
    }
    return IBTFO_OK;
}

ibtfo_status ibtfo_batch_progress(ibtfo_batch *b, ibtfo_progress *out, int *active, int n)
{
    ibtfo_status s = ibtfo_batch_progress_enqueue(b);
    if (s != IBTFO_OK)
        return s;
    return ibtfo_batch_progress_read(b, out, active, n, 1);
}

ibtfo_status ibtfo_batch_synchronize(ibtfo_batch *b)
{
    if (!b)
        return bfail(IBTFO_EINVAL, "null batch");
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->stream));
    return IBTFO_OK;
}

ibtfo_status ibtfo_batch_set_tiling(ibtfo_batch *b, int tile_shape, int ctas_per_sm)
{
    if (!b)
        return bfail(IBTFO_EINVAL, "null batch");
    if (tile_shape < 0 || tile_shape >= SHAPE_COUNT || ctas_per_sm < 0)
        return bfail(IBTFO_EINVAL, "bad tile_shape / ctas_per_sm");
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->stream));
    return set_shape(b, tile_shape, ctas_per_sm);
}

ibtfo_status ibtfo_batch_get_tiling(const ibtfo_batch *b, ibtfo_batch_tiling *t)
{
    if (!b || !t)
        return bfail(IBTFO_EINVAL, "null argument");
    std::memset(t, 0, sizeof(*t));
    t->tile_shape = b->cfg.tile_shape;
    t->ctas_per_sm = b->cfg.ctas_per_sm;
    t->max_ctas_per_sm = b->occupancy;
    t->grid = b->grid_sweep;
    long long n = 0;
    for (const Slot &s : b->slots)
        n += s.c ? (long long)s.tiles.size() : 0;
    t->tiles = n;
    return IBTFO_OK;
}

// Autotuner: every tile shape x resident-CTA count (1, 2, ..., the occupancy
// limit) runs `steps` real steps of the current cases, timed with events on
// the batch stream; the fastest is kept.  The steps advance the cases: the
// state is the same bit for bit under every tiling (each cell's update and
// the CFL maxima do not depend on the tiling; only the order of the mass
// partial sums does), so the search costs time, not results.
ibtfo_status ibtfo_batch_autotune(ibtfo_batch *b, int steps, ibtfo_batch_tiling *best, ibtfo_batch_tiling *trials,
                                  int max_trials, int *n_trials)
{
    if (!b || steps <= 0)
        return bfail(IBTFO_EINVAL, "null batch or steps <= 0");
    cudaSetDevice(b->device);
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    float best_ms = -1.0f;
    int best_shape = b->cfg.tile_shape, best_ctas = b->cfg.ctas_per_sm, nt = 0;
    ibtfo_status rs = IBTFO_OK;
    for (int shape = 0; shape < SHAPE_COUNT && rs == IBTFO_OK; shape++)
    {
        BatchKernel k = batch_kernel(b->cfg.scheme, b->cfg.riemann, b->cfg.limiter, b->cfg.precision, shape);
        const int occ = k.prepare ? k.prepare() : 0;
        for (int ctas = 1; ctas <= occ && rs == IBTFO_OK; ctas++)
        {
            rs = ibtfo_batch_set_tiling(b, shape, ctas);
            if (rs != IBTFO_OK)
                break;
            rs = ibtfo_batch_advance(b, 1); // upload + warm-up step
            if (rs != IBTFO_OK)
                break;
            cudaEventRecord(e0, b->stream);
            enqueue_steps(b, steps);
            cudaEventRecord(e1, b->stream);
            cudaError_t e = cudaEventSynchronize(e1);
            if (e != cudaSuccess)
            {
                rs = bcuda(e, "autotune");
                break;
            }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms /= steps;
            if (trials && nt < max_trials)
            {
                ibtfo_batch_tiling &t = trials[nt];
                ibtfo_batch_get_tiling(b, &t);
                t.ms_per_step = ms;
            }
            nt++;
            if (best_ms < 0.0f || ms < best_ms)
            {
                best_ms = ms;
                best_shape = shape;
                best_ctas = ctas;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rs != IBTFO_OK)
        return rs;
    if (n_trials)
        *n_trials = nt;
    rs = ibtfo_batch_set_tiling(b, best_shape, best_ctas);
    if (rs == IBTFO_OK && best)
    {
        ibtfo_batch_get_tiling(b, best);
        best->ms_per_step = best_ms;
    }
    return rs;
}

} // extern "C"
