// Serving loop: solves arrive as requests, are admitted against a device-
// memory budget, run together in one batch (continuous batching), and
// retire when their own loop ends (t_end or max_iter).
//
// No counterpart in the reference (one case per process, Test/Sod/Sod.cpp).
// Each scheduling round (ibtfo_server_pump):
//   1. queue the next chunk of steps of every active case (graph launches);
//   2. read the progress snapshot taken after the previous chunk, while the
//      GPU runs the new one;
//   3. take the cases whose loop has ended out of the batch (no host wait),
//      queue the copy of their density on their own stream (ordered after
//      the steps already queued) and move them to a retiring list;
//   4. finish the retiring cases whose stream is idle: stamp the result,
//      free the case, return its bytes to the budget;
//   5. admit arrived requests in arrival order while the budget and the
//      active-case limit allow: create the case, set up its geometry and
//      initial state on the GPU, release the set-up arrays, add it to the batch;
//   6. queue the snapshot after the new chunk.
// A case gives the same result in the mix as alone: the batch runs the
// same tile body (bit for bit with the one-case kernels).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ibtfo.h"
#include "internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Live
{
    ibtfo_case *c = nullptr;
    ibtfo_request req{};
    long long bytes = 0;
    double admitted = 0.0;
};

struct Retiring
{
    ibtfo_case *c = nullptr;
    ibtfo_result res{};
    long long bytes = 0;
};

} // namespace

struct ibtfo_server
{
    ibtfo_server_config cfg{};
    ibtfo_batch *batch = nullptr;
    std::mutex mu; // pending, done, stats counters touched by submit/poll
    std::deque<ibtfo_request> pending;
    std::vector<ibtfo_result> done;
    std::map<int, Live> live; // batch slot -> case
    std::vector<Retiring> retiring;
    long long bytes_in_use = 0, peak_bytes = 0;
    Clock::time_point t0;
    bool started = false;
    bool snapshot_pending = false;
    bool tuned = false;
    ibtfo_server_stats st{};
    std::vector<ibtfo_progress> prog;
    std::vector<int> act;
};

namespace {

double now_s(const ibtfo_server *s)
{
    return std::chrono::duration<double>(Clock::now() - s->t0).count();
}

ibtfo_status sfail(ibtfo_status code, const std::string &m)
{
    ibtfo::set_last_error(m.c_str());
    return code;
}

ibtfo_config config_of(const ibtfo_server *s, const ibtfo_request &r)
{
    ibtfo_config k{};
    k.n_x = r.n_x;
    k.n_y = r.n_y;
    k.num_ghost_cell = 2;
    k.lo_x = r.lo_x;
    k.lo_y = r.lo_y;
    k.hi_x = r.hi_x;
    k.hi_y = r.hi_y;
    k.gamma = r.gamma;
    k.cfl_number = r.cfl_number;
    k.psy_time = r.t_end;
    k.max_iter = r.max_iter > 0 ? r.max_iter : 2147483647;
    k.scheme = s->cfg.scheme;
    k.riemann = s->cfg.riemann;
    k.limiter = s->cfg.limiter;
    k.boundary = r.boundary;
    k.global_boundary = r.global_boundary;
    k.precision = s->cfg.precision;
    k.time_advance = s->cfg.time_advance;
    return k;
}

void finish_failed(ibtfo_server *s, const ibtfo_request &r, ibtfo_status code, double t)
{
    ibtfo_result res{};
    res.id = r.id;
    res.status = code;
    res.arrival = r.arrival;
    res.admitted = t;
    res.finished = t;
    std::lock_guard<std::mutex> lk(s->mu);
    s->done.push_back(res);
    s->st.completed++;
    s->st.failed++;
}

// create, set up and add one case; IBTFO_OK, or the error the request fails with
ibtfo_status admit_one(ibtfo_server *s, const ibtfo_request &r, long long resident)
{
    const ibtfo_config k = config_of(s, r);
    ibtfo_case *c = nullptr;
    ibtfo_status e = ibtfo_create(&k, &c);
    if (e == IBTFO_OK)
        e = ibtfo_setup_bodies(c, r.bodies, std::min(std::max(r.n_bodies, 0), IBTFO_MAX_BODIES));
    if (e == IBTFO_OK)
        e = ibtfo_init_x_split(c, r.x_split, r.left, r.right);
    if (e == IBTFO_OK)
        e = ibtfo_release_geometry(c);
    int slot = -1;
    if (e == IBTFO_OK)
        e = ibtfo_batch_add(s->batch, c, &slot);
    if (e != IBTFO_OK)
    {
        if (c)
            ibtfo_destroy(c);
        return e;
    }
    Live L;
    L.c = c;
    L.req = r;
    L.bytes = resident;
    L.admitted = now_s(s);
    s->live[slot] = L;
    s->bytes_in_use += resident;
    s->peak_bytes = std::max(s->peak_bytes, s->bytes_in_use);
    return IBTFO_OK;
}

void admit(ibtfo_server *s)
{
    for (;;)
    {
        ibtfo_request r;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->pending.empty())
                return;
            r = s->pending.front();
        }
        const double t = now_s(s);
        if (r.arrival > t)
            return; // not arrived yet (requests are kept in arrival order)
        if (s->cfg.max_active > 0 && (int)s->live.size() >= s->cfg.max_active)
            return;
        const ibtfo_config k = config_of(s, r);
        long long resident = 0, setup = 0;
        ibtfo_status e = ibtfo_case_bytes(&k, &resident, &setup);
        if (e == IBTFO_OK && setup > s->cfg.memory_budget)
            e = IBTFO_ENOMEM; // can never fit
        if (e == IBTFO_OK && s->bytes_in_use + setup > s->cfg.memory_budget)
            return; // wait for memory to free up (first come, first served)
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->pending.pop_front();
        }
        if (e == IBTFO_OK)
            e = admit_one(s, r, resident);
        if (e != IBTFO_OK)
        {
            finish_failed(s, r, e, t);
            continue;
        }
        std::lock_guard<std::mutex> lk(s->mu);
        s->st.admitted++;
    }
}

// cases whose loop ended in the last snapshot leave the batch
ibtfo_status retire_finished(ibtfo_server *s)
{
    const int n = ibtfo_batch_num_slots(s->batch);
    if ((int)s->prog.size() < n)
    {
        s->prog.resize(n);
        s->act.resize(n);
    }
    ibtfo_status e = ibtfo_batch_progress_read(s->batch, s->prog.data(), s->act.data(), n, 1);
    if (e != IBTFO_OK)
        return e;
    for (auto it = s->live.begin(); it != s->live.end();)
    {
        const int slot = it->first;
        if (slot >= n || s->act[slot])
        {
            ++it;
            continue;
        }
        Live &L = it->second;
        const ibtfo_progress &p = s->prog[slot];
        e = ibtfo_batch_remove(s->batch, slot);
        if (e != IBTFO_OK)
            return e;
        Retiring R;
        R.c = L.c;
        R.bytes = L.bytes;
        R.res.id = L.req.id;
        R.res.status = IBTFO_OK;
        R.res.iter = p.iter;
        R.res.nan_cells = p.nan_cells;
        R.res.now_t = p.now_t;
        R.res.mass = p.mass;
        R.res.mass_start = p.mass_start;
        R.res.arrival = L.req.arrival;
        R.res.admitted = L.admitted;
        if (L.req.density_out)
        {
            e = ibtfo_get_density(L.c, L.req.density_out, 0);
            if (e != IBTFO_OK)
                R.res.status = e;
        }
        s->retiring.push_back(R);
        it = s->live.erase(it);
    }
    return IBTFO_OK;
}

void finish_retiring(ibtfo_server *s, bool wait)
{
    for (auto it = s->retiring.begin(); it != s->retiring.end();)
    {
        ibtfo_status q = wait ? ibtfo_synchronize(it->c) : ibtfo_query(it->c);
        if (q == IBTFO_ETIMEOUT)
        {
            ++it;
            continue;
        }
        it->res.finished = now_s(s);
        if (q != IBTFO_OK && it->res.status == IBTFO_OK)
            it->res.status = q;
        ibtfo_destroy(it->c);
        s->bytes_in_use -= it->bytes;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->done.push_back(it->res);
            s->st.completed++;
            if (it->res.status != IBTFO_OK)
                s->st.failed++;
        }
        it = s->retiring.erase(it);
    }
}

} // namespace

extern "C" {

ibtfo_status ibtfo_server_create(const ibtfo_server_config *cfg, ibtfo_server **out)
{
    if (!cfg || !out)
        return sfail(IBTFO_EINVAL, "null argument");
    *out = nullptr;
    ibtfo_server *s = new ibtfo_server();
    s->cfg = *cfg;
    if (s->cfg.chunk_steps <= 0)
        s->cfg.chunk_steps = 32;
    if (s->cfg.memory_budget <= 0)
    {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        s->cfg.memory_budget = (long long)(0.8 * (double)fr);
    }
    ibtfo_batch_config bc{};
    bc.scheme = cfg->scheme;
    bc.riemann = cfg->riemann;
    bc.limiter = cfg->limiter;
    bc.precision = cfg->precision;
    bc.tile_shape = cfg->tile_shape >= 0 ? cfg->tile_shape : IBTFO_TILE_32x8;
    bc.ctas_per_sm = cfg->ctas_per_sm;
    bc.graph_steps = std::min(16, s->cfg.chunk_steps);
    bc.time_advance = cfg->time_advance;
    ibtfo_status e = ibtfo_batch_create(&bc, &s->batch);
    if (e != IBTFO_OK)
    {
        delete s;
        return e;
    }
    s->tuned = cfg->tile_shape >= 0;
    s->t0 = Clock::now();
    *out = s;
    return IBTFO_OK;
}

ibtfo_status ibtfo_server_destroy(ibtfo_server *s)
{
    if (!s)
        return IBTFO_OK;
    ibtfo_batch_synchronize(s->batch);
    for (auto &kv : s->live)
        ibtfo_destroy(kv.second.c);
    for (auto &r : s->retiring)
        ibtfo_destroy(r.c);
    ibtfo_batch_destroy(s->batch);
    delete s;
    return IBTFO_OK;
}

ibtfo_status ibtfo_server_submit(ibtfo_server *s, const ibtfo_request *r)
{
    if (!s || !r)
        return sfail(IBTFO_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    // keep arrival order (stable for equal arrivals)
    auto it = s->pending.end();
    while (it != s->pending.begin() && (it - 1)->arrival > r->arrival)
        --it;
    s->pending.insert(it, *r);
    s->st.submitted++;
    return IBTFO_OK;
}

ibtfo_status ibtfo_server_start(ibtfo_server *s)
{
    if (!s)
        return sfail(IBTFO_EINVAL, "null server");
    s->t0 = Clock::now();
    s->started = true;
    return IBTFO_OK;
}

double ibtfo_server_clock(const ibtfo_server *s) { return s ? now_s(s) : 0.0; }

ibtfo_status ibtfo_server_pump(ibtfo_server *s, int *busy)
{
    if (!s)
        return sfail(IBTFO_EINVAL, "null server");
    if (!s->started)
        ibtfo_server_start(s);
    ibtfo_status e = IBTFO_OK;
    const bool stepping = !s->live.empty();
    if (stepping)
    {
        e = ibtfo_batch_advance(s->batch, s->cfg.chunk_steps);
        if (e != IBTFO_OK)
            return e;
        s->st.chunks++;
        s->st.steps += s->cfg.chunk_steps;
    }
    if (s->snapshot_pending)
    {
        e = retire_finished(s);
        s->snapshot_pending = false;
        if (e != IBTFO_OK)
            return e;
    }
    finish_retiring(s, false);
    admit(s);
    if (!s->tuned && (int)s->live.size() >= 4)
    {
        ibtfo_batch_tiling best;
        e = ibtfo_batch_autotune(s->batch, 2, &best, nullptr, 0, nullptr);
        if (e != IBTFO_OK)
            return e;
        s->tuned = true;
    }
    if (!s->live.empty())
    {
        e = ibtfo_batch_progress_enqueue(s->batch);
        if (e != IBTFO_OK)
            return e;
        s->snapshot_pending = true;
    }
    s->st.peak_active = std::max(s->st.peak_active, (int)s->live.size());
    if (busy)
    {
        std::lock_guard<std::mutex> lk(s->mu);
        *busy = (!s->live.empty() || !s->retiring.empty() || !s->pending.empty()) ? 1 : 0;
    }
    return IBTFO_OK;
}

ibtfo_status ibtfo_server_run(ibtfo_server *s, double max_seconds)
{
    if (!s)
        return sfail(IBTFO_EINVAL, "null server");
    if (!s->started)
        ibtfo_server_start(s);
    const double t_stop = now_s(s) + (max_seconds > 0 ? max_seconds : 1e300);
    for (;;)
    {
        int busy = 0;
        ibtfo_status e = ibtfo_server_pump(s, &busy);
        if (e != IBTFO_OK)
            return e;
        if (!busy)
            return IBTFO_OK;
        if (now_s(s) > t_stop)
            return sfail(IBTFO_ETIMEOUT, "ibtfo_server_run: time limit reached with work left");
        if (s->live.empty())
        {
            // nothing on the GPU: wait for the next arrival or a retiring copy
            double next = 1e300;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                if (!s->pending.empty())
                    next = s->pending.front().arrival;
            }
            const double wait = std::min(next - now_s(s), 0.002);
            if (wait > 0)
                std::this_thread::sleep_for(std::chrono::duration<double>(wait));
        }
    }
}

int ibtfo_server_poll(ibtfo_server *s, ibtfo_result *out, int max)
{
    if (!s || !out || max <= 0)
        return 0;
    std::lock_guard<std::mutex> lk(s->mu);
    const int n = std::min<int>(max, (int)s->done.size());
    std::copy(s->done.begin(), s->done.begin() + n, out);
    s->done.erase(s->done.begin(), s->done.begin() + n);
    return n;
}

ibtfo_status ibtfo_server_stats_get(ibtfo_server *s, ibtfo_server_stats *out)
{
    if (!s || !out)
        return sfail(IBTFO_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->pending = (int)s->pending.size();
    out->active = (int)s->live.size();
    out->retiring = (int)s->retiring.size();
    out->bytes_in_use = s->bytes_in_use;
    out->peak_bytes = s->peak_bytes;
    out->memory_budget = s->cfg.memory_budget;
    ibtfo_batch_tiling t;
    if (ibtfo_batch_get_tiling(s->batch, &t) == IBTFO_OK)
    {
        out->tile_shape = t.tile_shape;
        out->ctas_per_sm = t.ctas_per_sm;
    }
    return IBTFO_OK;
}

} // extern "C"
