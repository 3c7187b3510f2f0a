#!/usr/bin/env python
"""Benchmark of the GB300 IBTFO time step on the inclined-channel workload.

Workload: inclined Sod channel with ghost-fluid walls, 2048x1024 cells on
[0,2]x[0,1], channel width 0.25 at 30 degrees, IDWBaseGFM walls, MUSCL +
HLLC + minmod, CFL 0.45, FP64 -- the reference's plain path.  One step = one
iteration of the reference loop body (Advance, Boundary, Global_Boundary,
ComputeDt, CaculateMass) over the whole grid.  Inputs are synthetic (the
case plug-in in ibtfo_gb300/cases.py); the loop's t_end is lifted so that
every timed iteration does its full work.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput in
Gcell-updates/s (interior cells x steps / time), timed per step with CUDA
events on the case's stream, L2 flushed between steps; `e2e` is the same
metric through the C ABI with the state in pinned host memory, copied in
and out every step.  With N > 1 (torchrun) every rank runs an independent
replica of the case on its own GPU ("replicas only": the path has no
cross-GPU exchange) and value sums all ranks' work over the slowest rank's
time.  `--impl reference` times the reference algorithm on the host cores
instead (the CPU oracle, OpenMP over all cores), rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

BYTES_PER_CELL = 65  # 32 B state read + 32 B state write + 1 B cell type (FP64)
METRIC = "Gcell-updates/s"


def workload():
    from ibtfo_gb300 import cases
    return cases.inclined_channel(2048, 1024)


PRECISION = os.environ.get("IBTFO_BENCH_PRECISION", "fp64_fast")


def profile_run(args):
    """Plain stepping of one workload (for profiler captures): set up, warm up,
    run `--steps` steps, print ms/step.  No CPU leg, no extra legs."""
    import torch
    from ibtfo_gb300 import cases
    if args.workload == "vortex":
        w, inputs = cases.vortex_periodic(args.size), vortex_inputs
        if args.riemann:
            w.riemann = args.riemann
    elif args.workload == "obstacles":
        w, inputs = cases.shock_obstacles(args.size, args.size // 2), obstacle_inputs
    else:
        w, inputs = cases.inclined_channel(args.size, args.size // 2), channel_inputs
    r = gpu_arm(args, 0, 1, 0, precision=args.precision, e2e=False, w=w, inputs=inputs, steps=args.steps)
    print(json.dumps({"workload": w.name, "precision": args.precision, "steps": args.steps,
                      "ms_per_step": r["step_ms"] / args.steps, "sweep_ms": r["sweep_ms"] / args.steps,
                      "Gcell_updates_per_s": w.grid.n_x * w.grid.n_y * args.steps / (r["step_ms"] * 1e-3) / 1e9}))
    torch.cuda.synchronize()


L2_NOTE = "flushed between timed steps (256 MiB write)"


def config_json(w):
    """The workload, the same dict in both arms.  The arithmetic each arm
    runs is the line's own "precision" key (the GPU arm's precision key, or
    "fp64", the reference's strict binary64, for the reference arm)."""
    g = w.grid
    return {"workload": w.name, "n_x": g.n_x, "n_y": g.n_y, "domain": [g.lo_x, g.lo_y, g.hi_x, g.hi_y],
            "scheme": w.scheme, "riemann": w.riemann, "limiter": w.limiter, "boundary": w.boundary,
            "cfl": w.cfl, "gamma": w.gamma}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_value(key):
    """A per-launch figure of the headline sweep from the committed ncu
    summary (a line `key: value ...`), or None."""
    p = os.path.join(ROOT, "profiles", "sweep_inclined_channel.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def profiled_traffic():
    """DRAM bytes per sweep launch from the committed ncu summary, or None."""
    return profiled_value("traffic_bytes_per_launch_full_grid")


def link_rate(nbytes, reps=10):
    """Host link of this box: GB/s of page-locked host -> device and device ->
    host copies of `nbytes` (CUDA events on one stream, after a warm-up)."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    out = {}
    for name, (dst, src) in (("h2d", (d, h)), ("d2h", (h, d))):
        with torch.cuda.stream(s):
            dst.copy_(src, non_blocking=True)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(reps):
                dst.copy_(src, non_blocking=True)
            e1.record(s)
        s.synchronize()
        out[name + "_gbs"] = reps * nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9
    return out


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ CPU leg
def cpu_oracle_rate(w, steps=None, warmup=1, budget_s=15.0):
    """Times the CPU oracle (the reference algorithm restated in C, OpenMP
    over all host cores) on the workload's full grid.  Returns
    (Gcell-updates/s, ms/step, cores, steps)."""
    import oracle
    from ibtfo_gb300 import cases
    g = w.grid
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    o = oracle.OracleCase(g.n_x, g.n_y, g.ng, (g.lo_x, g.lo_y), (g.hi_x, g.hi_y), w.gamma, w.cfl, w.scheme,
                          w.riemann, w.limiter, w.boundary, w.gbc)
    phi = cases.channel_phi(g)
    o.setup_geometry(phi)
    u0 = cases.channel_init(g, o.get("XYCOORD").reshape(-1, 6)[:, 5], w.gamma)
    o.set_initial_state(u0)
    if warmup:
        o.run(warmup)
    t0 = time.perf_counter()
    o.run(1)
    t1 = time.perf_counter() - t0
    if steps is None:
        steps = int(max(1, min(50, budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    o.close()
    ms = 1e3 * dt / steps
    return g.n_x * g.n_y / (ms * 1e-3) / 1e9, ms, cores, steps


# ------------------------------------------------------------------ GPU leg
def channel_inputs(w, case):
    from ibtfo_gb300 import cases
    phi = cases.channel_phi(w.grid)
    case.setup_geometry(phi)
    case.set_state(cases.channel_init(w.grid, case.cell_types(), w.gamma))


def vortex_inputs(w, case):
    from ibtfo_gb300 import cases
    phi, u0 = cases.isentropic_vortex(w.grid)
    case.setup_geometry(phi)
    case.set_state(u0)


def obstacle_inputs(w, case):
    import ibtfo_gb300 as ib
    from ibtfo_gb300 import cases
    case.setup_bodies(obstacle_bodies(ib, cases.random_obstacles()))
    case.init_x_split(0.5, cases.post_shock(3.0), (1.0, 0.0, 0.0, 1.0))
    case.release_geometry()


def vortex_errors(w, rhos):
    """Density errors of the FP32 compensated form against the FP64 path (the
    path pinned to the oracle) after the same steps, and of both against the
    analytic vortex at the time each integrated: relative L1 and L-inf."""
    from ibtfo_gb300 import cases
    g = w.grid

    def rel(a, b):
        d = np.abs(a - b)
        return {"l1": float(d.sum() / np.abs(b).sum()), "linf": float(d.max() / np.abs(b).max())}

    (r64, t64), (r32, t32) = rhos["fp64_fast"], rhos["fp32c"]
    out = {"fp32c_vs_fp64": rel(r32, r64), "t_fp64": t64, "t_fp32c": t32}
    for name, r, t in (("fp64", r64, t64), ("fp32c", r32, t32)):
        _, ex = cases.isentropic_vortex(g, t=t)
        out[f"{name}_vs_analytic"] = rel(r, ex.reshape(g.N, g.M, 4)[g.ng:-g.ng, g.ng:-g.ng, 0])
    return out


def vortex_period_leg(n_big=4096, n_pair=1024, perturb=1e-7):
    """The vortex workload advected one full period (t = 10, the loop's
    t_end): the FP32 form at n_big^2 (steps, seconds, density against the
    analytic vortex at its loop time); at n_pair^2 the FP32 form, fp64_fast
    to the same step count, and fp64_fast from an initial state perturbed by
    `perturb` (relative, seeded) -- the FP64 run's own sensitivity, the scale
    against which the FP32 form's distance from FP64 is read."""
    import ibtfo_gb300 as ib
    from ibtfo_gb300 import cases

    def rel(a, b):
        d = np.abs(a - b)
        return {"l1": float(d.sum() / np.abs(b).sum()), "linf": float(d.max() / np.abs(b).max())}

    def run(n, prec, max_iter=2 ** 31 - 1, pert=0.0):
        w = cases.vortex_periodic(n)
        g = w.grid
        phi, u0 = cases.isentropic_vortex(g)
        if pert:
            u0 = u0.reshape(-1, 4) * (1.0 + pert * np.random.default_rng(3).standard_normal((g.M * g.N, 4)))
        with ib.Case.from_workload(w, precision=prec, max_iter=max_iter) as c:
            c.setup_geometry(phi)
            c.set_state(np.ascontiguousarray(u0).reshape(-1))
            t0 = time.perf_counter()
            p = c.run()
            secs = time.perf_counter() - t0
            rho = c.density()
        _, ex = cases.isentropic_vortex(g, t=p["now_t"])
        return p, rho, secs, ex.reshape(g.N, g.M, 4)[g.ng:-g.ng, g.ng:-g.ng, 0]

    w = cases.vortex_periodic(n_big)
    out = {"t_end": w.t_end, "scheme": w.scheme, "riemann": w.riemann, "time": w.time, "cfl": w.cfl}
    p, rho, secs, ex = run(n_big, "fp32c")
    out[f"fp32c_{n_big}"] = {"steps": p["iter"], "now_t": p["now_t"], "seconds": secs,
                             "Gcell_updates_per_s": n_big * n_big * p["iter"] / secs / 1e9,
                             "vs_analytic": rel(rho, ex), "nan_cells": p["nan_cells"]}
    p32, r32, s32, e32 = run(n_pair, "fp32c")
    p64, r64, s64, e64 = run(n_pair, "fp64_fast", max_iter=p32["iter"])
    pp, rp, _, _ = run(n_pair, "fp64_fast", max_iter=p32["iter"], pert=perturb)
    out[f"pair_{n_pair}"] = {"steps": [p32["iter"], p64["iter"]], "seconds": [s32, s64],
                             "fp32c_vs_fp64": rel(r32, r64), "fp64_perturbed_vs_fp64": rel(rp, r64),
                             "perturbation": perturb, "fp64_vs_analytic": rel(r64, e64),
                             "fp32c_vs_analytic": rel(r32, e32)}
    return out


def max_over_ranks(values, world, device):
    """Element-wise maximum of per-rank timings over all ranks (the slowest
    replica sets the whole job's time); identity for one rank."""
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_rate(world, cells, steps, seconds):
    """Whole-job cell updates per second (Gcell-updates/s): every replica
    advanced `cells` cells `steps` times within `seconds`."""
    return world * cells * steps / seconds / 1e9


def gpu_arm(args, rank, world, local_rank, precision=None, e2e=True, w=None, inputs=channel_inputs, steps=None,
            snapshot=False):
    import torch
    import ibtfo_gb300 as ib

    torch.cuda.set_device(local_rank)
    w = w or workload()
    g = w.grid
    cells = g.n_x * g.n_y
    stream = torch.cuda.Stream()
    c = ib.Case.from_workload(w, t_end=1e300, max_iter=2 ** 31 - 1, precision=precision or PRECISION)
    c.set_stream(stream.cuda_stream)
    inputs(w, c)
    p_start = c.progress()
    K = steps or args.steps
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > 129 MB L2

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            c.enqueue_sweep()
            c.enqueue_boundary()
    stream.synchronize()

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(K)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = ib.launch_count()
    with ClockSampler(local_rank) as clk:
        with torch.cuda.stream(stream):
            for k in range(K):
                flush.fill_(float(k))
                ev[k][0].record(stream)
                c.enqueue_sweep()
                ev[k][1].record(stream)
                c.enqueue_boundary()
                ev[k][2].record(stream)
        torch.cuda.synchronize()
    launches = ib.launch_count() - launches0
    if world > 1:
        torch.distributed.barrier()
    step_ms = sum(e[0].elapsed_time(e[2]) for e in ev)
    sweep_ms = sum(e[0].elapsed_time(e[1]) for e in ev)
    prog = c.progress()
    rho = None
    if snapshot:
        # interior density after warm-up + K steps, and the time it represents
        # (now_t advances by the dt computed after each step: dt_0 + ... + dt_{n-1})
        rho = c.get_state().reshape(g.N, g.M, 4)[g.ng:-g.ng, g.ng:-g.ng, 0].copy()
        rho_t = prog["now_t"] - prog["dt"] + p_start["dt"]

    # end to end through the C ABI with host buffers (pinned)
    e2e_steps = max(1, min(K, 100)) if e2e else 1
    pin = ib.PinnedBuffer(g.M * g.N * 4)
    c.get_state_ptr(pin.ptr)
    # warm-up: the first in-place call copies every row in (both state buffers
    # then agree with the array outside the cells later calls copy); the
    # second captures the step's CUDA graph for this array
    c.step_host_ptr(pin.ptr, pin.ptr)
    c.step_host_ptr(pin.ptr, pin.ptr)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        # one reference loop iteration on the host array: the state goes in,
        # the step runs, the new state and the loop scalars come back
        c.step_host_ptr(pin.ptr, pin.ptr)
    e2e_s = time.perf_counter() - t0
    e2e_bytes = c.step_host_bytes(in_place=True)
    pin.close()
    link = link_rate(g.M * g.N * 4 * 8) if e2e else None
    if link is not None:
        link["numa_nodes"] = len([d for d in os.listdir("/sys/devices/system/node") if d.startswith("node")]) \
            if os.path.isdir("/sys/devices/system/node") else None

    step_ms, sweep_ms, e2e_s = max_over_ranks([step_ms, sweep_ms, e2e_s], world, "cuda")
    res = {"step_ms": step_ms, "sweep_ms": sweep_ms, "e2e_s": e2e_s, "e2e_steps": e2e_steps, "e2e_bytes": e2e_bytes,
           "link": link,
           "cells": cells,
           "launches": launches, "clocks": clk.summary(), "progress": prog, "M": g.M, "N": g.N}
    if snapshot:
        res["rho"], res["rho_t"] = rho, rho_t
    c.close()
    return res


def served_request(ib, r, arrival, density_out=None):
    from ibtfo_gb300 import cases
    post = cases.post_shock(r.mach)
    return ib.request(r.id, r.n_x, r.n_y, (0.0, 0.0), (r.width, r.height), r.t_end,
                      bodies=[ib.circle(r.xc, r.yc, r.radius)], x_split=r.x_shock, left=post,
                      right=(1.0, 0.0, 0.0, 1.0), arrival=arrival, cfl=r.cfl, density_out=density_out)


def obstacle_bodies(ib, obstacles):
    return [ib.circle(o.xc, o.yc, o.a) if o.kind == "circle" else ib.ellipse(o.xc, o.yc, o.a, o.b, o.theta)
            for o in obstacles]


def ccm_leg(steps=40, warmup=3, n_x=8192, n_y=4096, full=False):
    """Mach 3 shock over 24 seeded obstacles with cut cells (8192x4096 on
    [0,4]x[0,2]): set-up time (level set, cut-cell geometry, mixing lists,
    initial state, all on the GPU), then `steps` timed steps of the FP32 form
    with HLL_Toro and with Steger-Warming and of FP64 with HLL_Toro; the FP32
    density against FP64's after the same steps.  full: also the FP32
    HLL_Toro run to t_end = 1.0."""
    import torch
    import ibtfo_gb300 as ib
    from ibtfo_gb300 import cases
    w = cases.shock_obstacles(n_x, n_y)
    g = w.grid
    cells = g.n_x * g.n_y
    obs = cases.random_obstacles()
    post = cases.post_shock(3.0)
    out = {"workload": f"{w.name}: Mach 3 shock at x = 0.5 over {len(obs)} seeded circles/ellipses (seed 20261203), "
                       f"cut cells, CFL {w.cfl}", "cells": cells, "steps": steps, "legs": {}}
    rho = {}
    peak = measured_peaks()[0]
    for riemann, prec in (("HLL_Toro", "fp32c"), ("StegerWarming", "fp32c"), ("HLL_Toro", "fp64_fast")):
        stream = torch.cuda.Stream()
        with ib.Case.from_workload(w, riemann=riemann, precision=prec, t_end=1e300, max_iter=2 ** 31 - 1) as c:
            c.set_stream(stream.cuda_stream)
            t0 = time.perf_counter()
            c.setup_bodies(obstacle_bodies(ib, obs))
            c.init_x_split(0.5, post, (1.0, 0.0, 0.0, 1.0))
            c.release_geometry()
            setup_s = time.perf_counter() - t0
            with torch.cuda.stream(stream):
                for _ in range(warmup):
                    c.enqueue_sweep()
                    c.enqueue_boundary()
            stream.synchronize()
            ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
            with torch.cuda.stream(stream):
                for k in range(steps):
                    ev[k][0].record(stream)
                    c.enqueue_sweep()
                    ev[k][1].record(stream)
                    c.enqueue_boundary()
                    ev[k][2].record(stream)
            torch.cuda.synchronize()
            step_ms = sum(e[0].elapsed_time(e[2]) for e in ev)
            sweep_ms = sum(e[0].elapsed_time(e[1]) for e in ev)
            p = c.progress()
            out["legs"][f"{riemann}/{prec}"] = {
                "value": job_rate(1, cells, steps, step_ms * 1e-3), "unit": METRIC, "ms_per_step": step_ms / steps,
                "sweep_and_mixing_ms": sweep_ms / steps,
                "roofline_frac": BYTES_PER_CELL * cells / (sweep_ms / steps * 1e-3) / 1e9 / peak,
                "setup_s": setup_s, "nan_cells": p["nan_cells"], "now_t": p["now_t"]}
            if riemann == "HLL_Toro":
                rho[prec] = c.density()
    a, b = rho["fp32c"], rho["fp64_fast"]
    d = np.abs(a - b)
    out["fp32c_vs_fp64_density"] = {"l1": float(d.sum() / np.abs(b).sum()), "linf": float(d.max() / np.abs(b).max()),
                                    "after_steps": warmup + steps}
    if full:
        with ib.Case.from_workload(w, riemann="HLLC", precision="fp32c", max_iter=2 ** 31 - 1) as c:
            c.setup_bodies(obstacle_bodies(ib, obs))
            c.init_x_split(0.5, post, (1.0, 0.0, 0.0, 1.0))
            c.release_geometry()
            t0 = time.perf_counter()
            p = c.run()
            secs = time.perf_counter() - t0
        out["to_t_end"] = {"t_end": w.t_end, "steps": p["iter"], "seconds": secs, "nan_cells": p["nan_cells"],
                           "Gcell_updates_per_s": job_rate(1, cells, p["iter"], secs)}
    return out


def serve_leg(n_requests=64, rates=(1.0, 4.0), precision="fp32c", plain_precision="fp64_fast",
              max_cells=2048 * 2048):
    """The served batch stream (the first `n_requests` of the seed-42 stream,
    grids log-uniform over 128^2..max_cells): cases/s and p50/p99 latency of
    the server at each arrival rate (None: all requests at t = 0, the
    server's capacity); the same requests run plainly one after another in
    `plain_precision` (timed: cases/s of the plain path); each served density
    against the plain one, both at t_end and at the served run's step count
    (the loop stops at the first now_t >= t_end with no clipping,
    Test/Sod/Sod.cpp:123,176, so runs whose dt sequences differ in rounding
    can stop one step apart; the matched-step figure is the arithmetic
    error).

    Solver, time integration and CFL: cases.SERVE_RIEMANN (HLL with Toro's
    wave speeds and the positivity safeguards), cases.SERVE_TIME (RK2) at
    cases.SERVE_CFL (0.45); cases.py gives the measurements behind them."""
    import ibtfo_gb300 as ib
    from ibtfo_gb300 import cases
    base = cases.served_stream(n_requests, 1.0, seed=42, max_cells=max_cells)
    cells = sum(r.n_x * r.n_y for r in base)
    riemann, tadv = cases.SERVE_RIEMANN, cases.SERVE_TIME
    bufs = {r.id: ib.PinnedBuffer(r.n_x * r.n_y) for r in base}
    out = {"workload": f"shock over a cylinder, the first {n_requests} requests of the seed-42 stream, "
                       f"cells per request log-uniform over 128^2..{max_cells} "
                       f"(grids {min(r.n_x * r.n_y for r in base)}..{max(r.n_x * r.n_y for r in base)} cells, "
                       f"{cells} cells in all; Mach {min(r.mach for r in base):.2f}..{max(r.mach for r in base):.2f}), "
                       f"MUSCL + {riemann} + minmod, Time = {tadv}, IDWBaseGFM, CFL {base[0].cfl}, 1.5 crossings; "
                       f"all {n_requests} served and run plainly, nothing extrapolated",
           "served_precision": precision, "plain_precision": plain_precision, "rates": []}
    served = None
    for rate in rates:
        arrivals = [0.0] * n_requests if rate is None else \
            [r.arrival for r in cases.served_stream(n_requests, rate, seed=42, max_cells=max_cells)]
        with ib.Server(riemann=riemann, precision=precision, chunk_steps=32, tile_shape="auto", time=tadv) as srv:
            for r, a in zip(base, arrivals):
                srv.submit(served_request(ib, r, a, density_out=bufs[r.id]))
            srv.start()
            srv.run(max_seconds=1200)
            res = srv.poll(max_results=n_requests + 8)
            st = srv.stats()
        res = sorted(res, key=lambda q: q["id"])
        lat = sorted(x["finished"] - x["arrival"] for x in res)
        span = max(x["finished"] for x in res)
        cell_updates = sum(r.n_x * r.n_y * x["iter"] for r, x in zip(base, res))
        out["rates"].append({
            "rate_per_s": rate if rate is not None else "all at t=0", "cases": len(res),
            "failed": sum(1 for x in res if x["status"] != 0), "seconds": span, "cases_per_s": len(res) / span,
            "Gcell_updates_per_s": cell_updates / span / 1e9,
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "peak_active": st["peak_active"], "peak_bytes": st["peak_bytes"],
            "tiling": {"shape": ib.TILE_SHAPES_BY_ID.get(st["tile_shape"]), "ctas_per_sm": st["ctas_per_sm"]}})
        if served is None:
            served = res
    served_rho = {k: b.array.copy() for k, b in bufs.items()}
    for b in bufs.values():
        b.close()
    # the same requests run plainly, one after another
    l1_end, l1_match, linf_match, iters_equal = [], [], [], 0
    plain_s = 0.0
    for r, sres in zip(base, served):
        it_s = sres["iter"]
        with ib.Case(r.n_x, r.n_y, lo=(0.0, 0.0), hi=(r.width, r.height), cfl=r.cfl, t_end=r.t_end,
                     max_iter=2 ** 31 - 1, scheme="MUSCL", riemann=riemann, boundary="IDWBaseGFM",
                     precision=plain_precision, time=tadv) as c:
            t0 = time.perf_counter()
            c.setup_bodies([ib.circle(r.xc, r.yc, r.radius)])
            c.init_x_split(r.x_shock, cases.post_shock(r.mach), (1.0, 0.0, 0.0, 1.0))
            c.advance(it_s)  # the loop stops early if it reaches t_end first
            rho_match = c.density().reshape(-1) if c.progress()["iter"] == it_s else None
            p = c.run()
            plain_s += time.perf_counter() - t0
            rho_end = c.density().reshape(-1)
            iters_equal += int(p["iter"] == it_s)
            while p["iter"] < it_s:  # the served run took more steps: continue past t_end (untimed)
                p = c.step()
            if rho_match is None:
                rho_match = c.density().reshape(-1)
        a = served_rho[r.id]
        l1_end.append(float(np.abs(a - rho_end).sum() / np.abs(rho_end).sum()))
        l1_match.append(float(np.abs(a - rho_match).sum() / np.abs(rho_match).sum()))
        linf_match.append(float(np.abs(a - rho_match).max() / np.abs(rho_match).max()))
    cell_updates = sum(r.n_x * r.n_y * x["iter"] for r, x in zip(base, served))
    out["plain"] = {"seconds": plain_s, "cases_per_s": n_requests / plain_s,
                    "Gcell_updates_per_s": cell_updates / plain_s / 1e9}
    # the served rate at the highest arrival rate (capacity-limited: 4 requests/s is above what the
    # GPU retires) against the plain path's
    out["served_vs_plain_cases_per_s"] = max(x["cases_per_s"] for x in out["rates"]) / out["plain"]["cases_per_s"]
    out["density_l1_vs_plain"] = {"at": "the served run's step count", "max": max(l1_match),
                                  "median": float(np.median(l1_match)),
                                  "within_1e-5": sum(1 for e in l1_match if e <= 1e-5), "of": len(l1_match)}
    out["density_linf_vs_plain"] = {"max": max(linf_match), "median": float(np.median(linf_match))}
    out["density_l1_vs_plain_at_t_end"] = {"max": max(l1_end), "median": float(np.median(l1_end)),
                                           "within_1e-5": sum(1 for e in l1_end if e <= 1e-5),
                                           "same_step_count": iters_equal, "of": len(l1_end)}
    worst = sorted(range(len(base)), key=lambda k: -l1_match[k])[:5]
    out["worst_requests"] = [{"id": base[k].id, "grid": [base[k].n_x, base[k].n_y], "mach": base[k].mach,
                              "steps": served[k]["iter"], "l1": l1_match[k], "linf": linf_match[k]} for k in worst]
    out["nan_results"] = sum(1 for x in served if x["nan_cells"])
    return out


def fp64_roofline(sweep_s):
    """The bound of the FP64 sweep: FP64 thread instructions per launch (DADD
    + DMUL + DFMA, from the committed ncu capture of the same launch) per
    second of the CUDA-event-timed sweep, against this GPU's FP64 pipe rate
    measured now (ibtfo_fp64_pipe_rate: independent DFMA chains on every SM)."""
    import ibtfo_gb300 as ib
    ops = profiled_value("fp64_thread_inst_per_launch_full_grid")
    peak, _ = ib.fp64_pipe_rate(16384)
    out = {"bound": "fp64 pipe", "unit": "G FP64 thread-inst/s", "peak": peak / 1e9,
           "peak_source": "measured in this run (DFMA chains, CUDA events)", "ops_per_launch": ops,
           "ops_source": "ncu sm__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum of one launch "
                         "(profiles/sweep_inclined_channel.md)"}
    if ops:
        out["achieved"] = ops / sweep_s / 1e9
        out["frac"] = out["achieved"] / out["peak"]
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-workload", dest="workload", choices=("channel", "vortex", "obstacles"), default=None,
                    help="only step this workload (profiler captures)")
    ap.add_argument("--size", type=int, default=4096, help="grid size for --profile-workload")
    ap.add_argument("--riemann", default=None, help="Riemann key for --profile-workload vortex")
    ap.add_argument("--precision", default=PRECISION, choices=("fp64", "fp64_fast", "fp32c"))
    ap.add_argument("--serve-requests", type=int, default=64, help="requests of the served-stream leg (0: skip)")
    ap.add_argument("--serve-max-cells", type=int, default=2048 * 2048, help="largest request grid (cells)")
    ap.add_argument("--serve-only", action="store_true", help="run only the served-stream leg")
    ap.add_argument("--ccm-only", action="store_true", help="run only the cut-cell (shock over obstacles) leg")
    ap.add_argument("--ccm-full", action="store_true", help="cut-cell leg: also run to t_end = 1.0")
    ap.add_argument("--no-ccm", action="store_true", help="skip the cut-cell leg")
    ap.add_argument("--no-period", action="store_true", help="skip the vortex's one-period leg")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.workload:
        profile_run(args)
        return 0
    if args.ccm_only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"ccm": ccm_leg(full=args.ccm_full)}), flush=True)
        return 0
    if args.serve_only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"serve": serve_leg(args.serve_requests, max_cells=args.serve_max_cells)}), flush=True)
        return 0

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    w = workload()
    g = w.grid
    cells = g.n_x * g.n_y

    if args.impl == "reference":
        if rank != 0:
            return 0
        rate, ms, cores, n = cpu_oracle_rate(w, steps=args.steps, warmup=args.warmup)
        sample = f"{args.warmup} warm-up + {n} timed steps of the full {g.n_x}x{g.n_y} grid"
        line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": METRIC, "n_gpus": world,
                "steps": n, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config_json(w), "precision": "fp64", "l2": "n/a (host cores)",
                "cpu_baseline": {"value": rate, "unit": METRIC, "cores": cores, "kind": "port", "sample": sample},
                "e2e": {"value": rate, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0

    if world > 1:
        import torch
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, ms, cores, n = cpu_oracle_rate(w)
        cpu = {"value": rate, "unit": METRIC, "cores": cores, "kind": "port",
               "sample": f"1 warm-up + {n} timed steps of the full {g.n_x}x{g.n_y} grid, OpenMP over {cores} threads"}

    r = gpu_arm(args, rank, world, local_rank)
    # the other FP64 precision, timed the same way (steps only), for comparison
    other = "fp64" if PRECISION == "fp64_fast" else "fp64_fast"
    r2 = gpu_arm(args, rank, world, local_rank, precision=other, e2e=False)
    # the isentropic-vortex workload (4096^2, periodic, MHM + HLLC) in the FP64
    # path and in the FP32 compensated precision form
    from ibtfo_gb300 import cases as _cases
    wv = _cases.vortex_periodic(4096)
    kv = max(10, min(args.steps, 100))
    forms = {}
    rhos = {}
    for prec in ("fp64_fast", "fp32c"):
        rv = gpu_arm(args, rank, world, local_rank, precision=prec, e2e=False, w=wv, inputs=vortex_inputs, steps=kv,
                     snapshot=(rank == 0))
        cv = wv.grid.n_x * wv.grid.n_y
        sw_s = rv["sweep_ms"] * 1e-3 / kv
        sweeps = 2 if wv.time == "RK2" else 1  # an RK2 step reads and writes the state twice
        forms[prec] = {"value": job_rate(world, cv, kv, rv["step_ms"] * 1e-3), "unit": METRIC,
                       "steps": args.warmup + kv, "sweep_ms": rv["sweep_ms"] / kv, "sweeps_per_step": sweeps,
                       "roofline_frac": sweeps * BYTES_PER_CELL * cv / sw_s / 1e9 / measured_peaks()[0]}
        rhos[prec] = (rv.get("rho"), rv.get("rho_t"))
    # for comparison: the FP32 sweep with the plain (not difference-form) face
    # solve, as the contact-restoring HLLC with single steps runs it
    wp = _cases.vortex_periodic(4096, riemann="HLLC_Toro", time="SingleStep")
    rp = gpu_arm(args, rank, world, local_rank, precision="fp32c", e2e=False, w=wp, inputs=vortex_inputs, steps=kv)
    forms["fp32c_plain_face_solve"] = {
        "riemann": wp.riemann, "time": wp.time, "value": job_rate(world, cv, kv, rp["step_ms"] * 1e-3), "unit": METRIC,
        "sweep_ms": rp["sweep_ms"] / kv,
        "roofline_frac": BYTES_PER_CELL * cv / (rp["sweep_ms"] * 1e-3 / kv) / 1e9 / measured_peaks()[0]}
    if rank == 0:
        forms["errors"] = vortex_errors(wv, rhos)
        if not args.no_period:
            forms["one_period"] = vortex_period_leg()
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    if rank != 0:
        return 0
    # the cut-cell workload (rank 0)
    ccm = None if args.no_ccm else ccm_leg(full=args.ccm_full)
    # the served stream (rank 0; replicas would serve their own streams)
    serve = None
    if args.serve_requests > 0:
        serve = serve_leg(args.serve_requests, max_cells=args.serve_max_cells)
    K = args.steps
    step_s = r["step_ms"] * 1e-3
    value = job_rate(world, cells, K, step_s)
    sweep_s = r["sweep_ms"] * 1e-3 / K
    peak, peak_kind = measured_peaks()
    achieved = BYTES_PER_CELL * cells / sweep_s / 1e9
    traffic = profiled_traffic()
    e2e_val = job_rate(world, cells, r["e2e_steps"], r["e2e_s"])
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K, "warmup": args.warmup,
            "ms_per_step": r["step_ms"] / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": config_json(w), "precision": PRECISION, "l2": L2_NOTE,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_source": peak_kind, "kernel": "sweep_kernel",
                         "algorithmic_bytes_per_cell": BYTES_PER_CELL, "sweep_ms": r["sweep_ms"] / K,
                         "fp64": fp64_roofline(sweep_s)},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": METRIC, "h2d_bytes_per_step": r["e2e_bytes"][0],
                    "d2h_bytes_per_step": r["e2e_bytes"][1], "steps": r["e2e_steps"],
                    "call": "ibtfo_step_host, in place on a page-locked host array",
                    "vs_device_resident": e2e_val / value, "link": r["link"]},
            "gpu_launches": r["launches"], "clocks": r["clocks"],
            "other_precision": {"precision": other, "value": job_rate(world, cells, K, r2["step_ms"] * 1e-3),
                                "unit": METRIC, "sweep_ms": r2["sweep_ms"] / K},
            "serve": serve,
            "cut_cells": ccm,
            "forms": {"workload": wv.name, "scheme": wv.scheme, "riemann": wv.riemann, "time": wv.time,
                      "cfl": wv.cfl, "boundary": "periodic", **forms},
            "final": {"iter": r["progress"]["iter"], "nan_cells": r["progress"]["nan_cells"]}}
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
