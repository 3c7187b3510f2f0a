"""ibtfo_gb300: GB300-native (sm_103a) IBTFO per-timestep solver.

Thin Python binding of the C ABI in include/ibtfo.h (libibtfo_gb300.so,
built in-tree by ibtfo_gb300/build.py).  The names follow the reference's
solver API: a `Case` is one problem with the reference's slot keys
(Scheme, Riemann, Limiter, Boundary) and .inp numbers; its methods map to
Psy_coord/Level_Set/Scheme_Index (setup_geometry), Initialize (set_state),
and the time-loop body (advance/step/run).

There is no CPU fallback: importing works without a GPU, but every solver
call needs the compiled library and a CUDA device and raises if either is
missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libibtfo_gb300.so")

SCHEMES = {"MUSCL": 0, "MHM": 1, "Godunov": 2, "Lax": 3}
TIME_ADVANCES = {"SingleStep": 0, "RK2": 1}
RIEMANNS = {"HLL": 0, "HLLC": 1, "PVRS": 2, "StegerWarming": 3, "HLLC_Toro": 4, "HLL_Toro": 5}
LIMITERS = {"minmod": 0, "VanLeer": 1}
BOUNDARIES = {"Regular": 0, "IDWBaseGFM": 1, "LinearBaseGFM": 2, "RiemannBaseGFM": 3, "BCGFM": 4, "HBCGFM": 5,
              "CCM": 6}
GLOBAL_BCS = {"walls": 0, "periodic": 1}
PRECISIONS = {"fp64": 0, "fp64_fast": 1, "fp32c": 2}

STATUS = {0: "OK", 1: "EINVAL", 2: "ENOMEM", 3: "ENAN", 4: "ETIMEOUT", 5: "ECUDA", 6: "ESTATE"}


class IbtfoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"IBTFO_{STATUS.get(code, code)}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("n_x", C.c_int), ("n_y", C.c_int), ("num_ghost_cell", C.c_int),
                ("lo_x", C.c_double), ("lo_y", C.c_double), ("hi_x", C.c_double), ("hi_y", C.c_double),
                ("gamma", C.c_double), ("cfl_number", C.c_double), ("psy_time", C.c_double),
                ("max_iter", C.c_int), ("scheme", C.c_int), ("riemann", C.c_int), ("limiter", C.c_int),
                ("boundary", C.c_int), ("global_boundary", C.c_int), ("precision", C.c_int),
                ("time_advance", C.c_int), ("reserved", C.c_int * 6)]


class Progress(C.Structure):
    _fields_ = [("iter", C.c_int), ("status", C.c_int), ("nan_cells", C.c_int), ("reserved", C.c_int),
                ("now_t", C.c_double), ("dt", C.c_double), ("mass", C.c_double), ("mass_start", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


# every entry point of include/ibtfo.h with its ctypes signature
_P = C.c_void_p
_DP = C.POINTER(C.c_double)
class BatchConfig(C.Structure):
    _fields_ = [("scheme", C.c_int), ("riemann", C.c_int), ("limiter", C.c_int), ("precision", C.c_int),
                ("tile_shape", C.c_int), ("ctas_per_sm", C.c_int), ("graph_steps", C.c_int),
                ("time_advance", C.c_int), ("reserved", C.c_int * 4)]


class BatchTiling(C.Structure):
    _fields_ = [("tile_shape", C.c_int), ("ctas_per_sm", C.c_int), ("max_ctas_per_sm", C.c_int), ("grid", C.c_int),
                ("tiles", C.c_longlong), ("ms_per_step", C.c_double), ("reserved", C.c_int * 4)]

    def as_dict(self):
        return {"tile_shape": TILE_SHAPES_BY_ID[self.tile_shape], "ctas_per_sm": self.ctas_per_sm,
                "max_ctas_per_sm": self.max_ctas_per_sm, "grid": self.grid, "tiles": self.tiles,
                "ms_per_step": self.ms_per_step}


class Body(C.Structure):
    _fields_ = [("kind", C.c_int), ("reserved", C.c_int), ("xc", C.c_double), ("yc", C.c_double),
                ("a", C.c_double), ("b", C.c_double), ("theta", C.c_double)]


def circle(xc, yc, r):
    return Body(0, 0, xc, yc, r, r, 0.0)


def ellipse(xc, yc, a, b, theta):
    return Body(1, 0, xc, yc, a, b, theta)


MAX_BODIES = 8


class ServerConfig(C.Structure):
    _fields_ = [("scheme", C.c_int), ("riemann", C.c_int), ("limiter", C.c_int), ("precision", C.c_int),
                ("memory_budget", C.c_longlong), ("max_active", C.c_int), ("chunk_steps", C.c_int),
                ("tile_shape", C.c_int), ("ctas_per_sm", C.c_int), ("time_advance", C.c_int),
                ("reserved", C.c_int * 5)]


class Request(C.Structure):
    _fields_ = [("id", C.c_longlong), ("arrival", C.c_double), ("n_x", C.c_int), ("n_y", C.c_int),
                ("lo_x", C.c_double), ("lo_y", C.c_double), ("hi_x", C.c_double), ("hi_y", C.c_double),
                ("gamma", C.c_double), ("cfl_number", C.c_double), ("t_end", C.c_double), ("max_iter", C.c_int),
                ("boundary", C.c_int), ("global_boundary", C.c_int), ("n_bodies", C.c_int),
                ("bodies", Body * MAX_BODIES), ("x_split", C.c_double), ("left", C.c_double * 4),
                ("right", C.c_double * 4), ("density_out", C.c_void_p), ("reserved", C.c_int * 8)]


class Result(C.Structure):
    _fields_ = [("id", C.c_longlong), ("status", C.c_int), ("iter", C.c_int), ("nan_cells", C.c_int),
                ("reserved", C.c_int), ("now_t", C.c_double), ("mass", C.c_double), ("mass_start", C.c_double),
                ("arrival", C.c_double), ("admitted", C.c_double), ("finished", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("admitted", C.c_longlong), ("completed", C.c_longlong),
                ("failed", C.c_longlong), ("pending", C.c_int), ("active", C.c_int), ("retiring", C.c_int),
                ("peak_active", C.c_int), ("bytes_in_use", C.c_longlong), ("peak_bytes", C.c_longlong),
                ("memory_budget", C.c_longlong), ("chunks", C.c_longlong), ("steps", C.c_longlong),
                ("tile_shape", C.c_int), ("ctas_per_sm", C.c_int), ("reserved", C.c_int * 6)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


TILE_SHAPES = {"32x8": 0, "32x16": 1, "64x8": 2}
TILE_SHAPES_BY_ID = {v: k for k, v in TILE_SHAPES.items()}


SIGNATURES = {
    "ibtfo_abi_version": (C.c_int, []),
    "ibtfo_last_error": (C.c_char_p, []),
    "ibtfo_launch_count": (C.c_longlong, []),
    "ibtfo_create": (C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
    "ibtfo_destroy": (C.c_int, [_P]),
    "ibtfo_set_stream": (C.c_int, [_P, _P]),
    "ibtfo_setup_geometry": (C.c_int, [_P, _DP]),
    "ibtfo_get_geometry": (C.c_int, [_P, _DP]),
    "ibtfo_num_sch": (C.c_int, [_P]),
    "ibtfo_get_scheme_index": (C.c_int, [_P, _DP]),
    "ibtfo_num_ghost_cells": (C.c_int, [_P]),
    "ibtfo_get_cut_cells": (C.c_int, [_P, _DP, _DP, _DP]),
    "ibtfo_set_state": (C.c_int, [_P, _DP]),
    "ibtfo_get_state": (C.c_int, [_P, _DP, _DP]),
    "ibtfo_put_state": (C.c_int, [_P, _DP]),
    "ibtfo_step_host": (C.c_int, [_P, _DP, _DP, C.POINTER(Progress)]),
    "ibtfo_step_host_bytes": (C.c_int, [_P, C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "ibtfo_advance": (C.c_int, [_P, C.c_int]),
    "ibtfo_enqueue_sweep": (C.c_int, [_P]),
    "ibtfo_enqueue_boundary": (C.c_int, [_P]),
    "ibtfo_step": (C.c_int, [_P, C.POINTER(Progress)]),
    "ibtfo_run": (C.c_int, [_P, C.c_int, C.POINTER(Progress)]),
    "ibtfo_get_progress": (C.c_int, [_P, C.POINTER(Progress)]),
    "ibtfo_synchronize": (C.c_int, [_P]),
    "ibtfo_dt_mass_noalloc": (C.c_int, [_P, C.c_longlong, C.c_int, _P, C.c_int, C.c_int, C.c_int, C.c_double,
                                        C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, _P, _P]),
    "ibtfo_inp_open": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "ibtfo_inp_parse": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "ibtfo_inp_close": (None, [_P]),
    "ibtfo_inp_get": (C.c_int, [_P, C.c_char_p, C.c_double, _DP]),
    "ibtfo_inp_get_string": (C.c_int, [_P, C.c_char_p, C.c_char_p, C.c_int]),
    "ibtfo_config_from_inp": (C.c_int, [_P, C.POINTER(Config)]),
    "ibtfo_case_phi": (C.c_int, [C.c_char_p, _P, C.POINTER(Config), _DP]),
    "ibtfo_case_init": (C.c_int, [C.c_char_p, _P, C.POINTER(Config), _DP, _DP]),
    "ibtfo_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(_P)]),
    "ibtfo_host_free": (C.c_int, [_P]),
    "ibtfo_fp64_pipe_rate": (C.c_int, [C.c_int, _DP, _DP]),
    "ibtfo_fast_math_eval": (C.c_int, [C.c_int, _DP, _DP, C.c_int]),
    "ibtfo_query": (C.c_int, [_P]),
    "ibtfo_write_vtk": (C.c_int, [_P, C.c_char_p, C.c_int]),
    "ibtfo_write_vtk_async": (C.c_int, [_P, C.c_char_p, C.c_int]),
    "ibtfo_output_wait": (C.c_int, [_P]),
    "ibtfo_save_checkpoint": (C.c_int, [_P, C.c_char_p]),
    "ibtfo_load_checkpoint": (C.c_int, [_P, C.c_char_p]),
    "ibtfo_setup_bodies": (C.c_int, [_P, C.POINTER(Body), C.c_int]),
    "ibtfo_init_x_split": (C.c_int, [_P, C.c_double, _DP, _DP]),
    "ibtfo_post_shock_state": (C.c_int, [C.c_double, C.c_double, _DP, _DP]),
    "ibtfo_release_geometry": (C.c_int, [_P]),
    "ibtfo_get_density": (C.c_int, [_P, _DP, C.c_int]),
    "ibtfo_case_bytes": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "ibtfo_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(_P)]),
    "ibtfo_server_destroy": (C.c_int, [_P]),
    "ibtfo_server_submit": (C.c_int, [_P, C.POINTER(Request)]),
    "ibtfo_server_start": (C.c_int, [_P]),
    "ibtfo_server_clock": (C.c_double, [_P]),
    "ibtfo_server_pump": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "ibtfo_server_run": (C.c_int, [_P, C.c_double]),
    "ibtfo_server_poll": (C.c_int, [_P, C.POINTER(Result), C.c_int]),
    "ibtfo_server_stats_get": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "ibtfo_batch_create": (C.c_int, [C.POINTER(BatchConfig), C.POINTER(_P)]),
    "ibtfo_batch_destroy": (C.c_int, [_P]),
    "ibtfo_batch_set_stream": (C.c_int, [_P, _P]),
    "ibtfo_batch_add": (C.c_int, [_P, _P, C.POINTER(C.c_int)]),
    "ibtfo_batch_remove": (C.c_int, [_P, C.c_int]),
    "ibtfo_batch_size": (C.c_int, [_P]),
    "ibtfo_batch_num_slots": (C.c_int, [_P]),
    "ibtfo_batch_case": (_P, [_P, C.c_int]),
    "ibtfo_batch_advance": (C.c_int, [_P, C.c_int]),
    "ibtfo_batch_progress_enqueue": (C.c_int, [_P]),
    "ibtfo_batch_progress_read": (C.c_int, [_P, C.POINTER(Progress), C.POINTER(C.c_int), C.c_int, C.c_int]),
    "ibtfo_batch_progress": (C.c_int, [_P, C.POINTER(Progress), C.POINTER(C.c_int), C.c_int]),
    "ibtfo_batch_synchronize": (C.c_int, [_P]),
    "ibtfo_batch_set_tiling": (C.c_int, [_P, C.c_int, C.c_int]),
    "ibtfo_batch_get_tiling": (C.c_int, [_P, C.POINTER(BatchTiling)]),
    "ibtfo_batch_autotune": (C.c_int, [_P, C.c_int, C.POINTER(BatchTiling), C.POINTER(BatchTiling), C.c_int,
                                       C.POINTER(C.c_int)]),
}

_I = C.c_int
_D = C.c_double
# include/ibtfo_ref.h: the reference's entry points over host arrays
REF_SIGNATURES = {
    "ibtfo_ref_configure": (None, [_I] * 6),
    "ibtfo_ref_status": (_I, []),
    "ibtfo_ref_Psy_coord": (None, [_D, _D, _D, _D, _I, _I, _I, _DP, _I, _I]),
    "ibtfo_ref_Level_Set": (None, [_I, _I, _I, _DP, _I, _I]),
    "ibtfo_ref_Scheme_Index": (None, [_I, _I, _I, _DP, _DP, _I, _I]),
    "ibtfo_ref_TimeAdvance": (None, [_D, _D, _I, _I, _I, _D, _D, _DP, _DP, _DP, _DP, _DP, _I, _I]),
    "ibtfo_ref_Advance": (None, [_D, _D, _I, _I, _I, _D, _D, _DP, _DP, _DP, _DP, _I, _I]),
    "ibtfo_ref_Boundary": (None, [_I, _I, _I, _D, _DP, _DP, _DP, _DP, _I, _I]),
    "ibtfo_ref_Global_Boundary": (None, [_I, _I, _I, _D, _DP, _DP, _I, _I]),
    "ibtfo_ref_ComputeDt": (None, [_D, _D, _I, _I, _I, _D, _D, _DP, _DP, _DP, _I, _I]),
    "ibtfo_ref_CaculateMass": (None, [_D, _D, _I, _I, _I, _DP, _DP, _DP, _I, _I]),
    "ibtfo_ref_WriteData": (None, [_D, _D, _D, _D, _I, _I, _I, _I, _D, _D, _DP, _DP, _I, _I]),
    "ibtfo_ref_update_self": (None, [_DP]),
    "ibtfo_ref_update_device": (None, [_DP]),
    "ibtfo_ref_release": (None, [_DP]),
}

_lib = None


def lib():
    """The loaded C library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m ibtfo_gb300.build` (needs nvcc)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in list(SIGNATURES.items()) + list(REF_SIGNATURES.items()):
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(code):
    if code != 0:
        raise IbtfoError(code, lib().ibtfo_last_error().decode(errors="replace"))


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def launch_count() -> int:
    return lib().ibtfo_launch_count()


def fp64_pipe_rate(iters: int = 4096) -> tuple[float, float]:
    """(FP64 thread instructions per second, seconds of the timed launch) of
    the current GPU: independent DFMA chains on every SM, CUDA-event timed."""
    r, t = C.c_double(), C.c_double()
    _check(lib().ibtfo_fp64_pipe_rate(int(iters), C.byref(r), C.byref(t)))
    return r.value, t.value


FAST_MATH = {"rcp_f64": 0, "sqrt_f64": 1, "rcp_f32": 2, "sqrt_f32": 3, "div_f64": 4, "libsqrt_f64": 5,
             "div_f32": 6, "libsqrt_f32": 7}


def fast_math_eval(fn: str, x) -> np.ndarray:
    """The fast precisions' reciprocal / square root (or CUDA's IEEE ones)
    evaluated on the GPU at the values x (float64 in and out)."""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
    y = np.empty_like(x)
    _check(lib().ibtfo_fast_math_eval(FAST_MATH[fn], _dp(x), _dp(y), int(x.size)))
    return y


class Case:
    """One problem resident on the current CUDA device."""

    def __init__(self, n_x, n_y, ng=2, lo=(0.0, 0.0), hi=(1.0, 1.0), gamma=1.4, cfl=0.5, t_end=1.0,
                 max_iter=100000, scheme="MUSCL", riemann="HLL", limiter="minmod", boundary="Regular",
                 gbc="walls", precision="fp64", time="SingleStep"):
        L = lib()
        cfg = Config(n_x, n_y, ng, lo[0], lo[1], hi[0], hi[1], gamma, cfl, t_end, max_iter,
                     SCHEMES[scheme], RIEMANNS[riemann], LIMITERS[limiter], BOUNDARIES[boundary], GLOBAL_BCS[gbc],
                     PRECISIONS[precision], TIME_ADVANCES[time])
        h = _P()
        _check(L.ibtfo_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.cfg = cfg
        self.n_x, self.n_y, self.ng = n_x, n_y, ng
        self.M, self.N = n_x + 2 * ng, n_y + 2 * ng
        self.nsch = L.ibtfo_num_sch(h)

    @classmethod
    def from_workload(cls, w, **over):
        g = w.grid
        kw = dict(n_x=g.n_x, n_y=g.n_y, ng=g.ng, lo=(g.lo_x, g.lo_y), hi=(g.hi_x, g.hi_y), gamma=w.gamma, cfl=w.cfl,
                  t_end=w.t_end, scheme=w.scheme, riemann=w.riemann, limiter=w.limiter, boundary=w.boundary,
                  gbc=w.gbc, time=getattr(w, "time", "SingleStep"))
        kw.update(over)
        return cls(**kw)

    def close(self):
        if getattr(self, "h", None):
            lib().ibtfo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---------------------------------------------------------- set-up
    def setup_geometry(self, phi):
        phi = np.ascontiguousarray(phi, dtype=np.float64).reshape(-1)
        if phi.size != self.M * self.N:
            raise ValueError("phi must have M*N values")
        _check(lib().ibtfo_setup_geometry(self.h, _dp(phi)))

    def get_geometry(self):
        out = np.empty(self.M * self.N * 6)
        _check(lib().ibtfo_get_geometry(self.h, _dp(out)))
        return out

    def get_scheme_index(self):
        out = np.empty(self.M * self.N * self.nsch)
        _check(lib().ibtfo_get_scheme_index(self.h, _dp(out)))
        return out

    @property
    def num_ghost_cells(self):
        return lib().ibtfo_num_ghost_cells(self.h)

    def cut_cells(self):
        """(alpha, ax, ay), each (N, M), of a cut-cell case."""
        a, x, y = (np.empty(self.M * self.N) for _ in range(3))
        _check(lib().ibtfo_get_cut_cells(self.h, _dp(a), _dp(x), _dp(y)))
        return a.reshape(self.N, self.M), x.reshape(self.N, self.M), y.reshape(self.N, self.M)

    def cell_types(self):
        return self.get_geometry().reshape(-1, 6)[:, 5].copy()

    def set_state(self, u0):
        u0 = np.ascontiguousarray(u0, dtype=np.float64).reshape(-1)
        if u0.size != self.M * self.N * 4:
            raise ValueError("u0 must have M*N*4 values")
        _check(lib().ibtfo_set_state(self.h, _dp(u0)))

    def set_state_ptr(self, host_ptr: int):
        """set_state from a raw host address (e.g. pinned memory), M*N*4 doubles."""
        _check(lib().ibtfo_set_state(self.h, C.cast(C.c_void_p(host_ptr), _DP)))

    def get_state(self, u_new=False):
        uo = np.empty(self.M * self.N * 4)
        un = np.empty(self.M * self.N * 4) if u_new else None
        _check(lib().ibtfo_get_state(self.h, _dp(uo), _dp(un) if un is not None else None))
        return (uo, un) if u_new else uo

    def put_state(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        if u.size != self.M * self.N * 4:
            raise ValueError("u must have M*N*4 values")
        _check(lib().ibtfo_put_state(self.h, _dp(u)))

    def put_state_ptr(self, host_ptr: int):
        _check(lib().ibtfo_put_state(self.h, C.cast(C.c_void_p(host_ptr), _DP)))

    def get_state_ptr(self, host_ptr: int):
        _check(lib().ibtfo_get_state(self.h, C.cast(C.c_void_p(host_ptr), _DP), None))

    def step_host_ptr(self, in_ptr: int, out_ptr: int):
        """One step on host buffers (raw addresses, M*N*4 doubles each; may be
        the same): put the state, step, read the new state back; returns the
        progress.  In place, from the second call on the same buffer, only
        the cells a step reads go in and only those it can change come back;
        solid cells keep what the buffer holds."""
        p = Progress()
        _check(lib().ibtfo_step_host(self.h, C.cast(C.c_void_p(in_ptr), _DP), C.cast(C.c_void_p(out_ptr), _DP),
                                     C.byref(p)))
        return p.as_dict()

    def step_host_bytes(self, in_place=True):
        """(host-to-device, device-to-host) bytes of one step_host_ptr call
        (in place: a call after the first on the same buffer)."""
        a, b = C.c_longlong(), C.c_longlong()
        _check(lib().ibtfo_step_host_bytes(self.h, 1 if in_place else 0, C.byref(a), C.byref(b)))
        return a.value, b.value

    # ---------------------------------------------------------- stepping
    def set_stream(self, stream_ptr: int | None):
        _check(lib().ibtfo_set_stream(self.h, C.c_void_p(stream_ptr) if stream_ptr else None))

    def advance(self, nsteps: int):
        _check(lib().ibtfo_advance(self.h, int(nsteps)))

    def enqueue_sweep(self):
        _check(lib().ibtfo_enqueue_sweep(self.h))

    def enqueue_boundary(self):
        _check(lib().ibtfo_enqueue_boundary(self.h))

    def step(self):
        p = Progress()
        _check(lib().ibtfo_step(self.h, C.byref(p)))
        return p.as_dict()

    def run(self, stop_on_nan=False):
        p = Progress()
        _check(lib().ibtfo_run(self.h, 1 if stop_on_nan else 0, C.byref(p)))
        return p.as_dict()

    def progress(self):
        p = Progress()
        _check(lib().ibtfo_get_progress(self.h, C.byref(p)))
        return p.as_dict()

    def synchronize(self):
        _check(lib().ibtfo_synchronize(self.h))

    def setup_bodies(self, bodies):
        """Geometry from analytic bodies (circle()/ellipse()), phi built on the GPU."""
        arr = (Body * max(len(bodies), 1))(*bodies)
        _check(lib().ibtfo_setup_bodies(self.h, arr, len(bodies)))

    def init_x_split(self, x_split, left, right):
        """Initial primitive states left of / right of x = x_split, built on the GPU."""
        L = np.ascontiguousarray(left, dtype=np.float64)
        R = np.ascontiguousarray(right, dtype=np.float64)
        _check(lib().ibtfo_init_x_split(self.h, float(x_split), _dp(L), _dp(R)))

    def release_geometry(self):
        _check(lib().ibtfo_release_geometry(self.h))

    def density(self):
        out = np.empty(self.n_x * self.n_y)
        _check(lib().ibtfo_get_density(self.h, _dp(out), 1))
        return out.reshape(self.n_y, self.n_x)

    def write_vtk(self, path, binary=False, wait=True):
        """VTK file of the current state (the reference's WriteData layout).
        wait=False writes it off the step path: the snapshot is taken in order
        with the steps and the file is written while stepping continues
        (output_wait() joins it)."""
        fn = lib().ibtfo_write_vtk if wait else lib().ibtfo_write_vtk_async
        _check(fn(self.h, os.fsencode(path), 1 if binary else 0))

    def output_wait(self):
        _check(lib().ibtfo_output_wait(self.h))

    def save_checkpoint(self, path):
        _check(lib().ibtfo_save_checkpoint(self.h, os.fsencode(path)))

    def load_checkpoint(self, path):
        _check(lib().ibtfo_load_checkpoint(self.h, os.fsencode(path)))

    def idle(self) -> bool:
        """True when nothing queued on the case's stream is pending (does not wait)."""
        code = lib().ibtfo_query(self.h)
        if code == 4:
            return False
        _check(code)
        return True


class Batch:
    """Many cases stepped together (persistent batched sweep, CUDA graphs).

    Every case must share the batch's scheme, Riemann solver, limiter and
    precision; `add` takes a Case whose state is set.  A case in a batch is
    stepped by the batch only; its own get_state / progress stay valid after
    `synchronize`."""

    def __init__(self, scheme="MUSCL", riemann="HLL", limiter="minmod", precision="fp32c", tile_shape="32x8",
                 ctas_per_sm=0, graph_steps=16, time="SingleStep"):
        cfg = BatchConfig(SCHEMES[scheme], RIEMANNS[riemann], LIMITERS[limiter], PRECISIONS[precision],
                          TILE_SHAPES[tile_shape], ctas_per_sm, graph_steps, TIME_ADVANCES[time])
        h = _P()
        _check(lib().ibtfo_batch_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.cases = {}

    def close(self):
        if getattr(self, "h", None):
            lib().ibtfo_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add(self, case: Case) -> int:
        slot = C.c_int()
        _check(lib().ibtfo_batch_add(self.h, case.h, C.byref(slot)))
        self.cases[slot.value] = case
        return slot.value

    def remove(self, slot: int):
        _check(lib().ibtfo_batch_remove(self.h, int(slot)))
        return self.cases.pop(slot, None)

    def __len__(self):
        return lib().ibtfo_batch_size(self.h)

    @property
    def num_slots(self):
        return lib().ibtfo_batch_num_slots(self.h)

    def set_stream(self, stream_ptr: int | None):
        _check(lib().ibtfo_batch_set_stream(self.h, C.c_void_p(stream_ptr) if stream_ptr else None))

    def advance(self, nsteps: int):
        _check(lib().ibtfo_batch_advance(self.h, int(nsteps)))

    def progress(self):
        """{slot: (progress dict, active)} for every occupied slot (waits)."""
        n = self.num_slots
        arr = (Progress * max(n, 1))()
        act = (C.c_int * max(n, 1))()
        _check(lib().ibtfo_batch_progress(self.h, arr, act, n))
        return {k: (arr[k].as_dict(), bool(act[k])) for k in range(n) if k in self.cases}

    def progress_enqueue(self):
        _check(lib().ibtfo_batch_progress_enqueue(self.h))

    def progress_read(self, wait=True):
        """Like progress() for the last enqueued snapshot; None if not ready (wait=False)."""
        n = self.num_slots
        arr = (Progress * max(n, 1))()
        act = (C.c_int * max(n, 1))()
        code = lib().ibtfo_batch_progress_read(self.h, arr, act, n, 1 if wait else 0)
        if code == 4 and not wait:
            return None
        _check(code)
        return {k: (arr[k].as_dict(), bool(act[k])) for k in range(n) if k in self.cases}

    def synchronize(self):
        _check(lib().ibtfo_batch_synchronize(self.h))

    def set_tiling(self, tile_shape="32x8", ctas_per_sm=0):
        _check(lib().ibtfo_batch_set_tiling(self.h, TILE_SHAPES[tile_shape], int(ctas_per_sm)))

    def tiling(self):
        t = BatchTiling()
        _check(lib().ibtfo_batch_get_tiling(self.h, C.byref(t)))
        return t.as_dict()

    def autotune(self, steps=8, max_trials=64):
        best = BatchTiling()
        trials = (BatchTiling * max_trials)()
        n = C.c_int()
        _check(lib().ibtfo_batch_autotune(self.h, int(steps), C.byref(best), trials, max_trials, C.byref(n)))
        return best.as_dict(), [trials[i].as_dict() for i in range(min(n.value, max_trials))]


def post_shock_state(mach, gamma=1.4, pre=(1.0, 0.0, 0.0, 1.0)):
    pre = np.ascontiguousarray(pre, dtype=np.float64)
    out = np.empty(4)
    _check(lib().ibtfo_post_shock_state(float(mach), float(gamma), _dp(pre), _dp(out)))
    return tuple(out)


def case_bytes(cfg: "Config"):
    r, s = C.c_longlong(), C.c_longlong()
    _check(lib().ibtfo_case_bytes(C.byref(cfg), C.byref(r), C.byref(s)))
    return r.value, s.value


def request(id, n_x, n_y, lo, hi, t_end, bodies=(), x_split=0.0, left=(1.0, 0.0, 0.0, 1.0),
            right=(1.0, 0.0, 0.0, 1.0), arrival=0.0, gamma=1.4, cfl=0.45, boundary="IDWBaseGFM", gbc="walls",
            max_iter=0, density_out=None):
    """A Request; density_out: optional PinnedBuffer (or integer address) of n_x*n_y doubles."""
    if len(bodies) > MAX_BODIES:
        raise ValueError(f"at most {MAX_BODIES} bodies")
    r = Request()
    r.id, r.arrival, r.n_x, r.n_y = int(id), float(arrival), int(n_x), int(n_y)
    r.lo_x, r.lo_y, r.hi_x, r.hi_y = float(lo[0]), float(lo[1]), float(hi[0]), float(hi[1])
    r.gamma, r.cfl_number, r.t_end, r.max_iter = float(gamma), float(cfl), float(t_end), int(max_iter)
    r.boundary, r.global_boundary = BOUNDARIES[boundary], GLOBAL_BCS[gbc]
    r.n_bodies = len(bodies)
    for k, b in enumerate(bodies):
        r.bodies[k] = b
    r.x_split = float(x_split)
    r.left[:] = [float(v) for v in left]
    r.right[:] = [float(v) for v in right]
    if density_out is not None:
        r.density_out = density_out.ptr if hasattr(density_out, "ptr") else int(density_out)
    return r


class Server:
    """Continuous-batching request loop (native; see ibtfo_server_* in ibtfo.h)."""

    def __init__(self, scheme="MUSCL", riemann="HLLC", limiter="minmod", precision="fp32c", memory_budget=0,
                 max_active=0, chunk_steps=32, tile_shape="32x8", ctas_per_sm=0, time="SingleStep"):
        cfg = ServerConfig(SCHEMES[scheme], RIEMANNS[riemann], LIMITERS[limiter], PRECISIONS[precision],
                           int(memory_budget), int(max_active), int(chunk_steps),
                           -1 if tile_shape == "auto" else TILE_SHAPES[tile_shape], int(ctas_per_sm),
                           TIME_ADVANCES[time])
        h = _P()
        _check(lib().ibtfo_server_create(C.byref(cfg), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().ibtfo_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, req: "Request"):
        _check(lib().ibtfo_server_submit(self.h, C.byref(req)))

    def start(self):
        _check(lib().ibtfo_server_start(self.h))

    def clock(self):
        return lib().ibtfo_server_clock(self.h)

    def pump(self):
        busy = C.c_int()
        _check(lib().ibtfo_server_pump(self.h, C.byref(busy)))
        return bool(busy.value)

    def run(self, max_seconds=0.0):
        _check(lib().ibtfo_server_run(self.h, float(max_seconds)))

    def poll(self, max_results=4096):
        out = (Result * max_results)()
        n = lib().ibtfo_server_poll(self.h, out, max_results)
        return [out[i].as_dict() for i in range(n)]

    def stats(self):
        st = ServerStats()
        _check(lib().ibtfo_server_stats_get(self.h, C.byref(st)))
        return st.as_dict()


class Inp:
    """A parsed .inp file (the reference's ParamReader rules)."""

    def __init__(self, path=None, text=None):
        h = _P()
        if text is not None:
            _check(lib().ibtfo_inp_parse(text.encode(), C.byref(h)))
        else:
            _check(lib().ibtfo_inp_open(str(path).encode(), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().ibtfo_inp_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get(self, key, default=0.0):
        v = C.c_double()
        found = lib().ibtfo_inp_get(self.h, key.encode(), float(default), C.byref(v))
        return v.value, bool(found)

    def get_string(self, key):
        buf = C.create_string_buffer(256)
        return buf.value.decode() if lib().ibtfo_inp_get_string(self.h, key.encode(), buf, 256) else None

    def config(self):
        cfg = Config()
        _check(lib().ibtfo_config_from_inp(self.h, C.byref(cfg)))
        return cfg


def case_phi(name, cfg, inp=None):
    n = (cfg.n_x + 2 * cfg.num_ghost_cell) * (cfg.n_y + 2 * cfg.num_ghost_cell)
    out = np.empty(n)
    _check(lib().ibtfo_case_phi(name.encode(), inp.h if inp else None, C.byref(cfg), _dp(out)))
    return out


def case_init(name, cfg, xycoord, inp=None):
    xy = np.ascontiguousarray(xycoord, dtype=np.float64).reshape(-1)
    out = np.empty(xy.size // 6 * 4)
    _check(lib().ibtfo_case_init(name.encode(), inp.h if inp else None, C.byref(cfg), _dp(xy), _dp(out)))
    return out


def config(n_x, n_y, ng=2, lo=(0.0, 0.0), hi=(1.0, 1.0), gamma=1.4, cfl=0.5, t_end=1.0, max_iter=100000,
           scheme="MUSCL", riemann="HLL", limiter="minmod", boundary="Regular", gbc="walls", precision="fp64",
           time="SingleStep"):
    return Config(n_x, n_y, ng, lo[0], lo[1], hi[0], hi[1], gamma, cfl, t_end, max_iter, SCHEMES[scheme],
                  RIEMANNS[riemann], LIMITERS[limiter], BOUNDARIES[boundary], GLOBAL_BCS[gbc], PRECISIONS[precision],
                  TIME_ADVANCES[time])


class PinnedBuffer:
    """Page-locked host buffer of float64 (cudaHostAlloc through the C ABI)."""

    def __init__(self, n):
        p = _P()
        _check(lib().ibtfo_host_alloc(8 * n, C.byref(p)))
        self.ptr = p.value
        self.n = n
        self.array = np.ctypeslib.as_array(C.cast(p, _DP), shape=(n,))

    def close(self):
        if self.ptr:
            lib().ibtfo_host_free(C.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
