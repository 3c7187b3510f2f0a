"""CPU oracle (test infrastructure only).

Python access to the plain-C FP64 restatement of the reference solver in
oracle/ibtfo_oracle.c, plus a reader for the reference-harness record format.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; the product (ibtfo_gb300) never does.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")


def reference_dir() -> str | None:
    """Root of the reference's source checkout (the directory holding Src/ and
    Test/): $IBTFO_REFERENCE_DIR, else a directory named `reference` beside
    this repository.  None when neither holds the sources (e.g. on a machine
    that only runs the built library)."""
    cand = os.environ.get("IBTFO_REFERENCE_DIR") or \
        os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    return cand if os.path.isdir(os.path.join(cand, "Src")) else None

SCHEMES = {"MUSCL": 0, "MHM": 1, "Godunov": 2, "Lax": 3}
TIME_ADVANCES = {"SingleStep": 0, "RK2": 1}
RIEMANNS = {"HLL": 0, "HLLC": 1, "PVRS": 2, "StegerWarming": 3}
LIMITERS = {"minmod": 0, "VanLeer": 1}
BOUNDARIES = {"Regular": 0, "IDWBaseGFM": 1, "LinearBaseGFM": 2, "RiemannBaseGFM": 3, "BCGFM": 4, "HBCGFM": 5}
GLOBAL_BCS = {"walls": 0, "periodic": 1}


def build(force: bool = False) -> str:
    """Compile liboracle.so (gcc, -O2 -ffp-contract=off -fopenmp)."""
    srcs = [os.path.join(HERE, "ibtfo_oracle.c"), os.path.join(HERE, "ccm_oracle.c")]
    if not force and os.path.exists(LIB_PATH) and \
            os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(s) for s in srcs):
        return LIB_PATH
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=c11"] + srcs + \
        ["-o", LIB_PATH, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER(C.c_double)
        L.or_create.restype = C.c_void_p
        L.or_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.or_destroy.argtypes = [C.c_void_p]
        L.or_set_time_advance.argtypes = [C.c_void_p, C.c_int]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_num_sch.argtypes = [C.c_void_p]
        L.or_setup_geometry.argtypes = [C.c_void_p, P]
        L.or_set_initial_state.argtypes = [C.c_void_p, P]
        L.or_run.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, P, P]
        L.or_run.restype = C.c_int
        L.or_advance.argtypes = [C.c_void_p, C.c_double]
        for f in ("or_boundary", "or_global_boundary"):
            getattr(L, f).argtypes = [C.c_void_p]
        for f in ("or_compute_dt", "or_mass"):
            getattr(L, f).argtypes = [C.c_void_p]
            getattr(L, f).restype = C.c_double
        L.or_array_len.argtypes = [C.c_void_p, C.c_int]
        L.or_array_len.restype = C.c_long
        L.or_get.argtypes = [C.c_void_p, C.c_int, P]
        L.or_put.argtypes = [C.c_void_p, C.c_int, P]
        L.or_scalars.argtypes = [C.c_void_p, P]
        L.or_iter.argtypes = [C.c_void_p]
        L.or_iter.restype = C.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleCase:
    """One case on the CPU oracle (FP64, reference array-of-structures layout)."""

    def __init__(self, n_x, n_y, ng=2, lo=(0.0, 0.0), hi=(1.0, 1.0), gamma=1.4, cfl=0.5, scheme="MUSCL",
                 riemann="HLL", limiter="minmod", boundary="Regular", gbc="walls", time="SingleStep"):
        self.L = lib()
        self.n_x, self.n_y, self.ng = n_x, n_y, ng
        self.M, self.N = n_x + 2 * ng, n_y + 2 * ng
        h = self.L.or_create(n_x, n_y, ng, lo[0], lo[1], hi[0], hi[1], gamma, cfl, SCHEMES[scheme],
                             RIEMANNS[riemann], LIMITERS[limiter], BOUNDARIES[boundary], GLOBAL_BCS[gbc])
        if not h:
            raise ValueError("oracle rejected the configuration")
        self.h = h
        self.L.or_set_time_advance(h, TIME_ADVANCES[time])
        self.nsch = self.L.or_num_sch(h)

    def close(self):
        if self.h:
            self.L.or_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setup_geometry(self, phi):
        phi = np.ascontiguousarray(phi, dtype=np.float64).reshape(-1)
        assert phi.size == self.M * self.N
        self.L.or_setup_geometry(self.h, _p(phi))

    def set_initial_state(self, u0):
        u0 = np.ascontiguousarray(u0, dtype=np.float64).reshape(-1)
        assert u0.size == self.M * self.N * 4
        self.L.or_set_initial_state(self.h, _p(u0))

    def run(self, nsteps, t_end=1e300, max_iter=2 ** 31 - 1):
        dts = np.zeros(max(nsteps, 1))
        ms = np.zeros(max(nsteps, 1))
        n = self.L.or_run(self.h, nsteps, t_end, max_iter, _p(dts), _p(ms))
        return dts[:n], ms[:n]

    def get(self, which):
        idx = {"U_OLD": 0, "U_NEW": 1, "XYCOORD": 2, "SCHEME_IDX": 3, "U_TMP": 4}[which]
        n = self.L.or_array_len(self.h, idx)
        out = np.empty(n)
        self.L.or_get(self.h, idx, _p(out))
        return out

    def put(self, which, arr):
        idx = {"U_OLD": 0, "U_NEW": 1, "XYCOORD": 2, "SCHEME_IDX": 3, "U_TMP": 4}[which]
        arr = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
        assert arr.size == self.L.or_array_len(self.h, idx)
        self.L.or_put(self.h, idx, _p(arr))

    def scalars(self):
        out = np.zeros(4)
        self.L.or_scalars(self.h, _p(out))
        return {"dt": out[0], "now_t": out[1], "mass_start": out[2], "mass_now": out[3],
                "iter": self.L.or_iter(self.h)}


def set_threads(n: int):
    lib().or_set_threads(int(n))


def read_ref_record(path: str) -> dict:
    """Reads one record written by oracle/harness/harness_main.cpp."""
    with open(path, "rb") as f:
        data = f.read()
    assert data[:8] == b"IBTFOREF", "not a reference-harness record"
    M, N, ng, nsch, iters, _ver = struct.unpack_from("<6i", data, 8)
    off = 8 + 24
    now_t, dt = struct.unpack_from("<2d", data, off)
    off += 16
    cells = M * N

    def take(n):
        nonlocal off
        a = np.frombuffer(data, dtype="<f8", count=n, offset=off).copy()
        off += 8 * n
        return a

    rec = {"M": M, "N": N, "ng": ng, "num_sch": nsch, "iters": iters, "now_t": now_t, "dt": dt}
    rec["dts"] = take(iters + 1)
    rec["masses"] = take(iters + 1)
    rec["phi"] = take(cells)
    rec["u_init"] = take(cells * 4)
    rec["xycoord"] = take(cells * 6)
    rec["scheme_idx"] = take(cells * nsch)
    rec["u_old"] = take(cells * 4)
    rec["u_new"] = take(cells * 4)
    assert off == len(data)
    return rec


# ------------------------------------------------------------------ cut cells

CCM_RIEMANNS = {"StegerWarming": 3, "HLLC_Toro": 4, "HLL_Toro": 5}


def _ccm_lib():
    L = lib()
    if not getattr(L, "_ccm_ready", False):
        P = C.POINTER(C.c_double)
        L.ccm_create.restype = C.c_void_p
        L.ccm_create.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_double] * 7 + [C.c_int] * 4
        L.ccm_destroy.argtypes = [C.c_void_p]
        L.ccm_setup.argtypes = [C.c_void_p, P]
        L.ccm_set_state.argtypes = [C.c_void_p, P]
        L.ccm_run.argtypes = [C.c_void_p, C.c_int, P, P]
        L.ccm_run.restype = C.c_int
        L.ccm_get_state.argtypes = [C.c_void_p, P]
        L.ccm_get_geometry.argtypes = [C.c_void_p, P, P, P, C.POINTER(C.c_ubyte)]
        L.ccm_scalars.argtypes = [C.c_void_p, P]
        L._ccm_ready = True
    return L


class CcmOracle:
    """One cut-cell case on the CPU (FP64 restatement of the library's cut-cell method)."""

    def __init__(self, n_x, n_y, ng=2, lo=(0.0, 0.0), hi=(1.0, 1.0), gamma=1.4, cfl=0.45, t_end=1e300,
                 scheme="MUSCL", riemann="HLL_Toro", limiter="minmod", gbc="walls"):
        self.L = _ccm_lib()
        self.n_x, self.n_y, self.ng = n_x, n_y, ng
        self.M, self.N = n_x + 2 * ng, n_y + 2 * ng
        self.h = self.L.ccm_create(n_x, n_y, ng, lo[0], lo[1], hi[0], hi[1], gamma, cfl, t_end, SCHEMES[scheme],
                                   CCM_RIEMANNS[riemann], LIMITERS[limiter], 1 if gbc == "periodic" else 0)

    def close(self):
        if getattr(self, "h", None):
            self.L.ccm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setup(self, phi):
        phi = np.ascontiguousarray(phi, dtype=np.float64).reshape(-1)
        assert phi.size == self.M * self.N
        self.L.ccm_setup(self.h, _p(phi))

    def set_state(self, u0):
        u0 = np.ascontiguousarray(u0, dtype=np.float64).reshape(-1)
        assert u0.size == self.M * self.N * 4
        self.L.ccm_set_state(self.h, _p(u0))

    def run(self, nsteps):
        dts, ms = np.zeros(max(nsteps, 1)), np.zeros(max(nsteps, 1))
        n = self.L.ccm_run(self.h, nsteps, _p(dts), _p(ms))
        return dts[:n], ms[:n]

    def get_state(self):
        out = np.empty(self.M * self.N * 4)
        self.L.ccm_get_state(self.h, _p(out))
        return out

    def geometry(self):
        n = self.M * self.N
        a, ax, ay = np.empty(n), np.empty(n), np.empty(n)
        t = np.empty(n, dtype=np.uint8)
        self.L.ccm_get_geometry(self.h, _p(a), _p(ax), _p(ay), t.ctypes.data_as(C.POINTER(C.c_ubyte)))
        shp = (self.N, self.M)
        return a.reshape(shp), ax.reshape(shp), ay.reshape(shp), t.reshape(shp)

    def scalars(self):
        out = np.zeros(6)
        self.L.ccm_scalars(self.h, _p(out))
        return {"dt": out[0], "now_t": out[1], "mass": out[2], "mass_start": out[3], "iter": int(out[4]),
                "exchanges": int(out[5])}
