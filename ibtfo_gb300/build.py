"""Build step of the package: compiles the CUDA sources in ibtfo_gb300/csrc/
for sm_103a into ibtfo_gb300/libibtfo_gb300.so (in-tree, git-ignored).

    python -m ibtfo_gb300.build [--jobs N] [--force]

Translation units compile in parallel.  Device code is compiled without
floating-point contraction (the reference's expressions evaluate to the same
binary64 values) except in the *_fast.cu and *_f32.cu units (fp64_fast and FP32 forms);
host code is compiled without contraction so that coordinates and other
host-side values match the reference bit for bit on every host architecture.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libibtfo_gb300.so")
CLI = os.path.join(HERE, "ibtfo_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                  "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build ibtfo_gb300")
    return cand


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    nv = nvcc()
    objs, todo = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            todo.append((s, o))

    def compile_one(so):
        s, o = so
        flags = list(NVFLAGS)
        if os.path.basename(s).endswith(("_fast.cu", "_f32.cu")):
            flags[flags.index("-fmad=false")] = "-fmad=true"  # fp64_fast and FP32 units contract multiply-adds
        cmd = [nv] + flags + ["-c", s, "-o", o]
        if s.endswith(".cpp"):
            cmd = [nv, "-x", "cu"] + NVFLAGS + ["-c", s, "-o", o]
        p = subprocess.run(cmd, capture_output=True, text=True)
        return s, p.returncode, p.stdout + p.stderr

    errors = []
    with cf.ThreadPoolExecutor(jobs or min(8, os.cpu_count() or 4)) as ex:
        for s, rc, out in ex.map(compile_one, todo):
            if rc != 0:
                errors.append(f"{os.path.basename(s)}:\n{out}")
            elif verbose and out.strip():
                print(out)
    if errors:
        raise RuntimeError("CUDA build failed:\n" + "\n".join(errors))
    if todo or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n" + p.stdout + p.stderr)
        os.replace(tmp, LIB)
    cli_src = os.path.join(HERE, "cli", "ibtfo_run.cpp")
    if os.path.exists(cli_src) and (force or _newer(CLI, [cli_src, LIB])):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), cli_src,
               "-L" + HERE, "-libtfo_gb300", "-Wl,-rpath,$ORIGIN", "-o", CLI]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("ibtfo_run build failed:\n" + p.stdout + p.stderr)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(a.force, a.jobs, a.verbose))
    return 0


if __name__ == "__main__":
    sys.exit(main())
