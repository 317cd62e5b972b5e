"""Builds libpn.so in-tree (pn_gb300/_lib/) for sm_103a.

The CUDA sources are compiled with nvcc (one -gencode, arch=compute_103a,code=sm_103a), the
host C utilities with gcc, in parallel; the shared library links the CUDA runtime statically
so it loads without torch.  Run ``python -m pn_gb300.build`` or call :func:`build`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libpn.so")
CLI = os.path.join(HERE, "cli", "pn_run.c")
EXE = os.path.join(OUT, "pn_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]
CC_FLAGS = ["-O2", "-fPIC", "-std=gnu11", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    c = sorted(f for f in os.listdir(CSRC) if f.endswith(".c"))
    return cu, c


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile (incrementally) and link libpn.so; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    cu, c = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "pn.h"))
    jobs = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj])
    for f in c:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["gcc"] + CC_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lm"])
    if force or _stale(EXE, [CLI, LIB]):
        # the command-line driver (the reference's main loop on the device-resident API)
        _run(["gcc"] + CC_FLAGS + [CLI, "-L" + OUT, "-lpn", "-Wl,-rpath," + OUT, "-lm", "-o", EXE])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
