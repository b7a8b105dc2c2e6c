"""Builds librbtp.so (the sm_103a CUDA library behind include/rbtp.h) and the drop-in host rb3d.

Every CUDA translation unit is compiled for sm_103a only, in parallel, into _build/, and linked
into rbtp/_lib/librbtp.so inside this package directory (in-tree, so test and bench processes
load it from here).  Host code is compiled with -ffp-contract=off so that host-side arithmetic
(particle placement, diagnostics formulas) gives identical results on x86-64 and aarch64.

Usage:  python rbtp_build.py [--clean] [--jobs N] [--no-host]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "rbtp", "_lib")
LIB = os.path.join(LIBDIR, "librbtp.so")
RB3D = os.path.join(LIBDIR, "rb3d")

SOURCES = ["lbm_step.cu", "batch_step.cu", "particles.cu", "diagnostics.cu", "api.cu", "batch.cu", "server.cu", "noalloc.cu", "calib.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-I" + os.path.join(REPO, "include"),
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + res.stdout)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _arch_guard() -> None:
    """Objects built on another machine architecture (x86-64 here, aarch64 on the GPU hosts) are
    discarded so a copied tree never links stale foreign objects."""
    import platform
    stamp = os.path.join(BUILD, "ARCH")
    mach = platform.machine()
    try:
        old = open(stamp).read().strip()
    except OSError:
        old = None
    if old != mach:
        for d in (BUILD, LIBDIR):
            if os.path.isdir(d):
                shutil.rmtree(d)
        os.makedirs(BUILD, exist_ok=True)
        with open(stamp, "w") as fh:
            fh.write(mach + "\n")


def build(jobs: int = 0, host: bool = True, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    _arch_guard()
    os.makedirs(LIBDIR, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, h) for h in ("rbtp_internal.cuh", "step_node.cuh", "handle.cuh")]
    headers.append(os.path.join(REPO, "include", "rbtp.h"))
    objs, todo = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers + [os.path.abspath(__file__)]):
            todo.append([nv] + NVCC_FLAGS + ["-c", s, "-o", o])
    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            for fut in [ex.submit(_run, c) for c in todo]:
                fut.result()
    if todo or _stale(LIB, objs):
        _run([nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    if host:
        main = os.path.join(HOST, "rb3d_main.cpp")
        if os.path.exists(main) and _stale(RB3D, [main, LIB, os.path.join(HOST, "parameters.h")]):
            _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(REPO, "include"),
                  "-I" + HOST, main, "-o", RB3D, "-L" + LIBDIR, "-lrbtp", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("built", LIB)
    return LIB


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--clean", action="store_true")
    ap.add_argument("--jobs", type=int, default=0)
    ap.add_argument("--no-host", action="store_true")
    a = ap.parse_args()
    if a.clean and os.path.isdir(BUILD):
        shutil.rmtree(BUILD)
    build(a.jobs, host=not a.no_host, verbose=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
