"""Helpers of the reference-pin tests: build the driver that runs the reference's own kernels
(oracle/ref_pin/ref_driver.cpp over oracle/_ref/<case>.cubin), write its inputs, run it and read its
outputs.  Test infrastructure only."""
import os
import subprocess
import sys

import numpy as np

from conftest import REPO
from rbtp import Config, derive

sys.path.insert(0, os.path.join(REPO, "oracle", "ref_pin"))
import cases  # noqa: E402

REF = os.path.join(REPO, "oracle", "_ref")
DRIVER_SRC = os.path.join(REPO, "oracle", "ref_pin", "ref_driver.cpp")
DRIVER = os.path.join(REF, "ref_driver")


def have_cubins() -> bool:
    return os.path.exists(os.path.join(REF, "ref_single.cubin"))


def build_driver() -> str:
    for libdir in ("/usr/local/cuda/lib64/stubs", "/usr/local/cuda/targets/sbsa-linux/lib/stubs",
                   "/usr/local/cuda/targets/x86_64-linux/lib/stubs"):
        if os.path.exists(os.path.join(libdir, "libcuda.so")):
            break
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I/usr/local/cuda/include", DRIVER_SRC, "-o", DRIVER,
                        "-L" + libdir, "-lcuda"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return DRIVER


def cfg_of(case: str, **over) -> Config:
    """librbtp / oracle configuration of a pin case (no output cadence, FP64 storage)."""
    v = cases.values(case, **over)
    v.update(nend=1 << 30, ndiag=0, nflowout=0, nnuout=0, nout_p=0, storage=0)
    return Config.defaults(**v)


def write_inputs(d, cfg, f=None, g=None, f7=None, parts=None, **extra):
    """cfg.txt (the constants the driver sets, plus `extra` keys such as synthetic/seed/amp or
    sample_stride) and the binary start state (omitted with synthetic=1)."""
    der = derive(cfg)
    keys = dict(lx=cfg.lx, ly=cfg.ly, lz=cfg.lz, npart=der.npart, radius=der.particle_radius,
                mass=der.particle_mass, inertia=der.particle_inertia,
                heat_capacity=der.particle_heat_capacity, cp_fluid=cfg.cp_fluid,
                rho_particle_ratio=cfg.rho_particle_ratio, tau=der.tau, tauc=der.tauc, grav0=der.grav0,
                beta=cfg.beta, t_hot=cfg.t_hot, t_cold=cfg.t_cold, t_ref=cfg.t_ref, diff=der.diff,
                visc=cfg.visc, repforce_scale=cfg.repforce_scale, rep_min_gap=cfg.rep_min_gap,
                rep_min_gap_w=cfg.rep_min_gap_w, particle_fraction=cfg.particle_fraction,
                cp_particle_ratio=cfg.cp_particle_ratio)
    keys.update(extra)
    with open(os.path.join(d, "cfg.txt"), "w") as fh:
        for k, v in keys.items():
            fh.write(f"{k} {float(v)!r}\n")
    if f is not None:
        f.tofile(os.path.join(d, "f.bin"))
        g.tofile(os.path.join(d, "g.bin"))
        f7.tofile(os.path.join(d, "flow7.bin"))
    if parts is not None:
        np.ascontiguousarray(parts).tofile(os.path.join(d, "particles.bin"))


def run(driver, case, base, cfg, f, g, f7, parts, steps, timeout=900, **extra):
    """Run `steps` reference steps from the given start; returns the output directory."""
    ind, outd = base / "in", base / "out"
    ind.mkdir(parents=True)
    outd.mkdir()
    write_inputs(str(ind), cfg, f, g, f7, parts, **extra)
    r = subprocess.run([driver, os.path.join(REF, case + ".cubin"), str(ind), str(steps), str(outd)],
                       capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stdout + r.stderr
    return outd


def run_nu(driver, case, base, cfg, f, g, f7, parts, steps, every, timeout=1800, **extra):
    """Nu rows (output_nu's 7 columns) of the reference's kernels every `every` steps."""
    ind = base / "in"
    ind.mkdir(parents=True)
    write_inputs(str(ind), cfg, f, g, f7, parts, **extra)
    out = base / "nu.bin"
    r = subprocess.run([driver, os.path.join(REF, case + ".cubin"), str(ind), "nu", str(steps), str(every),
                        str(out)], capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stdout + r.stderr
    return np.fromfile(out).reshape(-1, 7)


def links_from(path):
    """(node, dir, pid, q) of a links dump, sorted by (node, dir)."""
    a = np.fromfile(path, dtype=np.float64).reshape(-1, 4)
    order = np.lexsort((a[:, 1], a[:, 0]))
    a = a[order]
    return a[:, 0].astype(np.int64), a[:, 1].astype(np.int64), a[:, 2].astype(np.int64), a[:, 3]
