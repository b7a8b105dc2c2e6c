"""The drop-in host rb3d (the reference's main.cu surface: parameters.h macros, output cadence and
files) built against a small case and run on the GPU: its Nu_*.txt rows must be the library's own
rbtp_nu values for the same case (to the %15.6E text precision), the binary files must have the
reference's sizes, and a restart from its files (CONTINUOUS_STEPS) must continue the run."""
import glob
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO
from rbtp import Solver, workloads as W

pytestmark = pytest.mark.gpu

HOST = os.path.join(REPO, "rb-thermoparticles_gb300", "host")
LIBDIR = os.path.join(REPO, "rb-thermoparticles_gb300", "rbtp", "_lib")

CASE = dict(lx=48, ly=48, lz=24, rayleigh=1e6, prandtl=0.71, activate_particles=1,
            particle_fraction=0.04, particle_diam_frac=8.0 / 48.0, rho_particle_ratio=1.0)


def _parameters_h(continuous, nend):
    c = CASE
    visc = W.visc_rule(c["lx"], c["rayleigh"], c["prandtl"])
    return f"""#ifndef PARAMETERS_H
#define PARAMETERS_H
#define CONTINUOUS_STEPS {continuous}
#define LX {c['lx']}
#define LY {c['ly']}
#define LZ {c['lz']}
#define LXY (LX * LY)
#define LXYZ (LX * LY * LZ)
#define NPOP 27
#define NEND {nend}
#define NDIAG 10
#define NFLOWOUT 20
#define NNUOUT 10
#define NOUT_P 20
#define RAYLEIGH {c['rayleigh']!r}
#define PRANDTL {c['prandtl']!r}
#define T_HOT 1.0
#define T_COLD 0.0
#define T_REF 0.5
#define BETA 0.0000625
#define VISC {visc!r}
#define RHO0 1.0
#define ACTIVATE_PARTICLES {c['activate_particles']}
#define PARTICLE_FRACTION {c['particle_fraction']!r}
#define PARTICLE_DIAM_FRAC ({c['particle_diam_frac']!r})
#define CP_PARTICLE_RATIO 10.0
#define CP_FLUID 1.0
#define RHO_PARTICLE_RATIO {c['rho_particle_ratio']!r}
#define REPFORCE_SCALE 2.0e-4
#define PARTICLE_INIT_TEMP (T_COLD + T_HOT)/2
#define PARTICLE_RAND_SEED 86143
#define REP_MIN_GAP 2.0
#define REP_MIN_GAP_W 2.0
#define REP_STF0 0.025
#define REP_STF1 0.002
#define REP_STF0_W 0.025
#define REP_STF1_W 0.002
#define BLOCK_X 8
#define BLOCK_Y 8
#define BLOCK_Z 4
#define RBTP_STORAGE 0
#endif
"""


def _build_and_run(tmp, continuous, nend, name):
    # the driver includes "parameters.h" from its own directory first: build a copy beside the
    # case's parameters.h, as a user of the reference edits parameters.h next to main.cu
    src_dir = tmp / ("src_" + name)
    src_dir.mkdir()
    (src_dir / "parameters.h").write_text(_parameters_h(continuous, nend))
    (src_dir / "rb3d_main.cpp").write_text(open(os.path.join(HOST, "rb3d_main.cpp")).read())
    exe = str(tmp / name)
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I" + str(src_dir), "-I" + os.path.join(REPO, "include"),
                        str(src_dir / "rb3d_main.cpp"), "-o", exe, "-L" + LIBDIR, "-lrbtp",
                        "-Wl,-rpath," + LIBDIR], capture_output=True, text=True, timeout=240)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], cwd=str(tmp), capture_output=True, text=True, timeout=240)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Simulation completed." in r.stdout


def _cfg():
    return W.config("plain_fp64", **CASE)


def test_rb3d_outputs_and_restart(lib_built, tmp_path):
    _build_and_run(tmp_path, 0, 40, "rb3d_a")
    s = Solver(_cfg())
    out = tmp_path / s.output_dir()
    L = 48 * 48 * 24
    assert (out / "fg000000040.dat").stat().st_size == 2 * 27 * L * 8
    assert (out / "000000040.dat").stat().st_size == 7 * L * 8
    assert (out / "000000020.dat").stat().st_size == 7 * L * 8
    stats = (out / "statistics.dat").read_text().split("\n")
    assert len([x for x in stats if x.strip()]) == 4                  # steps 10, 20, 30, 40
    assert (out / "pos" / "pos_000000020.txt").exists() and (out / "pos" / "pos_000000020.bin").exists()
    nu_file = glob.glob(str(out / "Nu_*.txt"))
    assert len(nu_file) == 1
    rows = np.loadtxt(nu_file[0]).reshape(-1, 7)
    assert list(rows[:, 0]) == [10, 20, 30, 40]
    # the library's own Nu rows for the same case
    s.initialize()
    for k, step in enumerate((10, 20, 30, 40)):
        s.step(10, macros_last=True)
        ref = np.array(s.nu(step))
        assert np.allclose(rows[k], ref, rtol=2e-6, atol=1e-12), (step, rows[k], ref)
    # restart from the files rb3d wrote, 40 -> 60, against the uninterrupted library run
    _build_and_run(tmp_path, 40, 60, "rb3d_b")
    rows = np.loadtxt(nu_file[0]).reshape(-1, 7)
    assert list(rows[:, 0]) == [10, 20, 30, 40, 50, 60]
    for k, step in enumerate((50, 60)):
        s.step(10, macros_last=True)
        ref = np.array(s.nu(step))
        # fluid Nu columns (top, bottom, bulk fluid) continue bit for bit; the bulk and particle
        # parts average u_x T over solid nodes, which a restart from files does not carry
        assert np.allclose(rows[4 + k][[3, 4, 5]], ref[[3, 4, 5]], rtol=2e-6, atol=1e-12), (step, rows[4 + k], ref)
