"""Where the reference method itself leaves the physical regime, recorded with the oracle (the FP64
restatement of the reference step, pinned against the reference's kernels elsewhere).

1. Density ratio 1.5 with spheres of diameter 16 at LX = 320.  The reference's gravity is
   g0 = Ra visc^2 / (beta dT LX^3 Pr) = 0.02 / (beta LX) with its u0 rule for VISC and its fixed
   BETA = 6.25e-5 (globals.cu:26-28), so g0 = 1 lattice unit at LX = 320, and the particle
   buoyancy (1 - 1/rho_r) g0 of move.cu:47,63 accelerates every sphere by 1/3 lattice unit per
   step^2.  The box here is 320x64x32 with four spheres: the particle-laden benchmark
   configuration's LX (so its g0), sphere size, Ra and Pr, with fewer spheres so the oracle runs
   in seconds.  Recorded: the density deviation passes -0.5 (half the rest density) at step 3,
   the spheres stay in the box through step 11 and leave it at step 12.  At density ratio 1.0
   (no particle buoyancy) the same case stays near rest.
2. Three requests of the serving benchmark's mix, all 32x32x16 cavities (g0 = 10 lattice units)
   holding 137-143 spheres of diameter 3.2 (about 15 % solid): request 14 (Ra = 2.9e7, relaxation
   time 0.505), request 8 (Ra = 5.7e6, 0.511) and request 7 (Ra = 7.9e5, 0.525).  Spheres leave the
   box at step 2889 (request 14), step 2692 (request 8, density deviation beyond 0.5 from step 929)
   and step 18183 (request 7), within the requests' horizons; the density deviation exceeds 0.5 in
   magnitude long before.  The CUDA path reports RBTP_ERR_NONFINITE for them.  Request 7 takes
   about three minutes of oracle time and runs with RBTP_SLOW_TESTS=1.
"""
import math
import os

import numpy as np
import pytest

from rbtp import derive, workloads as W


def _ratio_case(ratio):
    d, n = 16.0, 4
    v = 4.0 * math.pi * (d / 2) ** 3 / 3.0
    return W.config("plain_fp64", lx=320, ly=64, lz=32, rayleigh=1e8, activate_particles=1,
                    particle_diam_frac=d / 320.0, particle_fraction=(n + 0.5) * v / (320 * 64 * 32),
                    rho_particle_ratio=ratio, cp_particle_ratio=10.0, particle_init_temp=0.5)


def _inside(p, cfg):
    return bool(np.all(np.isfinite(p[:, :3])) and np.all((p[:, 0] >= 0) & (p[:, 0] < cfg.lx)
                                                          & (p[:, 1] >= 0) & (p[:, 1] < cfg.ly)
                                                          & (p[:, 2] >= 0) & (p[:, 2] < cfg.lz)))


def _run_until_escape(oracle_mod, cfg, max_steps, start=None):
    """Step the oracle one step at a time until a sphere leaves the box (the run stops there, so
    no step ever starts from an escaped sphere).  Returns per-step (speed max, rho min, rho max)
    and the escape step (None if none)."""
    o = oracle_mod.Oracle(cfg)
    o.initialize()
    if start is not None:
        o.load_state(*start, o.particles())
    rec, escape = [], None
    for k in range(1, max_steps + 1):
        o.step(1)
        p = o.particles()
        rho = o.macros()["rho"]
        rec.append((np.sqrt((p[:, 3:6] ** 2).sum(1)).max(), rho.min(), rho.max()))
        if not _inside(p, cfg):
            escape = k
            break
    o.close()
    return np.array(rec), escape


def test_density_ratio_1p5_leaves_the_physical_regime(oracle_mod):
    cfg = _ratio_case(1.5)
    der = derive(cfg)
    assert der.npart == 4 and der.particle_radius == 8.0 and abs(der.grav0 - 1.0) < 1e-3
    f, g, f7 = W.initial_state(cfg)
    rec, escape = _run_until_escape(oracle_mod, cfg, 14, start=(f, g, f7))
    buoy = (1.0 - 1.0 / 1.5) * der.grav0
    assert abs(rec[0, 0] - buoy) < 1e-3 * buoy          # step 1: v = (1 - 1/rho_r) g0 (move.cu:47)
    assert rec[1, 1] > -1e-3 and rec[2, 1] < -0.5        # density deviation passes -0.5 at step 3
    assert rec[3, 0] > 1.0                               # faster than one lattice unit per step
    assert escape == 12
    # at ratio 1.0 the same start stays near rest for twice as long
    rec1, escape1 = _run_until_escape(oracle_mod, _ratio_case(1.0), 24, start=(f, g, f7))
    assert escape1 is None
    assert rec1[:, 0].max() < 1e-3 and np.abs(rec1[:, 1:]).max() < 1e-2


def _serving_request(k):
    cfgs = W.ensemble(16, seed=3, storage=0)
    horizons = np.random.default_rng(3).integers(2000, 50001, size=16)
    return cfgs[k], int(horizons[k])


@pytest.mark.parametrize("k,escape_step", [
    (14, 2889),
    (8, 2692),
    pytest.param(7, 18183, marks=pytest.mark.skipif(not os.environ.get("RBTP_SLOW_TESTS"),
                                                    reason="three minutes of oracle time; RBTP_SLOW_TESTS=1")),
])
def test_serving_requests_that_fail_diverge_in_the_oracle(oracle_mod, k, escape_step):
    cfg, horizon = _serving_request(k)
    der = derive(cfg)
    assert (cfg.lx, cfg.ly, cfg.lz) == (32, 32, 16) and der.npart >= 137 and der.tau < 0.53
    rec, escape = _run_until_escape(oracle_mod, cfg, escape_step)
    assert escape == escape_step < horizon
    assert np.abs(rec[:-1, 1:]).max() > 0.5              # |density deviation| > 0.5 before it
