"""Seeded synthetic workloads of the RB-ThermoParticles hot path.

The reference ships no datasets or fixtures; its cases are compile-time macro sets.  These
functions produce the configurations and initial states used by the tests and the benchmark:

  plain_fp64     64x64x32,   Ra=1e6, Pr=0.71, single phase
  production     320x320x160, Ra=1e8, Pr=0.71, single phase
  particle_laden 320x320x160, Ra=1e8, 1000 spheres of diameter 16 (density ratio 1.5)

Viscosity follows the rule VISC = 0.1414 * LX * sqrt(Pr / Ra), which keeps the reference's free-fall
velocity u0 = sqrt(g0 beta dT LX) at 0.1414 with BETA fixed (src_lbm/globals.cu:26-30).

Initial state ("restart fixture"): rho deviation 0, u = 0, T(x) = 1 - (x + 1/2)/LX plus a uniform
perturbation in [-amp, amp] drawn from SplitMix64 keyed by (seed, node index).  In the reference's
deviation form that is f_i = 0 and g_i = w_i T (src_lbm/initial.cu:362-397 with rho = 0, u = 0).
"""
from __future__ import annotations

import math

import numpy as np

from . import Config

W = np.array([8 / 27] + [2 / 27] * 6 + [1 / 54] * 12 + [1 / 216] * 8)
CX = np.array([0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1, 0, 1, 0, -1, 0, 1, -1, -1, 1, 1, -1, -1, 1])
CY = np.array([0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0, -1, 0, 1, 0, -1, 1, 1, -1, -1, 1, 1, -1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1])
OPP = np.array([0, 3, 4, 1, 2, 6, 5, 9, 10, 7, 8, 17, 18, 15, 16, 13, 14, 11, 12, 25, 26, 23, 24, 21, 22, 19, 20])


def splitmix64_uniform(seed: int, n: int) -> np.ndarray:
    """n doubles in [0, 1): SplitMix64 output k (k = 1..n) of the stream with the given seed."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def visc_rule(lx: int, ra: float, pr: float) -> float:
    return 0.1414 * lx * math.sqrt(pr / ra)


def config(name: str, storage: int = 0, **over) -> Config:
    """Named configurations; keyword overrides win."""
    if name == "plain_fp64":
        kw = dict(lx=64, ly=64, lz=32, rayleigh=1e6, prandtl=0.71, activate_particles=0,
                  particle_fraction=0.0)
    elif name == "production":
        kw = dict(lx=320, ly=320, lz=160, rayleigh=1e8, prandtl=0.71, activate_particles=0,
                  particle_fraction=0.0)
    elif name == "particle_laden":
        # floor(L * frac / V) = 1000 spheres of radius 8 (PARTICLE_DIAM_FRAC = 16/320)
        v = 4.0 * math.pi * 8.0 ** 3 / 3.0
        kw = dict(lx=320, ly=320, lz=160, rayleigh=1e8, prandtl=0.71, activate_particles=1,
                  particle_diam_frac=16.0 / 320.0, particle_fraction=1000.5 * v / (320 * 320 * 160),
                  rho_particle_ratio=1.5, cp_particle_ratio=10.0, particle_init_temp=0.5)
    else:
        raise KeyError(name)
    kw.update(over)
    kw.setdefault("visc", visc_rule(kw["lx"], kw["rayleigh"], kw["prandtl"]))
    kw["storage"] = storage
    # outputs only when asked for explicitly
    kw.setdefault("nend", 1 << 30)
    kw.setdefault("ndiag", 0)
    kw.setdefault("nflowout", 0)
    kw.setdefault("nnuout", 0)
    kw.setdefault("nout_p", 0)
    return Config.defaults(**kw)


def initial_state(cfg: Config, seed: int = 1, amp: float = 1e-3):
    """(f, g, flow7) of the linear-conduction start with a seeded perturbation."""
    lx, ly, lz = cfg.lx, cfg.ly, cfg.lz
    L = lx * ly * lz
    x = np.arange(L) % lx
    T = cfg.t_hot - (x + 0.5) / lx * (cfg.t_hot - cfg.t_cold)
    T = T + amp * (2.0 * splitmix64_uniform(seed, L) - 1.0)
    f = np.zeros(27 * L)
    g = (W[:, None] * T[None, :]).reshape(-1)
    flow7 = np.zeros(7 * L)
    flow7[4 * L:5 * L] = T
    return f, g, flow7


def ensemble(n: int = 256, seed: int = 2, storage: int = 1, max_spheres: int = 200,
             sizes=(32, 48, 64, 96, 128)):
    """Configurations of the batched ensemble: LY drawn from `sizes`, LX = LY, LZ = LY/2, Ra
    log-uniform in [1e5, 1e8], Pr uniform in [0.7, 7], VISC by the u0 rule, 0..max_spheres spheres of
    diameter 0.1 LY (density ratio 1.0, the reference default), per-cavity placement seeds."""
    rng = np.random.default_rng(seed)
    cfgs = []
    for k in range(n):
        ly = int(rng.choice(sizes))
        lx, lz = ly, ly // 2
        ra = float(10.0 ** rng.uniform(5.0, 8.0))
        pr = float(rng.uniform(0.7, 7.0))
        ns = int(rng.integers(0, max_spheres + 1))
        r = 0.5 * 0.1 * lx
        vol = 4.0 * math.pi * r ** 3 / 3.0
        # the densest rejection-sampled packing is bounded; keep the fraction workable
        ns = min(ns, int(0.15 * lx * ly * lz / vol))
        over = dict(lx=lx, ly=ly, lz=lz, rayleigh=ra, prandtl=pr)
        if ns > 0:
            over.update(activate_particles=1, particle_diam_frac=0.1,
                        particle_fraction=(ns + 0.5) * vol / (lx * ly * lz), rho_particle_ratio=1.0,
                        particle_rand_seed=86143 + k)
        cfgs.append(config("plain_fp64", storage=storage, **over))
    return cfgs
