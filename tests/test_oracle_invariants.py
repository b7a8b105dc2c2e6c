"""Physical invariants of the oracle's step (main.cu:32-85 restated): exact mass conservation with
bounce-back walls, invariance of the quiescent state, the conduction solution, zero force on a
resting sphere in quiescent fluid, and determinism."""
import numpy as np
import pytest

from rbtp import workloads as W


def _small(**kw):
    base = dict(lx=16, ly=12, lz=10, rayleigh=1e5)
    base.update(kw)
    return W.config("plain_fp64", **base)


def test_mass_conservation(oracle_mod):
    cfg = _small()
    o = oracle_mod.Oracle(cfg)
    f, g, f7 = W.initial_state(cfg)
    o.load_state(f, g, f7)
    o.step(50)
    f2, _ = o.fg()
    assert abs(f2.sum()) < 1e-13  # deviation-form mass: walls are pure bounce-back


def test_quiescent_rest_is_invariant(oracle_mod):
    # no buoyancy and walls at T_REF: the deviation-form rest state f = 0, g_i = w_i T_REF is a
    # fixed point of the step
    cfg = _small(beta=0.0, t_hot=0.5, t_cold=0.5)
    o = oracle_mod.Oracle(cfg)
    f0 = np.zeros(27 * cfg.nodes)
    g0 = (W.W[:, None] * np.full(cfg.nodes, 0.5)[None, :]).reshape(-1)
    o.load_state(f0, g0)
    o.step(20)
    f1, g1 = o.fg()
    assert np.abs(f1).max() < 1e-16
    assert np.abs(g1 - g0).max() < 1e-15


def test_fresh_init_reproduces_reference_g(oracle_mod):
    # init_g evaluates the equilibrium with the rho field that init_f set to RHO0 = 1 although the
    # populations are in deviation form (initial.cu:350,372): g_0 = (2 w_0 - 1) T0, g_i = 2 w_i T0
    cfg = _small()
    o = oracle_mod.Oracle(cfg)
    o.initialize()
    f, g = o.fg()
    T0 = cfg.t_ref
    assert np.all(f == 0.0)
    g = g.reshape(27, -1)
    assert np.allclose(g[0], (2 * W.W[0] - 1) * T0, rtol=0, atol=1e-16)
    assert np.allclose(g[1:], (2 * W.W[1:, None]) * T0, rtol=0, atol=1e-16)
    assert np.allclose(g.sum(0), T0, atol=1e-15)


def test_conduction_profile(oracle_mod):
    # beta = 0: pure diffusion between the half-way Dirichlet walls converges to a profile within
    # the anti-bounce-back wall error of T = 1 - (x + 1/2)/LX; it is antisymmetric about the
    # mid-plane, so the two wall Nusselt numbers agree, and with u = 0 the bulk Nu is exactly 1
    cfg = _small(lx=12, ly=4, lz=4, beta=0.0, visc=0.1)
    o = oracle_mod.Oracle(cfg)
    f, g, f7 = W.initial_state(cfg, amp=1e-2)
    o.load_state(f, g, f7)
    o.step(3000)
    o.step(1)
    m = o.macros()
    x = np.arange(cfg.nodes) % cfg.lx
    T_lin = 1.0 - (x + 0.5) / cfg.lx
    assert np.abs(m["phi"] - T_lin).max() < 1e-3
    dev = (m["phi"] - T_lin).reshape(cfg.lz, cfg.ly, cfg.lx)
    assert np.abs(dev + dev[:, :, ::-1]).max() < 1e-12
    _, _, nub, nut, nubot, _, _ = o.nu(3001)
    assert nut == pytest.approx(nubot, abs=1e-12)
    assert nut == pytest.approx(1.0, abs=2e-2)
    assert nub == 1.0


def test_resting_sphere_in_quiescent_fluid_feels_no_hydrodynamic_force(oracle_mod):
    import math
    cfg = _small(lx=24, ly=24, lz=24, beta=0.0, t_hot=0.5, t_cold=0.5, activate_particles=1,
                 particle_diam_frac=8.0 / 24.0, particle_fraction=1.5 * (4 / 3 * math.pi * 64) / 24 ** 3)
    o = oracle_mod.Oracle(cfg)
    assert o.npart == 1
    f = np.zeros(27 * cfg.nodes)
    g = (W.W[:, None] * np.full(cfg.nodes, 0.5)[None, :]).reshape(-1)
    parts = np.zeros((1, 33))
    parts[0, :3] = [12.0, 12.0, 12.0]
    parts[0, 30] = 0.5
    o.load_state(f, g, None, parts)
    o.step(3)
    p = o.particles()[0]
    assert np.abs(p[6:9]).max() < 1e-13   # force accumulator
    assert np.abs(p[21:24]).max() < 1e-13  # torque
    assert np.abs(p[3:6]).max() < 1e-13    # velocity stays zero


def test_oracle_is_deterministic(oracle_mod):
    cfg = _small()
    outs = []
    for _ in range(2):
        o = oracle_mod.Oracle(cfg)
        f, g, f7 = W.initial_state(cfg)
        o.load_state(f, g, f7)
        o.step(5)
        outs.append(o.fg())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
