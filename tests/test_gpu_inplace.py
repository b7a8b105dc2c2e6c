"""The in-place AA population storage: even steps read natural slots and write post-collision
populations swapped in place, odd steps gather from and scatter to the neighbours' slots, and the
particle kernels (IBB, refill) and the exports address the slots by the parity of the step just
taken.  Every step is compared with the oracle, so both parities of every kernel are checked, with
spheres moving away from the x walls so that new fluid appears next to the Dirichlet walls (the
refill after an odd step then reads populations that the step's scatter turned into wall images)."""
import numpy as np
import pytest

from conftest import rel_l2
from rbtp import Solver, derive, workloads as W

pytestmark = pytest.mark.gpu


def _check(s, o, tol):
    fs, gs = s.fg()
    fo, go = o.fg()
    assert rel_l2(gs, go) < tol and np.linalg.norm(fs - fo) / np.linalg.norm(go) < tol
    ms, mo = s.macros(), o.macros()
    for k in ("rho", "ux", "uy", "uz", "phi", "force_x"):
        den = max(np.linalg.norm(mo[k]), 1e-3 * np.linalg.norm(mo["phi"]))
        assert np.linalg.norm(ms[k] - mo[k]) / den < tol, k
    assert np.array_equal(s.flags(), o.flags())
    ps, po = s.particles(), o.particles()
    scale = np.maximum(np.abs(po).max(0), 1e-300)
    assert np.all(np.abs(ps - po).max(0) <= 1e-10 * scale + 1e-15)


def test_every_step_of_both_parities_against_the_oracle(lib_built, oracle_mod):
    cfg = W.config("plain_fp64", lx=48, ly=48, lz=24, activate_particles=1, particle_diam_frac=8.0 / 48.0,
                   particle_fraction=0.04, rho_particle_ratio=1.0)
    n = derive(cfg).npart
    s, o = Solver(cfg), oracle_mod.Oracle(cfg)
    o.initialize()
    p = o.particles()
    rng = np.random.default_rng(17)
    # two spheres next to the x walls, moving away from them; the others drift
    p[0, :3] = (4.0 + 1.07, 12.3, 12.1)
    p[1, :3] = (48.0 - 4.0 - 1.13, 36.2, 11.9)
    p[:, 3:6] = 0.01 * rng.standard_normal((n, 3))
    p[0, 3], p[1, 3] = 0.08, -0.08
    p[:, 18:21] = 0.002 * rng.standard_normal((n, 3))
    p[:, 30] = 0.5 + 0.2 * rng.standard_normal(n)
    f, g, f7 = W.initial_state(cfg, seed=8, amp=1e-2)
    s.load_state(f, g, f7, p)
    o.load_state(f, g, f7, p)
    refilled = near_wall = 0
    for k in range(1, 41):
        s.step(1, macros_last=True)
        o.step(1)
        a, b = s.new_fluid(), o.new_fluid()
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), k
        refilled += len(a[0])
        x = a[0] % cfg.lx
        near_wall += int(np.sum((x < 3) | (x > cfg.lx - 4)))
        if k <= 6 or k % 4 == 0:            # both parities early, then every fourth step
            _check(s, o, 1e-12)
    assert refilled > 50
    assert near_wall > 0                     # new fluid next to the x walls was refilled
