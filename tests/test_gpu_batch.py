"""Batched execution (rbtp_batch_*): cavities of different sizes, Ra, Pr and sphere counts advanced
together by one persistent launch per step must give the same results as each cavity stepped
alone.  Tolerances: FP64 storage 1e-12 relative L2 of the populations (the batched kernel runs the
same per-node code, so agreement is normally exact); FP32 storage 1e-6; shifted-FP16 storage 1e-3
(a last-bit difference of an FP32 intermediate can round a stored half differently).  Particle integer
structures (solid owners) must be identical.
"""
import math

import numpy as np
import pytest

from conftest import rel_l2
from rbtp import Batch, RbtpError, Solver, STORE_F16S, STORE_F32, STORE_F64, workloads as W

pytestmark = pytest.mark.gpu


def _cfgs(storage):
    return [
        W.config("plain_fp64", lx=40, ly=32, lz=16, rayleigh=3e5, storage=storage),
        # extents that are not multiples of the batched tile (32 or 64 wide, 4 planes deep)
        W.config("plain_fp64", lx=24, ly=48, lz=18, rayleigh=2e6, prandtl=3.0, storage=storage),
        W.config("plain_fp64", lx=48, ly=48, lz=24, activate_particles=1, particle_diam_frac=8.0 / 48.0,
                 particle_fraction=0.04, storage=storage),
        W.config("plain_fp64", lx=32, ly=32, lz=32, activate_particles=1, particle_diam_frac=6.0 / 32.0,
                 particle_fraction=0.03, rayleigh=5e5, particle_rand_seed=7, storage=storage),
    ]


def _start(cfg, k):
    s = Solver(cfg)
    if cfg.activate_particles:
        s.initialize()
        f, g, f7 = W.initial_state(cfg, seed=20 + k)
        s.load_state(f, g, f7, s.particles())
    else:
        s.load_state(*W.initial_state(cfg, seed=20 + k))
    return s


@pytest.mark.parametrize("storage,tol", [(STORE_F64, 1e-12), (STORE_F32, 1e-6), (STORE_F16S, 1e-3)])
def test_batch_matches_individual_runs(lib_built, storage, tol):
    cfgs = _cfgs(storage)
    alone = [_start(c, k) for k, c in enumerate(cfgs)]
    mixed = [_start(c, k) for k, c in enumerate(cfgs)]
    b = Batch(storage)
    for s in mixed:
        b.add(s)
    for s in alone:
        s.step(25)
    b.step(25)
    st = b.stats()
    assert st["members"] == 4 and st["tuned"] == 1 and st["graph"] == 1
    for a, m in zip(alone, mixed):
        assert m.istep == a.istep == 25
        fa, ga = a.fg()
        fm, gm = m.fg()
        assert rel_l2(gm, ga) < tol
        assert np.linalg.norm(fm - fa) / np.linalg.norm(ga) < tol
        if a.npart:
            assert np.array_equal(a.flags(), m.flags())
            pa, pm = a.particles(), m.particles()
            assert np.abs(pa - pm).max() <= 1e3 * tol * max(1.0, np.abs(pa).max())


def test_launch_shapes_give_identical_results(lib_built):
    cfgs = _cfgs(STORE_F32)
    outs = []
    for shape, grid in ((0, 152 * 4), (1, 152 * 8), (0, 100000)):
        ss = [_start(c, k) for k, c in enumerate(cfgs)]
        b = Batch(STORE_F32)
        for s in ss:
            b.add(s)
        b.set_launch(shape, grid)
        b.step(12)
        outs.append([s.fg()[1] for s in ss])
        b.close()
    for o in outs[1:]:
        for x, y in zip(outs[0], o):
            assert np.array_equal(x, y)


def test_membership_changes_and_sampling(lib_built):
    cfgs = _cfgs(STORE_F32)
    ss = [_start(c, k) for k, c in enumerate(cfgs)]
    ref = [_start(c, k) for k, c in enumerate(cfgs)]
    b = Batch(STORE_F32)
    b.add(ss[0], sample_every=10)
    b.add(ss[2], sample_every=10)
    b.step(10)
    assert ss[0].nu(10)[0] == 10.0        # macros materialised by the sampling cadence
    b.add(ss[1], sample_every=5)           # joins while the others are running
    b.remove(ss[0])                        # leaves; keeps its state and stays usable alone
    b.step(10)
    ss[0].step(10)
    for k, steps in ((0, 20), (1, 10), (2, 20)):
        ref[k].step(steps)
        assert ss[k].istep == ref[k].istep
        assert rel_l2(ss[k].fg()[1], ref[k].fg()[1]) < 1e-6
    assert ss[1].nu(ss[1].istep)[0] == 10.0


def test_stop_steps_and_device_sampling(lib_built):
    """Members stop at their own steps inside one batch call and sample Nu on the device on their
    own cadence; each member's state and Nu rows equal a solo run of exactly its steps (FP64: the
    state to 1e-12 relative L2, the Nu rows to 1e-10 relative — the batched reduction is the solo
    one, chunk by chunk)."""
    cfgs = _cfgs(STORE_F64)
    stops, every, nsteps = [7, 30, 19, 0], [5, 10, 0, 6], 30
    alone = [_start(c, k) for k, c in enumerate(cfgs)]
    mixed = [_start(c, k) for k, c in enumerate(cfgs)]
    b = Batch(STORE_F64)
    for s, st, ev in zip(mixed, stops, every):
        b.add(s)
        b.set_sampling(s, ev)
        b.set_stop(s, st)
    b.launch(nsteps)
    with pytest.raises(RbtpError) as e:          # members are busy while the steps are in flight
        mixed[0].fg()
    assert e.value.status == -7
    b.wait()
    for k, (a, m) in enumerate(zip(alone, mixed)):
        n = stops[k] if stops[k] > 0 else nsteps
        assert m.istep == n
        want = sorted({s for s in range(1, n + 1) if every[k] and s % every[k] == 0} |
                      ({n} if stops[k] > 0 else set()))
        rows, done = [], 0
        for s in want:
            a.step(s - done, macros_last=True)
            done = s
            rows.append(a.nu(s))
        if done < n:
            a.step(n - done)
        got = b.samples(m)
        assert got.shape == (len(want), 7)
        np.testing.assert_allclose(got, np.array(rows), rtol=1e-10, atol=1e-12)
        assert b.samples(m).shape == (0, 7)      # drained
        fa, ga = a.fg()
        fm, gm = m.fg()
        assert rel_l2(gm, ga) < 1e-12
        assert np.linalg.norm(fm - fa) / np.linalg.norm(ga) < 1e-12


def test_sample_ring_overrun_is_reported(lib_built):
    cfg = _cfgs(STORE_F32)[0]
    s = _start(cfg, 0)
    b = Batch(STORE_F32)
    b.add(s)
    b.set_sampling(s, 1)
    b.step(70)                                   # 70 samples into a 64-slot ring
    with pytest.raises(RbtpError) as e:
        b.samples(s)
    assert e.value.status == -8
    got = b.samples(s)                           # the ring was resynchronised to the newest 64
    assert got.shape == (0, 7)


def test_particle_kernel_width_does_not_change_results(lib_built):
    """Alone, each of three cavities has fewer than 608 spheres (wide per-particle CTAs); batched
    together they have more (narrow CTAs).  Solid flags, link sets and states must not differ."""
    v = 4.0 * math.pi * 2.0 ** 3 / 3.0
    cfgs = [W.config("plain_fp64", lx=64, ly=64, lz=32, activate_particles=1, particle_diam_frac=4.0 / 64.0,
                     particle_fraction=250.5 * v / (64 * 64 * 32), rho_particle_ratio=1.0,
                     particle_rand_seed=100 + k, storage=STORE_F32) for k in range(3)]
    alone = [_start(c, k) for k, c in enumerate(cfgs)]
    mixed = [_start(c, k) for k, c in enumerate(cfgs)]
    assert all(s.npart == 250 for s in alone)
    b = Batch(STORE_F32)
    for s in mixed:
        b.add(s)
    assert b.stats()["total_particles"] == 750
    for s in alone:
        s.step(12)
    b.step(12)
    for a, m in zip(alone, mixed):
        assert np.array_equal(a.flags(), m.flags())
        la, lm = a.links(), m.links()
        for x, y in zip(la[:3], lm[:3]):
            assert np.array_equal(x, y)
        assert np.abs(la[3] - lm[3]).max() < 1e-5      # q from FP32 positions
        assert rel_l2(m.fg()[1], a.fg()[1]) < 1e-6
