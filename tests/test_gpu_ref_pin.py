"""Reference pin: the reference's own CUDA kernels, compiled from its sources for each case
(oracle/ref_pin/build_ref.py -> oracle/_ref/<case>.cubin) and driven by a restatement of its host
loop (oracle/ref_pin/ref_driver.cpp), are run on the GPU from the same initial state as the oracle
and librbtp.  This pins the oracle (and the CUDA path) against the reference's device arithmetic.

Tolerances: solid owners, IBB link sets (node, direction, particle) and new-fluid lists bit-exact;
link q within 1e-13 (the reference is compiled with FMA contraction, the oracle without); fields
within 1e-12 relative L2 after the stated number of steps; particle columns within 1e-9 of each
column's scale (the reference sums forces with atomics in arbitrary order).
"""
import math
import os
import sys

import numpy as np
import pytest

import refpin
from conftest import REPO, rel_l2
from rbtp import Solver, derive, workloads as W

pytestmark = pytest.mark.gpu

STEPS = 60


def _fields_close(fi, gi, fr, gr, tol=1e-12):
    assert rel_l2(gi, gr) < tol, rel_l2(gi, gr)
    assert np.linalg.norm(fi - fr) / np.linalg.norm(gr) < tol


def _macros_close(m, mr, tol=1e-12):
    for k, name in enumerate(["rho", "ux", "uy", "uz", "phi", "force_x"]):
        den = max(np.linalg.norm(mr[k]), 1e-3 * np.linalg.norm(mr[4]))
        assert np.linalg.norm(m[name] - mr[k]) / den < tol, name


def _columns_close(pi, pr, tol=1e-9):
    scale = np.maximum(np.abs(pr).max(0), 1e-300)
    assert np.all(np.abs(pi - pr).max(0) <= tol * scale + 1e-15), np.abs(pi - pr).max(0) / scale


def test_reference_pin_single_phase(ref_driver, oracle_mod, tmp_path):
    case = "ref_single"
    cfg = refpin.cfg_of(case)
    f, g, f7 = W.initial_state(cfg, seed=11)
    out = refpin.run(ref_driver, case, tmp_path, cfg, f, g, f7, None, STEPS)
    L = cfg.nodes
    fr = np.fromfile(out / "f.bin")
    gr = np.fromfile(out / "g.bin")
    mr = np.fromfile(out / "macros.bin").reshape(6, L)
    o = oracle_mod.Oracle(cfg)
    o.load_state(f, g, f7)
    o.step(STEPS)
    s = Solver(cfg)
    s.load_state(f, g, f7)
    s.step(STEPS, macros_last=True)
    for impl in (o, s):     # the oracle and librbtp, each against the reference's kernels
        _fields_close(*impl.fg(), fr, gr)
        _macros_close(impl.macros(), mr)


def test_reference_pin_config1_100_and_1000_steps(ref_driver, oracle_mod, tmp_path):
    """The plain FP64 parity configuration (64x64x32, Ra = 1e6, Pr = 0.71, seeded +-1e-3 start):
    f, g and the macroscopic fields of librbtp and of the oracle within 1e-12 relative L2 of the
    reference's kernels after 100 steps, and librbtp still within 1e-12 after 1000 steps (the
    configuration's run length; 1.4e-15 measured)."""
    case = "ref_config1"
    cfg = refpin.cfg_of(case)
    assert (cfg.lx, cfg.ly, cfg.lz) == (64, 64, 32) and cfg.rayleigh == 1e6
    L = cfg.nodes
    f, g, f7 = W.initial_state(cfg, seed=1)
    out100 = refpin.run(ref_driver, case, tmp_path / "s100", cfg, f, g, f7, None, 100)
    out1000 = refpin.run(ref_driver, case, tmp_path / "s1000", cfg, f, g, f7, None, 1000)
    o = oracle_mod.Oracle(cfg)
    o.load_state(f, g, f7)
    o.step(100)
    s = Solver(cfg)
    s.load_state(f, g, f7)
    s.step(100, macros_last=True)
    fr, gr = np.fromfile(out100 / "f.bin"), np.fromfile(out100 / "g.bin")
    mr = np.fromfile(out100 / "macros.bin").reshape(6, L)
    for impl in (o, s):
        _fields_close(*impl.fg(), fr, gr)
        _macros_close(impl.macros(), mr)
    s.step(900, macros_last=True)
    fs, gs = s.fg()
    fr, gr = np.fromfile(out1000 / "f.bin"), np.fromfile(out1000 / "g.bin")
    mr = np.fromfile(out1000 / "macros.bin").reshape(6, L)
    err = max(rel_l2(gs, gr), np.linalg.norm(fs - fr) / np.linalg.norm(gr))
    print(f"64x64x32 Ra=1e6 after 1000 steps: relative L2 {err:.3e}")
    _fields_close(fs, gs, fr, gr)
    _macros_close(s.macros(), mr)


def _particle_state(oracle_mod, cfg, seed=5):
    o = oracle_mod.Oracle(cfg)
    o.initialize()                       # glibc placement of pinit.cu:97-144
    p = o.particles()
    rng = np.random.default_rng(seed)
    p[:, 3:6] = 0.03 * rng.standard_normal((len(p), 3))    # moving spheres -> refill events
    p[:, 18:21] = 0.003 * rng.standard_normal((len(p), 3))
    p[:, 30] = 0.5 + 0.1 * rng.standard_normal(len(p))
    return p


def test_reference_pin_particles(ref_driver, oracle_mod, tmp_path):
    case = "ref_particles"
    cfg = refpin.cfg_of(case)
    parts = _particle_state(oracle_mod, cfg)
    assert len(parts) == derive(cfg).npart > 1
    f, g, f7 = W.initial_state(cfg, seed=12)
    out = refpin.run(ref_driver, case, tmp_path, cfg, f, g, f7, parts, STEPS)
    o = oracle_mod.Oracle(cfg)
    o.load_state(f, g, f7, parts)
    s = Solver(cfg)
    s.load_state(f, g, f7, parts)
    # loaded state: owners and link sets
    own0 = np.fromfile(out / "owner0.bin", dtype=np.int32)
    assert np.array_equal(o.flags(), own0) and np.array_equal(s.flags(), own0)
    rn, rd, rp, rq = refpin.links_from(out / "links0.bin")
    for impl in (o, s):
        node, d, pid, q = impl.links()
        assert np.array_equal(node, rn) and np.array_equal(d, rd) and np.array_equal(pid, rp)
        assert np.abs(q - rq).max() < 1e-13
    o.step(STEPS)
    s.step(STEPS, macros_last=True)
    fr, gr = np.fromfile(out / "f.bin"), np.fromfile(out / "g.bin")
    pr = np.fromfile(out / "particles.bin").reshape(-1, 33)
    own = np.fromfile(out / "owner.bin", dtype=np.int32)
    nf = np.fromfile(out / "newfluid.bin", dtype=np.int32).reshape(-1, 2)
    for impl in (o, s):
        _fields_close(*impl.fg(), fr, gr)
        _columns_close(impl.particles(), pr)
        assert np.array_equal(impl.flags(), own)
        node, pid = impl.new_fluid()
        order = np.argsort(nf[:, 0], kind="stable")
        assert np.array_equal(node, nf[order, 0]) and np.array_equal(pid, nf[order, 1])
    rn, rd, rp, rq = refpin.links_from(out / "links.bin")
    for impl in (o, s):
        node, d, pid, q = impl.links()
        assert np.array_equal(node, rn) and np.array_equal(d, rd) and np.array_equal(pid, rp)
        assert np.abs(q - rq).max() < 1e-10


# The eight spheres of radius 4 of the particle case (48x48x24), placed by hand: two pairs inside
# the contact range REP_MIN_GAP = 2 of each other (gaps 1.0 and about 0.5) and four spheres within
# REP_MIN_GAP_W = 2 of a wall (x = 0, y = LY, z = 0, and x = LX together with z = LZ).
CONTACT_POSITIONS = [(12.13, 12.07, 12.21), (12.13, 21.07, 12.21),          # pair, gap 1.0
                     (30.11, 12.17, 12.09), (38.61, 12.47, 12.29),          # pair, gap ~0.51
                     (5.23, 36.19, 12.11),                                  # wall x = 0, gap 1.23
                     (24.07, 43.31, 12.17),                                 # wall y = 48, gap 0.69
                     (36.03, 36.11, 5.53),                                  # wall z = 0, gap 1.53
                     (43.19, 24.13, 19.03)]                                 # walls x = 48, z = 24


def _contact_forces(p, cfg):
    """pforces.cu:6-76 restated in numpy: the soft-sphere pair and wall forces at positions p."""
    der = derive(cfg)
    r, coeff = der.particle_radius, der.particle_mass * cfg.repforce_scale
    F = np.zeros((len(p), 3))

    def law(gap, mg, s0, s1):
        overlap = -gap if gap < 0 else 0.0
        fac = (mg - gap) / mg
        return coeff * (fac * fac / s0 + overlap / (mg * s1))

    for a in range(len(p)):
        for b in range(a + 1, len(p)):
            d = p[a] - p[b]
            dist = math.sqrt(d @ d)
            if dist - 2 * r < cfg.rep_min_gap:
                lf = law(dist - 2 * r, cfg.rep_min_gap, cfg.rep_stf0, cfg.rep_stf1)
                F[a] += lf * d / dist
                F[b] -= lf * d / dist
    dims = (cfg.lx, cfg.ly, cfg.lz)
    for a in range(len(p)):
        for ax in range(3):
            for gap, sign in ((p[a, ax] - r, 1.0), (dims[ax] - p[a, ax] - r, -1.0)):
                if gap < cfg.rep_min_gap_w:
                    F[a, ax] += sign * law(gap, cfg.rep_min_gap_w, cfg.rep_stf0_w, cfg.rep_stf1_w)
    return F


def test_reference_pin_contact_and_wall_forces(ref_driver, oracle_mod, tmp_path):
    """Spheres inside the contact range of each other and of the walls: the force, torque and
    history columns of librbtp and of the oracle after 1 and after 10 steps agree with the
    reference's kernels (repulsive_pair_kernel / repulsive_wall_kernel, pforces.cu:6-76, beside
    the IBB momentum exchange) to 1e-9 of each column's scale.  The contact forces are at least
    1e-3 of the step-1 force scale, so that comparison resolves the contact law to 1e-6."""
    case = "ref_particles"
    cfg = refpin.cfg_of(case)
    n = derive(cfg).npart
    assert n == len(CONTACT_POSITIONS)
    rng = np.random.default_rng(21)
    p = np.zeros((n, 33))
    p[:, :3] = CONTACT_POSITIONS
    p[:, 3:6] = 0.003 * rng.standard_normal((n, 3))
    p[:, 18:21] = 0.0003 * rng.standard_normal((n, 3))
    p[:, 30] = 0.5 + 0.1 * rng.standard_normal(n)
    fc = _contact_forces(p[:, :3], cfg)
    touched = np.abs(fc).max(1) > 0
    assert touched.all()               # every sphere feels a contact or a wall
    f, g, f7 = W.initial_state(cfg, seed=13)
    for steps in (1, 10):
        out = refpin.run(ref_driver, case, tmp_path / f"s{steps}", cfg, f, g, f7, p, steps)
        pr = np.fromfile(out / "particles.bin").reshape(-1, 33)
        if steps == 1:
            # force (columns 6-8) = IBB momentum exchange + contact forces of the start positions
            ibb = pr[:, 6:9] - fc
            print("contact / IBB force per touched sphere:",
                  np.abs(fc[touched]).max(1) / np.maximum(np.abs(ibb[touched]).max(1), 1e-300))
            assert np.all(np.abs(fc[touched]).max(1) > 1e-3 * np.abs(pr[:, 6:9]).max())
        o = oracle_mod.Oracle(cfg)
        o.load_state(f, g, f7, p)
        o.step(steps)
        s = Solver(cfg)
        s.load_state(f, g, f7, p)
        s.step(steps, macros_last=True)
        for impl in (o, s):
            pi = impl.particles()
            _columns_close(pi, pr)
            # force, force history, torque and torque history columns by name
            for cols in (slice(6, 9), slice(9, 12), slice(12, 15), slice(21, 24), slice(24, 27), slice(27, 30)):
                scale = max(np.abs(pr[:, cols]).max(), 1e-300)
                assert np.abs(pi[:, cols] - pr[:, cols]).max() <= 1e-9 * scale
            assert np.array_equal(impl.flags(), np.fromfile(out / "owner.bin", dtype=np.int32))
        cs, co = s.contacts(), o.contacts()
        assert np.array_equal(cs[0], co[0]) and np.array_equal(cs[1], co[1])
        fr, gr = np.fromfile(out / "f.bin"), np.fromfile(out / "g.bin")
        _fields_close(*s.fg(), fr, gr)
        s.close()
        o.close()


@pytest.mark.parametrize("case", ["ref_single", "ref_particles"])
def test_librbtp_against_reference_golden_fixtures(lib_built, oracle_mod, case):
    """librbtp from the same inputs as tests/golden/make_golden.py reproduces the fixtures the
    reference's kernels produced (the pin without the reference's cubins: runs everywhere)."""
    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    import make_golden as MG
    from test_oracle_golden import check_against_golden
    data = dict(np.load(os.path.join(REPO, "tests", "golden", case + ".npz")))
    cfg, f, g, f7, parts = MG.inputs(case, oracle_mod)
    s = Solver(cfg)
    s.load_state(f, g, f7, parts)
    if parts is not None:
        npart = len(parts)
        assert np.array_equal(MG.solid_counts(s.flags(), npart), data["solid0"])
        node, d, pid, q = s.links()
        got = MG.link_checksums(node, d, pid, q, npart)
        assert np.array_equal(got[:, :3], data["links0"][:, :3])
        assert np.all(np.abs(got[:, 3] - data["links0"][:, 3]) <= 1e-12 * np.maximum(data["links0"][:, 0], 1))
    s.step(MG.STEPS, macros_last=True)
    check_against_golden(s, case, data)
