"""Reference pin: the reference's own CUDA kernels, compiled from its sources for each case
(oracle/ref_pin/build_ref.py -> oracle/_ref/<case>.cubin) and driven by a restatement of its host
loop (oracle/ref_pin/ref_driver.cpp), are run on the GPU from the same initial state as the oracle
and librbtp.  This pins the oracle (and the CUDA path) against the reference's device arithmetic.

Tolerances: solid owners, IBB link sets (node, direction, particle) and new-fluid lists bit-exact;
link q within 1e-13 (the reference is compiled with FMA contraction, the oracle without); fields
within 1e-12 relative L2 after the stated number of steps.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import REPO, rel_l2
from rbtp import Config, Solver, derive, workloads as W

sys.path.insert(0, os.path.join(REPO, "oracle", "ref_pin"))
import cases  # noqa: E402

pytestmark = pytest.mark.gpu

REF = os.path.join(REPO, "oracle", "_ref")
DRIVER_SRC = os.path.join(REPO, "oracle", "ref_pin", "ref_driver.cpp")
DRIVER = os.path.join(REF, "ref_driver")
STEPS = 60


@pytest.fixture(scope="module")
def driver(lib_built, oracle_mod):
    if not os.path.exists(os.path.join(REF, "ref_single.cubin")):
        pytest.skip("reference pin cubins are built only where the reference sources exist")
    for libdir in ("/usr/local/cuda/lib64/stubs", "/usr/local/cuda/targets/sbsa-linux/lib/stubs",
                   "/usr/local/cuda/targets/x86_64-linux/lib/stubs"):
        if os.path.exists(os.path.join(libdir, "libcuda.so")):
            break
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I/usr/local/cuda/include", DRIVER_SRC, "-o", DRIVER,
                        "-L" + libdir, "-lcuda"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return DRIVER


def _cfg(case):
    v = cases.values(case)
    v.update(nend=1 << 30, ndiag=0, nflowout=0, nnuout=0, nout_p=0, storage=0)
    return Config.defaults(**v)


def _write_inputs(d, cfg, f, g, f7, parts):
    der = derive(cfg)
    keys = dict(lx=cfg.lx, ly=cfg.ly, lz=cfg.lz, npart=der.npart, radius=der.particle_radius,
                mass=der.particle_mass, inertia=der.particle_inertia,
                heat_capacity=der.particle_heat_capacity, cp_fluid=cfg.cp_fluid,
                rho_particle_ratio=cfg.rho_particle_ratio, tau=der.tau, tauc=der.tauc, grav0=der.grav0,
                beta=cfg.beta, t_hot=cfg.t_hot, t_cold=cfg.t_cold, t_ref=cfg.t_ref, diff=der.diff,
                visc=cfg.visc, repforce_scale=cfg.repforce_scale, rep_min_gap=cfg.rep_min_gap,
                rep_min_gap_w=cfg.rep_min_gap_w)
    with open(os.path.join(d, "cfg.txt"), "w") as fh:
        for k, v in keys.items():
            fh.write(f"{k} {float(v)!r}\n")
    f.tofile(os.path.join(d, "f.bin"))
    g.tofile(os.path.join(d, "g.bin"))
    f7.tofile(os.path.join(d, "flow7.bin"))
    if parts is not None:
        np.ascontiguousarray(parts).tofile(os.path.join(d, "particles.bin"))


def _run(driver, case, tmp_path, f, g, f7, parts, steps):
    ind, outd = tmp_path / "in", tmp_path / "out"
    ind.mkdir()
    outd.mkdir()
    cfg = _cfg(case)
    _write_inputs(str(ind), cfg, f, g, f7, parts)
    r = subprocess.run([driver, os.path.join(REF, case + ".cubin"), str(ind), str(steps), str(outd)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return outd


def _links_from(path):
    a = np.fromfile(path, dtype=np.float64).reshape(-1, 4)
    order = np.lexsort((a[:, 1], a[:, 0]))
    a = a[order]
    return a[:, 0].astype(np.int64), a[:, 1].astype(np.int64), a[:, 2].astype(np.int64), a[:, 3]


def test_reference_pin_single_phase(driver, oracle_mod, tmp_path):
    case = "ref_single"
    cfg = _cfg(case)
    f, g, f7 = W.initial_state(cfg, seed=11)
    out = _run(driver, case, tmp_path, f, g, f7, None, STEPS)
    L = cfg.nodes
    fr = np.fromfile(out / "f.bin")
    gr = np.fromfile(out / "g.bin")
    mr = np.fromfile(out / "macros.bin").reshape(6, L)
    o = oracle_mod.Oracle(cfg)
    o.load_state(f, g, f7)
    o.step(STEPS)
    fo, go = o.fg()
    s = Solver(cfg)
    s.load_state(f, g, f7)
    s.step(STEPS, macros_last=True)
    fs, gs = s.fg()
    scale = np.linalg.norm(go)
    # oracle vs the reference's kernels
    assert rel_l2(go, gr) < 1e-12 and np.linalg.norm(fo - fr) / scale < 1e-12
    # librbtp vs the reference's kernels
    assert rel_l2(gs, gr) < 1e-12 and np.linalg.norm(fs - fr) / scale < 1e-12
    mo, ms = o.macros(), s.macros()
    for k, name in enumerate(["rho", "ux", "uy", "uz", "phi", "force_x"]):
        den = max(np.linalg.norm(mr[k]), 1e-3 * np.linalg.norm(mr[4]))
        assert np.linalg.norm(mo[name] - mr[k]) / den < 1e-12, name
        assert np.linalg.norm(ms[name] - mr[k]) / den < 1e-12, name


def _particle_state(oracle_mod, cfg, seed=5):
    o = oracle_mod.Oracle(cfg)
    o.initialize()                       # glibc placement of pinit.cu:97-144
    p = o.particles()
    rng = np.random.default_rng(seed)
    p[:, 3:6] = 0.03 * rng.standard_normal((len(p), 3))    # moving spheres -> refill events
    p[:, 18:21] = 0.003 * rng.standard_normal((len(p), 3))
    p[:, 30] = 0.5 + 0.1 * rng.standard_normal(len(p))
    return p


def test_reference_pin_particles(driver, oracle_mod, tmp_path):
    case = "ref_particles"
    cfg = _cfg(case)
    L = cfg.nodes
    parts = _particle_state(oracle_mod, cfg)
    assert len(parts) == derive(cfg).npart > 1
    f, g, f7 = W.initial_state(cfg, seed=12)
    out = _run(driver, case, tmp_path, f, g, f7, parts, STEPS)
    o = oracle_mod.Oracle(cfg)
    o.load_state(f, g, f7, parts)
    s = Solver(cfg)
    s.load_state(f, g, f7, parts)
    # loaded state: owners and link sets
    own0 = np.fromfile(out / "owner0.bin", dtype=np.int32)
    assert np.array_equal(o.flags(), own0) and np.array_equal(s.flags(), own0)
    rn, rd, rp, rq = _links_from(out / "links0.bin")
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
        fi, gi = impl.fg()
        assert rel_l2(gi, gr) < 1e-12
        assert np.linalg.norm(fi - fr) / np.linalg.norm(gr) < 1e-12
        pi = impl.particles()
        scale = np.maximum(np.abs(pr).max(0), 1e-300)
        assert np.all(np.abs(pi - pr).max(0) <= 1e-9 * scale + 1e-15)
        assert np.array_equal(impl.flags(), own)
        node, pid = impl.new_fluid()
        order = np.argsort(nf[:, 0], kind="stable")
        assert np.array_equal(node, nf[order, 0]) and np.array_equal(pid, nf[order, 1])
    rn, rd, rp, rq = _links_from(out / "links.bin")
    for impl in (o, s):
        node, d, pid, q = impl.links()
        assert np.array_equal(node, rn) and np.array_equal(d, rd) and np.array_equal(pid, rp)
        assert np.abs(q - rq).max() < 1e-10


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
