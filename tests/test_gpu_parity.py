"""GPU parity of librbtp (called through its C ABI) against the CPU oracle.

Tolerances (FP64 storage): populations and macroscopic fields within 1e-12 relative L2 after 100
steps; integer structures (solid flags, owners, IBB link sets, new-fluid lists, contact pairs)
bit-exact at identical particle states.  FP32/FP16 storage is compared with looser, stated
tolerances.
"""
import math
import os

import numpy as np
import pytest

from conftest import rel_l2
from rbtp import Solver, RbtpError, STORE_F32, STORE_F16S, derive, workloads as W

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


@pytest.fixture(scope="module")
def env(lib_built, oracle_mod):
    return oracle_mod


def _pair(oracle_mod, cfg):
    return Solver(cfg), oracle_mod.Oracle(cfg)


def _compare_fields(s, o, tol=TOL64, macros=True):
    fs, gs = s.fg()
    fo, go = o.fg()
    # f is in deviation form (values ~1e-3): compare against the population scale of g as well
    assert rel_l2(gs, go) < tol, rel_l2(gs, go)
    assert np.linalg.norm(fs - fo) / max(np.linalg.norm(go), 1e-300) < tol
    if np.linalg.norm(fo) > 0:
        assert rel_l2(fs, fo) < 1e3 * tol
    if macros:
        ms, mo = s.macros(), o.macros()
        for k in ("rho", "ux", "uy", "uz", "phi", "force_x"):
            scale = max(np.linalg.norm(mo[k]), np.linalg.norm(mo["phi"]) * 1e-3)
            assert np.linalg.norm(ms[k] - mo[k]) / scale < tol, k


def test_single_phase_fp64_100_steps(env):
    cfg = W.config("plain_fp64")
    s, o = _pair(env, cfg)
    f, g, f7 = W.initial_state(cfg)
    s.load_state(f, g, f7)
    o.load_state(f, g, f7)
    s.step(1, macros_last=True)
    o.step(1)
    _compare_fields(s, o, tol=1e-14)
    s.step(99, macros_last=True, flow_last=True)
    o.step(99)
    _compare_fields(s, o)
    ns, no = np.array(s.nu(100)), np.array(o.nu(100))
    assert np.allclose(ns, no, rtol=1e-10, atol=1e-12), (ns, no)
    assert np.allclose(s.means(), o.means(), rtol=1e-9, atol=1e-15)
    assert np.allclose(s.profile(), o.profile(), rtol=1e-9, atol=1e-15)
    ts, ks = s.dissipation()
    to, ko = o.dissipation()
    assert rel_l2(ts, to) < 1e-10 and rel_l2(ks, ko) < 1e-10


def test_fresh_init_fp64(env):
    cfg = W.config("plain_fp64", lx=40, ly=24, lz=20)
    s, o = _pair(env, cfg)
    s.initialize()
    o.initialize()
    _compare_fields(s, o, tol=1e-15)
    s.step(30, macros_last=True)
    o.step(30)
    _compare_fields(s, o)


def test_size_independent_properties_fullsize_fp64(env):
    # 320x320x160: exact mass conservation (bounce-back walls) and finite, bounded fields
    cfg = W.config("production")
    s = Solver(cfg)
    f, g, f7 = W.initial_state(cfg)
    s.load_state(f, g, f7)
    s.step(10, macros_last=True)
    fs, gs = s.fg()
    assert abs(fs.sum()) < 1e-9
    m = s.means()
    assert np.all(np.isfinite(m)) and abs(m[3] - 0.5) < 1e-3
    row = s.nu(10)
    assert np.all(np.isfinite(row))


# measured: FP32 phi 1.1e-6, ux 7e-6, Nu 5e-5; shifted FP16 phi 1.4e-6, ux 3.2e-4, Nu 7e-6
@pytest.mark.parametrize("storage,tol_phi,tol_u,tol_nu", [(STORE_F32, 5e-6, 1e-4, 1e-3),
                                                          (STORE_F16S, 2e-5, 3e-3, 1e-3)])
def test_reduced_storage_against_fp64(env, storage, tol_phi, tol_u, tol_nu):
    cfg = W.config("plain_fp64", storage=storage)
    s = Solver(cfg)
    o = env.Oracle(W.config("plain_fp64"))
    f, g, f7 = W.initial_state(cfg)
    s.load_state(f, g, f7)
    o.load_state(f, g, f7)
    # the first step after a load is an even step: it collides the natural slots (no gather)
    s.step(1, macros_last=True)
    o.step(1)
    assert rel_l2(s.macros()["phi"], o.macros()["phi"]) < 1e-6
    s.step(99, macros_last=True)
    o.step(99)
    ms, mo = s.macros(), o.macros()
    assert rel_l2(ms["phi"], mo["phi"]) < tol_phi
    assert rel_l2(ms["ux"], mo["ux"]) < tol_u
    ns, no = s.nu(100), o.nu(100)
    # the wall Nusselt numbers difference T_wall - T(x = 1/2), which amplifies storage rounding
    assert abs(ns[4] - no[4]) / abs(no[4]) < tol_nu


def _particle_cfg(**kw):
    base = dict(lx=64, ly=64, lz=32, activate_particles=1, particle_diam_frac=8.0 / 64.0,
                particle_fraction=0.02, rho_particle_ratio=1.0)
    base.update(kw)
    return W.config("plain_fp64", **base)


def _links_equal(s, o):
    a, b = s.links(), o.links()
    assert len(a[0]) == len(b[0])
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    assert np.array_equal(a[3], b[3])  # q bit-exact


def test_particles_init_and_links_bit_exact(env):
    cfg = _particle_cfg()
    s, o = _pair(env, cfg)
    assert s.npart == o.npart == 9
    s.initialize()
    o.initialize()
    assert np.array_equal(s.particles(), o.particles())   # glibc rand placement, pinit.cu:97-144
    assert np.array_equal(s.flags(), o.flags())
    _links_equal(s, o)
    _compare_fields(s, o, tol=1e-15)


def test_particles_fp64_100_steps(env):
    cfg = _particle_cfg()
    s, o = _pair(env, cfg)
    s.initialize()
    o.initialize()
    f, g, f7 = W.initial_state(cfg)
    p = o.particles()
    s.load_state(f, g, f7, p)
    o.load_state(f, g, f7, p)
    s.step(1, macros_last=True)
    o.step(1)
    _compare_fields(s, o, tol=1e-13)
    ps, po = s.particles(), o.particles()
    assert np.abs(ps - po).max() <= 1e-12 * max(1.0, np.abs(po).max())
    assert np.array_equal(s.flags(), o.flags())
    s.step(99, macros_last=True)
    o.step(99)
    _compare_fields(s, o)
    ps, po = s.particles(), o.particles()
    scale = np.maximum(np.abs(po).max(0), 1e-300)
    assert np.all(np.abs(ps - po).max(0) <= 1e-10 * scale + 1e-16)
    assert np.array_equal(s.flags(), o.flags())
    ns, no = np.array(s.nu(100)), np.array(o.nu(100))
    assert np.allclose(ns, no, rtol=1e-9, atol=1e-12)


def test_many_particles_take_the_narrow_launch_path(env):
    """700 spheres (more than the 608 that switch the per-particle kernels to 128-thread CTAs): the
    solid flags and link set at load are bit-exact against the oracle, and 10 FP64 steps agree."""
    v = 4.0 * math.pi * 2.0 ** 3 / 3.0
    cfg = _particle_cfg(lx=96, ly=96, lz=48, particle_diam_frac=4.0 / 96.0,
                        particle_fraction=700.5 * v / (96 * 96 * 48))
    s, o = _pair(env, cfg)
    assert s.npart == o.npart == 700
    s.initialize()
    o.initialize()
    assert np.array_equal(s.particles(), o.particles())
    assert np.array_equal(s.flags(), o.flags())
    _links_equal(s, o)
    f, g, f7 = W.initial_state(cfg, seed=4)
    p = o.particles()
    s.load_state(f, g, f7, p)
    o.load_state(f, g, f7, p)
    s.step(10, macros_last=True)
    o.step(10)
    _compare_fields(s, o)
    assert np.array_equal(s.flags(), o.flags())


def _rejected_candidates(env, X, r):
    """Candidates (fluid node, direction whose neighbour lies in the sphere) of one isolated sphere
    that fail the reference's ray-sphere test (links.cu:7-23) on rounding."""
    rsq = r * r
    lo, hi = np.floor(X - r - 2).astype(int), np.ceil(X + r + 2).astype(int)
    out = []
    for ix in range(lo[0], hi[0] + 1):
        for iy in range(lo[1], hi[1] + 1):
            for iz in range(lo[2], hi[2] + 1):
                x0, y0, z0 = ix + 0.5, iy + 0.5, iz + 0.5
                dx, dy, dz = x0 - X[0], y0 - X[1], z0 - X[2]
                if dx * dx + dy * dy + dz * dz <= rsq:
                    continue
                for ip in range(1, 27):
                    ex, ey, ez = x0 + W.CX[ip] - X[0], y0 + W.CY[ip] - X[1], z0 + W.CZ[ip] - X[2]
                    if ex * ex + ey * ey + ez * ez > rsq:
                        continue
                    if not env.link_q(ip, x0, y0, z0, X[0], X[1], X[2], rsq)[0]:
                        out.append((ix, iy, iz, ip))
    return out


def _rejecting_spheres(env, r, nodes, rng):
    """Centres X = n + 1/2 - r u (u a random unit vector) put the node centre n on the sphere up to
    rounding; kept when some candidate ray then rounds to q just above 1 and is rejected."""
    out = []
    for n in nodes:
        for _ in range(400):
            u = rng.standard_normal(3)
            X = np.asarray(n, dtype=float) + 0.5 - r * u / np.linalg.norm(u)
            if _rejected_candidates(env, X, r):
                out.append(X)
                break
    return out


@pytest.mark.parametrize("storage", [0, STORE_F32])
@pytest.mark.parametrize("narrow", [False, True])
def test_links_with_rejected_candidates(env, narrow, storage):
    """Spheres placed so that candidate rays round off the surface: the link build's compaction
    path (taken only by candidate groups that hold a rejected ray) gives the oracle's link set on
    both launch widths (512-thread CTAs below 608 spheres, 128 above) and in FP64 and FP32
    storage."""
    if narrow:
        v = 4.0 * math.pi * 2.0 ** 3 / 3.0
        cfg = _particle_cfg(lx=96, ly=96, lz=48, particle_diam_frac=4.0 / 96.0,
                            particle_fraction=700.5 * v / (96 * 96 * 48), storage=storage)
        nodes = [(8 + 9 * a, 8 + 9 * b, 24) for a in range(2) for b in range(8)]
        free_x = (30.0, 92.0)
    else:
        cfg = _particle_cfg(particle_fraction=0.01, storage=storage)
        nodes = [(10, 12 + 14 * b, 16) for b in range(3)] + [(24, 12 + 14 * b, 16) for b in range(3)]
        free_x = (38.0, 58.0)
    s, o = _pair(env, cfg)
    n = s.npart
    r = float(derive(cfg).particle_radius)
    rng = np.random.default_rng(11)
    placed = _rejecting_spheres(env, r, nodes[:n], rng)
    assert len(placed) >= min(3, n)
    p = np.zeros((n, 33))
    p[:, 30] = 0.5
    p[:len(placed), :3] = placed
    rest = n - len(placed)
    p[len(placed):, 0] = rng.uniform(*free_x, rest)
    p[len(placed):, 1] = rng.uniform(r + 1, cfg.ly - r - 1, rest)
    p[len(placed):, 2] = rng.uniform(r + 1, cfg.lz - r - 1, rest)
    f, g, f7 = W.initial_state(cfg)
    s.load_state(f, g, f7, p)
    o.load_state(f, g, f7, p)
    assert np.array_equal(s.flags(), o.flags())
    if storage == 0:
        _links_equal(s, o)
    else:
        a, b = s.links(), o.links()
        assert len(a[0]) == len(b[0])
        for x, y in zip(a[:3], b[:3]):
            assert np.array_equal(x, y)
        # q in FP32 away from its decision edges: the cancellation in -b - sqrt(disc) leaves a few
        # 1e-6 (3.2e-6 measured)
        np.testing.assert_allclose(a[3], b[3], rtol=0, atol=1e-5)


def test_links_contacts_new_fluid_bit_exact_at_identical_state(env):
    # hand-placed spheres: two pairs inside the contact range, one near a wall
    cfg = _particle_cfg(particle_fraction=0.01)
    s, o = _pair(env, cfg)
    n = s.npart
    assert n >= 4
    rng = np.random.default_rng(7)
    p = np.zeros((n, 33))
    p[:, 30] = 0.5
    base = [(20.3, 20.1, 16.2), (28.9, 20.6, 16.0), (40.2, 40.7, 12.3), (40.9, 48.6, 13.1)]
    for k in range(n):
        if k < len(base):
            p[k, :3] = base[k]
        else:
            p[k, :3] = [10 + 44 * rng.random(), 8 + 48 * rng.random(), 6 + 20 * rng.random()]
    p[:, 3:6] = 0.02 * rng.standard_normal((n, 3))
    p[:, 18:21] = 0.002 * rng.standard_normal((n, 3))
    f, g, f7 = W.initial_state(cfg)
    s.load_state(f, g, f7, p)
    o.load_state(f, g, f7, p)
    assert np.array_equal(s.flags(), o.flags())
    _links_equal(s, o)
    s.step(1)
    o.step(1)
    cs, co = s.contacts(), o.contacts()
    assert len(cs[0]) >= 2
    assert np.array_equal(cs[0], co[0]) and np.array_equal(cs[1], co[1])
    # Force (columns 6-8) = IBB momentum exchange + the contact and wall forces of the step's start
    # positions (pforces.cu:6-76); torque (21-23).  The contact sums run in the same ascending-
    # partner order on both sides; the IBB sums in a fixed tree order here and link order in the
    # oracle, so the columns agree to rounding.
    ps, po = s.particles(), o.particles()
    for cols in (slice(6, 9), slice(9, 12), slice(12, 15), slice(21, 24)):
        scale = max(np.abs(po[:, cols]).max(), 1e-300)
        assert np.abs(ps[:, cols] - po[:, cols]).max() <= 1e-12 * scale, cols
    assert np.abs(po[:2, 6:9]).max() > 0.1                # the first pair is in contact
    assert np.array_equal(s.flags(), o.flags())
    nfs, nfo = s.new_fluid(), o.new_fluid()
    assert np.array_equal(nfs[0], nfo[0]) and np.array_equal(nfs[1], nfo[1])
    # identical particle state -> identical links
    s.load_state(*s.fg(), None, ps)
    o.load_state(*s.fg(), None, ps)
    assert np.array_equal(s.flags(), o.flags())
    _links_equal(s, o)


def test_gpu_is_deterministic(env):
    cfg = _particle_cfg()
    outs = []
    for _ in range(2):
        s = Solver(cfg)
        s.initialize()
        s.step(20, macros_last=True)
        outs.append((s.fg(), s.particles(), s.nu(20)))
        s.close()
    (f1, g1), p1, n1 = outs[0]
    (f2, g2), p2, n2 = outs[1]
    assert np.array_equal(f1, f2) and np.array_equal(g1, g2)
    assert np.array_equal(p1, p2) and n1 == n2


def test_nonfinite_watchdog(env):
    cfg = W.config("plain_fp64", lx=16, ly=16, lz=8)
    s = Solver(cfg)
    f, g, f7 = W.initial_state(cfg)
    g = g.copy()
    g[12345 % g.size] = np.nan
    s.load_state(f, g, f7)
    with pytest.raises(RbtpError) as e:
        s.step(2)
    assert e.value.status == -4


def test_restart_files_roundtrip(env, tmp_path):
    cfg = W.config("plain_fp64", lx=32, ly=24, lz=16, nflowout=10)
    s = Solver(cfg)
    f, g, f7 = W.initial_state(cfg)
    s.load_state(f, g, f7)
    s.step(10)
    d = str(tmp_path)
    s.output_flow(10, d)
    s.output_fg(10, d)
    r = Solver(cfg)
    r.load_restart(d, 10)
    assert r.istep == 10
    s.step(7, macros_last=True)
    r.step(7, macros_last=True)
    fa, ga = s.fg()
    fb, gb = r.fg()
    assert np.array_equal(fa, fb) and np.array_equal(ga, gb)
    # a truncated restart file is rejected with an error status, not an exit
    with open(tmp_path / "fg000000010.dat", "r+b") as fh:
        fh.truncate(1000)
    with pytest.raises(RbtpError) as e:
        Solver(cfg).load_restart(d, 10)
    assert e.value.status == -6


def test_particle_restart_is_exact_with_the_binary_sidecar(env, tmp_path):
    """pos/pos_%09d.txt keeps the reference's %14.6e format; the pos_%09d.bin sidecar written beside
    it holds the same rows exactly, so a restart from the files continues bit for bit at every
    fluid node and in the particle state.  (Solid nodes carry no physics: the flow file holds the
    rigid-body velocity and particle temperature there, as output_flow writes them, so their own
    populations differ after a restart, in the reference as here, and never reach a fluid node.)
    Without the sidecar the text file is read as the reference reads it (7 significant digits)."""
    cfg = W.config("plain_fp64", lx=48, ly=48, lz=24, activate_particles=1, particle_diam_frac=8.0 / 48.0,
                   particle_fraction=0.04, nflowout=10)
    s = Solver(cfg)
    s.initialize()
    s.step(10)
    d = str(tmp_path)
    s.output_flow(10, d)
    s.output_fg(10, d)
    s.output_particles(10, d)
    p10 = s.particles()
    r = Solver(cfg)
    r.load_restart(d, 10)
    assert np.array_equal(r.particles(), s.particles()) and np.array_equal(r.flags(), s.flags())
    s.step(7, macros_last=True)
    r.step(7, macros_last=True)
    fluid = s.flags() < 0
    assert np.array_equal(fluid, r.flags() < 0)
    L = cfg.nodes
    fa, ga = (x.reshape(27, L)[:, fluid] for x in s.fg())
    fb, gb = (x.reshape(27, L)[:, fluid] for x in r.fg())
    assert np.array_equal(fa, fb) and np.array_equal(ga, gb)
    assert np.array_equal(r.particles(), s.particles())
    na, nb = s.nu(17), r.nu(17)
    # Nu from fluid nodes (bulk fluid part, top, bottom) is identical; the particle part of the
    # bulk Nu averages u_x T over solid nodes (output_statis.cu), which hold no physics
    assert (na[3], na[4], na[5]) == (nb[3], nb[4], nb[5])
    os.remove(os.path.join(d, "pos", "pos_000000010.bin"))
    t = Solver(cfg)
    t.load_restart(d, 10)
    assert np.all(np.abs(t.particles() - p10) <= 5.000001e-7 * np.abs(p10))   # %14.6e rounding
