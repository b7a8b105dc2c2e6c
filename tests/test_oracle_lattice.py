"""Oracle checks that need no GPU: lattice tables, derived constants, closed-form geometry.

The reference has no tests or golden vectors; these analytic invariants pin the oracle's
restatement of src_lbm/initial.cu:276-286, src_lbm/globals.cu:18-33,126-169 and
src_part/links.cu:7-23.
"""
import math

import numpy as np
import pytest

from rbtp import Config, workloads as W


def test_d3q27_tables():
    c = np.stack([W.CX, W.CY, W.CZ], 1)
    assert len({tuple(v) for v in c}) == 27
    assert np.all(c[W.OPP] == -c)
    assert np.all(W.OPP[W.OPP] == np.arange(27))
    assert abs(W.W.sum() - 1.0) < 1e-15
    # isotropy: sum w c_a c_b = delta/3, sum w c_a c_b c_c c_d = (d_ab d_cd + ...)/9
    m2 = np.einsum("i,ia,ib->ab", W.W, c, c)
    assert np.allclose(m2, np.eye(3) / 3, atol=1e-15)
    m4 = np.einsum("i,ia,ib,ic,id->abcd", W.W, c, c, c, c)
    d = np.eye(3)
    iso = (np.einsum("ab,cd->abcd", d, d) + np.einsum("ac,bd->abcd", d, d) + np.einsum("ad,bc->abcd", d, d)) / 9
    assert np.allclose(m4, iso, atol=1e-15)
    assert np.allclose(np.einsum("i,ia->a", W.W, c), 0)


def test_derived_constants(oracle_mod):
    cfg = Config.defaults()
    d = oracle_mod.derive(cfg)
    LX = 320.0
    grav0 = 1.0e7 * 0.01206 ** 2 / (0.0000625 * 1.0 * LX ** 3 * 0.71)
    assert d.grav0 == pytest.approx(grav0, rel=1e-15)
    assert d.tau == 3 * 0.01206 + 0.5
    assert d.tauc == pytest.approx(3 * 0.01206 / 0.71 + 0.5, rel=1e-15)
    assert d.particle_radius == 8.0
    vol = 4 * math.pi * 8.0 ** 3 / 3
    assert d.npart == math.floor(320 * 320 * 160 * 0.05 / vol)
    assert d.particle_inertia == pytest.approx(0.4 * vol * 64, rel=1e-14)


def test_derived_matches_library_formula(oracle_mod, lib_built):
    import rbtp
    for name in ("plain_fp64", "production", "particle_laden"):
        cfg = W.config(name)
        a, b = oracle_mod.derive(cfg), rbtp.derive(cfg)
        for f, _ in a._fields_:
            assert getattr(a, f) == getattr(b, f), (name, f)
    assert rbtp.derive(W.config("particle_laden")).npart == 1000


def test_visc_rule_reproduces_u0():
    cfg = W.config("production")
    import oracle_py
    d = oracle_py.derive(cfg)
    assert d.u0 == pytest.approx(0.1414, rel=1e-3)
    assert d.grav0 == pytest.approx(1.0, rel=2e-3)


@pytest.mark.parametrize("ip", range(1, 27))
def test_link_q_closed_form(oracle_mod, ip):
    # node centre at the origin, sphere of radius r on the ray x0 + t c at distance t0 |c|
    c = np.array([W.CX[ip], W.CY[ip], W.CZ[ip]], dtype=float)
    r, t_hit = 0.6, 0.3
    center = (t_hit + r / np.linalg.norm(c)) * c
    ok, q = oracle_mod.link_q(ip, 0.0, 0.0, 0.0, *center, r * r)
    assert ok
    assert q == pytest.approx(t_hit, abs=1e-14)
    # a sphere behind the node does not produce a link
    ok, _ = oracle_mod.link_q(ip, 0.0, 0.0, 0.0, *(-3 * c), r * r)
    assert not ok


def test_link_set_symmetry(oracle_mod):
    # a sphere centred on a node centre: the link set is invariant under the cube symmetries
    cfg = W.config("plain_fp64", lx=32, ly=32, lz=32, activate_particles=1,
                   particle_diam_frac=9.0 / 32.0, particle_fraction=1.2 * (4 / 3 * math.pi * 4.5 ** 3) / 32 ** 3)
    o = oracle_mod.Oracle(cfg)
    assert o.npart == 1
    f, g, f7 = W.initial_state(cfg)
    parts = np.zeros((1, 33))
    parts[0, :3] = [16.5, 16.5, 16.5]
    o.load_state(f, g, f7, parts)
    node, d, pid, q = o.links()
    assert len(node) > 0 and np.all(pid == 0)
    x, y, z = node % 32, (node // 32) % 32, node // 1024
    key = {(int(a), int(b), int(cc), int(dd)): qq for a, b, cc, dd, qq in zip(x, y, z, d, q)}
    dirs = np.stack([W.CX, W.CY, W.CZ], 1)
    lut = {tuple(v): i for i, v in enumerate(dirs)}
    for (a, b, cc, dd), qq in key.items():
        # mirror x -> 32 - 1 - x about the sphere centre (node 16): x' = 32 - x
        m = (32 - a, b, cc, lut[(-W.CX[dd], W.CY[dd], W.CZ[dd])])
        assert m in key and key[m] == pytest.approx(qq, abs=1e-14)
        # swap x <-> y
        s = (b, a, cc, lut[(W.CY[dd], W.CX[dd], W.CZ[dd])])
        assert s in key and key[s] == pytest.approx(qq, abs=1e-14)
