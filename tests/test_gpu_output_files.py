"""The output layer against independent writers.

1. Byte for byte: the drop-in host rb3d (rbtp_write_* through the C ABI) writes the reference's
   files for a particle-laden case; the oracle's restatement of the reference's writers
   (oracle/rbtp_oracle_io.c: output_statis.cu:64-109,111-223,225-285, output_flow.cu:5-127,
   output_part.cu:4-115), fed with the library's own values for the same run, must produce the
   same bytes in every file: statistics.dat, Nu_%.2e.txt, Profile_%.2e.txt, %09d.dat (with the
   solid-node overwrite), fg%09d.dat and pos/pos_%09d.txt.
2. Numerically, with spheres present: the library's volume means, x-profiles and %09d.dat fields
   (solid nodes at the rigid-body velocity and particle temperature, overwrite_particle_nodes of
   output_statis.cu:5-60 and output_flow.cu:5-60) against the oracle's own run.
"""
import filecmp
import os

import numpy as np
import pytest

from conftest import rel_l2
from rbtp import Solver, workloads as W
from test_gpu_rb3d import CASE, _build_and_run

pytestmark = pytest.mark.gpu


def _cfg():
    return W.config("plain_fp64", nend=20, ndiag=10, nflowout=20, nnuout=10, nout_p=20, **CASE)


def test_rb3d_files_match_the_reference_writers_byte_for_byte(lib_built, oracle_mod, tmp_path):
    run_dir = tmp_path / "rb3d"
    run_dir.mkdir()
    _build_and_run(run_dir, 0, 20, "rb3d")
    cfg = _cfg()
    s = Solver(cfg)
    ra = cfg.rayleigh
    sub = oracle_mod.output_dirname(cfg.rayleigh, cfg.prandtl)
    assert sub == s.output_dir()
    ref_dir = str(tmp_path / "oracle" / sub)
    os.makedirs(ref_dir)
    # the library's values of the same run, written by the oracle's writers in main.cu's order
    s.initialize()
    oracle_mod.write_particles(ref_dir, 0, s.particles())
    s.step(10)
    oracle_mod.write_statistics(ref_dir, 10, s.means())
    oracle_mod.write_nu(ref_dir, ra, s.nu(10))
    oracle_mod.write_profile(ref_dir, ra, 10, s.profile())
    s.step(10)
    m = s.macros()
    ted, ked = s.dissipation()
    fields = np.concatenate([m["rho"], m["ux"], m["uy"], m["uz"], m["phi"], ted, ked])
    oracle_mod.write_statistics(ref_dir, 20, s.means())
    oracle_mod.write_flow(ref_dir, 20, cfg, fields, s.flags(), s.particles())
    oracle_mod.write_particles(ref_dir, 20, s.particles())
    oracle_mod.write_nu(ref_dir, ra, s.nu(20))
    oracle_mod.write_profile(ref_dir, ra, 20, s.profile())
    oracle_mod.write_fg(ref_dir, 20, *s.fg())
    got_dir = run_dir / sub
    names = []
    for root, _, files in os.walk(ref_dir):
        for fn in files:
            rel = os.path.relpath(os.path.join(root, fn), ref_dir)
            names.append(rel)
            assert filecmp.cmp(os.path.join(ref_dir, rel), str(got_dir / rel), shallow=False), rel
    assert sorted(names) == sorted(["statistics.dat", f"Nu_{ra:.2e}.txt", f"Profile_{ra:.2e}.txt",
                                    "000000020.dat", "fg000000020.dat", os.path.join("pos", "pos_000000000.txt"),
                                    os.path.join("pos", "pos_000000020.txt")])
    s.close()


def test_particle_present_diagnostics_against_the_oracle(lib_built, oracle_mod, tmp_path):
    cfg = W.config("plain_fp64", nflowout=20, **CASE)
    s, o = Solver(cfg), oracle_mod.Oracle(cfg)
    o.initialize()
    p = o.particles()
    rng = np.random.default_rng(9)
    p[:, 3:6] = 0.02 * rng.standard_normal((len(p), 3))
    p[:, 18:21] = 0.005 * rng.standard_normal((len(p), 3))
    p[:, 30] = 0.5 + 0.2 * rng.standard_normal(len(p))
    f, g, f7 = W.initial_state(cfg, seed=2)
    s.load_state(f, g, f7, p)
    o.load_state(f, g, f7, p)
    s.step(20, macros_last=True)
    o.step(20)
    assert np.array_equal(s.flags(), o.flags())
    solid = s.flags() >= 0
    assert solid.sum() > 1000
    ms, mo = s.means(), o.means()
    scale = np.abs(mo).max()
    assert np.all(np.abs(ms - mo) <= 1e-10 * scale), (ms, mo)
    ps, po = s.profile(), o.profile()
    assert np.all(np.abs(ps - po) <= 1e-10 * np.abs(po).max(0)), np.abs(ps - po).max(0)
    ns, no = np.array(s.nu(20)), np.array(o.nu(20))
    assert np.allclose(ns, no, rtol=1e-9, atol=1e-12)
    # %09d.dat: the library's writer against the oracle's writer on the oracle's own state
    a_dir, b_dir = tmp_path / "lib", tmp_path / "oracle"
    s.output_flow(20, str(a_dir))
    mo = o.macros()
    to, ko = o.dissipation()
    oracle_mod.write_flow(str(b_dir), 20, cfg, np.concatenate([mo["rho"], mo["ux"], mo["uy"], mo["uz"],
                                                                 mo["phi"], to, ko]), o.flags(), o.particles())
    L = cfg.nodes
    a = np.fromfile(a_dir / "000000020.dat").reshape(7, L)
    b = np.fromfile(b_dir / "000000020.dat").reshape(7, L)
    assert np.all(a[0][solid] == cfg.rho0) and np.all(a[5][solid] == 0.0) and np.all(a[6][solid] == 0.0)
    for k in range(7):
        den = max(np.linalg.norm(b[k]), 1e-3 * np.linalg.norm(b[4]))
        assert np.linalg.norm(a[k] - b[k]) / den < 1e-10, k
    # solid nodes carry the owning sphere's rigid-body motion and temperature
    assert rel_l2(a[4][solid], b[4][solid]) < 1e-12
