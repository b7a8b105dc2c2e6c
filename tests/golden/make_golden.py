#!/usr/bin/env python3
"""Golden fixtures from the reference's own CUDA kernels (TEST INFRASTRUCTURE ONLY).

The reference ships no tests or golden vectors, so these fixtures are made by running its kernels:
`oracle/ref_pin/build_ref.py` compiles the reference's sources per case into
`oracle/_ref/<case>.cubin` (only where the reference sources exist), and
`oracle/ref_pin/ref_driver.cpp` issues them in the order of its host loop (main.cu:32-85) from a
seeded start.  This script runs that driver on a GPU for the two pin cases and stores compact
outputs in `tests/golden/<case>.npz`:

* `macros`: rho, ux, uy, uz, phi, F_x after STEPS steps at 1024 fixed nodes (`nodes`);
* `f`, `g`: all 27 populations at 256 of those nodes (`pop_nodes`);
* `f_norm`, `g_norm`: per-direction L2 norms of the whole f and g arrays;
* particle case: `particles` (33 columns after STEPS steps), per-particle solid-node counts and
  link checksums (count, sum of node indices, sum of directions, sum of q) of the loaded state
  (`*0`) and after STEPS steps, and the new-fluid list of the last step.

The inputs are not stored: `inputs(case)` rebuilds them (seeded SplitMix64 start of
rbtp/workloads.py, the oracle's glibc sphere placement plus seeded velocities), and the tests call
the same function.  usage (on a machine with a GPU and the built cubins):

    python tests/golden/make_golden.py [out_dir]
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "rb-thermoparticles_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle", "ref_pin"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

STEPS = 60
CASES = ("ref_single", "ref_particles")
SEEDS = {"ref_single": 11, "ref_particles": 12}


def config(case):
    import cases
    from rbtp import Config
    v = cases.values(case)
    v.update(nend=1 << 30, ndiag=0, nflowout=0, nnuout=0, nout_p=0, storage=0)
    return Config.defaults(**v)


def inputs(case, oracle_mod):
    """(cfg, f, g, flow7, particles or None) of a pin case."""
    from rbtp import workloads as W
    cfg = config(case)
    f, g, f7 = W.initial_state(cfg, seed=SEEDS[case])
    parts = None
    if cfg.activate_particles:
        o = oracle_mod.Oracle(cfg)
        o.initialize()                       # glibc placement of pinit.cu:97-144
        parts = o.particles()
        o.close()
        rng = np.random.default_rng(5)
        parts[:, 3:6] = 0.03 * rng.standard_normal((len(parts), 3))     # moving spheres: refill
        parts[:, 18:21] = 0.003 * rng.standard_normal((len(parts), 3))
        parts[:, 30] = 0.5 + 0.1 * rng.standard_normal(len(parts))
    return cfg, f, g, f7, parts


def sample_nodes(L):
    nodes = np.sort(np.random.default_rng(0).choice(L, 1024, replace=False))
    return nodes, nodes[::4]


def link_checksums(node, d, pid, q, npart):
    out = np.zeros((npart, 4))
    for k in range(npart):
        m = pid == k
        out[k] = (m.sum(), node[m].astype(np.float64).sum(), d[m].astype(np.float64).sum(), q[m].sum())
    return out


def solid_counts(owner, npart):
    return np.bincount(owner[owner >= 0], minlength=npart).astype(np.int64)


def _driver():
    ref = os.path.join(REPO, "oracle", "_ref")
    exe = os.path.join(ref, "ref_driver")
    src = os.path.join(REPO, "oracle", "ref_pin", "ref_driver.cpp")
    libdir = next(d for d in ("/usr/local/cuda/lib64/stubs", "/usr/local/cuda/targets/sbsa-linux/lib/stubs",
                              "/usr/local/cuda/targets/x86_64-linux/lib/stubs")
                  if os.path.exists(os.path.join(d, "libcuda.so")))
    subprocess.run(["g++", "-O2", "-std=c++17", "-I/usr/local/cuda/include", src, "-o", exe, "-L" + libdir,
                    "-lcuda"], check=True)
    return ref, exe


def run_reference(case, oracle_mod, ref, exe):
    from rbtp import derive
    cfg, f, g, f7, parts = inputs(case, oracle_mod)
    der = derive(cfg)
    with tempfile.TemporaryDirectory() as d:
        ind, outd = os.path.join(d, "in"), os.path.join(d, "out")
        os.makedirs(ind)
        os.makedirs(outd)
        keys = dict(lx=cfg.lx, ly=cfg.ly, lz=cfg.lz, npart=der.npart, radius=der.particle_radius,
                    mass=der.particle_mass, inertia=der.particle_inertia,
                    heat_capacity=der.particle_heat_capacity, cp_fluid=cfg.cp_fluid,
                    rho_particle_ratio=cfg.rho_particle_ratio, tau=der.tau, tauc=der.tauc, grav0=der.grav0,
                    beta=cfg.beta, t_hot=cfg.t_hot, t_cold=cfg.t_cold, t_ref=cfg.t_ref, diff=der.diff,
                    visc=cfg.visc, repforce_scale=cfg.repforce_scale, rep_min_gap=cfg.rep_min_gap,
                    rep_min_gap_w=cfg.rep_min_gap_w)
        with open(os.path.join(ind, "cfg.txt"), "w") as fh:
            for k, v in keys.items():
                fh.write(f"{k} {float(v)!r}\n")
        f.tofile(os.path.join(ind, "f.bin"))
        g.tofile(os.path.join(ind, "g.bin"))
        f7.tofile(os.path.join(ind, "flow7.bin"))
        if parts is not None:
            np.ascontiguousarray(parts).tofile(os.path.join(ind, "particles.bin"))
        subprocess.run([exe, os.path.join(ref, case + ".cubin"), ind, str(STEPS), outd], check=True,
                       timeout=600)
        L = cfg.nodes
        fr = np.fromfile(os.path.join(outd, "f.bin")).reshape(27, L)
        gr = np.fromfile(os.path.join(outd, "g.bin")).reshape(27, L)
        mr = np.fromfile(os.path.join(outd, "macros.bin")).reshape(6, L)
        nodes, pop_nodes = sample_nodes(L)
        out = dict(steps=STEPS, nodes=nodes, pop_nodes=pop_nodes, macros=mr[:, nodes],
                   f=fr[:, pop_nodes], g=gr[:, pop_nodes], f_norm=np.linalg.norm(fr, axis=1),
                   g_norm=np.linalg.norm(gr, axis=1))
        if parts is not None:
            npart = len(parts)

            def links(path):
                a = np.fromfile(path, dtype=np.float64).reshape(-1, 4)
                return (a[:, 0].astype(np.int64), a[:, 1].astype(np.int64), a[:, 2].astype(np.int64), a[:, 3])

            out.update(particles=np.fromfile(os.path.join(outd, "particles.bin")).reshape(-1, 33),
                       solid0=solid_counts(np.fromfile(os.path.join(outd, "owner0.bin"), dtype=np.int32), npart),
                       solid=solid_counts(np.fromfile(os.path.join(outd, "owner.bin"), dtype=np.int32), npart),
                       links0=link_checksums(*links(os.path.join(outd, "links0.bin")), npart),
                       links=link_checksums(*links(os.path.join(outd, "links.bin")), npart),
                       newfluid=np.fromfile(os.path.join(outd, "newfluid.bin"), dtype=np.int32).reshape(-1, 2))
    return out


def main() -> int:
    import oracle_py
    out_dir = sys.argv[1] if len(sys.argv) > 1 else HERE
    os.makedirs(out_dir, exist_ok=True)
    ref, exe = _driver()
    for case in CASES:
        data = run_reference(case, oracle_py, ref, exe)
        np.savez_compressed(os.path.join(out_dir, f"{case}.npz"), **data)
        print(case, {k: np.shape(v) for k, v in data.items()})
    return 0


if __name__ == "__main__":
    sys.exit(main())
