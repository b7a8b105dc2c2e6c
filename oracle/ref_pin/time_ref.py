#!/usr/bin/env python3
"""Time the reference's own CUDA kernels on this GPU (TEST INFRASTRUCTURE / MEASUREMENT ONLY).

The kernels are the reference's sources compiled for sm_103a into oracle/_ref/<case>.cubin by
build_ref.py (cases.TIMING: the 320x320x160 benchmark workloads); ref_driver.cpp issues them in the
order of the reference's host loop (main.cu:35-85 with the particle wrappers), including its
device-to-device copies, and times `--steps` steps after `--warmup` steps on the seeded synthetic
start of rbtp/workloads.py.  The CUB prefix sums of build_links / refill_nodes are host scans in the
driver and are excluded from `ms_per_step` (reported separately).

usage: python oracle/ref_pin/time_ref.py [--case ref_production|ref_particle_laden] [--warmup 3] [--steps 10]
prints one JSON line.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "rb-thermoparticles_gb300"))
import cases  # noqa: E402

REF = os.path.join(REPO, "oracle", "_ref")
DRIVER = os.path.join(REF, "ref_driver")


def build_driver() -> str:
    libdir = None
    for d in ("/usr/local/cuda/lib64/stubs", "/usr/local/cuda/targets/sbsa-linux/lib/stubs",
              "/usr/local/cuda/targets/x86_64-linux/lib/stubs"):
        if os.path.exists(os.path.join(d, "libcuda.so")):
            libdir = d
            break
    cmd = ["g++", "-O2", "-std=c++17", "-I/usr/local/cuda/include", os.path.join(HERE, "ref_driver.cpp"),
           "-o", DRIVER, "-lcuda"]
    if libdir:
        cmd.insert(-1, "-L" + libdir)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return DRIVER


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="ref_production", choices=sorted(cases.TIMING))
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--steps", type=int, default=10)
    args = ap.parse_args()
    cubin = os.path.join(REF, args.case + ".cubin")
    if not os.path.exists(cubin):
        print(json.dumps({"case": args.case, "unavailable": "reference cubin not built (needs the reference sources)"}))
        return 0
    from rbtp import Config, Solver, derive  # noqa: E402

    v = cases.values(args.case)
    v.update(nend=1 << 30, ndiag=0, nflowout=0, nnuout=0, nout_p=0, storage=1)
    cfg = Config.defaults(**v)
    der = derive(cfg)
    driver = build_driver()
    with tempfile.TemporaryDirectory() as d:
        keys = dict(lx=cfg.lx, ly=cfg.ly, lz=cfg.lz, npart=der.npart, radius=der.particle_radius,
                    mass=der.particle_mass, inertia=der.particle_inertia,
                    heat_capacity=der.particle_heat_capacity, cp_fluid=cfg.cp_fluid,
                    rho_particle_ratio=cfg.rho_particle_ratio, tau=der.tau, tauc=der.tauc,
                    grav0=der.grav0, beta=cfg.beta, t_hot=cfg.t_hot, t_cold=cfg.t_cold, t_ref=cfg.t_ref,
                    diff=der.diff, visc=cfg.visc, repforce_scale=cfg.repforce_scale,
                    rep_min_gap=cfg.rep_min_gap, rep_min_gap_w=cfg.rep_min_gap_w, synthetic=1, seed=1,
                    amp=1e-3)
        with open(os.path.join(d, "cfg.txt"), "w") as fh:
            for k, val in keys.items():
                fh.write(f"{k} {float(val)!r}\n")
        if der.npart > 0:
            s = Solver(cfg)
            s.initialize()          # the reference's glibc placement (pinit.cu:97-144)
            s.particles().tofile(os.path.join(d, "particles.bin"))
            s.close()
        r = subprocess.run([driver, cubin, d, "time", str(args.warmup), str(args.steps)],
                           capture_output=True, text=True, timeout=3000)
    if r.returncode != 0:
        print(json.dumps({"case": args.case, "error": (r.stdout + r.stderr)[-400:]}))
        return 1
    tok = r.stdout.split()
    i = tok.index("ref_time")
    kv = dict(zip(tok[i + 1::2], tok[i + 2::2]))
    ms = float(kv["ms_per_step"])
    print(json.dumps({
        "case": args.case, "nodes": int(kv["nodes"]), "npart": int(kv["npart"]), "links": int(kv["links"]),
        "steps": int(kv["steps"]), "warmup": int(kv["warmup"]), "ms_per_step": ms,
        "ms_per_step_with_host_scans": float(kv["ms_per_step_with_host_scans"]),
        "mlups": int(kv["nodes"]) / (ms * 1e-3) / 1e6,
        "nonfinite_phi_nodes_after_run": int(kv["nonfinite"]),
        "what": "reference kernels (its sources, nvcc -O3 sm_103a, FP64) in its host-loop order incl. D2D copies",
    }))
    return 0


if __name__ == "__main__":
    sys.exit(main())
