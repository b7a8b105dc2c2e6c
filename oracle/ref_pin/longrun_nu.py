#!/usr/bin/env python3
"""Long-run time-averaged Nusselt numbers of librbtp's FP64 path against the reference's own kernels
on chaotic convection (TEST INFRASTRUCTURE ONLY; needs a GPU and oracle/_ref/ref_config1.cubin).

The configuration is the plain FP64 parity case: 64x64x32, Ra = 1e6, Pr = 0.71, seeded +-1e-3
starts.  Both codes run each seed for --steps steps from the same start; the Nu row of output_nu
(output_statis.cu:111-223) is taken every --every steps (by the reference-pin driver on the
reference's d_ux/d_phi, by rbtp_nu on librbtp) and averaged over the last two thirds.  Convection
at this Ra is chaotic, so the trajectories part after a few thousand steps and only the
statistics compare: the script prints, per seed and over seeds, the time averages, the relative
difference of the means, and that difference in standard errors of the difference.

    python oracle/ref_pin/longrun_nu.py [--seeds 1,2,3] [--steps 60000] [--every 100] [--out file]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import tempfile
import time
from pathlib import Path

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "rb-thermoparticles_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))

import numpy as np  # noqa: E402

import refpin  # noqa: E402  (tests/refpin.py: driver build and I/O helpers)
from rbtp import Solver, workloads as W  # noqa: E402

KEYS = ("nu_bulk", "nu_top", "nu_bottom")


def ours(cfg, seed, steps, every):
    s = Solver(cfg)
    s.load_state(*W.initial_state(cfg, seed=seed))
    rows = []
    for _ in range(steps // every):
        s.step(every, macros_last=True)
        rows.append(s.nu(s.istep))
    s.close()
    return np.array(rows)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--seeds", default="1,2,3")
    ap.add_argument("--steps", type=int, default=60000)
    ap.add_argument("--every", type=int, default=100)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    seeds = [int(v) for v in a.seeds.split(",")]
    import rbtp_build
    rbtp_build.build(host=False)
    driver = refpin.build_driver()
    cfg = refpin.cfg_of("ref_config1")
    res = {"workload": "64x64x32 Ra=1e6 Pr=0.71, seeded +-1e-3 starts (plain FP64 parity case)",
           "steps": a.steps, "sample_every": a.every, "average_over": "last 2/3 of each run",
           "seeds": seeds, "per_seed": {}}
    vals = {"reference": [], "librbtp": []}
    t_ref = t_ours = 0.0
    for seed in seeds:
        f, g, f7 = W.initial_state(cfg, seed=seed)
        with tempfile.TemporaryDirectory() as d:
            t0 = time.perf_counter()
            rr = refpin.run_nu(driver, "ref_config1", Path(d), cfg, None, None, None, None, a.steps, a.every,
                               timeout=7200, synthetic=1, seed=seed, amp=1e-3)
            t_ref += time.perf_counter() - t0
        t0 = time.perf_counter()
        ro = ours(cfg, seed, a.steps, a.every)
        t_ours += time.perf_counter() - t0
        assert np.array_equal(rr[:, 0], ro[:, 0])
        # the two runs agree row by row until chaos parts them: first sample where they differ by 1e-6
        diff = np.abs(ro[:, 2] - rr[:, 2]) / np.abs(rr[:, 2])
        part = int(rr[np.argmax(diff > 1e-6), 0]) if np.any(diff > 1e-6) else None
        keep = slice(len(rr) // 3, None)
        mr, mo = rr[keep, 2:5].mean(0), ro[keep, 2:5].mean(0)
        vals["reference"].append(mr)
        vals["librbtp"].append(mo)
        res["per_seed"][str(seed)] = {"reference": dict(zip(KEYS, map(float, mr))),
                                      "librbtp": dict(zip(KEYS, map(float, mo))),
                                      "rows_agree_to_1e-6_until_step": part}
        del f, g, f7
        print(f"seed {seed}: reference {mr}, librbtp {mo}, parted at step {part}", flush=True)
    n = len(seeds)
    R, O = np.array(vals["reference"]), np.array(vals["librbtp"])
    res["reference_seconds"] = round(t_ref, 1)
    res["librbtp_seconds"] = round(t_ours, 1)
    for j, k in enumerate(KEYS):
        d = O[:, j].mean() - R[:, j].mean()
        se = math.sqrt(O[:, j].var(ddof=1) / n + R[:, j].var(ddof=1) / n) if n > 1 else float("nan")
        res[k] = {"reference_mean": float(R[:, j].mean()), "librbtp_mean": float(O[:, j].mean()),
                  "reference_std": float(R[:, j].std(ddof=1)) if n > 1 else None,
                  "librbtp_std": float(O[:, j].std(ddof=1)) if n > 1 else None,
                  "rel_diff_of_means": float(d / R[:, j].mean()),
                  "diff_in_standard_errors": float(d / se) if se > 0 else None}
    line = json.dumps(res)
    print(line)
    if a.out:
        with open(a.out, "w") as fh:
            fh.write(line + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
