#!/usr/bin/env python3
"""Benchmark of the RB-ThermoParticles hot path on GB300: MLUPS and %HBM roofline.

Workload (headline): 320x320x160 single-phase Rayleigh-Benard, Ra=1e8, Pr=0.71, D3Q27 f+g, seeded
linear-conduction start, populations stored in FP32 (FP32 arithmetic).  The same workload is also
timed with FP64 storage/arithmetic (the parity path) and shifted-FP16 storage, and the
particle-laden variant (1000 spheres of diameter 16) with FP64 and FP32 storage; those appear as
sub-objects of the one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one full time step of the whole lattice (16.384 M nodes).  `value` = MLUPS with the state
resident in HBM, timed with CUDA events on the library's stream; the populations (7.3 GB at FP32)
exceed L2, so no flush is needed between steps.  `e2e` runs the same K steps through the public C
ABI starting from host (numpy) buffers: the state upload and the Nu / mean-field read-back are
inside the timed region.  `--impl reference` times the CPU oracle (the restated reference step,
OpenMP FP64) on a bounded slab of the same workload with all host threads.

Multi-GPU: the path does not shard (one cavity per GPU); N>1 runs N independent replicas, takes
the max time over ranks and reports the aggregate ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "rb-thermoparticles_gb300"))

MEASURED_PEAKS = os.path.join(REPO, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one k_step launch, the mean of one
# even-step and one odd-step launch of the in-place storage, from one-pass ncu captures of
# `python bench.py --only production:<storage> --steps 4 --warmup 3` (FP32, shifted FP16: the
# 320x320x160 workload itself) and `... --only production:f64 --grid 192x192x96 ...` (FP64, 3.1 GB
# per launch, scaled to 16,384,000 nodes by the node count; its reads are exactly 440 B per node,
# its writes 423 B per node because L2 still holds part of them when the kernel ends).  The
# captures' summary is kept with the other ncu summaries.  Algorithmic bytes per launch:
# 16,384,000 nodes x bytes_per_node.
NCU_DRAM_BYTES = {
    "f32": ((3.607174144e9 + 3.569068288e9) + (3.604580352e9 + 3.557273600e9)) / 2,
    "f16s": ((1.835989248e9 + 1.781190144e9) + (1.835062016e9 + 1.772242432e9)) / 2,
    "f64": ((1.558169344e9 + 1.497404672e9) + (1.557334528e9 + 1.492732416e9)) / 2 * 16384000 / (192 * 192 * 96),
}


# FP64 work of one FP64 k_step node update, from one ncu capture of an odd and an even launch
# (k_step<0,1,0>, k_step<0,0,0>) on 128x128x64 (1,048,576 nodes) with `python bench.py --only
# production:f64 --grid 128x128x64 --steps 4 --warmup 3`:
# smsp__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum per node, odd / even:
# 167.41 / 167.00 DFMA, 189.15 / 189.00 DADD, 68.23 / 68.00 DMUL, i.e. 424.4 FP64 arithmetic
# instructions (426.4 with the FP64 compares and conversions) and 591.6 flops (an FMA counts 2)
# per node on average.
_FP64_DFMA, _FP64_DADD, _FP64_DMUL = (167.41 + 167.00) / 2, (189.15 + 189.00) / 2, (68.23 + 68.00) / 2
FP64_FLOPS_PER_NODE = 2 * _FP64_DFMA + _FP64_DADD + _FP64_DMUL
FP64_INST_PER_NODE = _FP64_DFMA + _FP64_DADD + _FP64_DMUL


def bytes_per_node(storage: int) -> int:
    """Algorithmic HBM bytes per lattice-node update: read+write 27 f and 27 g populations plus
    read+write of the buoyancy auxiliary F_x (FP64 with FP64 storage; FP32 with the float storage
    modes, which compute F_x in FP32): 880, 440 and 224 bytes."""
    s = {0: 8, 1: 4, 2: 2}[storage]
    return 2 * 54 * s + 2 * (8 if storage == 0 else 4)


def hbm_peak():
    try:
        with open(MEASURED_PEAKS) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ----------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ----------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        # raw samples: $RBTP_CLOCKS_DIR if set (to keep them), else the system temporary directory
        self.path = os.path.join(os.environ.get("RBTP_CLOCKS_DIR") or tempfile.gettempdir(),
                                 f"rbtp_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        try:
            for line in open(self.path):
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9 and p[1].isdigit():
                    rows.append(p)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [int(r[1]) for r in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, n in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": int(rows[0][2]), "reasons": sorted(reasons),
                "samples": len(rows)}


# ----------------------------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------------------------
def _events(torch, solver):
    import ctypes
    ptr = ctypes.c_void_p()
    solver.lib.rbtp_get_stream(solver.handle, ctypes.byref(ptr))
    stream = torch.cuda.ExternalStream(ptr.value)
    return stream, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def time_variant(torch, name, storage, steps, warmup, dist=None, keep_state=False, **over):
    """Device-timed MLUPS of one variant with the state resident in HBM."""
    from rbtp import Solver, workloads as W
    cfg = W.config(name, storage=storage, **over)
    s = Solver(cfg)
    f, g, f7 = W.initial_state(cfg)
    if cfg.activate_particles:
        s.initialize()          # seeded sphere placement (pinit.cu:97-144)
        s.load_state(f, g, f7, s.particles())
    else:
        s.load_state(f, g, f7)
    del f, g, f7
    s.step(warmup)
    stream, e0, e1 = _events(torch, s)
    _barrier(dist)
    torch.cuda.synchronize()
    e0.record(stream)
    s.step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ms = _max_over_ranks(torch, dist, ms)
    L = cfg.nodes
    out = {"workload": name + "".join(f" {k}={v}" for k, v in over.items()),
           "storage": ["f64", "f32", "f16s"][storage], "ms_per_step": ms / steps,
           "mlups": L * steps / (ms * 1e-3) / 1e6, "nodes": L,
           "launches_per_step": 1 if not cfg.activate_particles else 14}
    if cfg.activate_particles:
        out["npart"] = s.npart
    if keep_state:
        return out, s
    s.close()
    return out


def e2e_variant(torch, name, storage, steps, dist=None):
    """Same metric through the public API from host buffers: state upload, K steps, Nu + means
    read-back, all inside the timed region."""
    import numpy as np
    from rbtp import Solver, workloads as W
    cfg = W.config(name, storage=storage)
    s = Solver(cfg)
    # the step's inputs sit in pinned (page-locked) host buffers, as a serving front end keeps them
    pinned = []
    for a in W.initial_state(cfg):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = a
        pinned.append(t)
    f, g, f7 = (t.numpy() for t in pinned)
    # the same call sequence once untimed (first-use allocations, module loading)
    s.load_state(f, g, f7)
    s.step(2, macros_last=True)
    s.nu(s.istep)
    s.means()
    _barrier(dist)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.load_state(f, g, f7)          # returns once the import has completed on the device
    t_up = time.perf_counter()
    s.step(steps, macros_last=True)
    row = s.nu(s.istep)
    means = s.means()
    t1 = time.perf_counter()
    sec = _max_over_ranks(torch, dist, (t1 - t0) * 1e3) * 1e-3
    assert np.all(np.isfinite(row)) and np.all(np.isfinite(means))
    h2d = f.nbytes + g.nbytes + f7.nbytes
    d2h = 7 * 8 + 4 * 8 + 10 * 8 * cfg.lx  # Nu row, means, per-plane sums
    s.close()
    return {"value": cfg.nodes * steps / sec / 1e6, "unit": "MLUPS",
            "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
            "seconds": sec, "upload_seconds": t_up - t0, "upload_gbs": h2d / (t_up - t0) / 1e9,
            "host_buffers": "pinned (page-locked); the import kernel reads them in place over the host link",
            "includes": "FP64 state upload from host (f, g, 7 flow fields) + K steps + Nu/means read-back"}


def batch_variant(torch, steps: int, warmup: int, n: int = 256) -> dict:
    """Batched ensemble: n independent cavities (LY in {32,48,64,96,128}, LX = LY, LZ = LY/2, Ra
    log-uniform 1e5..1e8, Pr 0.7..7, 0..200 spheres of diameter 0.1 LY), FP32 storage, advanced in
    lockstep by one persistent launch per step under a CUDA graph.  Reports aggregate MLUPS and
    the p50/p99 device time of single batch steps."""
    import numpy as np
    from rbtp import Batch, Solver, workloads as W
    cfgs = W.ensemble(n, storage=1)
    t0 = time.perf_counter()
    solvers = []
    for c in cfgs:
        s = Solver(c)
        s.initialize()
        solvers.append(s)
    b = Batch(1)
    for s in solvers:
        b.add(s)
    setup = time.perf_counter() - t0
    from rbtp import RbtpError
    failed_calls = []

    def bstep(k):
        # a member that goes non-finite makes the batch call report it (the others keep stepping);
        # the count of such members is taken at the end from their Nu samples
        try:
            b.step(k)
        except RbtpError as exc:
            failed_calls.append(exc.status)

    bstep(warmup + 16)                  # autotuner (8 candidates x 2 steps) + warm-up
    bstep(steps)
    st = b.stats()
    lat = []
    for _ in range(min(steps, 50)):
        bstep(1)
        lat.append(b.stats()["last_step_ms"])
    # one more step with every member sampled: members whose Nu row is not finite ended non-finite
    for s in solvers:
        b.set_sampling(s, 1)
    bstep(1)
    nonfinite = 0
    for s in solvers:
        try:
            rows = b.samples(s)
        except RbtpError:
            rows = np.full((1, 7), np.nan)
        if len(rows) == 0 or not np.all(np.isfinite(rows)):
            nonfinite += 1
    out = {"workload": f"{n} cavities, LY in {{32..128}}, 0-200 spheres, FP32 storage",
           "cavities": n, "nodes": st["nodes"], "spheres": st["total_particles"],
           "ms_per_step": st["last_step_ms"], "mlups": st["nodes"] / st["last_step_ms"] / 1e3,
           "step_ms_p50": float(np.percentile(lat, 50)), "step_ms_p99": float(np.percentile(lat, 99)),
           "tile_shape": ["32x4", "64x2"][st["tile_shape"]], "persistent_grid": st["grid"],
           "cuda_graph": bool(st["graph"]), "setup_seconds": round(setup, 2),
           "steps_run": warmup + 16 + steps + min(steps, 50) + 1,
           "members_nonfinite_at_end": nonfinite, "batch_calls_reporting_nonfinite": len(failed_calls)}
    b.close()
    for s in solvers:
        s.close()
    return out


def _stream(cfgs, horizons, arrivals, tick: int, every: int = 500) -> dict:
    """One Poisson stream through a fresh server; latency = completion - scheduled arrival."""
    import numpy as np
    from rbtp import Server
    n = len(cfgs)
    srv = Server(1, hbm_budget=180e9)
    t0 = srv.stats()["clock"]
    ids, k, peak, trace = [], 0, 0, []
    while True:
        now = srv.stats()["clock"] - t0
        while k < n and arrivals[k] <= now:
            ids.append(srv.submit(cfgs[k], int(horizons[k]), every))
            k += 1
        a, q = srv.tick(tick)
        peak = max(peak, a)
        st = srv.stats()
        trace.append((st["clock"] - t0, st["node_updates"]))
        if k == n and a == 0 and q == 0:
            break
        if a == 0 and q == 0 and k < n:
            time.sleep(max(0.0, min(0.05, arrivals[k] - (srv.stats()["clock"] - t0))))
    st = srv.stats()
    lat, ok, failed = [], 0, {}
    for i, rid in enumerate(ids):
        p = srv.poll(rid)
        _, _, done = srv.times(rid)
        if p["state"] == Server.DONE:
            ok += 1
            lat.append(done - t0 - arrivals[i])
        else:
            failed[str(i)] = p["status"]
    srv.close()
    span = max(st["clock"] - t0 - arrivals[0], 1e-9)
    # node updates up to the last arrival (the stream is still feeding the server then)
    t_last = arrivals[-1]
    upd_last = max([u for t, u in trace if t <= t_last] or [0.0])
    t_at = max([t for t, u in trace if t <= t_last] or [arrivals[0]])
    return {"rate_per_s": float(n / arrivals[-1]) if arrivals[-1] > 0 else "all at t=0",
            "completed": ok, "failed_status": failed,
            "latency_p50_s": float(np.percentile(lat, 50)) if lat else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if lat else None,
            "served_mlups": st["node_updates"] / span / 1e6,
            "served_mlups_until_last_arrival": (upd_last / (t_at - arrivals[0]) / 1e6
                                                if t_at > arrivals[0] else None),
            "peak_active": peak, "makespan_s": round(span, 3), "ticks": len(trace),
            "node_updates": st["node_updates"]}


def serving_variant(n: int = 16, rates=(0.5, 4.0), seed: int = 3, tick: int = 250,
                    batched_mlups=None) -> dict:
    """Serving: n solve requests drawn like the batched ensemble (sizes, Ra, Pr, spheres) with
    horizons uniform in [2000, 50000] steps and Nu sampled every 500 steps, arriving as a Poisson
    stream (the same requests at each swept rate, requests/s), admitted by footprint within 180 GB,
    FP32 storage.  Beside it: the same requests solved one after another by the plain FP64 path,
    estimated from 100 timed steps of each (after 10 warm-up steps) times its horizon."""
    import numpy as np
    from rbtp import Solver, workloads as W
    rng = np.random.default_rng(seed)
    cfgs = W.ensemble(n, seed=seed, storage=1)
    horizons = rng.integers(2000, 50001, size=n)
    gaps = rng.exponential(1.0, size=n)
    streams = {}
    for rate in rates:
        streams[str(rate)] = _stream(cfgs, horizons, np.cumsum(gaps / rate), tick)
    # the same requests all present at once: offline batching of the same work
    offline = _stream(cfgs, horizons, np.zeros(n), tick)
    # sequential plain FP64 solves of the same requests
    seq_s, work = 0.0, 0.0
    for c, h in zip(W.ensemble(n, seed=seed, storage=0), horizons):
        s = Solver(c)
        s.initialize()
        s.step(10)
        s.synchronize()
        t0 = time.perf_counter()
        s.step(100)
        s.synchronize()
        seq_s += (time.perf_counter() - t0) / 100 * int(h)
        work += float(c.nodes) * int(h)
        s.close()
    top = streams[str(max(rates))]
    out = {"requests": n, "tick_steps": tick, "sample_every": 500, "horizons": "uniform 2000..50000",
           "streams": streams, "offline_same_requests": offline,
           "latency_p50_s": top["latency_p50_s"], "latency_p99_s": top["latency_p99_s"],
           "served_mlups": top["served_mlups"], "completed": top["completed"],
           "sequential_fp64_mlups": work / seq_s / 1e6,
           "sequential_fp64_makespan_s": round(seq_s, 1),
           "sequential_fp64_method": "estimate: each request's plain FP64 solve timed over 100 steps "
                                     "(after 10 warm-up steps) and scaled to its horizon"}
    for rate, st in streams.items():
        st["served_over_batched"] = st["served_mlups"] / offline["served_mlups"]
    out["served_over_sequential_fp64"] = top["served_mlups"] / out["sequential_fp64_mlups"]
    # served throughput against batched throughput of the same requests (all present at t=0), and
    # against the 256-cavity ensemble (a 16-times larger concurrent load)
    out["served_over_batched"] = top["served_mlups"] / offline["served_mlups"]
    if batched_mlups:
        out["served_over_ensemble_batched"] = top["served_mlups"] / batched_mlups
    return out


def nu_accuracy(steps: int = 60000, every: int = 100, seeds=(1, 2, 3)) -> dict:
    """Time-averaged Nusselt numbers of FP32 and shifted-FP16 storage against the FP64 path (the
    parity-tested path) on 64x64x32, Ra=1e6, Pr=0.71, averaged over the last two thirds of the
    run.  Convection at this Ra is chaotic, so each mode runs from several seeded perturbations:
    the spread of the FP64 runs is the noise floor of a time average of this length, and the
    difference of the per-mode means is compared with the standard error of that difference."""
    import numpy as np
    from rbtp import Solver, workloads as W
    out = {"workload": "64x64x32 Ra=1e6 Pr=0.71, seeded starts", "steps": steps, "sample_every": every,
           "average_over": "last 2/3 of each run", "seeds": list(seeds)}
    keys = ("nu_bulk", "nu_top", "nu_bottom")
    per = {}
    for st, name in ((0, "f64"), (1, "f32"), (2, "f16s")):
        vals = []
        t0 = time.perf_counter()
        for seed in seeds:
            cfg = W.config("plain_fp64", storage=st)
            s = Solver(cfg)
            s.load_state(*W.initial_state(cfg, seed=seed))
            rows = []
            for _ in range(steps // every):
                s.step(every, macros_last=True)
                rows.append(s.nu(s.istep))
            s.close()
            r = np.array(rows)[len(rows) // 3:]
            vals.append(r[:, 2:5].mean(0))
        per[name] = np.array(vals)
        out[name + "_seconds"] = round(time.perf_counter() - t0, 3)
        out[name] = {k: {"mean": float(per[name][:, j].mean()), "std": float(per[name][:, j].std(ddof=1)),
                         "per_seed": [float(v) for v in per[name][:, j]]} for j, k in enumerate(keys)}
    n = len(seeds)
    for name in ("f32", "f16s"):
        out[name]["rel_diff_of_means_vs_f64"] = {}
        out[name]["diff_in_standard_errors"] = {}
        for j, k in enumerate(keys):
            d = per[name][:, j].mean() - per["f64"][:, j].mean()
            se = math.sqrt(per[name][:, j].var(ddof=1) / n + per["f64"][:, j].var(ddof=1) / n)
            out[name]["rel_diff_of_means_vs_f64"][k] = float(d / per["f64"][:, j].mean())
            out[name]["diff_in_standard_errors"][k] = float(d / se) if se > 0 else None
    out["steady"] = nu_accuracy_steady()
    return out


def nu_accuracy_steady(steps: int = 60000, every: int = 500) -> dict:
    """Time-averaged Nusselt numbers of FP32 and shifted-FP16 storage against FP64 on steady
    convection (64x64x32, Ra=3e4, Pr=0.71, seeded +-1e-2 start; one steady roll after ~30k steps),
    where no chaotic noise floor blurs the comparison; average over the last third."""
    import numpy as np
    from rbtp import Solver, workloads as W
    out = {"workload": "64x64x32 Ra=3e4 Pr=0.71 (steady convection), seeded +-1e-2 start",
           "steps": steps, "sample_every": every, "average_over": "last 1/3 of the run"}
    series = {}
    for st, name in ((0, "f64"), (1, "f32"), (2, "f16s")):
        cfg = W.config("plain_fp64", rayleigh=3e4, storage=st)
        s = Solver(cfg)
        s.load_state(*W.initial_state(cfg, seed=1, amp=1e-2))
        rows = []
        for _ in range(steps // every):
            s.step(every, macros_last=True)
            rows.append(s.nu(s.istep))
        series[name] = np.array(rows)
        s.close()
    keep = slice(2 * len(series["f64"]) // 3, None)
    for name in series:
        r = series[name][keep]
        out[name] = {"nu_bulk": float(r[:, 2].mean()), "nu_top": float(r[:, 3].mean()),
                     "nu_bottom": float(r[:, 4].mean())}
    for name in ("f32", "f16s"):
        out[name]["rel_err_vs_f64"] = {k: abs(out[name][k] / out["f64"][k] - 1.0)
                                       for k in ("nu_bulk", "nu_top", "nu_bottom")}
    return out


def nu_production(steps: int = 20000, every: int = 100) -> dict:
    """Nu error of the float storage modes at the production configuration: 320x320x160, Ra=1e8,
    Pr=0.71, the seeded +-1e-3 start, `steps` steps in FP64, FP32-store and shifted-FP16 storage
    from the same start, Nu sampled every `every` steps; time averages over the second half of the
    run and their relative differences from FP64.  At this Ra the flow is chaotic after a few
    free-fall times (LX / u0 = 2263 steps), so each float run follows FP64 only until rounding
    differences grow: the step at which each series first departs from FP64 by 1 % is reported
    beside the averages."""
    import numpy as np
    from rbtp import Solver, workloads as W
    out = {"workload": "production single-phase RB 320x320x160, Ra=1e8, Pr=0.71, seeded +-1e-3 start",
           "steps": steps, "sample_every": every, "average_over": "second half of the run"}
    series = {}
    for st, name in ((0, "f64"), (1, "f32"), (2, "f16s")):
        cfg = W.config("production", storage=st)
        s = Solver(cfg)
        f, g, f7 = W.initial_state(cfg)
        s.load_state(f, g, f7)
        del f, g, f7
        t0 = time.perf_counter()
        rows = []
        for _ in range(steps // every):
            s.step(every, macros_last=True)
            rows.append(s.nu(s.istep))
        out[name + "_seconds"] = round(time.perf_counter() - t0, 1)
        s.close()
        series[name] = np.array(rows)
    half = slice(len(series["f64"]) // 2, None)
    keys = ("nu_bulk", "nu_top", "nu_bottom")
    for name, r in series.items():
        out[name] = {k: float(r[half, 2 + j].mean()) for j, k in enumerate(keys)}
        out[name]["series_nu_bulk"] = [round(float(v), 5) for v in r[:, 2]]
    for name in ("f32", "f16s"):
        out[name]["rel_err_vs_f64"] = {k: out[name][k] / out["f64"][k] - 1.0 for k in keys}
        dev = np.abs(series[name][:, 2] / series["f64"][:, 2] - 1.0)
        out[name]["departs_from_f64_by_1pct_at_step"] = (int(series[name][np.argmax(dev > 0.01), 0])
                                                         if np.any(dev > 0.01) else None)
    out["f32_within_1pct"] = all(abs(v) < 0.01 for v in out["f32"]["rel_err_vs_f64"].values())
    out["f16s_within_1pct"] = all(abs(v) < 0.01 for v in out["f16s"]["rel_err_vs_f64"].values())
    return out


def cpu_baseline(steps: int = 3, nz: int = 40):
    """The oracle (FP64 OpenMP restatement of the reference step) on a slab of the production
    grid, all host threads."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_py
    from rbtp import workloads as W
    threads = oracle_py.set_threads(os.cpu_count() or 1)
    cfg = W.config("production", lz=nz)
    o = oracle_py.Oracle(cfg)
    f, g, f7 = W.initial_state(cfg)
    o.load_state(f, g, f7)
    del f, g, f7
    o.step(1)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": cfg.nodes * steps / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{cfg.lx}x{cfg.ly}x{cfg.lz} slab of the 320x320x160 single-phase workload, "
                      f"{steps} steps, FP64 oracle"}


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(torch, dist, v):
    """The largest of the ranks' values (the slowest replica sets the step time)."""
    if dist is None:
        return v
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args) -> dict:
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as td
        torch.cuda.set_device(local)
        td.init_process_group("nccl")
        dist = td
    else:
        torch.cuda.set_device(0)
    import rbtp_build
    if rank == 0 or world == 1:
        rbtp_build.build(host=False)
    _barrier(dist)
    peak, peak_src = hbm_peak()

    # headline: FP32 storage, clocks sampled over its timed region
    with ClockSampler(local) as clk:
        head = time_variant(torch, "production", 1, args.steps, args.warmup, dist)
    clocks = clk.summary()
    def guarded(fn, *a, **k):
        try:
            return fn(*a, **k)
        except Exception as exc:  # a failing variant is reported, the headline still prints
            return {"error": f"{type(exc).__name__}: {exc}"}

    fp64 = guarded(time_variant, torch, "production", 0, args.steps, args.warmup, dist)
    f16 = guarded(time_variant, torch, "production", 2, args.steps, args.warmup, dist)
    # Spheres at the reference's default density ratio 1.0: with ratio 1.5 the reference's particle
    # buoyancy (1 - 1/1.5) g0 accelerates every sphere by 0.33 lattice units per step^2 and the
    # spheres pile up against the x = LX wall within ~20 steps (move.cu:47,63).
    psteps = max(3, min(args.steps, 20))
    p64 = guarded(time_variant, torch, "particle_laden", 0, psteps, args.warmup, dist, rho_particle_ratio=1.0)
    p32 = guarded(time_variant, torch, "particle_laden", 1, psteps, args.warmup, dist, rho_particle_ratio=1.0)
    e2e = guarded(e2e_variant, torch, "production", 1, args.steps, dist)
    nua = guarded(nu_accuracy) if rank == 0 else None
    bat = guarded(batch_variant, torch, args.steps, args.warmup)
    srv = guarded(serving_variant, batched_mlups=bat.get("mlups"))

    def roof(v):
        b = bytes_per_node(["f64", "f32", "f16s"].index(v["storage"]))
        achieved = v["nodes"] * b / (v["ms_per_step"] * 1e-3) / 1e9
        traffic = NCU_DRAM_BYTES.get(v["storage"]) if v["workload"] == "production" else None
        return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_src,
                "bytes_per_node": b, "traffic": traffic,
                "algorithmic_bytes": v["nodes"] * b}

    for v in (head, fp64, f16, p64, p32):
        if "error" not in v:
            v["roofline"] = roof(v)
    # the FP64 path is bound by the FP64 pipe: its compute roofline against the measured FMA rate
    from rbtp import fp64_fma_rate
    dfma = guarded(fp64_fma_rate)
    fp64_compute = None
    if "mlups" in fp64 and isinstance(dfma, float) and dfma > 0:
        achieved = fp64["nodes"] * FP64_FLOPS_PER_NODE / (fp64["ms_per_step"] * 1e-3)
        fp64_compute = {"bound": "fp64", "achieved": round(achieved / 1e12, 4), "peak": round(dfma / 1e12, 4),
                        "unit": "TFLOP/s", "frac": round(achieved / dfma, 4),
                        "peak_source": "measured: rbtp_fp64_fma_rate microkernel (independent DFMA chains, CUDA events)",
                        "flops_per_node": round(FP64_FLOPS_PER_NODE, 1),
                        "fp64_instructions_per_node": round(FP64_INST_PER_NODE, 1),
                        # DADD and DMUL occupy the FP64 pipe like DFMA: the share of its issue rate
                        "fp64_instruction_frac": round(fp64["nodes"] * FP64_INST_PER_NODE
                                                       / (fp64["ms_per_step"] * 1e-3) / (dfma / 2), 4)}
        fp64["compute_roofline"] = fp64_compute
    value = head["mlups"] * world
    line = {
        "metric": "MLUPS (lattice-node updates/s), 320x320x160 D3Q27 f+g RB step, FP32-store",
        "value": round(value, 1), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(head["ms_per_step"], 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded linear-conduction start (SplitMix64 +-1e-3 perturbation)",
        "config": {"workload": "production single-phase RB 320x320x160, Ra=1e8, Pr=0.71, FP32-store",
                   "arithmetic": "FP32 population storage and FP32 step arithmetic (FP64 reductions)",
                   "nodes": head["nodes"], "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                   "l2": "state (3.5 GB of populations, in place) exceeds L2; no flush needed"},
        "roofline": head["roofline"],
        "clocks": clocks,
        "gpu_launches": head["launches_per_step"] * args.steps,
        "e2e": e2e,
        "fp64_mlups": round(fp64["mlups"], 1) if "mlups" in fp64 else None,
        "fp64_roofline": fp64.get("roofline"),
        "fp64_compute_roofline": fp64_compute,
        "fp64": fp64, "fp16s": f16, "particle_laden_fp64": p64, "particle_laden_fp32": p32,
        "fp32_over_fp64": round(head["mlups"] / fp64["mlups"], 3) if "mlups" in fp64 else None,
        "nu_accuracy": nua,
        "batched_ensemble": bat,
        "serving": srv,
    }
    if rank == 0:
        try:
            line["cpu_baseline"] = cpu_baseline()
        except Exception as exc:  # reported, not fatal
            line["cpu_baseline"] = {"value": None, "error": str(exc)}
    if dist is not None:
        dist.destroy_process_group()
    return line if rank == 0 else None


def run_only(args) -> dict:
    """One variant on an optional smaller grid (profiling captures): --only production:f32."""
    import torch
    torch.cuda.set_device(0)
    import rbtp_build
    rbtp_build.build(host=False)
    name, st = args.only.split(":")
    if name == "batch":
        if st != "f32":
            raise SystemExit("the batched ensemble runs with FP32 storage")
        return batch_variant(torch, args.steps, args.warmup, n=args.cavities)
    over = {}
    if args.grid:
        lx, ly, lz = (int(v) for v in args.grid.lower().split("x"))
        over.update(lx=lx, ly=ly, lz=lz)
    if name == "particle_laden":
        over.setdefault("rho_particle_ratio", 1.0)
    v = time_variant(torch, name, ["f64", "f32", "f16s"].index(st), args.steps, args.warmup, None, **over)
    peak, src = hbm_peak()
    b = bytes_per_node(["f64", "f32", "f16s"].index(st))
    achieved = v["nodes"] * b / (v["ms_per_step"] * 1e-3) / 1e9
    v["roofline"] = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": src, "bytes_per_node": b}
    return v


def run_reference(args) -> dict | None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_py
    from rbtp import workloads as W
    threads = oracle_py.set_threads(os.cpu_count() or 1)
    nz = 16
    cfg = W.config("production", lz=nz)
    o = oracle_py.Oracle(cfg)
    f, g, f7 = W.initial_state(cfg)
    o.load_state(f, g, f7)
    del f, g, f7
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    dt = time.perf_counter() - t0
    v = cfg.nodes * args.steps / dt / 1e6
    sample = (f"{cfg.lx}x{cfg.ly}x{nz} slab of the 320x320x160 workload per step, "
              f"FP64 oracle (OpenMP restatement of the reference CUDA step)")
    return {"metric": "MLUPS (lattice-node updates/s), 320x320x160 D3Q27 f+g RB step, FP32-store",
            "value": round(v, 3), "unit": "MLUPS", "impl": "reference", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "dtype": "f64", "data": "synthetic",
            # the same workload as the default arm, timed on a bounded slab sample (cpu_baseline.sample)
            "config": {"workload": "production single-phase RB 320x320x160, Ra=1e8, Pr=0.71, FP32-store",
                       "arithmetic": "FP64 throughout: the reference's own precision (its step has no "
                                     "FP32 storage mode); compare with this library's FP64 path, "
                                     "fp64_mlups in the GPU arm's line",
                       "nodes": 320 * 320 * 160, "parallelism": "host cores"},
            "cpu_baseline": {"value": round(v, 3), "unit": "MLUPS", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": round(v, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--only", default=None, help="one variant, e.g. production:f32 (profiling)")
    ap.add_argument("--grid", default=None, help="grid override for --only, e.g. 128x128x64")
    ap.add_argument("--cavities", type=int, default=256, help="ensemble size for --only batch:f32")
    ap.add_argument("--serving-stress", action="store_true",
                    help="only the serving leg at a heavy load: 64 requests at 1, 4, 16 and 64 arrivals/s")
    ap.add_argument("--nu-production", type=int, default=0, metavar="STEPS",
                    help="only the production-size Nu accuracy leg (FP64 vs FP32 vs shifted FP16) over STEPS steps")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.serving_stress or args.nu_production:
        import torch
        torch.cuda.set_device(0)
        import rbtp_build
        rbtp_build.build(host=False)
        if args.nu_production:
            print(json.dumps(nu_production(args.nu_production)), flush=True)
        else:
            bat = batch_variant(torch, 20, 5)
            print(json.dumps({"batched_ensemble": bat,
                              "serving": serving_variant(n=64, rates=(1.0, 4.0, 16.0, 64.0),
                                                         batched_mlups=bat.get("mlups"))}), flush=True)
        return 0
    if args.only:
        line = run_only(args)
    else:
        line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
