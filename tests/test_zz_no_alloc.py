"""GPU test of rbtp_plane_sums_noalloc, the allocation-free variant of the per-plane diagnostic
sums, for callers that cannot allocate device memory (a host framework that owns the device memory
pool, or a loop that cannot afford cudaMalloc's implicit synchronisation).

The entry point is called through the C ABI on device buffers the test owns (allocated here with
torch — the entry point itself allocates nothing), twice in a row on different lattice states, and
each result is checked against the existing entry points rbtp_nu and rbtp_means of the same state.
This file is named so that pytest collects it after every other test.
"""
import ctypes as C

import numpy as np
import pytest

import rbtp
from rbtp import Solver, workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _nu_from_planes(pl, cfg, der):
    # the formulas of rbtp_nu (output_statis.cu:111-223) applied to the ten per-plane sums
    lx = cfg.lx
    sf, nf, sp, npp, ws, wc = (pl[k] for k in range(6))
    avg_f = sum(sf[i] / nf[i] for i in range(lx) if nf[i] > 0) / lx
    avg_p = sum(sp[i] / npp[i] for i in range(lx) if npp[i] > 0) / lx
    vf = cfg.particle_fraction
    ff = max(0.0, 1.0 - vf)
    cond = der.diff * (cfg.t_hot - cfg.t_cold) / lx
    nbf = ff + ff * (avg_f / cond)
    nbp = vf * cfg.cp_particle_ratio * (avg_p / cond)
    area = cfg.ly * cfg.lz
    scale = lx / (cfg.t_hot - cfg.t_cold)
    return np.array([nbf + nbp, ws[lx - 1] / area * scale, ws[0] / area * scale, nbf, nbp])


def _call(lib, torch, s, cfg):
    m = s.macros()
    dev = {k: torch.from_numpy(m[k]).cuda() for k in ("ux", "uy", "uz", "phi")}
    parts = s.npart > 0
    owner = torch.from_numpy(s.flags()).cuda() if parts else None
    state = torch.from_numpy(np.ascontiguousarray(s.particles().T)).cuda() if parts else None  # column-major
    out = torch.full((10 * cfg.lx,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ptr = lambda t: None if t is None else C.c_void_p(t.data_ptr())  # noqa: E731
    st = lib.rbtp_plane_sums_noalloc(ptr(dev["ux"]), ptr(dev["uy"]), ptr(dev["uz"]), ptr(dev["phi"]),
                                     ptr(owner), ptr(state), s.npart, cfg.lx, cfg.ly, cfg.lz,
                                     cfg.t_hot, cfg.t_cold, ptr(out), C.c_void_p(stream))
    assert st == 0, rbtp.STATUS.get(st, st)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(10, cfg.lx)


def test_noalloc_plane_sums_match_existing_entry_points(lib_built):
    torch = pytest.importorskip("torch")
    lib = rbtp.load_library()
    cfg = W.config("plain_fp64", lx=48, ly=48, lz=24, activate_particles=1,
                   particle_diam_frac=8.0 / 48.0, particle_fraction=0.04)
    der = rbtp.derive(cfg)
    s = Solver(cfg)
    s.initialize()
    for steps in (20, 7):   # two calls in a row, on different states
        s.step(steps, macros_last=True)
        pl = _call(lib, torch, s, cfg)
        assert np.all(np.isfinite(pl))
        row = np.array(s.nu(s.istep))
        ours = _nu_from_planes(pl, cfg, der)
        ref = row[[2, 3, 4, 5, 6]]
        assert np.allclose(ours, ref, rtol=TOL, atol=TOL), (ours, ref)
        means = pl[6:10].sum(axis=1) / cfg.nodes
        assert np.allclose(means, s.means(), rtol=TOL, atol=1e-15)


def test_noalloc_single_phase_ragged_planes(lib_built):
    """No particles (owner and particle state NULL) and lx = 200, not a multiple of the reduction's
    128-thread blocks; the x-profile too."""
    torch = pytest.importorskip("torch")
    lib = rbtp.load_library()
    cfg = W.config("plain_fp64", lx=200, ly=24, lz=20)
    der = rbtp.derive(cfg)
    s = Solver(cfg)
    s.load_state(*W.initial_state(cfg, seed=4, amp=1e-2))
    for steps in (15, 4):
        s.step(steps, macros_last=True)
        pl = _call(lib, torch, s, cfg)
        assert np.all(np.isfinite(pl))
        row = np.array(s.nu(s.istep))
        ours = _nu_from_planes(pl, cfg, der)
        assert np.allclose(ours, row[[2, 3, 4, 5, 6]], rtol=TOL, atol=TOL), (ours, row)
        assert np.allclose(pl[6:10].sum(axis=1) / cfg.nodes, s.means(), rtol=TOL, atol=1e-15)
        prof = (pl[6:10] / (cfg.ly * cfg.lz)).T
        assert np.allclose(prof, s.profile(), rtol=TOL, atol=1e-15)


def test_noalloc_rejects_oversized_lattice(lib_built):
    lib = rbtp.load_library()
    d = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = lib.rbtp_plane_sums_noalloc(d, d, d, d, None, None, 0, 4096, 8, 8, 1.0, 0.0, d, None)
    assert st == -8  # RBTP_ERR_CAPACITY
    # lattices rbtp_create would reject (fewer than 3 nodes along an axis)
    for dims in ((1, 8, 8), (8, 2, 8), (8, 8, 2)):
        assert lib.rbtp_plane_sums_noalloc(d, d, d, d, None, None, 0, *dims, 1.0, 0.0, d, None) == -9
