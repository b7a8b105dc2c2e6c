"""Continuous-batching server (rbtp_server_*): requests admitted while others run share the batched
launches; each result must be the same alone and in the mix (FP32 storage: identical Nu series —
the batched kernels compute each cavity independently — checked to 1e-6 relative); admission respects
the HBM budget; an oversized request fails with a status instead of blocking the queue forever."""
import numpy as np
import pytest

from rbtp import Server, STORE_F32, footprint, workloads as W

pytestmark = pytest.mark.gpu


def _req(k, **kw):
    base = [dict(lx=32, ly=32, lz=16, rayleigh=1e6),
            dict(lx=48, ly=48, lz=24, rayleigh=3e5, prandtl=2.0, activate_particles=1,
                 particle_diam_frac=8.0 / 48.0, particle_fraction=0.04),
            dict(lx=40, ly=24, lz=20, rayleigh=5e6, prandtl=0.9),
            dict(lx=32, ly=32, lz=32, activate_particles=1, particle_diam_frac=6.0 / 32.0,
                 particle_fraction=0.03, rayleigh=8e5, particle_rand_seed=11)][k]
    base.update(kw)
    return W.config("plain_fp64", storage=STORE_F32, **base)


def _drain(srv, ids, max_steps=50, submit_later=()):
    pending = list(submit_later)
    ticks = 0
    while True:
        a, q = srv.tick(max_steps)
        ticks += 1
        if pending and ticks in (2, 3):
            cfg, hz, ev = pending.pop(0)
            ids.append(srv.submit(cfg, hz, ev))
        if a == 0 and q == 0 and not pending:
            break
        assert ticks < 10000
    return ids


def test_same_result_alone_and_in_the_mix(lib_built):
    alone = Server(STORE_F32)
    rid = alone.submit(_req(1), 300, 40)
    _drain(alone, [rid])
    ref = alone.poll(rid)
    assert ref["state"] == Server.DONE and ref["steps_done"] == 300
    assert len(ref["series"]) == 300 // 40 + 1          # samples at 40, 80, ..., 280 and the last step
    mix = Server(STORE_F32)
    others = [mix.submit(_req(0), 170, 25), mix.submit(_req(3), 420, 60)]
    ids = _drain(mix, others, submit_later=[(_req(1), 300, 40), (_req(2), 90, 30)])
    got = mix.poll(ids[2])
    assert got["state"] == Server.DONE and got["steps_done"] == 300
    np.testing.assert_allclose(got["series"], ref["series"], rtol=1e-6, atol=1e-9)
    for i in ids:
        assert mix.poll(i)["state"] == Server.DONE


def test_admission_by_footprint(lib_built):
    cfgs = [_req(0), _req(2), _req(0, rayleigh=2e6), _req(2, prandtl=3.0)]
    budget = max(footprint(c) for c in cfgs) * 2.2       # at most two resident at a time
    srv = Server(STORE_F32, hbm_budget=budget)
    ids = [srv.submit(c, 120, 60) for c in cfgs]
    peak = 0
    for _ in range(1000):
        a, q = srv.tick(60)
        peak = max(peak, a)
        assert srv.stats()["used_bytes"] <= budget
        if a == 0 and q == 0:
            break
    assert peak == 2
    t = [srv.times(i) for i in ids]
    assert all(x[2] > 0 for x in t)
    assert t[0][1] <= t[1][1] <= t[2][1] <= t[3][1]      # admitted in arrival order


def test_oversized_request_fails_cleanly(lib_built):
    small = _req(0)
    srv = Server(STORE_F32, hbm_budget=footprint(small) * 1.5)
    big = srv.submit(_req(1), 50, 25)
    ok = srv.submit(small, 50, 25)
    for _ in range(100):
        a, q = srv.tick(25)
        if a == 0 and q == 0:
            break
    assert srv.poll(big)["state"] == Server.FAILED and srv.poll(big)["status"] == -3
    assert srv.poll(ok)["state"] == Server.DONE


def test_checkpoint_resume_mid_stream(lib_built, tmp_path):
    """A server checkpointed between ticks and restored into a fresh server finishes every request
    with the same Nu series as an uninterrupted server, bit for bit (exact state checkpoints)."""
    reqs = [(_req(1), 260, 40), (_req(0), 150, 25), (_req(3), 330, 60), (_req(2), 90, 30)]
    ref = Server(STORE_F32)
    rids = [ref.submit(*r) for r in reqs]
    _drain(ref, rids)
    srv = Server(STORE_F32)
    ids = [srv.submit(*r) for r in reqs]
    for _ in range(3):
        srv.tick(50)
    mid = [srv.poll(i)["state"] for i in ids]
    assert Server.ACTIVE in mid
    srv.checkpoint(str(tmp_path))
    srv.close()
    again = Server(STORE_F32)
    again.restore(str(tmp_path))
    _drain(again, ids)
    for a, b in zip(rids, ids):
        pa, pb = ref.poll(a), again.poll(b)
        assert pb["state"] == Server.DONE and pb["steps_done"] == pa["steps_done"]
        np.testing.assert_array_equal(pb["series"], pa["series"])


def test_handle_checkpoint_is_exact(lib_built, tmp_path):
    from rbtp import Solver, STORE_F16S
    for storage in (0, STORE_F32, STORE_F16S):
        cfg = W.config("plain_fp64", lx=48, ly=48, lz=24, activate_particles=1, particle_diam_frac=8.0 / 48.0,
                       particle_fraction=0.04, storage=storage)
        # after an odd number of steps the in-place array holds post-collision populations
        # swapped, after an even number post-streaming ones in natural order: both are exact
        for n0 in (13, 12):
            a = Solver(cfg)
            a.initialize()
            a.step(n0)
            path = str(tmp_path / f"h{storage}_{n0}.ckp")
            a.checkpoint_write(path)
            b = Solver(cfg)
            b.checkpoint_read(path)
            assert b.istep == n0
            a.step(9, macros_last=True)
            b.step(9, macros_last=True)
            fa, ga = a.fg()
            fb, gb = b.fg()
            assert np.array_equal(fa, fb) and np.array_equal(ga, gb)
            assert np.array_equal(a.particles(), b.particles()) and np.array_equal(a.flags(), b.flags())
            assert a.nu(n0 + 9) == b.nu(n0 + 9)
