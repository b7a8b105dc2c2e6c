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
