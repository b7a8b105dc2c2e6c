"""The state import of rbtp_load_state reads its FP64 sources in one pass, by one of two routes:
sources the device can read (page-locked host memory through its device alias, device memory)
are read in place by the import kernel; pageable host memory is copied in chunks of 2^20 nodes
through two staging slots.  All routes must leave the same storage state, bit for bit, in every
storage mode, with and without the flow fields.  The lattice here has three staging chunks, the
last one ragged."""
import numpy as np
import pytest

from rbtp import Solver, STORE_F16S, STORE_F32, STORE_F64, workloads as W

pytestmark = pytest.mark.gpu


def _state(s):
    f, g = s.fg()
    m = s.macros()
    return f, g, m


@pytest.mark.parametrize("storage", [STORE_F64, STORE_F32, STORE_F16S])
def test_import_routes_agree_bit_for_bit(lib_built, storage):
    torch = pytest.importorskip("torch")
    cfg = W.config("plain_fp64", lx=128, ly=128, lz=136, storage=storage)
    assert 2 * (1 << 20) < cfg.nodes < 3 * (1 << 20)
    f, g, f7 = W.initial_state(cfg, seed=3, amp=1e-2)
    rng = np.random.default_rng(5)
    f = 1e-3 * rng.standard_normal(f.size)            # nonzero f: moments are not trivial
    f7[:4 * cfg.nodes] = 1e-3 * rng.standard_normal(4 * cfg.nodes)
    f7[5 * cfg.nodes:] = rng.random(2 * cfg.nodes)
    pinned = [torch.from_numpy(a).pin_memory() for a in (f, g, f7)]
    dev = [torch.from_numpy(a).cuda() for a in (f, g, f7)]
    for with_flow in (True, False):
        ref = Solver(cfg)
        ref.load_state(f, g, f7 if with_flow else None)            # pageable: staged copies
        want = _state(ref)
        for route in ("pinned", "device"):
            s = Solver(cfg)
            src = pinned if route == "pinned" else dev
            if route == "pinned":
                s.load_state(src[0].numpy(), src[1].numpy(), src[2].numpy() if with_flow else None)
            else:
                s.load_state_ptr(src[0].data_ptr(), src[1].data_ptr(), src[2].data_ptr() if with_flow else None)
            got = _state(s)
            assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), (route, with_flow)
            for k in want[2]:
                assert np.array_equal(got[2][k], want[2][k]), (route, with_flow, k)
            if with_flow:
                ts, ks = s.dissipation()
                assert np.array_equal(ts, f7[5 * cfg.nodes:6 * cfg.nodes])
            s.step(3, macros_last=True)
            ref_after = Solver(cfg)
            ref_after.load_state(f, g, f7 if with_flow else None)
            ref_after.step(3, macros_last=True)
            a, b = s.fg(), ref_after.fg()
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
            s.close()
            ref_after.close()
        ref.close()
    if storage == STORE_F64:
        # FP64 storage holds the imported populations exactly
        assert np.array_equal(want[0], f) and np.array_equal(want[1], g)
