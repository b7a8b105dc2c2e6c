"""Reduced-precision storage against FP64 where the comparison is not blurred by chaos: steady
convection (32x32x16, Ra = 2e4, Pr = 0.71, one roll), time-averaged Nusselt numbers over the last
third of 24,000 steps.  Tolerance 1 % for FP32 and for shifted FP16 (the FP32 store agrees to
~2e-4, the FP16 store to a few 1e-3 at this size).  Shifted FP16 keeps g relative to the
conduction profile, which is what lets it resolve the onset of convection from a small
perturbation at all."""
import numpy as np
import pytest

from rbtp import Solver, STORE_F16S, STORE_F32, STORE_F64, workloads as W

pytestmark = pytest.mark.gpu


def _nu_series(storage, steps=24000, every=500):
    cfg = W.config("plain_fp64", lx=32, ly=32, lz=16, rayleigh=2e4, storage=storage)
    s = Solver(cfg)
    s.load_state(*W.initial_state(cfg, seed=1, amp=1e-2))
    rows = []
    for _ in range(steps // every):
        s.step(every, macros_last=True)
        rows.append(s.nu(s.istep))
    s.close()
    r = np.array(rows)
    return r[2 * len(r) // 3:, 2:5].mean(0)   # bulk, top, bottom


def test_steady_nusselt_of_reduced_storage_within_one_percent(lib_built):
    ref = _nu_series(STORE_F64)
    assert ref[0] > 1.5                        # convection developed (conduction gives 1)
    for storage in (STORE_F32, STORE_F16S):
        got = _nu_series(storage)
        assert np.all(np.abs(got / ref - 1.0) < 1e-2), (storage, got, ref)
