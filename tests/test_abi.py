"""The C-ABI library loads here (no GPU) and exports every entry point include/rbtp.h declares;
host-side logic that needs no device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import rbtp
from rbtp import workloads as W

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(REPO, "include", "rbtp.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set(re.findall(r"\b(rbtp_[a-z0-9_]+)\s*\(", src))
    names.discard("rbtp_config_fill_defaults")  # static inline helper, not exported
    return names


def test_library_exports_every_declared_symbol(lib_built):
    lib = C.CDLL(lib_built)
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, missing
    assert {n for n, _, _ in rbtp.SIGNATURES} == _declared()


def test_config_struct_matches_header(lib_built):
    lib = rbtp.load_library()
    c = rbtp.Config()
    lib.rbtp_config_default(C.byref(c))
    d = rbtp.Config.defaults()
    for name, _ in rbtp.Config._fields_:
        if name != "reserved":
            assert getattr(c, name) == getattr(d, name), name
    assert c.lx == 320 and c.lz == 160 and c.particle_rand_seed == 86143


def test_status_strings(lib_built):
    lib = rbtp.load_library()
    for code in rbtp.STATUS:
        assert lib.rbtp_status_string(code)
    assert b"sm_103a" in lib.rbtp_version()


def test_create_without_gpu_fails_loudly(lib_built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(rbtp.RbtpError) as e:
        rbtp.Solver(W.config("plain_fp64"))
    assert e.value.status in (-11, -1)


def test_splitmix_stream_is_stable():
    u = W.splitmix64_uniform(1, 4)
    # SplitMix64(seed=1) outputs, top 53 bits scaled to [0, 1)
    ref = np.array([0x910A2DEC89025CC1, 0xBEEB8DA1658EEC67, 0xF893A2EEFB32555E, 0x71C18690EE42C90B],
                   dtype=np.uint64)
    assert np.array_equal(u, (ref >> np.uint64(11)).astype(np.float64) / 2.0 ** 53)
    f, g, f7 = W.initial_state(W.config("plain_fp64", lx=8, ly=4, lz=4))
    assert np.all(f == 0) and abs(g.reshape(27, -1).sum(0) - f7[4 * 128:5 * 128]).max() < 1e-15


def test_workload_configs():
    p = W.config("particle_laden")
    d = rbtp.derive(p) if os.path.exists(rbtp.LIB_PATH) else None
    assert p.lx == 320 and p.rho_particle_ratio == 1.5
    if d is not None:
        assert d.npart == 1000 and d.particle_radius == 8.0


def test_footprint_covers_the_population_buffers(lib_built):
    """rbtp_footprint (the server's admission size) is host arithmetic: for every storage mode it
    covers the one in-place population array (27 L paired (f, g) slots, FP64 keeps separate f and
    g arrays) and not a second copy of it, orders the modes by their bytes, and grows with
    particles."""
    from rbtp import footprint
    L = 320 * 320 * 160
    pop = {0: 2 * 27 * L * 8, 1: 27 * L * 8, 2: 27 * L * 4}
    fp = {st: footprint(W.config("production", storage=st)) for st in (0, 1, 2)}
    for st in (0, 1, 2):
        assert pop[st] <= fp[st] < pop[st] + 16 * 8 * L     # plus at most 16 FP64 fields per node
        assert fp[st] < 2 * pop[st] or st == 2               # no second population buffer
    assert fp[0] > fp[1] > fp[2]
    assert footprint(W.config("particle_laden", storage=1)) > fp[1]
