"""ctypes wrapper of the CPU oracle (oracle/rbtp_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, as the reference against which the library is compared.  The product library never imports
it.  The interface mirrors rbtp.Solver so
that parity tests read the same on both sides.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "rb-thermoparticles_gb300"))
from rbtp import Config, Derived, NuRow, PARTICLE_COLS  # noqa: E402

_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_lib = None


def build() -> str:
    import platform
    import shutil
    stamp = os.path.join(HERE, "_build", "ARCH")
    try:
        old = open(stamp).read().strip()
    except OSError:
        old = None
    if old != platform.machine():
        shutil.rmtree(os.path.join(HERE, "_build"), ignore_errors=True)
        os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
        with open(stamp, "w") as fh:
            fh.write(platform.machine() + "\n")
    res = subprocess.run(["make", "-C", HERE], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        H = C.c_void_p
        sig = {
            "orc_create": (C.c_int, [C.POINTER(Config), C.POINTER(H)]),
            "orc_destroy": (None, [H]),
            "orc_set_threads": (C.c_int, [C.c_int]),
            "orc_get_threads": (C.c_int, []),
            "orc_init_fresh": (C.c_int, [H]),
            "orc_load_state": (C.c_int, [H, _DP, _DP, _DP, _DP]),
            "orc_step": (C.c_int, [H, C.c_int]),
            "orc_npart": (C.c_int, [H]),
            "orc_derive": (C.c_int, [C.POINTER(Config), C.POINTER(Derived)]),
            "orc_get_fg": (C.c_int, [H, _DP, _DP]),
            "orc_get_macros": (C.c_int, [H, _DP, _DP, _DP, _DP, _DP, _DP]),
            "orc_get_particles": (C.c_int, [H, _DP]),
            "orc_get_flags": (C.c_int, [H, _IP, _IP]),
            "orc_get_links": (C.c_int, [H, _IP, _IP, _IP, _IP, _DP, C.c_int]),
            "orc_get_new_fluid": (C.c_int, [H, _IP, _IP, _IP, C.c_int]),
            "orc_get_contacts": (C.c_int, [H, _IP, _IP, _IP, C.c_int]),
            "orc_nu": (C.c_int, [H, C.c_int, C.POINTER(NuRow)]),
            "orc_means": (C.c_int, [H, _DP]),
            "orc_profile": (C.c_int, [H, _DP]),
            "orc_dissipation": (C.c_int, [H, _DP, _DP]),
            "orc_link_q": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_double, _DP]),
            "orc_set_positions_and_build": (C.c_int, [H, _DP]),
            "orc_output_dirname": (C.c_int, [C.c_double, C.c_double, C.c_char_p, C.c_size_t]),
            "orc_write_statistics": (C.c_int, [C.c_char_p, C.c_int, _DP]),
            "orc_write_nu": (C.c_int, [C.c_char_p, C.c_double, C.POINTER(NuRow)]),
            "orc_write_profile": (C.c_int, [C.c_char_p, C.c_double, C.c_int, C.c_int, _DP]),
            "orc_write_flow": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _DP,
                                         _IP, _DP, C.c_int]),
            "orc_write_fg": (C.c_int, [C.c_char_p, C.c_int, C.c_long, _DP, _DP]),
            "orc_write_particles": (C.c_int, [C.c_char_p, C.c_int, C.c_int, _DP]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def _ck(st: int, what: str = "") -> None:
    if st != 0:
        raise RuntimeError(f"oracle call {what} failed with status {st}")


def _dp(a):
    return None if a is None else a.ctypes.data_as(_DP)


def _ip(a):
    return None if a is None else a.ctypes.data_as(_IP)


def set_threads(n: int) -> int:
    return lib().orc_set_threads(n)


def derive(cfg: Config) -> Derived:
    d = Derived()
    _ck(lib().orc_derive(C.byref(cfg), C.byref(d)), "derive")
    return d


def link_q(ip, x0, y0, z0, px, py, pz, rsq):
    q = C.c_double()
    ok = lib().orc_link_q(ip, x0, y0, z0, px, py, pz, rsq, C.byref(q))
    return bool(ok), q.value


class Oracle:
    def __init__(self, cfg: Config):
        self.cfg = cfg
        self.lib = lib()
        self._h = C.c_void_p()
        _ck(self.lib.orc_create(C.byref(cfg), C.byref(self._h)), "create")
        self.npart = self.lib.orc_npart(self._h)
        self.L = cfg.lx * cfg.ly * cfg.lz

    def close(self):
        if self._h:
            self.lib.orc_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def initialize(self):
        _ck(self.lib.orc_init_fresh(self._h), "init_fresh")

    def load_state(self, f, g, flow7=None, particles=None):
        f = np.ascontiguousarray(f, dtype=np.float64)
        g = np.ascontiguousarray(g, dtype=np.float64)
        flow7 = None if flow7 is None else np.ascontiguousarray(flow7, dtype=np.float64)
        particles = None if particles is None else np.ascontiguousarray(particles, dtype=np.float64)
        _ck(self.lib.orc_load_state(self._h, _dp(f), _dp(g), _dp(flow7), _dp(particles)), "load_state")

    def step(self, n=1):
        _ck(self.lib.orc_step(self._h, n), "step")

    def fg(self):
        f, g = np.empty(27 * self.L), np.empty(27 * self.L)
        _ck(self.lib.orc_get_fg(self._h, _dp(f), _dp(g)), "fg")
        return f, g

    def macros(self):
        out = [np.empty(self.L) for _ in range(6)]
        _ck(self.lib.orc_get_macros(self._h, *[_dp(a) for a in out]), "macros")
        return dict(zip(["rho", "ux", "uy", "uz", "phi", "force_x"], out))

    def particles(self):
        out = np.empty((self.npart, PARTICLE_COLS))
        if self.npart:
            _ck(self.lib.orc_get_particles(self._h, _dp(out)), "particles")
        return out

    def flags(self):
        o = np.empty(self.L, dtype=np.int32)
        _ck(self.lib.orc_get_flags(self._h, _ip(o), None), "flags")
        return o

    def flags_prev(self):
        o = np.empty(self.L, dtype=np.int32)
        _ck(self.lib.orc_get_flags(self._h, None, _ip(o)), "flags")
        return o

    def links(self):
        n = C.c_int()
        _ck(self.lib.orc_get_links(self._h, C.byref(n), None, None, None, None, 0), "links")
        k = n.value
        node, d, pid = (np.empty(k, dtype=np.int32) for _ in range(3))
        q = np.empty(k)
        _ck(self.lib.orc_get_links(self._h, C.byref(n), _ip(node), _ip(d), _ip(pid), _dp(q), k), "links")
        return node, d, pid, q

    def new_fluid(self):
        n = C.c_int()
        _ck(self.lib.orc_get_new_fluid(self._h, C.byref(n), None, None, 0), "new_fluid")
        node, pid = np.empty(n.value, dtype=np.int32), np.empty(n.value, dtype=np.int32)
        _ck(self.lib.orc_get_new_fluid(self._h, C.byref(n), _ip(node), _ip(pid), n.value), "new_fluid")
        return node, pid

    def contacts(self):
        n = C.c_int()
        _ck(self.lib.orc_get_contacts(self._h, C.byref(n), None, None, 0), "contacts")
        p, q = np.empty(n.value, dtype=np.int32), np.empty(n.value, dtype=np.int32)
        _ck(self.lib.orc_get_contacts(self._h, C.byref(n), _ip(p), _ip(q), n.value), "contacts")
        return p, q

    def nu(self, istep=0):
        r = NuRow()
        _ck(self.lib.orc_nu(self._h, istep, C.byref(r)), "nu")
        return r.as_tuple()

    def means(self):
        m = np.empty(4)
        _ck(self.lib.orc_means(self._h, _dp(m)), "means")
        return m

    def profile(self):
        p = np.empty(4 * self.cfg.lx)
        _ck(self.lib.orc_profile(self._h, _dp(p)), "profile")
        return p.reshape(self.cfg.lx, 4)

    def dissipation(self):
        ted, ked = np.empty(self.L), np.empty(self.L)
        _ck(self.lib.orc_dissipation(self._h, _dp(ted), _dp(ked)), "dissipation")
        return ted, ked

    def set_positions_and_build(self, pos_xyz):
        pos = np.ascontiguousarray(pos_xyz, dtype=np.float64).reshape(-1)
        _ck(self.lib.orc_set_positions_and_build(self._h, _dp(pos)), "set_positions")


# ---- the reference's output writers (oracle/rbtp_oracle_io.c), fed with the values to write ----
def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def output_dirname(rayleigh: float, prandtl: float) -> str:
    buf = C.create_string_buffer(256)
    _ck(lib().orc_output_dirname(rayleigh, prandtl, buf, 256), "output_dirname")
    return buf.value.decode()


def write_statistics(directory: str, istep: int, means) -> None:
    m = _f64(means)
    _ck(lib().orc_write_statistics(directory.encode(), istep, _dp(m)), "write_statistics")


def write_nu(directory: str, rayleigh: float, row) -> None:
    r = NuRow(*[float(v) for v in row])
    _ck(lib().orc_write_nu(directory.encode(), rayleigh, C.byref(r)), "write_nu")


def write_profile(directory: str, rayleigh: float, istep: int, profile) -> None:
    p = _f64(profile).reshape(-1)
    _ck(lib().orc_write_profile(directory.encode(), rayleigh, istep, len(p) // 4, _dp(p)), "write_profile")


def write_flow(directory: str, istep: int, cfg: Config, fields7, owner=None, rows=None) -> None:
    f7 = _f64(fields7).reshape(-1)
    own = None if owner is None else np.ascontiguousarray(owner, dtype=np.int32)
    r = None if rows is None else _f64(rows)
    np_ = 0 if r is None else len(r)
    _ck(lib().orc_write_flow(directory.encode(), istep, cfg.lx, cfg.ly, cfg.lz, cfg.rho0, _dp(f7), _ip(own),
                             _dp(r), np_), "write_flow")


def write_fg(directory: str, istep: int, f, g) -> None:
    f, g = _f64(f), _f64(g)
    _ck(lib().orc_write_fg(directory.encode(), istep, len(f) // 27, _dp(f), _dp(g)), "write_fg")


def write_particles(directory: str, istep: int, rows) -> None:
    r = _f64(rows)
    _ck(lib().orc_write_particles(directory.encode(), istep, len(r), _dp(r)), "write_particles")
