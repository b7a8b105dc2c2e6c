"""rbtp — Python binding of librbtp, the GB300 (sm_103a) RB-ThermoParticles hot path.

The reference has no Python or FFI layer: its interface is the set of host entry points of
include/lbm.h and include/particle.h (initialize, macrovar/collision/streaming launches from
main.cu, build_links, bounce_back_*, compute_particle_*, apply_repulsive_forces, update_particles,
refill_nodes, diag_flow, output_nu, output_profile, output_flow, output_fg, output_particles) over
compile-time macros in parameters.h.  `Solver` exposes the same operations, by the same names, on
top of the C ABI declared in include/rbtp.h; `Config` mirrors every parameters.h macro.

All compute runs in librbtp.so.  There is no CPU fallback: if the library or a CUDA device is
missing, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "librbtp.so")

RBTP_OK = 0
STATUS = {
    0: "RBTP_OK", -1: "RBTP_ERR_CUDA", -2: "RBTP_ERR_CONFIG", -3: "RBTP_ERR_OOM",
    -4: "RBTP_ERR_NONFINITE", -5: "RBTP_ERR_TIMEOUT", -6: "RBTP_ERR_IO", -7: "RBTP_ERR_STATE",
    -8: "RBTP_ERR_CAPACITY", -9: "RBTP_ERR_ARG", -10: "RBTP_ERR_PLACEMENT", -11: "RBTP_ERR_NODEVICE",
}
STORE_F64, STORE_F32, STORE_F16S = 0, 1, 2
STEP_MACROS_LAST = 1
STEP_FLOW_LAST = 2
PARTICLE_COLS = 33

# Column names of the particle-state rows (pos/pos_%09d.txt after the pid).
PARTICLE_COLUMNS = (
    ["x", "y", "z", "vx", "vy", "vz", "fx", "fy", "fz", "fx_prev", "fy_prev", "fz_prev",
     "fx_prev2", "fy_prev2", "fz_prev2", "theta_x", "theta_y", "theta_z", "omega_x", "omega_y",
     "omega_z", "tx", "ty", "tz", "tx_prev", "ty_prev", "tz_prev", "tx_prev2", "ty_prev2",
     "tz_prev2", "temp", "heat", "heat_prev"])


class RbtpError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {message}")


class Config(C.Structure):
    """Runtime mirror of parameters.h (field names are the lower-cased macro names)."""

    _fields_ = [
        ("lx", C.c_int), ("ly", C.c_int), ("lz", C.c_int),
        ("continuous_steps", C.c_int),
        ("nend", C.c_int), ("ndiag", C.c_int), ("nflowout", C.c_int), ("nnuout", C.c_int),
        ("nout_p", C.c_int),
        ("rayleigh", C.c_double), ("prandtl", C.c_double),
        ("t_hot", C.c_double), ("t_cold", C.c_double), ("t_ref", C.c_double),
        ("beta", C.c_double), ("visc", C.c_double), ("rho0", C.c_double),
        ("activate_particles", C.c_int), ("particle_rand_seed", C.c_int),
        ("particle_fraction", C.c_double), ("particle_diam_frac", C.c_double),
        ("cp_particle_ratio", C.c_double), ("cp_fluid", C.c_double),
        ("rho_particle_ratio", C.c_double), ("repforce_scale", C.c_double),
        ("particle_init_temp", C.c_double),
        ("rep_min_gap", C.c_double), ("rep_min_gap_w", C.c_double),
        ("rep_stf0", C.c_double), ("rep_stf1", C.c_double),
        ("rep_stf0_w", C.c_double), ("rep_stf1_w", C.c_double),
        ("storage", C.c_int),
        ("reserved", C.c_int * 7),
    ]

    @classmethod
    def defaults(cls, **kw) -> "Config":
        """parameters.h:4-53 defaults, then overrides."""
        c = cls()
        c.lx, c.ly, c.lz = 320, 320, 160
        c.continuous_steps = 0
        c.nend, c.ndiag, c.nflowout, c.nnuout, c.nout_p = 1000000, 125, 25000, 125, 125
        c.rayleigh, c.prandtl = 1.0e7, 0.71
        c.t_hot, c.t_cold, c.t_ref = 1.0, 0.0, 0.5
        c.beta, c.visc, c.rho0 = 0.0000625, 0.01206, 1.0
        c.activate_particles, c.particle_rand_seed = 1, 86143
        c.particle_fraction, c.particle_diam_frac = 0.05, 1.0 / 20.0
        c.cp_particle_ratio, c.cp_fluid, c.rho_particle_ratio = 10.0, 1.0, 1.0
        c.repforce_scale, c.particle_init_temp = 2.0e-4, (0.0 + 1.0) / 2
        c.rep_min_gap, c.rep_min_gap_w = 2.0, 2.0
        c.rep_stf0, c.rep_stf1, c.rep_stf0_w, c.rep_stf1_w = 0.025, 0.002, 0.025, 0.002
        c.storage = STORE_F64
        for k, v in kw.items():
            if not hasattr(c, k):
                raise KeyError(f"unknown config field {k!r}")
            setattr(c, k, v)
        return c

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}

    @property
    def nodes(self) -> int:
        return self.lx * self.ly * self.lz


class Derived(C.Structure):
    _fields_ = [
        ("tau", C.c_double), ("tauc", C.c_double), ("grav0", C.c_double), ("u0", C.c_double),
        ("diff", C.c_double), ("particle_radius", C.c_double), ("particle_volume", C.c_double),
        ("particle_mass", C.c_double), ("particle_inertia", C.c_double),
        ("particle_heat_capacity", C.c_double), ("npart", C.c_int), ("reserved", C.c_int),
    ]


class NuRow(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("step", "volume_fraction", "nu_bulk", "nu_top", "nu_bottom", "nu_bulk_fluid",
                 "nu_bulk_part")]

    def as_tuple(self):
        return tuple(getattr(self, n) for n, _ in self._fields_)


class BatchStats(C.Structure):
    _fields_ = [("members", C.c_int), ("tiles", C.c_int), ("total_particles", C.c_int),
                ("tile_shape", C.c_int), ("grid", C.c_int), ("graph", C.c_int), ("tuned", C.c_int),
                ("reserved", C.c_int), ("last_step_ms", C.c_double), ("nodes", C.c_double)]


_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_H = C.c_void_p

# (name, restype, argtypes) of every C-ABI entry point in include/rbtp.h
SIGNATURES = [
    ("rbtp_config_default", None, [C.POINTER(Config)]),
    ("rbtp_derive", C.c_int, [C.POINTER(Config), C.POINTER(Derived)]),
    ("rbtp_status_string", C.c_char_p, [C.c_int]),
    ("rbtp_version", C.c_char_p, []),
    ("rbtp_create", C.c_int, [C.POINTER(Config), C.POINTER(_H)]),
    ("rbtp_destroy", C.c_int, [_H]),
    ("rbtp_last_error", C.c_char_p, [_H]),
    ("rbtp_init_fresh", C.c_int, [_H]),
    ("rbtp_load_state", C.c_int, [_H, _DP, _DP, _DP, _DP]),
    ("rbtp_load_restart", C.c_int, [_H, C.c_char_p, C.c_int]),
    ("rbtp_step", C.c_int, [_H, C.c_int]),
    ("rbtp_step_ex", C.c_int, [_H, C.c_int, C.c_uint]),
    ("rbtp_current_step", C.c_int, [_H, _IP]),
    ("rbtp_synchronize", C.c_int, [_H]),
    ("rbtp_get_stream", C.c_int, [_H, C.POINTER(C.c_void_p)]),
    ("rbtp_get_fg", C.c_int, [_H, _DP, _DP]),
    ("rbtp_get_macros", C.c_int, [_H, _DP, _DP, _DP, _DP, _DP, _DP]),
    ("rbtp_get_particles", C.c_int, [_H, _DP]),
    ("rbtp_npart", C.c_int, [_H, _IP]),
    ("rbtp_get_flags", C.c_int, [_H, _IP, _IP]),
    ("rbtp_get_links", C.c_int, [_H, _IP, _IP, _IP, _IP, _DP, C.c_int]),
    ("rbtp_get_new_fluid", C.c_int, [_H, _IP, _IP, _IP, C.c_int]),
    ("rbtp_get_contacts", C.c_int, [_H, _IP, _IP, _IP, C.c_int]),
    ("rbtp_nu", C.c_int, [_H, C.c_int, C.POINTER(NuRow)]),
    ("rbtp_means", C.c_int, [_H, _DP]),
    ("rbtp_profile", C.c_int, [_H, _DP]),
    ("rbtp_dissipation", C.c_int, [_H, _DP, _DP]),
    ("rbtp_output_dirname", C.c_int, [_H, C.c_char_p, C.c_size_t]),
    ("rbtp_write_statistics", C.c_int, [_H, C.c_char_p, C.c_int]),
    ("rbtp_write_nu", C.c_int, [_H, C.c_char_p, C.c_int]),
    ("rbtp_write_profile", C.c_int, [_H, C.c_char_p, C.c_int]),
    ("rbtp_write_flow", C.c_int, [_H, C.c_char_p, C.c_int]),
    ("rbtp_write_fg", C.c_int, [_H, C.c_char_p, C.c_int]),
    ("rbtp_write_particles", C.c_int, [_H, C.c_char_p, C.c_int]),
    ("rbtp_checkpoint_write", C.c_int, [_H, C.c_char_p]),
    ("rbtp_checkpoint_read", C.c_int, [_H, C.c_char_p]),
    ("rbtp_batch_create", C.c_int, [C.c_int, C.POINTER(_H)]),
    ("rbtp_batch_destroy", C.c_int, [_H]),
    ("rbtp_batch_add", C.c_int, [_H, _H]),
    ("rbtp_batch_remove", C.c_int, [_H, _H]),
    ("rbtp_batch_set_sampling", C.c_int, [_H, _H, C.c_int]),
    ("rbtp_batch_step", C.c_int, [_H, C.c_int]),
    ("rbtp_batch_set_stop", C.c_int, [_H, _H, C.c_int]),
    ("rbtp_batch_samples", C.c_int, [_H, _H, C.POINTER(NuRow), C.c_int, C.POINTER(C.c_int)]),
    ("rbtp_batch_launch", C.c_int, [_H, C.c_int]),
    ("rbtp_batch_wait", C.c_int, [_H]),
    ("rbtp_batch_stats_get", C.c_int, [_H, C.POINTER(BatchStats)]),
    ("rbtp_batch_set_launch", C.c_int, [_H, C.c_int, C.c_int]),
    ("rbtp_footprint", C.c_int, [C.POINTER(Config), C.POINTER(C.c_size_t)]),
    ("rbtp_server_create", C.c_int, [C.c_int, C.c_double, C.c_int, C.POINTER(_H)]),
    ("rbtp_server_destroy", C.c_int, [_H]),
    ("rbtp_server_submit", C.c_int, [_H, C.POINTER(Config), C.c_int, C.c_int, _IP]),
    ("rbtp_server_tick", C.c_int, [_H, C.c_int, _IP, _IP]),
    ("rbtp_server_poll", C.c_int, [_H, C.c_int, _IP, _IP, C.POINTER(NuRow), C.c_int, _IP]),
    ("rbtp_server_request_times", C.c_int, [_H, C.c_int, _DP, _DP, _DP]),
    ("rbtp_server_stats", C.c_int, [_H, _DP, _DP, _DP, _DP]),
    ("rbtp_server_checkpoint", C.c_int, [_H, C.c_char_p]),
    ("rbtp_server_restore", C.c_int, [_H, C.c_char_p]),
    ("rbtp_fp64_fma_rate", C.c_int, [C.POINTER(C.c_double)]),
    ("rbtp_plane_sums_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                          C.c_double, C.c_void_p, C.c_void_p]),
]

_lib: Optional[C.CDLL] = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load librbtp.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise RbtpError(-1, f"{path} is missing; build it with rb-thermoparticles_gb300/rbtp_build.py")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = lib
    return lib


def derive(cfg: Config) -> Derived:
    d = Derived()
    _check(load_library().rbtp_derive(C.byref(cfg), C.byref(d)))
    return d


def _check(status: int, handle=None) -> None:
    if status != RBTP_OK:
        msg = ""
        if handle:
            raw = load_library().rbtp_last_error(handle)
            msg = raw.decode() if raw else ""
        raise RbtpError(status, msg)


def _dp(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_DP)


def _ip(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_IP)


class Solver:
    """One cavity on the GPU.  Method names follow the reference's host entry points."""

    def __init__(self, cfg: Config):
        self.lib = load_library()
        self.cfg = cfg
        self._h = C.c_void_p()
        _check(self.lib.rbtp_create(C.byref(cfg), C.byref(self._h)))
        n = C.c_int()
        _check(self.lib.rbtp_npart(self._h, C.byref(n)), self._h)
        self.npart = n.value
        self.L = cfg.lx * cfg.ly * cfg.lz

    # -- lifetime -----------------------------------------------------------------------------
    def close(self) -> None:
        if self._h:
            self.lib.rbtp_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- initialize() (initial.cu:240-333) ----------------------------------------------------
    def initialize(self) -> None:
        _check(self.lib.rbtp_init_fresh(self._h), self._h)

    def load_state(self, f: np.ndarray, g: np.ndarray, flow7: Optional[np.ndarray] = None,
                   particles: Optional[np.ndarray] = None) -> None:
        f = np.ascontiguousarray(f, dtype=np.float64)
        g = np.ascontiguousarray(g, dtype=np.float64)
        if flow7 is not None:
            flow7 = np.ascontiguousarray(flow7, dtype=np.float64)
        if particles is not None:
            particles = np.ascontiguousarray(particles, dtype=np.float64)
        _check(self.lib.rbtp_load_state(self._h, _dp(f), _dp(g), _dp(flow7), _dp(particles)), self._h)

    def load_state_ptr(self, f_addr: int, g_addr: int, flow7_addr: Optional[int] = None,
                       particles: Optional[np.ndarray] = None) -> None:
        """rbtp_load_state from raw addresses (device memory, page-locked or pageable host memory of
        27 L, 27 L and 7 L doubles), e.g. the data_ptr() of tensors."""
        if particles is not None:
            particles = np.ascontiguousarray(particles, dtype=np.float64)
        cast = lambda a: None if a is None else C.cast(C.c_void_p(a), _DP)  # noqa: E731
        _check(self.lib.rbtp_load_state(self._h, cast(f_addr), cast(g_addr), cast(flow7_addr), _dp(particles)),
               self._h)

    def load_restart(self, directory: str, step: int) -> None:
        _check(self.lib.rbtp_load_restart(self._h, directory.encode(), step), self._h)

    # -- the time loop (main.cu:32-85) --------------------------------------------------------
    def step(self, nsteps: int = 1, macros_last: bool = False, flow_last: bool = False) -> None:
        """Advance nsteps; macros_last materialises the macroscopic fields on the last step,
        flow_last also the dissipation fields of a flow-output step."""
        flags = (STEP_MACROS_LAST if macros_last else 0) | (STEP_FLOW_LAST if flow_last else 0)
        _check(self.lib.rbtp_step_ex(self._h, nsteps, flags), self._h)

    @property
    def istep(self) -> int:
        v = C.c_int()
        _check(self.lib.rbtp_current_step(self._h, C.byref(v)), self._h)
        return v.value

    def synchronize(self) -> None:
        _check(self.lib.rbtp_synchronize(self._h), self._h)

    # -- state export -------------------------------------------------------------------------
    def fg(self):
        f = np.empty(27 * self.L)
        g = np.empty(27 * self.L)
        _check(self.lib.rbtp_get_fg(self._h, _dp(f), _dp(g)), self._h)
        return f, g

    def macros(self):
        out = [np.empty(self.L) for _ in range(6)]
        _check(self.lib.rbtp_get_macros(self._h, *[_dp(a) for a in out]), self._h)
        return dict(zip(["rho", "ux", "uy", "uz", "phi", "force_x"], out))

    def particles(self) -> np.ndarray:
        out = np.empty((self.npart, PARTICLE_COLS))
        if self.npart:
            _check(self.lib.rbtp_get_particles(self._h, _dp(out)), self._h)
        return out

    def flags(self) -> np.ndarray:
        o = np.empty(self.L, dtype=np.int32)
        _check(self.lib.rbtp_get_flags(self._h, _ip(o), None), self._h)
        return o

    def links(self):
        n = C.c_int()
        _check(self.lib.rbtp_get_links(self._h, C.byref(n), None, None, None, None, 0), self._h)
        k = n.value
        node, d, pid = (np.empty(k, dtype=np.int32) for _ in range(3))
        q = np.empty(k)
        _check(self.lib.rbtp_get_links(self._h, C.byref(n), _ip(node), _ip(d), _ip(pid), _dp(q), k), self._h)
        k = n.value
        return node[:k], d[:k], pid[:k], q[:k]

    def new_fluid(self):
        n = C.c_int()
        _check(self.lib.rbtp_get_new_fluid(self._h, C.byref(n), None, None, 0), self._h)
        node, pid = np.empty(n.value, dtype=np.int32), np.empty(n.value, dtype=np.int32)
        _check(self.lib.rbtp_get_new_fluid(self._h, C.byref(n), _ip(node), _ip(pid), len(node)), self._h)
        return node, pid

    def contacts(self):
        n = C.c_int()
        _check(self.lib.rbtp_get_contacts(self._h, C.byref(n), None, None, 0), self._h)
        p, q = np.empty(n.value, dtype=np.int32), np.empty(n.value, dtype=np.int32)
        _check(self.lib.rbtp_get_contacts(self._h, C.byref(n), _ip(p), _ip(q), len(p)), self._h)
        return p, q

    # -- diagnostics (output_statis.cu) -------------------------------------------------------
    def nu(self, istep: int = 0) -> tuple:
        r = NuRow()
        _check(self.lib.rbtp_nu(self._h, istep, C.byref(r)), self._h)
        return r.as_tuple()

    def means(self) -> np.ndarray:
        m = np.empty(4)
        _check(self.lib.rbtp_means(self._h, _dp(m)), self._h)
        return m

    def profile(self) -> np.ndarray:
        p = np.empty(4 * self.cfg.lx)
        _check(self.lib.rbtp_profile(self._h, _dp(p)), self._h)
        return p.reshape(self.cfg.lx, 4)

    def dissipation(self):
        ted, ked = np.empty(self.L), np.empty(self.L)
        _check(self.lib.rbtp_dissipation(self._h, _dp(ted), _dp(ked)), self._h)
        return ted, ked

    # -- reference writers (output/*.cu) -------------------------------------------------------
    def output_dir(self) -> str:
        buf = C.create_string_buffer(256)
        _check(self.lib.rbtp_output_dirname(self._h, buf, 256), self._h)
        return buf.value.decode()

    def diag_flow(self, istep: int, directory: Optional[str] = None) -> None:
        _check(self.lib.rbtp_write_statistics(self._h, _b(directory), istep), self._h)

    def output_nu(self, istep: int, directory: Optional[str] = None) -> None:
        _check(self.lib.rbtp_write_nu(self._h, _b(directory), istep), self._h)

    def output_profile(self, istep: int, directory: Optional[str] = None) -> None:
        _check(self.lib.rbtp_write_profile(self._h, _b(directory), istep), self._h)

    def output_flow(self, istep: int, directory: Optional[str] = None) -> None:
        _check(self.lib.rbtp_write_flow(self._h, _b(directory), istep), self._h)

    def output_fg(self, istep: int, directory: Optional[str] = None) -> None:
        _check(self.lib.rbtp_write_fg(self._h, _b(directory), istep), self._h)

    def output_particles(self, istep: int, directory: Optional[str] = None) -> None:
        _check(self.lib.rbtp_write_particles(self._h, _b(directory), istep), self._h)

    def checkpoint_write(self, path: str) -> None:
        """Exact checkpoint of the whole step state (resumes bit for bit)."""
        _check(self.lib.rbtp_checkpoint_write(self._h, _b(path)), self._h)

    def checkpoint_read(self, path: str) -> None:
        _check(self.lib.rbtp_checkpoint_read(self._h, _b(path)), self._h)


class Batch:
    """Many cavities advanced in lockstep by one persistent launch per step (rbtp_batch_*)."""

    def __init__(self, storage: int = STORE_F32):
        self.lib = load_library()
        self._b = C.c_void_p()
        _check(self.lib.rbtp_batch_create(storage, C.byref(self._b)))
        self.members = []

    def add(self, solver: "Solver", sample_every: int = 0) -> None:
        st = self.lib.rbtp_batch_add(self._b, solver.handle)
        if st:
            raise RbtpError(st, "rbtp_batch_add")
        self.members.append(solver)
        if sample_every:
            _check(self.lib.rbtp_batch_set_sampling(self._b, solver.handle, sample_every))

    def remove(self, solver: "Solver") -> None:
        _check(self.lib.rbtp_batch_remove(self._b, solver.handle))
        self.members.remove(solver)

    def step(self, nsteps: int = 1) -> None:
        st = self.lib.rbtp_batch_step(self._b, nsteps)
        if st:
            raise RbtpError(st, "rbtp_batch_step")

    def launch(self, nsteps: int = 1) -> None:
        """Enqueue nsteps batch steps and return while they run (wait() ends them)."""
        st = self.lib.rbtp_batch_launch(self._b, nsteps)
        if st:
            raise RbtpError(st, "rbtp_batch_launch")

    def wait(self) -> None:
        st = self.lib.rbtp_batch_wait(self._b)
        if st:
            raise RbtpError(st, "rbtp_batch_wait")

    def set_sampling(self, solver: "Solver", every: int) -> None:
        """On-device Nu sampling every `every` steps (0: only at the stop step) into a ring."""
        _check(self.lib.rbtp_batch_set_sampling(self._b, solver.handle, every))

    def set_stop(self, solver: "Solver", stop_step: int) -> None:
        """The member stops advancing at step stop_step while the others go on."""
        _check(self.lib.rbtp_batch_set_stop(self._b, solver.handle, stop_step))

    def samples(self, solver: "Solver") -> np.ndarray:
        """Nu rows (step, volume fraction, Nu bulk/top/bottom, bulk fluid/particle) of the samples
        taken since the last call."""
        out = []
        buf = (NuRow * 64)()
        while True:
            n = C.c_int(0)
            st = self.lib.rbtp_batch_samples(self._b, solver.handle, buf, 64, C.byref(n))
            out.extend(buf[k].as_tuple() for k in range(n.value))
            if st:
                raise RbtpError(st, "rbtp_batch_samples")
            if n.value < 64:
                break
        return np.array(out, dtype=np.float64).reshape(-1, 7)

    def set_launch(self, shape: int, grid: int = 0) -> None:
        _check(self.lib.rbtp_batch_set_launch(self._b, shape, grid))

    def stats(self) -> dict:
        st = BatchStats()
        _check(self.lib.rbtp_batch_stats_get(self._b, C.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_ if f != "reserved"}

    def close(self) -> None:
        if self._b:
            self.lib.rbtp_batch_destroy(self._b)
            self._b = C.c_void_p()
            self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fp64_fma_rate() -> float:
    """Measured FP64 FMA rate of the current device in flop/s (rbtp_fp64_fma_rate)."""
    v = C.c_double()
    _check(load_library().rbtp_fp64_fma_rate(C.byref(v)))
    return v.value


def footprint(cfg: Config) -> int:
    b = C.c_size_t()
    _check(load_library().rbtp_footprint(C.byref(cfg), C.byref(b)))
    return b.value


class Server:
    """Continuous-batching solve server (rbtp_server_*): submit cases, tick, stream Nu series."""

    QUEUED, ACTIVE, DONE, FAILED = 0, 1, 2, 3

    def __init__(self, storage: int = STORE_F32, hbm_budget: float = 180e9, max_active: int = 0):
        self.lib = load_library()
        self._s = C.c_void_p()
        _check(self.lib.rbtp_server_create(storage, float(hbm_budget), max_active, C.byref(self._s)))

    def submit(self, cfg: Config, horizon: int, sample_every: int) -> int:
        rid = C.c_int()
        _check(self.lib.rbtp_server_submit(self._s, C.byref(cfg), horizon, sample_every, C.byref(rid)))
        return rid.value

    def tick(self, max_steps: int = 100):
        a, q = C.c_int(), C.c_int()
        _check(self.lib.rbtp_server_tick(self._s, max_steps, C.byref(a), C.byref(q)))
        return a.value, q.value

    def poll(self, rid: int):
        st, done, n = C.c_int(), C.c_int(), C.c_int()
        self.lib.rbtp_server_poll(self._s, rid, C.byref(st), C.byref(done), None, 0, C.byref(n))
        rows = (NuRow * max(n.value, 1))()
        status = self.lib.rbtp_server_poll(self._s, rid, C.byref(st), C.byref(done), rows, n.value, C.byref(n))
        series = np.array([r.as_tuple() for r in rows[:n.value]]).reshape(-1, 7)
        return {"state": st.value, "steps_done": done.value, "status": status, "series": series}

    def times(self, rid: int):
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        _check(self.lib.rbtp_server_request_times(self._s, rid, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def stats(self) -> dict:
        v = [C.c_double() for _ in range(4)]
        _check(self.lib.rbtp_server_stats(self._s, *[C.byref(x) for x in v]))
        return dict(zip(["node_updates", "steps", "used_bytes", "clock"], [x.value for x in v]))

    def checkpoint(self, directory: str) -> None:
        """Between ticks: write every request's record and exact state under directory."""
        _check(self.lib.rbtp_server_checkpoint(self._s, _b(directory)))

    def restore(self, directory: str) -> None:
        """Into a fresh server: resume the checkpointed requests."""
        _check(self.lib.rbtp_server_restore(self._s, _b(directory)))

    def close(self) -> None:
        if self._s:
            self.lib.rbtp_server_destroy(self._s)
            self._s = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _b(s: Optional[str]):
    return s.encode() if s else None


__all__ = ["Config", "Derived", "NuRow", "Solver", "Batch", "BatchStats", "Server", "footprint", "RbtpError", "load_library", "derive",
           "STORE_F64", "STORE_F32", "STORE_F16S", "PARTICLE_COLS", "PARTICLE_COLUMNS",
           "SIGNATURES", "LIB_PATH", "fp64_fma_rate"]
