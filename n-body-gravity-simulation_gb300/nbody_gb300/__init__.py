"""nbody_gb300 -- Python front end of the GB300 N-body engine.

A thin ctypes layer over the C ABI in ``include/nbody_c.h`` (the library
``libnbody_gb300.so`` next to this file).  The numerics all live in the CUDA
kernels; this module only moves numpy arrays across the boundary.  It raises
``NBodyError`` on every non-OK status and refuses to run when the library has
not been built (there is no CPU fallback).

    from nbody_gb300 import Sim, Config, DIRECT_MIXED, VELOCITY_VERLET
    sim = Sim(Config(method=DIRECT_MIXED, G=1.0, softening=1e-3), capacity=n)
    sim.load(x, y, z, vx, vy, vz, m)
    sim.step(VELOCITY_VERLET, dt=5e-4, nsteps=10)
    state = sim.read_state()
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# NBODY_GB300_LIB selects another build of the library (the device-checked one)
LIB_PATH = os.environ.get("NBODY_GB300_LIB") or os.path.join(HERE, "libnbody_gb300.so")
COMPAT_LIB_PATH = os.path.join(HERE, "libnbody_compat.so")

# nb_method
DIRECT_FP64, DIRECT_MIXED, BARNES_HUT = 0, 1, 2
# nb_integrator
EULER, EULER_CROMER, LEAPFROG, VELOCITY_VERLET, RK4 = 0, 1, 2, 3, 4

STATUS = {0: "NB_OK", 1: "NB_ERR_INVALID_ARGUMENT", 2: "NB_ERR_CUDA", 3: "NB_ERR_OUT_OF_MEMORY",
          4: "NB_ERR_CAPACITY", 5: "NB_ERR_NOT_LOADED", 6: "NB_ERR_DEVICE_FAULT",
          7: "NB_ERR_UNSUPPORTED", 8: "NB_ERR_IO", 9: "NB_ERR_CANCELLED"}

# Every function declared in include/nbody_c.h (checked by the tests).
EXPORTS = [
    "nb_config_default", "nb_create", "nb_destroy", "nb_set_config", "nb_get_config",
    "nb_load", "nb_load_device", "nb_bind_device", "nb_read_state", "nb_device_arrays",
    "nb_num_bodies",
    "nb_compute_forces", "nb_step", "nb_invalidate_forces", "nb_synchronize",
    "nb_diagnostics", "nb_bh_build", "nb_bh_get_info", "nb_bh_read_order", "nb_bh_read_nodes",
    "nb_gen_plummer", "nb_gen_disk_bulge", "nb_status_string", "nb_last_error", "nb_version",
    "nb_profile_enable", "nb_profile_read", "nb_kernel_launch_count",
    "nb_direct_mixed_forces_noalloc",
    "nb_particles_read", "nb_particles_write", "nb_load_particles", "nb_csv_append",
    "nb_checkpoint_save", "nb_checkpoint_load",
    "nb_ensemble_create", "nb_ensemble_destroy", "nb_ensemble_load", "nb_ensemble_read_state",
    "nb_ensemble_compute_forces", "nb_ensemble_step", "nb_ensemble_tune",
    "nb_ensemble_synchronize", "nb_ensemble_info", "nb_ensemble_profile",
    "nb_server_config_default", "nb_server_create", "nb_server_destroy", "nb_server_submit",
    "nb_server_tick", "nb_server_result", "nb_server_release", "nb_server_get_stats",
    "nb_server_cancel", "nb_debug_fail_device_allocations", "nb_debug_device_checks",
    "nb_debug_fp32_rate",
]
_NON_STATUS = {"nb_status_string", "nb_last_error", "nb_version", "nb_kernel_launch_count"}


class NBodyError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS.get(status, status)}: {msg}")
        self.status = status


class _Config(C.Structure):
    _fields_ = [("method", C.c_int), ("G", C.c_double), ("softening", C.c_double),
                ("theta", C.c_double), ("leaf_capacity", C.c_int), ("flags", C.c_int)]


class _Diag(C.Structure):
    _fields_ = [("kinetic", C.c_double), ("potential", C.c_double),
                ("potential_softened", C.c_double), ("total", C.c_double),
                ("total_softened", C.c_double), ("angular_momentum", C.c_double * 3),
                ("center_of_mass", C.c_double * 3), ("momentum", C.c_double * 3),
                ("mass", C.c_double)]


class _BHInfo(C.Structure):
    _fields_ = [("num_nodes", C.c_int), ("num_leaves", C.c_int), ("max_depth", C.c_int),
                ("split_levels", C.c_int), ("root", C.c_double * 4),
                ("interactions_m2p", C.c_uint64), ("interactions_p2p", C.c_uint64),
                ("interactions_total", C.c_uint64)]


class _Profile(C.Structure):
    _fields_ = [("kernel_launches", C.c_uint64), ("force_launches", C.c_uint64),
                ("force_kernel_ms", C.c_double)]


class _EnsembleInfo(C.Structure):
    _fields_ = [("num_systems", C.c_int), ("total_bodies", C.c_int64),
                ("interactions_per_eval", C.c_double), ("work_items", C.c_int),
                ("ipt_by_bucket", C.c_int * 32), ("graph_launches", C.c_uint64),
                ("graph_steps", C.c_int), ("force_launches", C.c_uint64),
                ("force_kernel_ms", C.c_double)]


class _ServerConfig(C.Structure):
    _fields_ = [("G", C.c_double), ("softening", C.c_double), ("theta", C.c_double),
                ("leaf_capacity", C.c_int), ("direct_max_n", C.c_int), ("dt", C.c_double),
                ("hbm_budget_bytes", C.c_size_t), ("pool_bodies", C.c_size_t)]


class _ServerStats(C.Structure):
    _fields_ = [("jobs_submitted", C.c_uint64), ("jobs_finished", C.c_uint64),
                ("jobs_running", C.c_int), ("jobs_queued", C.c_int),
                ("steps_done", C.c_uint64), ("ticks", C.c_uint64),
                ("interactions", C.c_double), ("busy_ms", C.c_double),
                ("step_ms_p50", C.c_double), ("step_ms_p99", C.c_double),
                ("queue_ms_p50", C.c_double), ("queue_ms_p99", C.c_double),
                ("max_running", C.c_int), ("peak_device_bytes", C.c_size_t),
                ("host_admit_ms", C.c_double), ("host_issue_ms", C.c_double),
                ("host_wait_ms", C.c_double), ("host_retire_ms", C.c_double),
                ("host_upload_ms", C.c_double), ("host_direct_ms", C.c_double),
                ("host_join_ms", C.c_double),
                ("jobs_failed", C.c_uint64), ("jobs_cancelled", C.c_uint64)]


def kernel_launch_count() -> int:
    """This library's kernel launches in the process so far."""
    return int(lib().nb_kernel_launch_count())


BH_QUADRUPOLE = 2  # NB_FLAG_BH_QUADRUPOLE
BH_REFERENCE_OPENING = 16  # NB_FLAG_BH_REFERENCE_OPENING: the reference's opening rule
MIXED_SORTED = 4  # NB_FLAG_MIXED_SORTED: force the Hilbert-sorted near/far kernel
MIXED_UNSORTED = 8  # NB_FLAG_MIXED_UNSORTED: force the all-pairs double-single kernel


def bh_reuse_flag(k: int) -> int:
    """NB_FLAG_BH_REUSE(k): rebuild the Barnes-Hut tree every k evaluations."""
    return (int(k) & 0xFF) << 8


@dataclass
class Config:
    method: int = DIRECT_MIXED
    G: float = 1.0
    softening: float = 0.0
    theta: float = 0.5
    leaf_capacity: int = 8
    flags: int = 0

    def _c(self) -> _Config:
        return _Config(self.method, self.G, self.softening, self.theta, self.leaf_capacity,
                       self.flags)


_lib = None


def library_path() -> str:
    return LIB_PATH


def lib():
    """Loads libnbody_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with "
            "`python n-body-gravity-simulation_gb300/build.py` (no CPU fallback exists)")
    L = C.CDLL(LIB_PATH)
    vp, dp, sz = C.c_void_p, C.POINTER(C.c_double), C.c_size_t
    L.nb_config_default.argtypes = [C.POINTER(_Config)]
    L.nb_create.argtypes = [C.POINTER(_Config), sz, vp, C.POINTER(vp)]
    L.nb_destroy.argtypes = [vp]
    L.nb_set_config.argtypes = [vp, C.POINTER(_Config)]
    L.nb_get_config.argtypes = [vp, C.POINTER(_Config)]
    L.nb_load.argtypes = [vp, sz] + [vp] * 7
    L.nb_load_device.argtypes = [vp, sz] + [vp] * 7
    L.nb_bind_device.argtypes = [vp, sz, vp]
    L.nb_read_state.argtypes = [vp] + [vp] * 10
    L.nb_device_arrays.argtypes = [vp, C.POINTER(vp)]
    L.nb_num_bodies.argtypes = [vp, C.POINTER(sz)]
    L.nb_compute_forces.argtypes = [vp]
    L.nb_step.argtypes = [vp, C.c_int, C.c_double, C.c_int]
    L.nb_invalidate_forces.argtypes = [vp]
    L.nb_synchronize.argtypes = [vp]
    L.nb_diagnostics.argtypes = [vp, C.POINTER(_Diag)]
    L.nb_bh_build.argtypes = [vp, C.POINTER(_BHInfo)]
    L.nb_bh_get_info.argtypes = [vp, C.POINTER(_BHInfo)]
    L.nb_bh_read_order.argtypes = [vp, vp, vp]
    L.nb_bh_read_nodes.argtypes = [vp, C.c_int] + [vp] * 7
    L.nb_gen_plummer.argtypes = [sz, C.c_uint64, C.c_double, C.c_double, C.c_double] + [vp] * 7
    L.nb_gen_disk_bulge.argtypes = ([sz, C.c_uint64] + [C.c_double] * 7 + [vp] * 7)
    L.nb_status_string.argtypes = [C.c_int]
    L.nb_status_string.restype = C.c_char_p
    L.nb_last_error.restype = C.c_char_p
    L.nb_version.restype = C.c_char_p
    L.nb_profile_enable.argtypes = [vp, C.c_int]
    L.nb_profile_read.argtypes = [vp, C.POINTER(_Profile), C.c_int]
    L.nb_kernel_launch_count.restype = C.c_uint64
    L.nb_direct_mixed_forces_noalloc.argtypes = ([sz] + [vp] * 4 + [C.c_double] * 2 +
                                                 [vp] * 3 + [vp])
    L.nb_particles_read.argtypes = [C.c_char_p, sz, C.POINTER(sz)] + [vp] * 7
    L.nb_particles_write.argtypes = [C.c_char_p, sz] + [vp] * 7
    L.nb_load_particles.argtypes = [vp, C.c_char_p]
    L.nb_csv_append.argtypes = [vp, C.c_char_p, C.c_int, vp, vp, C.c_int, C.c_int]
    L.nb_checkpoint_save.argtypes = [vp, C.c_char_p]
    L.nb_checkpoint_load.argtypes = [vp, C.c_char_p]
    L.nb_ensemble_create.argtypes = [C.POINTER(_Config), C.c_int, vp, vp, C.POINTER(vp)]
    L.nb_ensemble_destroy.argtypes = [vp]
    L.nb_ensemble_load.argtypes = [vp] + [vp] * 7
    L.nb_ensemble_read_state.argtypes = [vp] + [vp] * 10
    L.nb_ensemble_compute_forces.argtypes = [vp]
    L.nb_ensemble_step.argtypes = [vp, C.c_int, C.c_double, C.c_int]
    L.nb_ensemble_tune.argtypes = [vp, vp]
    L.nb_ensemble_synchronize.argtypes = [vp]
    L.nb_ensemble_info.argtypes = [vp, C.POINTER(_EnsembleInfo)]
    L.nb_ensemble_profile.argtypes = [vp, C.c_int]
    L.nb_server_config_default.argtypes = [C.POINTER(_ServerConfig)]
    L.nb_server_create.argtypes = [C.POINTER(_ServerConfig), C.POINTER(vp)]
    L.nb_server_destroy.argtypes = [vp]
    L.nb_server_submit.argtypes = [vp, sz] + [vp] * 7 + [C.c_int, C.POINTER(C.c_int64)]
    L.nb_server_tick.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.nb_server_result.argtypes = [vp, C.c_int64] + [vp] * 10
    L.nb_server_release.argtypes = [vp, C.c_int64]
    L.nb_server_get_stats.argtypes = [vp, C.POINTER(_ServerStats)]
    L.nb_server_cancel.argtypes = [vp, C.c_int64]
    L.nb_debug_fail_device_allocations.argtypes = [C.c_int]
    L.nb_debug_device_checks.argtypes = [C.POINTER(C.c_int)]
    L.nb_debug_fp32_rate.argtypes = [dp]
    for name in EXPORTS:
        f = getattr(L, name)
        if name not in _NON_STATUS:
            f.restype = C.c_int
    _lib = L
    return L


def _check(status: int, where: str):
    if status != 0:
        msg = lib().nb_last_error().decode(errors="replace")
        raise NBodyError(status, where, msg)


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(C.c_void_p)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


# ------------------------------------------------------------------ generators
def plummer(n: int, seed: int = 0, total_mass: float = 1.0, scale: float = 1.0,
            G: float = 1.0):
    """Equal-mass Plummer sphere (Aarseth-Henon-Wielen); returns
    (x, y, z, vx, vy, vz, m) as float64 arrays."""
    out = [np.empty(n) for _ in range(7)]
    _check(lib().nb_gen_plummer(n, seed, total_mass, scale, G, *map(_ptr, out)),
           "nb_gen_plummer")
    return tuple(out)


def disk_bulge(n: int, seed: int = 0, total_mass: float = 1.0, bulge_frac: float = 0.2,
               bulge_scale: float = 0.2, disk_scale: float = 1.0, disk_height: float = 0.05,
               dispersion: float = 0.1, G: float = 1.0):
    out = [np.empty(n) for _ in range(7)]
    _check(lib().nb_gen_disk_bulge(n, seed, total_mass, bulge_frac, bulge_scale, disk_scale,
                                   disk_height, dispersion, G, *map(_ptr, out)),
           "nb_gen_disk_bulge")
    return tuple(out)


def read_particles(path: str):
    """The reference's particle file (N, then "m x y z vx vy vz" per body);
    returns (x, y, z, vx, vy, vz, m) as float64 arrays."""
    n = C.c_size_t()
    bp = os.fsencode(path)
    _check(lib().nb_particles_read(bp, 0, C.byref(n), *([None] * 7)), "nb_particles_read")
    cols = [np.empty(n.value) for _ in range(7)]  # m x y z vx vy vz
    _check(lib().nb_particles_read(bp, n.value, C.byref(n), *map(_ptr, cols)),
           "nb_particles_read")
    m, x, y, z, vx, vy, vz = cols
    return x, y, z, vx, vy, vz, m


def write_particles(path: str, x, y, z, vx, vy, vz, m):
    cols = [_f64(v) for v in (m, x, y, z, vx, vy, vz)]
    _check(lib().nb_particles_write(os.fsencode(path), len(cols[0]), *map(_ptr, cols)),
           "nb_particles_write")


# ------------------------------------------------------------------ simulation
class Sim:
    """One simulation on the current CUDA device (nb_sim)."""

    def __init__(self, config: Config | None = None, capacity: int = 1,
                 stream: int | None = None):
        self._h = C.c_void_p()
        cfg = (config or Config())._c()
        _check(lib().nb_create(C.byref(cfg), capacity, C.c_void_p(stream or 0),
                               C.byref(self._h)), "nb_create")
        self.capacity = capacity

    def close(self):
        if self._h:
            lib().nb_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def config(self) -> Config:
        c = _Config()
        _check(lib().nb_get_config(self._h, C.byref(c)), "nb_get_config")
        return Config(c.method, c.G, c.softening, c.theta, c.leaf_capacity, c.flags)

    @config.setter
    def config(self, cfg: Config):
        c = cfg._c()
        _check(lib().nb_set_config(self._h, C.byref(c)), "nb_set_config")

    @property
    def n(self) -> int:
        v = C.c_size_t()
        _check(lib().nb_num_bodies(self._h, C.byref(v)), "nb_num_bodies")
        return v.value

    def load(self, x, y, z, vx, vy, vz, m):
        arrs = [_f64(a) for a in (x, y, z, vx, vy, vz, m)]
        n = len(arrs[0])
        if any(len(a) != n for a in arrs):
            raise ValueError("arrays differ in length")
        self._keep = arrs  # pageable sources stay alive until the copies ran
        _check(lib().nb_load(self._h, n, *map(_ptr, arrs)), "nb_load")
        _check(lib().nb_synchronize(self._h), "nb_synchronize")
        self._keep = None

    def load_pointers(self, n: int, ptrs, device: bool = False):
        """Loads from raw addresses (host pinned or device) without copies on
        the Python side; the caller keeps the memory alive until synchronize()."""
        f = lib().nb_load_device if device else lib().nb_load
        _check(f(self._h, n, *[C.c_void_p(p) for p in ptrs]), "nb_load")

    def read_state(self):
        n = self.n
        out = [np.empty(n) for _ in range(10)]
        _check(lib().nb_read_state(self._h, *map(_ptr, out)), "nb_read_state")
        keys = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "m"]
        return dict(zip(keys, out))

    def read_pointers(self, ptrs10):
        """Copies the state into raw host addresses (None / 0 skips a field)."""
        _check(lib().nb_read_state(self._h, *[C.c_void_p(p) if p else None for p in ptrs10]),
               "nb_read_state")

    def accelerations(self):
        s = self.read_state()
        return s["ax"], s["ay"], s["az"]

    def device_arrays(self):
        arr = (C.c_void_p * 10)()
        _check(lib().nb_device_arrays(self._h, arr), "nb_device_arrays")
        return [arr[k] for k in range(10)]

    def compute_forces(self):
        _check(lib().nb_compute_forces(self._h), "nb_compute_forces")

    def step(self, integrator: int, dt: float, nsteps: int = 1):
        _check(lib().nb_step(self._h, integrator, dt, nsteps), "nb_step")

    def invalidate_forces(self):
        _check(lib().nb_invalidate_forces(self._h), "nb_invalidate_forces")

    def synchronize(self):
        _check(lib().nb_synchronize(self._h), "nb_synchronize")

    def diagnostics(self) -> dict:
        d = _Diag()
        _check(lib().nb_diagnostics(self._h, C.byref(d)), "nb_diagnostics")
        return dict(kinetic=d.kinetic, potential=d.potential,
                    potential_softened=d.potential_softened, total=d.total,
                    total_softened=d.total_softened,
                    angular_momentum=list(d.angular_momentum),
                    center_of_mass=list(d.center_of_mass), momentum=list(d.momentum),
                    mass=d.mass)

    def profile(self, enable: bool = True):
        _check(lib().nb_profile_enable(self._h, int(enable)), "nb_profile_enable")

    def profile_read(self, reset: bool = True) -> dict:
        p = _Profile()
        _check(lib().nb_profile_read(self._h, C.byref(p), int(reset)), "nb_profile_read")
        return dict(kernel_launches=p.kernel_launches, force_launches=p.force_launches,
                    force_kernel_ms=p.force_kernel_ms)

    # -------------------------------------------------------------- files
    def load_particles(self, path: str):
        _check(lib().nb_load_particles(self._h, os.fsencode(path)), "nb_load_particles")

    def csv_append(self, path: str, bodies, names=None, header: bool = False,
                   precision: int = 15):
        """One trajectory-CSV row (positions of `bodies`, energies, L, COM)."""
        idx = np.ascontiguousarray(bodies, dtype=np.int32)
        arr = None
        if names is not None:
            enc = [os.fsencode(str(v)) for v in names]
            arr = (C.c_char_p * len(enc))(*enc)
        _check(lib().nb_csv_append(self._h, os.fsencode(path), len(idx), _ptr(idx),
                                   C.cast(arr, C.c_void_p) if arr is not None else None,
                                   int(header), precision), "nb_csv_append")

    def checkpoint_save(self, path: str):
        _check(lib().nb_checkpoint_save(self._h, os.fsencode(path)), "nb_checkpoint_save")

    def checkpoint_load(self, path: str):
        _check(lib().nb_checkpoint_load(self._h, os.fsencode(path)), "nb_checkpoint_load")

    # -------------------------------------------------------------- Barnes-Hut
    def bh_build(self) -> dict:
        """Builds the tree of the current positions (no walk) and reports it."""
        info = _BHInfo()
        _check(lib().nb_bh_build(self._h, C.byref(info)), "nb_bh_build")
        return _bh_info_dict(info)

    def bh_info(self) -> dict:
        """The last tree and walk (after a Barnes-Hut force evaluation)."""
        info = _BHInfo()
        _check(lib().nb_bh_get_info(self._h, C.byref(info)), "nb_bh_get_info")
        return _bh_info_dict(info)

    def bh_order(self):
        n = self.n
        codes = np.empty(n, np.uint64)
        order = np.empty(n, np.uint32)
        _check(lib().nb_bh_read_order(self._h, _ptr(codes), _ptr(order)), "nb_bh_read_order")
        return codes, order

    def bh_nodes(self, num_nodes: int) -> dict:
        """Node table (depth-first preorder) of the last tree."""
        a = dict(depth=np.empty(num_nodes, np.int32), prefix=np.empty(num_nodes, np.uint64),
                 first=np.empty(num_nodes, np.int32), count=np.empty(num_nodes, np.int32),
                 is_leaf=np.empty(num_nodes, np.int32), skip=np.empty(num_nodes, np.int32),
                 com_mass=np.empty((num_nodes, 4), np.float32))
        _check(lib().nb_bh_read_nodes(self._h, num_nodes, _ptr(a["depth"]), _ptr(a["prefix"]),
                                      _ptr(a["first"]), _ptr(a["count"]), _ptr(a["is_leaf"]),
                                      _ptr(a["skip"]), _ptr(a["com_mass"])),
               "nb_bh_read_nodes")
        return a


class Ensemble:
    """Many independent systems advanced together (nb_ensemble)."""

    def __init__(self, config: Config, sizes, stream: int | None = None):
        self._h = C.c_void_p()
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes, dtype=np.int64)])
        cfg = config._c()
        _check(lib().nb_ensemble_create(C.byref(cfg), len(self.sizes), _ptr(self.sizes),
                                        C.c_void_p(stream or 0), C.byref(self._h)),
               "nb_ensemble_create")

    def close(self):
        if self._h:
            lib().nb_ensemble_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def total(self) -> int:
        return int(self.offsets[-1])

    def load(self, x, y, z, vx, vy, vz, m):
        arrs = [_f64(a) for a in (x, y, z, vx, vy, vz, m)]
        if any(len(a) != self.total for a in arrs):
            raise ValueError("arrays must hold sum(sizes) bodies")
        _check(lib().nb_ensemble_load(self._h, *map(_ptr, arrs)), "nb_ensemble_load")

    def read_state(self):
        out = [np.empty(self.total) for _ in range(10)]
        _check(lib().nb_ensemble_read_state(self._h, *map(_ptr, out)), "nb_ensemble_read_state")
        keys = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "m"]
        return dict(zip(keys, out))

    def system(self, state: dict, s: int) -> dict:
        a, b = self.offsets[s], self.offsets[s + 1]
        return {k: v[a:b] for k, v in state.items()}

    def compute_forces(self):
        _check(lib().nb_ensemble_compute_forces(self._h), "nb_ensemble_compute_forces")

    def step(self, integrator: int, dt: float, nsteps: int = 1):
        _check(lib().nb_ensemble_step(self._h, integrator, dt, nsteps), "nb_ensemble_step")

    def tune(self):
        out = np.zeros(32, np.int32)
        _check(lib().nb_ensemble_tune(self._h, _ptr(out)), "nb_ensemble_tune")
        return out

    def synchronize(self):
        _check(lib().nb_ensemble_synchronize(self._h), "nb_ensemble_synchronize")

    def profile(self, enable: bool = True):
        _check(lib().nb_ensemble_profile(self._h, int(enable)), "nb_ensemble_profile")

    def info(self) -> dict:
        i = _EnsembleInfo()
        _check(lib().nb_ensemble_info(self._h, C.byref(i)), "nb_ensemble_info")
        return dict(num_systems=i.num_systems, total_bodies=i.total_bodies,
                    interactions_per_eval=i.interactions_per_eval, work_items=i.work_items,
                    ipt_by_bucket=list(i.ipt_by_bucket), graph_launches=i.graph_launches,
                    graph_steps=i.graph_steps, force_launches=i.force_launches,
                    force_kernel_ms=i.force_kernel_ms)


class Server:
    """Continuous-batching job server (nb_server)."""

    def __init__(self, **overrides):
        c = _ServerConfig()
        _check(lib().nb_server_config_default(C.byref(c)), "nb_server_config_default")
        for k, v in overrides.items():
            setattr(c, k, v)
        self._h = C.c_void_p()
        _check(lib().nb_server_create(C.byref(c), C.byref(self._h)), "nb_server_create")
        self.sizes = {}

    def close(self):
        if self._h:
            lib().nb_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, state, steps: int) -> int:
        arrs = [_f64(a) for a in state]
        jid = C.c_int64()
        _check(lib().nb_server_submit(self._h, len(arrs[0]), *map(_ptr, arrs), steps,
                                      C.byref(jid)), "nb_server_submit")
        self.sizes[jid.value] = len(arrs[0])
        return jid.value

    def tick(self):
        r, q = C.c_int(), C.c_int()
        _check(lib().nb_server_tick(self._h, C.byref(r), C.byref(q)), "nb_server_tick")
        return r.value, q.value

    def result(self, job_id: int):
        n = self.sizes[job_id]
        out = [np.empty(n) for _ in range(10)]
        _check(lib().nb_server_result(self._h, job_id, *map(_ptr, out)), "nb_server_result")
        return dict(zip(["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "m"], out))

    def release(self, job_id: int):
        _check(lib().nb_server_release(self._h, job_id), "nb_server_release")

    def cancel(self, job_id: int):
        """Cancels a queued or running job (nb_server_cancel)."""
        _check(lib().nb_server_cancel(self._h, job_id), "nb_server_cancel")

    def stats(self) -> dict:
        s = _ServerStats()
        _check(lib().nb_server_get_stats(self._h, C.byref(s)), "nb_server_get_stats")
        return {k: getattr(s, k) for k, _ in _ServerStats._fields_}

    def run_until_idle(self, max_ticks: int = 10**7):
        for _ in range(max_ticks):
            r, q = self.tick()
            if r == 0 and q == 0:
                return
        raise RuntimeError("server did not drain")


def ensemble_sizes(num_systems: int, lo: int, hi: int, seed: int):
    """N per system, log-uniform in [lo, hi] (SplitMix64 keyed by seed and
    system index, as the generators)."""
    out = np.empty(num_systems, np.int64)
    for s in range(num_systems):
        z = (seed * 0xD1B54A32D192ED03 ^ (s + 1) * 0x9E3779B97F4A7C15) & (2**64 - 1)
        z = (z + 0x9E3779B97F4A7C15) & (2**64 - 1)
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & (2**64 - 1)
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & (2**64 - 1)
        z ^= z >> 31
        u = ((z >> 11) + 0.5) / 2.0**53
        out[s] = int(np.floor(np.exp(np.log(lo) + u * (np.log(hi + 1) - np.log(lo)))))
    return np.clip(out, lo, hi)


def plummer_ensemble(sizes, seed: int = 0):
    """Concatenated Plummer spheres (G = M = a = 1), system s seeded with seed + s."""
    parts = [plummer(int(n), seed=seed + s) for s, n in enumerate(sizes)]
    return tuple(np.concatenate([p[k] for p in parts]) for k in range(7))


def _bh_info_dict(info) -> dict:
    return dict(num_nodes=info.num_nodes, num_leaves=info.num_leaves,
                max_depth=info.max_depth, split_levels=info.split_levels,
                root=list(info.root), interactions_m2p=info.interactions_m2p,
                interactions_p2p=info.interactions_p2p)


def version() -> str:
    return lib().nb_version().decode()


def debug_device_checks() -> bool:
    """nb_debug_device_checks: whether this library checks device indices;
    raises NBodyError (NB_ERR_DEVICE_FAULT, with the source line, index and
    bound) if a check failed since the last call."""
    enabled = C.c_int()
    _check(lib().nb_debug_device_checks(C.byref(enabled)), "nb_debug_device_checks")
    return bool(enabled.value)


def debug_fp32_rate() -> float:
    """nb_debug_fp32_rate: measured packed-FMA lane operations per second of
    the current device (register-only probe kernel)."""
    v = C.c_double(0.0)
    _check(lib().nb_debug_fp32_rate(C.byref(v)), "nb_debug_fp32_rate")
    return v.value


def debug_fail_device_allocations(after: int):
    """Test hook (nb_debug_fail_device_allocations): the device allocation
    after `after` more successful ones fails with NB_ERR_OUT_OF_MEMORY;
    negative disarms.  Host side only."""
    _check(lib().nb_debug_fail_device_allocations(int(after)),
           "nb_debug_fail_device_allocations")
