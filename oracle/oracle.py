"""ctypes front end of the CPU oracle (test infrastructure only).

Loads ``oracle/liboracle.so`` (the C restatement of the reference's CPU path,
``nbody_oracle.c``) and, when it was built in this checkout,
``oracle/_ref/libnbref.so`` (the reference's own CPU sources plus
``ref_shim.cpp``).  Only the tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` import this module; the GPU product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libnbref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")

EULER, EULER_CROMER, LEAPFROG, VERLET, RK4 = 0, 1, 2, 3, 4
DIRECT, BH_OPT, BH_PTR = 0, 1, 2
G_REF = 4.0 * np.pi * np.pi  # CPU/include/common.hpp:28


def build(with_ref: bool = True) -> None:
    args = ["bash", os.path.join(HERE, "build_ref.sh")]
    if not with_ref:
        args.append("--no-ref")
    subprocess.run(args, check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_ref=False)
        L = C.CDLL(LIB_PATH)
        L.orc_mt_size.restype = C.c_size_t
        L.orc_mt_seed.argtypes = [C.c_void_p, C.c_uint32]
        L.orc_mt_u32.argtypes = [C.c_void_p]
        L.orc_mt_u32.restype = C.c_uint32
        L.orc_mt_uniform.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.orc_mt_uniform.restype = C.c_double
        L.orc_gen_uniform_cube.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_forces_naive.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.c_double,
                                       _dp, _dp, _dp, C.c_int]
        L.orc_forces_naive_abs.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double,
                                           C.c_double, _dp, C.c_int]
        L.orc_forces_naive_rows.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp,
                                            C.c_double, C.c_double, _dp, _dp, _dp, C.c_int]
        L.orc_forces_bh_opt.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.c_double,
                                        C.c_double, C.c_int, _dp, _dp, _dp, C.c_int]
        L.orc_forces_bh_opt.restype = C.c_int
        L.orc_forces_bh_ptr.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.c_double,
                                        C.c_double, _dp, _dp, _dp, C.c_int]
        L.orc_bh_opt_dump.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_int, C.c_int, _i32p,
                                      _i32p, _i32p, _i64p, _i64p, _i64p]
        L.orc_bh_opt_dump.restype = C.c_int
        L.orc_step.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                               _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_int,
                               C.c_double, C.c_int, C.c_int]
        L.orc_step.restype = C.c_int
        L.orc_diagnostics.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double,
                                      C.c_double, _dp, C.c_int]
        L.orc_potential_energy_seq.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double]
        L.orc_potential_energy_seq.restype = C.c_double
        L.orc_root_cube.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
        L.orc_split_levels.argtypes = [C.c_double]
        L.orc_split_levels.restype = C.c_int
        L.orc_morton63.argtypes = [C.c_int, _dp, _dp, _dp, _u64p, _dp]
        L.orc_sort_codes.argtypes = [C.c_int, _u64p, _u64p, _u32p]
        L.orc_octree.argtypes = [C.c_int, _u64p, C.c_int, C.c_int, C.c_int, _i32p, _u64p,
                                 _i32p, _i32p, _i32p, _i32p, _i32p]
        L.orc_octree.restype = C.c_int
        L.orc_max_threads.restype = C.c_int
        L.orc_gen_plummer.argtypes = [C.c_int, C.c_uint64, C.c_double, C.c_double, C.c_double,
                                      _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_gen_disk_bulge.argtypes = [C.c_int, C.c_uint64, C.c_double, C.c_double,
                                         C.c_double, C.c_double, C.c_double, C.c_double,
                                         C.c_double, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    """The reference's own CPU classes (only where they were compiled here)."""
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.ref_G.restype = C.c_double
        R.ref_forces.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_double,
                                 C.c_double, C.c_int, _dp, _dp, _dp]
        R.ref_run.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                              _dp, _dp, _dp, C.c_double, C.c_double, C.c_int, C.c_double,
                              C.c_int]
        R.ref_diagnostics.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        R.ref_bh_opt_dump.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_int, C.c_int, _i32p,
                                      _i32p, _i32p, _i64p, _i64p, _i64p]
        R.ref_bh_opt_dump.restype = C.c_int
        _ref = R
    return _ref


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class MT19937:
    """std::mt19937 with libstdc++'s uniform_real_distribution<double>."""

    def __init__(self, seed: int):
        self._buf = C.create_string_buffer(lib().orc_mt_size())
        lib().orc_mt_seed(self._buf, seed)

    def u32(self) -> int:
        return lib().orc_mt_u32(self._buf)

    def uniform(self, a: float, b: float) -> float:
        return lib().orc_mt_uniform(self._buf, a, b)

    def uniform_cube(self, n: int, order: int = 0):
        """order 0: the CPU benchmark's draw order; 1: the CUDA benchmark's."""
        x, y, z, m = (np.empty(n) for _ in range(4))
        lib().orc_gen_uniform_cube(self._buf, n, order, x, y, z, m)
        return x, y, z, m


def threads() -> int:
    return lib().orc_max_threads()


def forces_naive(x, y, z, m, G, eps, nthreads=0):
    x, y, z, m = map(_c, (x, y, z, m))
    n = len(x)
    ax, ay, az = np.empty(n), np.empty(n), np.empty(n)
    lib().orc_forces_naive(n, x, y, z, m, G, eps * eps, ax, ay, az, nthreads)
    return ax, ay, az


def forces_abs_sum(x, y, z, m, G, eps, nthreads=0):
    """Per body sum_j |pair term| (the error scale of any FP evaluation)."""
    x, y, z, m = map(_c, (x, y, z, m))
    out = np.empty(len(x))
    lib().orc_forces_naive_abs(len(x), x, y, z, m, G, eps * eps, out, nthreads)
    return out


def forces_naive_rows(x, y, z, m, G, eps, i0, i1, nthreads=0):
    x, y, z, m = map(_c, (x, y, z, m))
    n = len(x)
    k = i1 - i0
    ax, ay, az = np.empty(k), np.empty(k), np.empty(k)
    lib().orc_forces_naive_rows(n, i0, i1, x, y, z, m, G, eps * eps, ax, ay, az, nthreads)
    return ax, ay, az


def forces_bh_opt(x, y, z, m, G, eps, theta, leaf_capacity=8, nthreads=0):
    x, y, z, m = map(_c, (x, y, z, m))
    n = len(x)
    ax, ay, az = np.empty(n), np.empty(n), np.empty(n)
    rc = lib().orc_forces_bh_opt(n, x, y, z, m, G, eps * eps, theta, leaf_capacity, ax, ay,
                                 az, nthreads)
    if rc < 0:
        raise RuntimeError("oracle node pool overflow")
    return ax, ay, az


def forces_bh_ptr(x, y, z, m, G, eps, theta, nthreads=0):
    x, y, z, m = map(_c, (x, y, z, m))
    n = len(x)
    ax, ay, az = np.empty(n), np.empty(n), np.empty(n)
    lib().orc_forces_bh_ptr(n, x, y, z, m, G, eps * eps, theta, ax, ay, az, nthreads)
    return ax, ay, az


def run(integrator, method, x, y, z, vx, vy, vz, m, G, eps, dt, nsteps, theta=0.5,
        leaf_capacity=8, nthreads=0):
    """Advance copies of the state by nsteps reference steps; returns
    (x, y, z, vx, vy, vz, ax, ay, az)."""
    st = [np.array(a, dtype=np.float64, copy=True) for a in (x, y, z, vx, vy, vz)]
    m = _c(m)
    n = len(m)
    ax, ay, az = np.zeros(n), np.zeros(n), np.zeros(n)
    rc = lib().orc_step(integrator, method, n, *st, m, ax, ay, az, G, eps * eps, theta,
                        leaf_capacity, dt, nsteps, nthreads)
    if rc != 0:
        raise RuntimeError("oracle step failed")
    return (*st, ax, ay, az)


def diagnostics(x, y, z, vx, vy, vz, m, G, eps, nthreads=0):
    out = np.empty(13)
    lib().orc_diagnostics(len(m), *map(_c, (x, y, z, vx, vy, vz, m)), G, eps * eps, out,
                          nthreads)
    keys = ["ke", "pe", "pe_soft", "lx", "ly", "lz", "comx", "comy", "comz", "px", "py",
            "pz", "mass"]
    return dict(zip(keys, out.tolist()))


def potential_energy_seq(x, y, z, m, G):
    return lib().orc_potential_energy_seq(len(m), *map(_c, (x, y, z, m)), G)


def root_cube(x, y, z):
    out = np.empty(4)
    lib().orc_root_cube(len(x), *map(_c, (x, y, z)), out)
    return out


def split_levels(size: float) -> int:
    return lib().orc_split_levels(size)


def morton63(x, y, z):
    n = len(x)
    codes = np.empty(n, dtype=np.uint64)
    root = np.empty(4)
    lib().orc_morton63(n, *map(_c, (x, y, z)), codes, root)
    return codes, root


def sort_codes(codes):
    codes = np.ascontiguousarray(codes, dtype=np.uint64)
    n = len(codes)
    sc = np.empty(n, dtype=np.uint64)
    order = np.empty(n, dtype=np.uint32)
    lib().orc_sort_codes(n, codes, sc, order)
    return sc, order


def octree(sorted_codes, leaf_capacity, levels, max_nodes=None):
    sc = np.ascontiguousarray(sorted_codes, dtype=np.uint64)
    n = len(sc)
    if max_nodes is None:
        max_nodes = 8 * n + 64
    arrs = dict(depth=np.empty(max_nodes, np.int32), prefix=np.empty(max_nodes, np.uint64),
                first=np.empty(max_nodes, np.int32), count=np.empty(max_nodes, np.int32),
                is_leaf=np.empty(max_nodes, np.int32),
                first_child=np.empty(max_nodes, np.int32),
                nchild=np.empty(max_nodes, np.int32))
    nn = lib().orc_octree(n, sc, leaf_capacity, levels, max_nodes, arrs["depth"],
                          arrs["prefix"], arrs["first"], arrs["count"], arrs["is_leaf"],
                          arrs["first_child"], arrs["nchild"])
    if nn < 0:
        raise RuntimeError("octree node buffer too small")
    return {k: v[:nn].copy() for k, v in arrs.items()}


def bh_opt_dump(x, y, z, m, leaf_capacity, use_ref=False):
    """Node list of the CPU node-pool tree: depth, count, leaf, cell coords."""
    n = len(x)
    max_out = 8 * n + 1000
    depth, count, leaf = (np.empty(max_out, np.int32) for _ in range(3))
    cx, cy, cz = (np.empty(max_out, np.int64) for _ in range(3))
    f = ref().ref_bh_opt_dump if use_ref else lib().orc_bh_opt_dump
    nn = f(n, *map(_c, (x, y, z, m)), leaf_capacity, max_out, depth, count, leaf, cx, cy, cz)
    if nn < 0:
        raise RuntimeError("dump failed")
    return dict(depth=depth[:nn], count=count[:nn], is_leaf=leaf[:nn], cx=cx[:nn],
                cy=cy[:nn], cz=cz[:nn])


def error_stats(a_test, a_ref):
    """The reference benchmark's error statistics
    (CPU/tests/test2_ForceBenchmark.cpp:84-150): mean/max absolute |da| and
    mean/max relative |da|/|a_ref| over bodies with |a_ref| > 1e-12 (the mean
    divides by N, as the reference does)."""
    ax, ay, az = a_test
    rx, ry, rz = a_ref
    d = np.sqrt((ax - rx) ** 2 + (ay - ry) ** 2 + (az - rz) ** 2)
    r = np.sqrt(rx * rx + ry * ry + rz * rz)
    n = len(d)
    mask = r > 1e-12
    rel = np.where(mask, d / np.where(mask, r, 1.0), 0.0)
    return dict(avg_abs=float(d.sum() / n), max_abs=float(d.max(initial=0.0)),
                avg_rel=float(rel.sum() / n), max_rel=float(rel.max(initial=0.0)))


def plummer(n, seed=0, total_mass=1.0, scale=1.0, G=1.0):
    """The engine's seeded Plummer sphere, restated (section 8 of the C file):
    (x, y, z, vx, vy, vz, m) as float64 arrays, the same bits as the engine's
    generator."""
    out = [np.empty(n) for _ in range(7)]
    lib().orc_gen_plummer(n, seed, total_mass, scale, G, *out)
    return tuple(out)


def disk_bulge(n, seed=0, total_mass=1.0, bulge_frac=0.2, bulge_scale=0.2, disk_scale=1.0,
               disk_height=0.05, dispersion=0.1, G=1.0):
    """The engine's seeded Plummer bulge + exponential disk, restated."""
    out = [np.empty(n) for _ in range(7)]
    lib().orc_gen_disk_bulge(n, seed, total_mass, bulge_frac, bulge_scale, disk_scale,
                             disk_height, dispersion, G, *out)
    return tuple(out)
