"""CPU-side checks of the C ABI: the library builds, loads and exports every
function that include/*.h declares; host-only entry points (generators,
status strings) work without a GPU."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "nbody_c.h")


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(nb_\w+)\s*\(", text):
            # declarations start a line with a return type: skip macro bodies
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_core_api():
    names = declared_functions()
    for must in ("nb_create", "nb_load", "nb_compute_forces", "nb_step", "nb_diagnostics",
                 "nb_read_state", "nb_destroy"):
        assert must in names


def test_library_exports_every_declared_symbol(nb):
    L = nb.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_header(nb):
    """The Python front end binds exactly the functions the header declares."""
    assert set(nb.EXPORTS) == set(declared_functions())


def test_status_strings_and_version(nb):
    L = nb.lib()
    assert L.nb_status_string(0) == b"ok"
    assert L.nb_status_string(4) == b"capacity exceeded"
    assert L.nb_status_string(9) == b"cancelled"
    # every status the header declares has its own string and a Python name
    codes = [int(c) for c in re.findall(r"NB_(?:OK|ERR_[A-Z_]+) = (\d+)", open(HEADER).read())]
    assert sorted(codes) == list(range(len(codes)))
    assert set(codes) == set(nb.STATUS)
    names = {L.nb_status_string(c) for c in codes}
    assert len(names) == len(codes) and b"unknown status" not in names
    assert b"sm_103a" in L.nb_version()


def test_plummer_generator_deterministic_and_virial(nb, oracle):
    a = nb.plummer(2000, seed=3)
    b = nb.plummer(2000, seed=3)
    c = nb.plummer(2000, seed=4)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    assert not np.array_equal(a[0], c[0])
    x, y, z, vx, vy, vz, m = a
    assert m.sum() == pytest.approx(1.0)
    assert abs(np.sum(m * x)) < 1e-12 and abs(np.sum(m * vx)) < 1e-12
    d = oracle.diagnostics(x, y, z, vx, vy, vz, m, 1.0, 0.0)
    q = 2 * d["ke"] / abs(d["pe"])  # virial ratio, 1 in equilibrium
    assert 0.85 < q < 1.15


def test_disk_bulge_generator(nb):
    x, y, z, vx, vy, vz, m = nb.disk_bulge(4000, seed=1)
    assert m.sum() == pytest.approx(1.0)
    r_disk = np.hypot(x[800:], y[800:])
    assert 0.5 < np.median(r_disk) < 3.0          # exponential disk, scale length 1
    assert np.median(np.abs(z[800:])) < 0.2       # thin: sech^2 height 0.05
    # disk rotates: specific angular momentum about z is positive on average
    assert np.mean(x[800:] * vy[800:] - y[800:] * vx[800:]) > 0


def test_generator_rejects_bad_arguments(nb):
    with pytest.raises(nb.NBodyError):
        nb.plummer(10, total_mass=-1.0)


def test_create_fails_cleanly_without_gpu(nb):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(nb.NBodyError) as e:
        nb.Sim(nb.Config(), capacity=16)
    assert e.value.status in (2, 3)  # NB_ERR_CUDA / out of memory: no device


def test_normal_build_has_no_device_checks(nb):
    """nb_debug_device_checks needs no GPU: the normal build reports that its
    kernels carry no index checks (the checked build is tested on the GPU)."""
    assert nb.debug_device_checks() is False
