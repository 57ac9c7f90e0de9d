"""The reference's C++ host API on top of the engine (libnbody_compat.so).

CPU checks (here): the compat headers lay out every class exactly as the
reference's CUDA/include headers do (so objects built against either header set
can be shared), and -- where the reference checkout exists -- the reference's
own CUDA test programs compile unchanged against its own headers and link
against libnbody_compat.so with no unresolved symbol.
GPU checks: drivers written against the compat headers, in the style of the
reference's tests, run on the GPU and agree with the CPU oracle.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import PKG_DIR, REPO, ref_root

REF = ref_root() or ""
COMPAT_INC = os.path.join(PKG_DIR, "compat", "include")
LIBDIR = os.path.join(PKG_DIR, "nbody_gb300")
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc(args, cwd):
    r = subprocess.run([NVCC, "-std=c++17", *args], cwd=cwd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def _probe(tmp_path, inc):
    exe = tmp_path / ("probe_" + os.path.basename(os.path.dirname(inc)))
    _nvcc(["-x", "cu", "-I", inc, os.path.join(REPO, "tests", "compat", "layout_probe.cpp"),
           "-o", str(exe)], tmp_path)
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "CUDA", "include")),
                    reason="reference checkout not present")
def test_layout_matches_reference_headers(tmp_path):
    ours = _probe(tmp_path, COMPAT_INC)
    theirs = _probe(tmp_path, os.path.join(REF, "CUDA", "include"))
    assert ours == theirs
    assert "BarnesHutForceCalculator 368" in ours


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "CUDA", "tests")),
                    reason="reference checkout not present")
@pytest.mark.parametrize("test", ["test1_EarthSun", "test2_ForceBenchmark",
                                  "test5_barnesHutBenchmark"])
def test_reference_tests_link_unchanged(nb, tmp_path, test):
    src = os.path.join(REF, "CUDA", "tests", test + ".cu")
    _nvcc([*ARCH, "-I", os.path.join(REF, "CUDA", "include"), src, "-o", str(tmp_path / test),
           "-L", LIBDIR, "-lnbody_compat", "-lnbody_gb300", "-Xlinker", "-rpath=" + LIBDIR],
          tmp_path)
    assert (tmp_path / test).exists()


def build_driver(tmp_path, name):
    exe = tmp_path / name
    _nvcc([*ARCH, "-O2", "-I", COMPAT_INC, "-I", os.path.join(REPO, "include"),
           os.path.join(REPO, "tests", "compat", name + ".cu"), "-o", str(exe), "-L", LIBDIR,
           "-lnbody_compat", "-lnbody_gb300", "-Xlinker", "-rpath=" + LIBDIR], tmp_path)
    return str(exe)


@pytest.mark.gpu
def test_compat_forces_driver(nb, oracle, tmp_path):
    exe = build_driver(tmp_path, "compat_forces")
    n = 3000
    out = tmp_path / "forces.bin"
    subprocess.run([exe, str(n), "42", str(out)], check=True, capture_output=True)
    raw = np.fromfile(out, dtype=np.float64)
    assert int(raw[0]) == n
    x, y, z, m = (raw[1 + k * n:1 + (k + 1) * n] for k in range(4))
    a_naive = raw[1 + 4 * n:1 + 7 * n].reshape(3, n)
    a_bh = raw[1 + 7 * n:1 + 10 * n].reshape(3, n)
    # the test program's std::mt19937 draws are the CUDA benchmark's order; the host
    # compiler may fuse libstdc++'s u*(b-a)+a into an FMA (Arm), so allow an ulp
    g = oracle.MT19937(42)
    ox, oy, oz, om = g.uniform_cube(n, order=1)
    assert np.allclose(x, ox, rtol=1e-15, atol=1e-13) and np.allclose(m, om, rtol=1e-15)
    ref = np.array(oracle.forces_naive(x, y, z, m, oracle.G_REF, 0.0))
    rel = np.linalg.norm(a_naive - ref, axis=0) / np.linalg.norm(ref, axis=0)
    assert rel.max() <= 1e-12
    cpu_bh = np.array(oracle.forces_bh_opt(x, y, z, m, oracle.G_REF, 0.0, 0.5, 8))
    e_gpu = np.linalg.norm(a_bh - ref, axis=0) / np.linalg.norm(ref, axis=0)
    e_cpu = np.linalg.norm(cpu_bh - ref, axis=0) / np.linalg.norm(ref, axis=0)
    assert e_gpu.mean() <= e_cpu.mean()
    times = raw[1 + 10 * n:]
    assert times[0] > 0 and times[1] > 0 and times[3] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("integ,code", [("euler", 0), ("euler-cromer", 1), ("leapfrog", 2),
                                        ("verlet", 3), ("rk4", 4)])
def test_compat_integrators_driver(nb, oracle, tmp_path, integ, code):
    exe = build_driver(tmp_path, "compat_orbit")
    out = tmp_path / "orbit.bin"
    subprocess.run([exe, integ, "366", str(out)], check=True, capture_output=True)
    got = np.fromfile(out, dtype=np.float64).reshape(10, 2)
    x = np.array([0.0, 1.0]); y = np.zeros(2); z = np.zeros(2)
    vx = np.zeros(2); vy = np.array([0.0, 2 * np.pi]); vz = np.zeros(2)
    m = np.array([1.0, 3.003e-6])
    ref = oracle.run(code, oracle.DIRECT, x, y, z, vx, vy, vz, m, oracle.G_REF, 0.0, 1 / 365,
                     366)
    # scale: the largest vector magnitude of the quantity (position, velocity,
    # acceleration) over both bodies
    for k in range(9):
        g3 = slice(3 * (k // 3), 3 * (k // 3) + 3)
        scale = max(np.sqrt((np.array(ref[g3]) ** 2).sum(axis=0)).max(), 1e-300)
        assert np.abs(got[k] - ref[k]).max() <= 1e-12 * scale, (integ, k)
