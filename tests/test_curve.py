"""The Hilbert-curve index and the order-preserving FP64 keys (csrc/nb_curve.cuh)
checked on the host: tests/curve_probe.cu is compiled with nvcc and run."""
import os
import shutil
import subprocess

from conftest import PKG_DIR, REPO

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def test_hilbert_index_and_order_keys(tmp_path):
    exe = tmp_path / "curve_probe"
    r = subprocess.run([NVCC, "-std=c++17", "-O2", "-I", os.path.join(PKG_DIR, "csrc"),
                        "-I", os.path.join(REPO, "include"),
                        os.path.join(REPO, "tests", "curve_probe.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "OK", out.stdout + out.stderr
