"""The device-checked build (build.py --checks, -DNB_DEVICE_CHECKS=1): every
kernel family runs with its index checks on, no check fails, and the results
are the same bits as the normal library's (the checks skip only accesses that
would be out of range, and none is).  Each library runs in a child process
(NBODY_GB300_LIB), since one process loads one build of the engine, with the
autotuners off (NB_AUTOTUNE=0): the mixed direct sums' bits do not depend on the
tuned CTA shape, but the all-pairs ensemble kernel's timed i-bodies per lane
would differ between two processes and change its summation order."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import PKG_DIR, REPO

pytestmark = pytest.mark.gpu


def run_workloads(lib_path, out):
    env = dict(os.environ, NBODY_GB300_LIB=lib_path, NB_AUTOTUNE="0")
    r = subprocess.run([sys.executable, os.path.join(REPO, "tests", "checked_workloads.py"),
                        str(out)], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return np.load(out)


def test_checked_build_runs_clean_and_matches(nb, tmp_path):
    sys.path.insert(0, PKG_DIR)
    import build as pkg_build
    checked = run_workloads(pkg_build.build(checks=True), tmp_path / "checked.npz")
    normal = run_workloads(nb.LIB_PATH, tmp_path / "normal.npz")
    assert bool(checked["enabled"]) and not bool(normal["enabled"])
    for k in normal.files:
        if k != "enabled":
            assert np.array_equal(checked[k], normal[k]), k
