"""The device-checked build (build.py --checks, -DNB_DEVICE_CHECKS=1): every
kernel family runs with its index checks on, no check fails, and the results
are the same bits as the normal library's (the checks skip only accesses that
would be out of range, and none is).  The checked library runs in a child
process (NBODY_GB300_LIB), since one process loads one build of the engine."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import PKG_DIR, REPO

pytestmark = pytest.mark.gpu


def test_checked_build_runs_clean_and_matches(nb, tmp_path):
    sys.path.insert(0, PKG_DIR)
    import build as pkg_build
    checked = pkg_build.build(checks=True)
    out = tmp_path / "checked.npz"
    env = dict(os.environ, NBODY_GB300_LIB=checked)
    r = subprocess.run([sys.executable, os.path.join(REPO, "tests", "checked_workloads.py"),
                        str(out)], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    got = np.load(out)
    assert bool(got["enabled"])
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import checked_workloads
    ref = checked_workloads.run(nb)
    assert not nb.debug_device_checks()  # the normal build has no checks
    for k, v in ref.items():
        assert np.array_equal(got[k], v), k
