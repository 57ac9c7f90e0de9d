"""Same input, same bits, in separate processes with the autotuners on.

The mixed kernels time several CTA shapes at the first evaluation of each
body count and keep the fastest.  The j-segments and (for the Hilbert-sorted
kernel) the chunks per warp are fixed by the body count alone, so the timed
choice changes only how work is scheduled, never the order in which a body's
terms are summed: two processes that run the same evaluations must agree bit
for bit.  Each case runs in two fresh child processes (NB_AUTOTUNE unset) and
compares the accelerations and the evolved state.
"""
import json
import os
import subprocess
import sys

import pytest

from conftest import PKG_DIR, REPO

pytestmark = pytest.mark.gpu

CHILD = r'''
import hashlib, json, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import nbody_gb300 as nb
case = sys.argv[2]
out = {}
if case == "bench_workload":
    # the benchmark workload: 65,536-body Plummer sphere, velocity Verlet
    st = nb.plummer(65536, seed=0)
    cfg = nb.Config(method=nb.DIRECT_MIXED, G=1.0, softening=1e-3)
    with nb.Sim(cfg, capacity=65536) as s:
        s.load(*st)
        s.step(nb.VELOCITY_VERLET, 5e-4, 12)
        cur = s.read_state()
elif case == "all_pairs_8192":
    st = nb.plummer(8192, seed=3)
    cfg = nb.Config(method=nb.DIRECT_MIXED, G=1.0, softening=1e-3, flags=nb.MIXED_UNSORTED)
    with nb.Sim(cfg, capacity=8192) as s:
        s.load(*st)
        s.step(nb.VELOCITY_VERLET, 5e-4, 3)
        cur = s.read_state()
for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"):
    out[k] = hashlib.sha256(np.ascontiguousarray(cur[k]).tobytes()).hexdigest()
print("DIGEST" + json.dumps(out))
'''


def _run(case):
    env = dict(os.environ)
    env.pop("NB_AUTOTUNE", None)
    r = subprocess.run([sys.executable, "-c", CHILD, PKG_DIR, case], env=env, cwd=REPO,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [l for l in r.stdout.splitlines() if l.startswith("DIGEST")]
    assert line, r.stdout[-2000:]
    return json.loads(line[0][6:])


@pytest.mark.parametrize("case", ["bench_workload", "all_pairs_8192"])
def test_two_processes_give_the_same_bits(case):
    a = _run(case)
    b = _run(case)
    assert a == b
