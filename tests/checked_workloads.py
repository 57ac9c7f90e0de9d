"""Workloads run both on the normal library and on the device-checked one
(build.py --checks) by tests/test_gpu_checks.py: every kernel family of the
engine on small inputs.  `python tests/checked_workloads.py OUT.npz` runs them
on the library NBODY_GB300_LIB names and saves the results; the run fails if
a device-side index check failed."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "n-body-gravity-simulation_gb300"))


def run(nb) -> dict:
    out = {}

    def sim_run(key, method, st, flags=0, steps=0, integ=None, theta=0.5):
        cfg = nb.Config(method=method, G=1.0, softening=1e-3, theta=theta, flags=flags)
        with nb.Sim(cfg, capacity=len(st[0])) as s:
            s.load(*st)
            s.compute_forces()
            if steps:
                s.step(integ, 1e-3, steps)
            r = s.read_state()
        for k in ("x", "ax", "ay", "az"):
            out[f"{key}_{k}"] = r[k]

    disk = nb.disk_bulge(30000, seed=11)
    plum = nb.plummer(20000, seed=12)
    sim_run("bh", nb.BARNES_HUT, disk, steps=3, integ=nb.LEAPFROG)
    sim_run("bh_reuse_quad", nb.BARNES_HUT, disk, flags=nb.bh_reuse_flag(2) | nb.BH_QUADRUPOLE,
            steps=3, integ=nb.LEAPFROG)
    sim_run("sorted", nb.DIRECT_MIXED, plum, flags=nb.MIXED_SORTED, steps=9,
            integ=nb.VELOCITY_VERLET)
    sim_run("unsorted", nb.DIRECT_MIXED, nb.plummer(5000, seed=13), flags=nb.MIXED_UNSORTED,
            steps=2, integ=nb.RK4)
    sim_run("fp64", nb.DIRECT_FP64, nb.plummer(2000, seed=14), steps=2, integ=nb.LEAPFROG)
    sizes = nb.ensemble_sizes(30, 32, 4096, 15)
    ens_state = nb.plummer_ensemble(sizes, seed=15)
    for key, flags in (("ens_sorted", 0), ("ens_unsorted", nb.MIXED_UNSORTED)):
        cfg = nb.Config(method=nb.DIRECT_MIXED, G=1.0, softening=1e-3, flags=flags)
        with nb.Ensemble(cfg, sizes) as e:
            e.load(*ens_state)
            e.step(nb.RK4, 1e-3, 3)
            r = e.read_state()
        out[f"{key}_x"], out[f"{key}_ax"] = r["x"], r["ax"]
    with nb.Server() as s:
        ids = [s.submit(nb.plummer(3000, seed=16), 4), s.submit(nb.disk_bulge(20000, seed=17), 4)]
        s.run_until_idle()
        for k, j in enumerate(ids):
            out[f"server{k}_x"] = s.result(j)["x"]
    return out


def main(path: str) -> int:
    import nbody_gb300 as nb
    res = run(nb)
    enabled = nb.debug_device_checks()  # raises on a failed check
    np.savez(path, enabled=np.array(enabled), **res)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1]))
