"""Files through a simulation on the GPU: particle-file load, the reference's
trajectory CSV (CPU/src/n-body.cpp, golden CPU/orbit.csv rows), and binary
checkpoints whose continuation is bit-identical to the uninterrupted run."""
import csv
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
COLS = ["earth_x", "earth_y", "earth_z", "sun_x", "sun_y", "sun_z", "kinetic_energy",
        "potential_energy", "total_energy", "angular_momentum_x", "angular_momentum_y",
        "angular_momentum_z", "center_of_mass_x", "center_of_mass_y", "center_of_mass_z"]


def test_load_particles_into_sim(nb, tmp_path):
    st = nb.plummer(1000, seed=3)
    p = str(tmp_path / "plummer.txt")
    nb.write_particles(p, *st)
    with nb.Sim(nb.Config(method=nb.DIRECT_FP64), capacity=1000) as s:
        s.load_particles(p)
        back = s.read_state()
        for k, name in enumerate(["x", "y", "z", "vx", "vy", "vz", "m"]):
            assert np.array_equal(back[name], st[k])
        with pytest.raises(nb.NBodyError) as e:
            s.load_particles(str(tmp_path / "missing.txt"))
        assert e.value.status == 8


def test_orbit_csv_matches_reference_file(nb, oracle, tmp_path):
    """Sun + Earth, velocity Verlet, dt = 1/365, 366 steps: the header, the
    first row (default stream format) and every later row (%.15f) as the
    reference writes them; values agree with CPU/orbit.csv to 1e-12 (the FP64
    force path is pinned at 1e-12 relative)."""
    x = np.array([0.0, 1.0]); y = np.zeros(2); z = np.zeros(2)
    vx = np.zeros(2); vy = np.array([0.0, 2 * np.pi]); vz = np.zeros(2)
    m = np.array([1.0, 3.003e-6])
    path = str(tmp_path / "orbit.csv")
    with nb.Sim(nb.Config(method=nb.DIRECT_FP64, G=oracle.G_REF, softening=0.0),
                capacity=2) as s:
        s.load(x, y, z, vx, vy, vz, m)
        s.csv_append(path, [1, 0], ["earth", "sun"], header=True, precision=-1)
        dt = 1.0 / 365.0
        for _ in range(int(1.0 / dt) + 1):
            s.step(nb.VELOCITY_VERLET, dt)
            s.csv_append(path, [1, 0], precision=15)
    lines = open(path).read().splitlines()
    assert lines[0] == ",".join(COLS)
    assert len(lines) == 1 + 367
    golden = {int(r["row"]): r for r in csv.DictReader(open(os.path.join(GOLDEN,
                                                                          "orbit_earth_sun.csv")))}
    first = open(os.path.join(GOLDEN, "orbit_earth_sun.csv")).read().splitlines()[1]
    assert lines[1] == first.split(",", 1)[1]  # "1,0,0,0,0,0,5.92768e-05,..."
    rows = list(csv.DictReader(lines))
    checked = 0
    for step, r in enumerate(rows):
        if step == 0 or step not in golden:
            continue
        assert all(len(r[c].split(".")[1]) == 15 for c in COLS)
        diff = max(abs(float(r[c]) - float(golden[step][c])) for c in COLS)
        assert diff <= 1e-12, (step, diff)
        checked += 1
    assert checked >= 17


@pytest.mark.parametrize("method,n,integ", [("fp64", 2000, "leapfrog"),
                                            ("mixed", 3000, "verlet"),
                                            ("bh", 6000, "leapfrog"),
                                            ("fp64", 500, "rk4")])
def test_checkpoint_resume_bit_identical(nb, tmp_path, method, n, integ):
    meth = {"fp64": nb.DIRECT_FP64, "mixed": nb.DIRECT_MIXED, "bh": nb.BARNES_HUT}[method]
    it = {"leapfrog": nb.LEAPFROG, "verlet": nb.VELOCITY_VERLET, "rk4": nb.RK4}[integ]
    cfg = nb.Config(method=meth, G=1.0, softening=0.01, theta=0.5)
    st = nb.plummer(n, seed=11)
    ck = str(tmp_path / "state.ck")
    dt = 1e-3
    with nb.Sim(cfg, capacity=n) as a:
        a.load(*st)
        a.step(it, dt, 5)
        a.checkpoint_save(ck)
        a.step(it, dt, 5)
        want = a.read_state()
    with nb.Sim(nb.Config(method=nb.DIRECT_FP64), capacity=n) as b:
        b.checkpoint_load(ck)
        assert b.config.method == meth
        b.step(it, dt, 5)
        got = b.read_state()
    for k in want:
        assert np.array_equal(want[k], got[k]), k


def test_checkpoint_errors(nb, tmp_path):
    bad = tmp_path / "bad.ck"
    bad.write_bytes(b"not a checkpoint at all")
    with nb.Sim(nb.Config(), capacity=10) as s:
        with pytest.raises(nb.NBodyError) as e:
            s.checkpoint_load(str(bad))
        assert e.value.status == 8
        st = nb.plummer(10, seed=1)
        s.load(*st)
        ck = str(tmp_path / "ten.ck")
        s.checkpoint_save(ck)
    with nb.Sim(nb.Config(), capacity=5) as small:
        with pytest.raises(nb.NBodyError) as e:
            small.checkpoint_load(ck)
        assert e.value.status == 4
