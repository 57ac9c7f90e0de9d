"""GPU integrators and diagnostics against the CPU oracle.

FP64 path: trajectories within 1e-12 (relative to the state's scale) of the
oracle's, which restates the reference's CPU integrators operation by
operation; the reference's leapfrog and velocity Verlet evaluate forces twice
per step, the GPU reuses the end-of-step force (the CUDA reference does the
same through is_first_step), which is the same value.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = {0: "euler", 1: "euler_cromer", 2: "leapfrog", 3: "verlet", 4: "rk4"}


def scaled_err(a, b):
    s = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / s


def run_gpu(nb, method, integ, state, G, eps, dt, steps):
    n = len(state[0])
    with nb.Sim(nb.Config(method=method, G=G, softening=eps), capacity=n) as s:
        s.load(*state)
        s.step(integ, dt, steps)
        return s.read_state()


@pytest.mark.parametrize("integ", [0, 1, 2, 3, 4])
def test_fp64_integrators_match_oracle(nb, oracle, integ):
    x, y, z, vx, vy, vz, m = nb.plummer(512, seed=5)
    G, eps, dt, steps = 1.0, 0.05, 1e-3, 10
    got = run_gpu(nb, nb.DIRECT_FP64, integ, (x, y, z, vx, vy, vz, m), G, eps, dt, steps)
    ref = oracle.run(integ, oracle.DIRECT, x, y, z, vx, vy, vz, m, G, eps, dt, steps)
    for k, key in enumerate(["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"]):
        assert scaled_err(got[key], ref[k]) <= 1e-12, (NAMES[integ], key)


@pytest.mark.parametrize("integ", [2, 3, 4])
def test_mixed_integrators_close_to_oracle(nb, oracle, integ):
    x, y, z, vx, vy, vz, m = nb.plummer(1024, seed=6)
    G, eps, dt, steps = 1.0, 0.01, 1e-3, 10
    got = run_gpu(nb, nb.DIRECT_MIXED, integ, (x, y, z, vx, vy, vz, m), G, eps, dt, steps)
    ref = oracle.run(integ, oracle.DIRECT, x, y, z, vx, vy, vz, m, G, eps, dt, steps)
    # a per-body force error <= 1e-6 |a| moves positions by ~1e-6 |a| (10 dt)^2
    # and velocities by ~1e-6 |a| 10 dt over the run
    for k, key in enumerate(["x", "y", "z"]):
        assert scaled_err(got[key], ref[k]) <= 1e-8, (NAMES[integ], key)
    for k, key in enumerate(["vx", "vy", "vz"]):
        assert scaled_err(got[key], ref[3 + k]) <= 1e-6, (NAMES[integ], key)
    for k, key in enumerate(["ax", "ay", "az"]):
        assert scaled_err(got[key], ref[6 + k]) <= 1e-5, (NAMES[integ], key)


def test_plummer_1024_leapfrog_100_steps(nb, oracle):
    """The plain-method workload: N = 1024 equal-mass Plummer sphere (G = 1,
    M = 1, a = 1, virial velocities, seed 0), eps = 0.01, leapfrog KDK,
    dt = 1e-3, 100 steps; per-body accelerations and total energy vs the
    oracle (FP64, 1e-12)."""
    x, y, z, vx, vy, vz, m = nb.plummer(1024, seed=0)
    G, eps, dt, steps = 1.0, 0.01, 1e-3, 100
    with nb.Sim(nb.Config(method=nb.DIRECT_FP64, G=G, softening=eps), capacity=1024) as s:
        s.load(x, y, z, vx, vy, vz, m)
        s.step(nb.LEAPFROG, dt, steps)
        got = s.read_state()
        d = s.diagnostics()
    ref = oracle.run(oracle.LEAPFROG, oracle.DIRECT, x, y, z, vx, vy, vz, m, G, eps, dt, steps)
    for k, key in enumerate(["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"]):
        assert scaled_err(got[key], ref[k]) <= 1e-12, key
    od = oracle.diagnostics(*ref[:6], m, G, eps)
    assert d["total_softened"] == pytest.approx(od["ke"] + od["pe_soft"], rel=1e-12)
    assert d["kinetic"] == pytest.approx(od["ke"], rel=1e-12)


def test_diagnostics_match_oracle(nb, oracle):
    x, y, z, vx, vy, vz, m = nb.plummer(3000, seed=8)
    G, eps = 1.0, 0.02
    with nb.Sim(nb.Config(method=nb.DIRECT_FP64, G=G, softening=eps), capacity=3000) as s:
        s.load(x, y, z, vx, vy, vz, m)
        d = s.diagnostics()
    o = oracle.diagnostics(x, y, z, vx, vy, vz, m, G, eps)
    assert d["kinetic"] == pytest.approx(o["ke"], rel=1e-12)
    assert d["potential"] == pytest.approx(o["pe"], rel=1e-12)
    assert d["potential_softened"] == pytest.approx(o["pe_soft"], rel=1e-12)
    assert d["mass"] == pytest.approx(o["mass"], rel=1e-14)
    L = np.array(d["angular_momentum"]); Lo = np.array([o["lx"], o["ly"], o["lz"]])
    assert np.abs(L - Lo).max() <= 1e-12 * max(np.abs(Lo).max(), 1e-3)
    c = np.array(d["center_of_mass"]); co = np.array([o["comx"], o["comy"], o["comz"]])
    assert np.abs(c - co).max() <= 1e-13
    p = np.array(d["momentum"]); po = np.array([o["px"], o["py"], o["pz"]])
    assert np.abs(p - po).max() <= 1e-13


def test_earth_sun_velocity_verlet(nb, oracle):
    """CUDA/tests/test1_EarthSun.cu: Sun + Earth, direct forces, velocity
    Verlet, dt = 1/365, 366 steps, G = 4 pi^2: trajectory equals the oracle's."""
    x = np.array([0.0, 1.0]); y = np.zeros(2); z = np.zeros(2)
    vx = np.zeros(2); vy = np.array([0.0, 2 * np.pi]); vz = np.zeros(2)
    m = np.array([1.0, 3.003e-6])
    G = oracle.G_REF
    got = run_gpu(nb, nb.DIRECT_FP64, nb.VELOCITY_VERLET, (x, y, z, vx, vy, vz, m), G, 0.0,
                  1 / 365, 366)
    ref = oracle.run(oracle.VERLET, oracle.DIRECT, x, y, z, vx, vy, vz, m, G, 0.0, 1 / 365, 366)
    for k, key in enumerate(["x", "y", "z", "vx", "vy", "vz"]):
        assert scaled_err(got[key], ref[k]) <= 1e-12, key


def test_steps_are_deterministic(nb):
    st = nb.plummer(2048, seed=1)
    a = run_gpu(nb, nb.DIRECT_MIXED, nb.VELOCITY_VERLET, st, 1.0, 1e-3, 5e-4, 20)
    b = run_gpu(nb, nb.DIRECT_MIXED, nb.VELOCITY_VERLET, st, 1.0, 1e-3, 5e-4, 20)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
