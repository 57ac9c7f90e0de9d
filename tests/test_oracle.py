"""Pins the CPU oracle (oracle/nbody_oracle.c) before any GPU result is
compared with it:
  - against the reference's published golden outputs (seed-42 force error
    tables, the Earth-Sun trajectory CPU/orbit.csv, std::mt19937 draws);
  - against the reference's own CPU classes compiled here (oracle/_ref), bit
    for bit, when that library was built (skipped elsewhere);
  - the 63-bit Morton / octree rule against the reference's node-pool tree.
"""
import csv
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _close6(a, b):
    """Printed with 6 significant digits by the reference."""
    return abs(a - b) <= 5e-6 * abs(b) + 1e-300


def test_mt19937_matches_std(oracle):
    fx = json.load(open(os.path.join(GOLDEN, "mt19937_seed42.json")))
    g = oracle.MT19937(42)
    assert [g.u32() for _ in range(8)] == fx["u32"]
    g = oracle.MT19937(42)
    assert [g.uniform(-100.0, 100.0) for _ in range(8)] == fx["uniform_m100_100"]


def test_force_benchmark_golden_tables(oracle):
    """CPU/tests/test2_ForceBenchmark.cpp with one rng(42) across 5 runs; the
    oracle's direct, pointer-BH and node-pool-BH forces must reproduce every
    printed error statistic.  N = 10000 cases are checked for runs 1-2 only
    to keep the CPU suite short (the generator still advances through them)."""
    fx = json.load(open(os.path.join(GOLDEN, "force_benchmark_seed42.json")))
    g = oracle.MT19937(42)
    G = oracle.G_REF
    checked = 0
    for run in fx["runs"]:
        for case in run["cases"]:
            n = case["n"]
            x, y, z, m = g.uniform_cube(n, order=0)
            if n >= 10000 and run["run"] > 2:
                continue
            a = oracle.forces_naive(x, y, z, m, G, 0.0)
            bh = oracle.error_stats(oracle.forces_bh_ptr(x, y, z, m, G, 0.0, 0.5), a)
            bo = oracle.error_stats(oracle.forces_bh_opt(x, y, z, m, G, 0.0, 0.5, 8), a)
            for key, want in case["bh"].items():
                assert _close6(bh[key], want), (run["run"], n, "bh", key, bh[key], want)
            for key, want in case["bh_opt"].items():
                assert _close6(bo[key], want), (run["run"], n, "bh_opt", key, bo[key], want)
            checked += 1
    assert checked >= 17


def test_orbit_csv_golden(oracle):
    """CPU/src/n-body.cpp: Sun + Earth, pointer BH theta 0.3, velocity Verlet,
    dt = 1/365, 366 steps, diagnostics after every step (printed %.15f)."""
    x = np.array([0.0, 1.0]); y = np.zeros(2); z = np.zeros(2)
    vx = np.zeros(2); vy = np.array([0.0, 2 * np.pi]); vz = np.zeros(2)
    m = np.array([1.0, 3.003e-6])
    G = oracle.G_REF
    rows = {int(r["row"]): r for r in csv.DictReader(open(os.path.join(GOLDEN,
                                                                        "orbit_earth_sun.csv")))}
    state = (x, y, z, vx, vy, vz)
    dt = 1.0 / 365.0
    checked = 0
    for step in range(0, 367):
        if step > 0:
            st = oracle.run(oracle.VERLET, oracle.BH_PTR, *state, m, G, 0.0, dt, 1, theta=0.3)
            state = st[:6]
        if step not in rows or step == 0:
            continue
        X, Y, Z, VX, VY, VZ = state
        d = oracle.diagnostics(X, Y, Z, VX, VY, VZ, m, G, 0.0)
        pe = oracle.potential_energy_seq(X, Y, Z, m, G)
        got = [X[1], Y[1], Z[1], X[0], Y[0], Z[0], d["ke"], pe, d["ke"] + pe, d["lx"], d["ly"],
               d["lz"], d["comx"], d["comy"], d["comz"]]
        r = rows[step]
        want = [r[k] for k in ["earth_x", "earth_y", "earth_z", "sun_x", "sun_y", "sun_z",
                               "kinetic_energy", "potential_energy", "total_energy",
                               "angular_momentum_x", "angular_momentum_y",
                               "angular_momentum_z", "center_of_mass_x", "center_of_mass_y",
                               "center_of_mass_z"]]
        # The published file was written on another machine; rebuilding the
        # reference here reproduces it to within 1e-14 (last printed digit).
        diff = max(abs(float("%.15f" % g_) - float(w)) for g_, w in zip(got, want))
        assert diff <= 2e-14, (step, diff)
        checked += 1
    assert checked > 60


def test_earth_sun_integrator_errors(oracle):
    """CPU/tests/test1_EarthSun.cpp: every integrator against a velocity-Verlet
    run, 365 steps; the known answers (velocity Verlet exact, leapfrog at the
    round-off level, RK4 ~3e-4 in position)."""
    x = np.array([0.0, 1.0]); y = np.zeros(2); z = np.zeros(2)
    vx = np.zeros(2); vy = np.array([0.0, 2 * np.pi]); vz = np.zeros(2)
    m = np.array([1.0, 3.003e-6])
    G = oracle.G_REF
    dt = 1.0 / 365.0
    ref = oracle.run(oracle.VERLET, oracle.DIRECT, x, y, z, vx, vy, vz, m, G, 0.0, dt, 365)

    def perr(s):
        return float(np.mean(np.sqrt((s[0] - ref[0]) ** 2 + (s[1] - ref[1]) ** 2 +
                                     (s[2] - ref[2]) ** 2)))

    errs = {k: perr(oracle.run(k, oracle.DIRECT, x, y, z, vx, vy, vz, m, G, 0.0, dt, 365))
            for k in (oracle.EULER, oracle.EULER_CROMER, oracle.LEAPFROG, oracle.VERLET,
                      oracle.RK4)}
    assert errs[oracle.VERLET] == 0.0
    assert errs[oracle.LEAPFROG] < 1e-12
    assert 1e-4 < errs[oracle.RK4] < 1e-3
    assert errs[oracle.EULER] > errs[oracle.EULER_CROMER] > errs[oracle.RK4]


needs_ref = pytest.mark.skipif(
    not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                    "libnbref.so")),
    reason="reference CPU sources were not compiled in this checkout")


@needs_ref
@pytest.mark.parametrize("method", [0, 1, 2])
def test_forces_bit_exact_vs_reference_build(oracle, method):
    g = oracle.MT19937(7)
    x, y, z, m = g.uniform_cube(700, order=0)
    R = oracle.ref()
    n = len(x)
    got = {0: lambda: oracle.forces_naive(x, y, z, m, oracle.G_REF, 0.1),
           1: lambda: oracle.forces_bh_opt(x, y, z, m, oracle.G_REF, 0.1, 0.6, 5),
           2: lambda: oracle.forces_bh_ptr(x, y, z, m, oracle.G_REF, 0.1, 0.6)}[method]()
    ra = [np.empty(n) for _ in range(3)]
    R.ref_forces(method, n, x, y, z, m, 0.1, 0.6, 5, *ra)
    for u, v in zip(got, ra):
        assert np.array_equal(u, v)


@needs_ref
@pytest.mark.parametrize("integ", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("method", [0, 1, 2])
def test_integrators_bit_exact_vs_reference_build(oracle, integ, method):
    g = oracle.MT19937(11)
    x, y, z, m = g.uniform_cube(300, order=1)
    rng = np.random.default_rng(3)
    vx, vy, vz = (rng.normal(size=300) for _ in range(3))
    dt, steps = 1e-3, 5
    mine = oracle.run(integ, method, x, y, z, vx, vy, vz, m, oracle.G_REF, 0.5, dt, steps,
                      theta=0.5, leaf_capacity=8)
    st = [a.copy() for a in (x, y, z, vx, vy, vz)]
    acc = [np.zeros(300) for _ in range(3)]
    oracle.ref().ref_run(integ, method, 300, *st, m, *acc, 0.5, 0.5, 8, dt, steps)
    for u, v in zip(mine, st + acc):
        assert np.array_equal(u, v)


@needs_ref
def test_diagnostics_vs_reference_build(oracle):
    g = oracle.MT19937(5)
    x, y, z, m = g.uniform_cube(200, order=0)
    rng = np.random.default_rng(0)
    vx, vy, vz = (rng.normal(size=200) for _ in range(3))
    out = np.empty(9)
    oracle.ref().ref_diagnostics(200, x, y, z, vx, vy, vz, m, out)
    d = oracle.diagnostics(x, y, z, vx, vy, vz, m, oracle.G_REF, 0.0)
    assert d["ke"] == out[0]
    assert oracle.potential_energy_seq(x, y, z, m, oracle.G_REF) == out[1]
    assert d["pe"] == pytest.approx(out[1], rel=1e-13)
    assert [d["lx"], d["ly"], d["lz"]] == list(out[3:6])
    assert [d["comx"], d["comy"], d["comz"]] == list(out[6:9])


def _canonical_oracle_tree(oracle, x, y, z, leaf):
    codes, root = oracle.morton63(x, y, z)
    sc, order = oracle.sort_codes(codes)
    levels = oracle.split_levels(root[3])
    t = oracle.octree(sc, leaf, levels)
    out = set()
    for d, p, c, lf in zip(t["depth"], t["prefix"], t["count"], t["is_leaf"]):
        # de-interleave the 3*d-bit prefix (x high) into per-axis cell indices
        cx = cy = cz = 0
        p = int(p)
        for k in range(int(d)):
            dig = (p >> (3 * (int(d) - 1 - k))) & 7
            cx = 2 * cx + ((dig >> 2) & 1)
            cy = 2 * cy + ((dig >> 1) & 1)
            cz = 2 * cz + (dig & 1)
        out.add((int(d), cx, cy, cz, int(c), bool(lf)))
    return out


def _canonical_cpu_tree(dump):
    return {(int(d), int(cx), int(cy), int(cz), int(c), bool(lf))
            for d, cx, cy, cz, c, lf in zip(dump["depth"], dump["cx"], dump["cy"], dump["cz"],
                                            dump["count"], dump["is_leaf"]) if c > 0}


@pytest.mark.parametrize("leaf", [1, 8, 16])
def test_octree_rule_equals_cpu_node_pool_tree(oracle, leaf):
    """The non-empty cells of the reference's node-pool tree (restated) equal
    the octree read off the sorted 63-bit Morton codes."""
    g = oracle.MT19937(42)
    x, y, z, m = g.uniform_cube(3000, order=0)
    dump = oracle.bh_opt_dump(x, y, z, m, leaf)
    assert _canonical_cpu_tree(dump) == _canonical_oracle_tree(oracle, x, y, z, leaf)


@needs_ref
@pytest.mark.parametrize("leaf", [1, 8])
def test_octree_rule_equals_reference_build_tree(oracle, leaf):
    g = oracle.MT19937(43)
    x, y, z, m = g.uniform_cube(2000, order=0)
    dump = oracle.bh_opt_dump(x, y, z, m, leaf, use_ref=True)
    assert _canonical_cpu_tree(dump) == _canonical_oracle_tree(oracle, x, y, z, leaf)


def test_sort_is_stable(oracle):
    codes = np.array([5, 3, 5, 1, 3, 5, 0], dtype=np.uint64)
    sc, order = oracle.sort_codes(codes)
    assert sc.tolist() == [0, 1, 3, 3, 5, 5, 5]
    assert order.tolist() == [6, 3, 1, 4, 0, 2, 5]


def test_split_levels(oracle):
    assert oracle.split_levels(200.0) == 21
    assert oracle.split_levels(1e-8) == 3   # 1e-8/2^3 = 1.25e-9 >= 1e-9 > 6.25e-10
    assert oracle.split_levels(1e-9) == 0


@pytest.mark.parametrize("kind,n,seed", [("plummer", 1, 0), ("plummer", 4097, 3),
                                         ("plummer", 65536, 0), ("disk_bulge", 5, 1),
                                         ("disk_bulge", 20000, 8)])
def test_oracle_generators_match_the_engine(oracle, nb, kind, n, seed):
    """The oracle's restated workload generators give the engine's bits, so
    the CPU arms of the benchmark build the same inputs without loading the
    engine library."""
    a = getattr(oracle, kind)(n, seed)
    b = getattr(nb, kind)(n, seed)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
