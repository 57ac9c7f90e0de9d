"""GPU batched ensemble (nb_ensemble_*) against the CPU oracle.

Tolerances are those of the mixed single-system path (tests/test_gpu_direct.py):
per body |da| <= 1e-6 sum_j |pair term|, and <= 1e-6 |a| where the sum is well
conditioned.  Bit-exact: a system gives the same forces and trajectory alone
and inside any ensemble, and the graph-replayed step loop equals the same steps
launched one by one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6


def make(nb, num, lo=32, hi=4096, seed=3):
    sizes = nb.ensemble_sizes(num, lo, hi, seed)
    return sizes, nb.plummer_ensemble(sizes, seed=seed * 1000)


def cfg(nb, eps=1e-2, flags=0):
    return nb.Config(method=nb.DIRECT_MIXED, G=1.0, softening=eps, flags=flags)


KERNELS = {"sorted": 0, "unsorted": 8}  # default / NB_FLAG_MIXED_UNSORTED


@pytest.mark.parametrize("kernel", KERNELS)
def test_forces_match_oracle(nb, oracle, kernel):
    """Both force launches: the default Hilbert-sorted near/far one and the
    all-pairs double-single one (NB_FLAG_MIXED_UNSORTED)."""
    sizes, st = make(nb, 40)
    with nb.Ensemble(cfg(nb, flags=KERNELS[kernel]), sizes) as e:
        e.load(*st)
        e.compute_forces()
        got = e.read_state()
        info = e.info()
    assert info["total_bodies"] == int(sizes.sum())
    assert info["interactions_per_eval"] == float(np.sum(sizes * (sizes - 1.0)))
    for s in range(len(sizes)):
        g = e.system(got, s)
        x, y, z, m = g["x"], g["y"], g["z"], g["m"]
        ref = oracle.forces_naive(x, y, z, m, 1.0, 1e-2)
        sabs = oracle.forces_abs_sum(x, y, z, m, 1.0, 1e-2)
        d = np.sqrt((g["ax"] - ref[0]) ** 2 + (g["ay"] - ref[1]) ** 2 + (g["az"] - ref[2]) ** 2)
        r = np.sqrt(ref[0] ** 2 + ref[1] ** 2 + ref[2] ** 2)
        assert (d / sabs).max() <= TOL, s
        well = sabs / r <= 10.0
        assert (d / r)[well].max(initial=0.0) <= TOL, s


@pytest.mark.parametrize("kernel", KERNELS)
def test_system_alone_equals_in_mix(nb, kernel):
    sizes, st = make(nb, 30, seed=5)
    with nb.Ensemble(cfg(nb, flags=KERNELS[kernel]), sizes) as e:
        e.load(*st)
        e.step(nb.RK4, 1e-3, 7)
        mix = e.read_state()
    for s in (0, 11, 29):
        a, b = int(np.sum(sizes[:s])), int(np.sum(sizes[:s + 1]))
        one = tuple(v[a:b] for v in st)
        with nb.Ensemble(cfg(nb, flags=KERNELS[kernel]), [sizes[s]]) as e1:
            e1.load(*one)
            e1.step(nb.RK4, 1e-3, 7)
            alone = e1.read_state()
        for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"):
            assert np.array_equal(alone[k], mix[k][a:b]), (s, k)


@pytest.mark.parametrize("kernel", KERNELS)
def test_graph_replay_equals_direct_launches(nb, kernel):
    """60 steps: two replayed 25-step chunks (the sorted kernel re-sorts
    before the second) and 10 direct steps, against 60 direct steps."""
    sizes, st = make(nb, 20, seed=6)
    out = []
    for profile in (False, True):  # profiling runs the steps without the graph
        with nb.Ensemble(cfg(nb, flags=KERNELS[kernel]), sizes) as e:
            e.load(*st)
            e.profile(profile)
            e.step(nb.RK4, 1e-3, 60)
            out.append(e.read_state())
            info = e.info()
            if not profile:
                assert info["graph_launches"] >= 1 and info["graph_steps"] >= 2
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k


@pytest.mark.parametrize("integ", ["rk4", "leapfrog"])
def test_trajectories_match_oracle(nb, oracle, integ):
    sizes, st = make(nb, 12, lo=32, hi=512, seed=7)
    it = nb.RK4 if integ == "rk4" else nb.LEAPFROG
    ot = oracle.RK4 if integ == "rk4" else oracle.LEAPFROG
    dt, steps = 1e-3, 10
    with nb.Ensemble(cfg(nb), sizes) as e:
        e.load(*st)
        e.step(it, dt, steps)
        got = e.read_state()
    for s in range(len(sizes)):
        g = e.system(got, s)
        a, b = e.offsets[s], e.offsets[s + 1]
        ref = oracle.run(ot, oracle.DIRECT, *(v[a:b] for v in st[:6]), st[6][a:b], 1.0, 1e-2,
                         dt, steps)
        for k, key in enumerate(["x", "y", "z"]):
            scale = np.abs(ref[k]).max()
            assert np.abs(g[key] - ref[k]).max() <= 1e-8 * scale, (s, key)
        for k, key in enumerate(["vx", "vy", "vz"]):
            scale = np.abs(ref[3 + k]).max()
            assert np.abs(g[key] - ref[3 + k]).max() <= 1e-6 * scale, (s, key)


def test_tune_reports_shapes(nb):
    sizes, st = make(nb, 50, seed=8)
    with nb.Ensemble(cfg(nb), sizes) as e:
        e.load(*st)
        ipt = e.tune()
        buckets = {int(np.log2(n)) for n in sizes}
        for b in buckets:
            assert ipt[b] in (1, 2, 4)
        info = e.info()
        assert info["work_items"] >= len(sizes)
