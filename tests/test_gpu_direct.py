"""GPU parity of the all-pairs force kernels against the CPU oracle.

Tolerances (written here, checked per body):
  FP64 path  : |a_gpu - a_ref| / |a_ref| <= 1e-12
  mixed path : |a_gpu - a_ref| / |a_ref| <= 1e-6
with the reference benchmark's convention that bodies with |a_ref| <= 1e-12
are excluded from the relative error (CPU/tests/test2_ForceBenchmark.cpp:102-112);
those must still agree to 1e-6 of the RMS acceleration.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_MIXED = 1e-6


def rel_errors(a, ref):
    d = np.sqrt(sum((u - v) ** 2 for u, v in zip(a, ref)))
    r = np.sqrt(sum(v * v for v in ref))
    rms = np.sqrt(np.mean(r * r)) if len(r) else 1.0
    mask = r > 1e-12
    rel = d[mask] / r[mask]
    return (rel.max() if rel.size else 0.0), (d.max() / rms if rms > 0 else d.max())


def cube(oracle, n, seed=42):
    g = oracle.MT19937(seed)
    x, y, z, m = g.uniform_cube(n, order=1)
    return x, y, z, np.zeros(n), np.zeros(n), np.zeros(n), m


def gpu_forces(nb, method, state, G, eps):
    n = len(state[0])
    with nb.Sim(nb.Config(method=method, G=G, softening=eps), capacity=max(n, 1)) as s:
        s.load(*state)
        s.compute_forces()
        return s.accelerations()


SIZES = [1, 2, 3, 31, 100, 255, 256, 257, 1000, 1025, 4097]


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("eps", [0.0, 0.5])
def test_fp64_matches_oracle(nb, oracle, n, eps):
    st = cube(oracle, n)
    a = gpu_forces(nb, nb.DIRECT_FP64, st, oracle.G_REF, eps)
    ref = oracle.forces_naive(st[0], st[1], st[2], st[6], oracle.G_REF, eps)
    mx, rms = rel_errors(a, ref)
    assert mx <= TOL_FP64 and rms <= TOL_FP64, (mx, rms)


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("eps", [0.0, 0.5])
def test_mixed_matches_oracle(nb, oracle, n, eps):
    st = cube(oracle, n)
    a = gpu_forces(nb, nb.DIRECT_MIXED, st, oracle.G_REF, eps)
    ref = oracle.forces_naive(st[0], st[1], st[2], st[6], oracle.G_REF, eps)
    mx, rms = rel_errors(a, ref)
    assert mx <= TOL_MIXED and rms <= TOL_MIXED, (mx, rms)


def test_single_body_feels_nothing(nb, oracle):
    st = tuple(np.array([v]) for v in (1.5, -2.0, 3.0, 0.1, 0.2, 0.3, 2.0))
    for method in (nb.DIRECT_FP64, nb.DIRECT_MIXED):
        a = gpu_forces(nb, method, st, 1.0, 0.0)
        assert all(v[0] == 0.0 for v in a)


@pytest.mark.parametrize("method", ["fp64", "mixed"])
def test_plummer_softened(nb, oracle, method):
    n = 4096
    x, y, z, vx, vy, vz, m = nb.plummer(n, seed=0)
    meth = nb.DIRECT_FP64 if method == "fp64" else nb.DIRECT_MIXED
    a = gpu_forces(nb, meth, (x, y, z, vx, vy, vz, m), 1.0, 1e-3)
    ref = oracle.forces_naive(x, y, z, m, 1.0, 1e-3)
    mx, rms = rel_errors(a, ref)
    tol = TOL_FP64 if method == "fp64" else TOL_MIXED
    assert mx <= tol and rms <= tol, (mx, rms)


def test_mixed_close_pairs_far_from_origin(nb, oracle):
    """Tight pairs at |x| ~ 1e3: the double-single displacement keeps the pair
    force accurate where an FP32 position (ulp ~ 6e-5) would not."""
    rng = np.random.default_rng(1)
    n = 512
    c = rng.uniform(-1, 1, size=(n // 2, 3)) * 1e3
    off = rng.normal(size=(n // 2, 3)) * 1e-3
    p = np.concatenate([c, c + off])
    x, y, z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
    m = rng.uniform(0.5, 2.0, n)
    zero = np.zeros(n)
    a = gpu_forces(nb, nb.DIRECT_MIXED, (x, y, z, zero, zero, zero, m), 1.0, 1e-4)
    ref = oracle.forces_naive(x, y, z, m, 1.0, 1e-4)
    mx, rms = rel_errors(a, ref)
    assert mx <= TOL_MIXED, mx


@pytest.mark.parametrize("method", ["fp64", "mixed"])
def test_forces_are_deterministic(nb, oracle, method):
    st = cube(oracle, 3000, seed=9)
    meth = nb.DIRECT_FP64 if method == "fp64" else nb.DIRECT_MIXED
    a1 = gpu_forces(nb, meth, st, 1.0, 0.01)
    a2 = gpu_forces(nb, meth, st, 1.0, 0.01)
    for u, v in zip(a1, a2):
        assert np.array_equal(u, v)


def test_capacity_and_empty_errors(nb, oracle):
    with nb.Sim(nb.Config(method=nb.DIRECT_MIXED), capacity=4) as s:
        with pytest.raises(nb.NBodyError) as e:
            s.compute_forces()
        assert e.value.status == 5  # nothing loaded
        big = tuple(np.zeros(5) for _ in range(7))
        with pytest.raises(nb.NBodyError) as e:
            s.load(*big)
        assert e.value.status == 4  # capacity
        with pytest.raises(nb.NBodyError) as e:
            s.step(99, 0.1)
        assert e.value.status == 1


def test_config_switch_between_paths(nb, oracle):
    st = cube(oracle, 700, seed=2)
    ref = oracle.forces_naive(st[0], st[1], st[2], st[6], 2.0, 0.3)
    with nb.Sim(nb.Config(method=nb.DIRECT_FP64, G=2.0, softening=0.3), capacity=700) as s:
        s.load(*st)
        s.compute_forces()
        assert rel_errors(s.accelerations(), ref)[0] <= TOL_FP64
        s.config = nb.Config(method=nb.DIRECT_MIXED, G=2.0, softening=0.3)
        s.compute_forces()
        assert rel_errors(s.accelerations(), ref)[0] <= TOL_MIXED
