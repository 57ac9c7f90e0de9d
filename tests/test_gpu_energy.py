"""Energy drift of the mixed-precision path against the FP64 path.

The stated target: over 1000 velocity-Verlet steps the drift of the softened
total energy on the mixed path stays within 2x that of the FP64 path run from
the same start (the FP64 path is itself pinned to the CPU oracle at 1e-12).
Checked on an 8192-body Plummer sphere (eps 1e-3, dt 5e-4) for the all-pairs
and the sorted near/far mixed kernels; the benchmark reports the same ratio at
65,536 bodies.
"""
import pytest

pytestmark = pytest.mark.gpu

N, EPS, DT, STEPS = 8192, 1e-3, 5e-4, 1000


def drift(nb, method, flags=0):
    st = nb.plummer(N, seed=0)
    with nb.Sim(nb.Config(method=method, G=1.0, softening=EPS, flags=flags), capacity=N) as s:
        s.load(*st)
        e0 = s.diagnostics()["total_softened"]
        s.step(nb.VELOCITY_VERLET, DT, STEPS)
        e1 = s.diagnostics()["total_softened"]
    return (e1 - e0) / abs(e0)


@pytest.fixture(scope="module")
def fp64_drift(nb):
    return drift(nb, nb.DIRECT_FP64)


@pytest.mark.parametrize("flags", [0, 4], ids=["all_pairs", "sorted"])
def test_mixed_drift_within_twice_fp64(nb, fp64_drift, flags):
    d = drift(nb, nb.DIRECT_MIXED, flags)
    assert abs(fp64_drift) > 0.0
    assert abs(d) <= 2.0 * abs(fp64_drift), (d, fp64_drift)
