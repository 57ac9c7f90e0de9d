"""The reference's own FP64 GPU kernel (the "plain FP64 GPU kernel" baseline of
the benchmark) computes the reference forces, and the engine's FP64 path agrees
with it to 1e-12 relative.

The kernel is computeAccelerationNaiveKernel (CUDA/src/force_calculator_naive.cu:4-59),
compiled for sm_103a from the reference source (oracle/build_ref.sh) and launched
as ForceCalculatorNaive::computeAccelerations does.  It folds G = 4 pi^2 into
every pair (force_calculator_naive.cu:45).  Skipped where the cubin was not
built (no reference sources on the build host).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel_max(a, ref):
    d = np.sqrt(sum((u - v) ** 2 for u, v in zip(a, ref)))
    r = np.sqrt(sum(v * v for v in ref))
    mask = r > 1e-12
    return float((d[mask] / r[mask]).max(initial=0.0))


@pytest.fixture(scope="module")
def ref_kernel():
    import ref_gpu
    if not ref_gpu.available():
        pytest.skip("reference cubin not built")
    k = ref_gpu.RefNaiveKernel()
    yield k
    k.close()


@pytest.mark.parametrize("n,eps", [(1, 0.0), (255, 0.01), (1000, 0.0), (1031, 0.5)])
def test_reference_kernel_matches_oracle(ref_kernel, oracle, n, eps):
    g = oracle.MT19937(42)
    x, y, z, m = g.uniform_cube(n, order=1)
    a = ref_kernel.forces(x, y, z, m, eps)
    ref = oracle.forces_naive(x, y, z, m, oracle.G_REF, eps)
    assert rel_max(a, ref) <= TOL


def test_engine_fp64_matches_reference_kernel(ref_kernel, nb, oracle):
    x, y, z, vx, vy, vz, m = nb.plummer(4096, seed=0)
    eps = 1e-3
    a_ref = ref_kernel.forces(x, y, z, m, eps)
    with nb.Sim(nb.Config(method=nb.DIRECT_FP64, G=oracle.G_REF, softening=eps),
                capacity=4096) as s:
        s.load(x, y, z, vx, vy, vz, m)
        s.compute_forces()
        a = s.accelerations()
    assert rel_max(a, a_ref) <= TOL
