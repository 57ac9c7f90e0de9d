"""Step graphs: on a capturable stream, nb_step captures one step into a CUDA
graph (the second of two like steps) and replays it.  A replayed run must give
the same bits as the same run stepped launch by launch (the legacy default
stream, which is never captured), across methods and integrators, and across
changes that must drop the graph (dt, integrator, a load, a config change)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CASES = [("fp64", "leapfrog"), ("fp64", "rk4"), ("fp64", "euler"), ("mixed", "verlet"),
         ("bh", "leapfrog"), ("bh", "verlet")]


def run(nb, method, integ, stream, steps=6, dt=1e-3, n=3000):
    meth = {"fp64": nb.DIRECT_FP64, "mixed": nb.DIRECT_MIXED, "bh": nb.BARNES_HUT}[method]
    it = {"leapfrog": nb.LEAPFROG, "verlet": nb.VELOCITY_VERLET, "rk4": nb.RK4,
          "euler": nb.EULER}[integ]
    st = nb.plummer(n, seed=17)
    cfg = nb.Config(method=meth, G=1.0, softening=0.01, theta=0.6)
    with nb.Sim(cfg, capacity=n, stream=stream) as s:
        s.load(*st)
        for _ in range(steps):
            s.step(it, dt, 1)
        s.synchronize()
        return s.read_state()


@pytest.mark.parametrize("method,integ", CASES)
def test_graph_replay_matches_direct_launches(nb, method, integ):
    side = torch.cuda.Stream()
    a = run(nb, method, integ, None)
    launches0 = nb.kernel_launch_count()
    b = run(nb, method, integ, side.cuda_stream)
    assert nb.kernel_launch_count() > launches0
    for k in a:
        assert np.array_equal(a[k], b[k]), (method, integ, k)


def test_graph_dropped_on_changes(nb):
    """dt change, integrator change, reload and config change between steps."""
    side = torch.cuda.Stream()
    n = 2000
    st = nb.plummer(n, seed=3)
    st2 = nb.plummer(n, seed=4)

    def script(stream):
        cfg = nb.Config(method=nb.DIRECT_FP64, G=1.0, softening=0.01)
        with nb.Sim(cfg, capacity=n, stream=stream) as s:
            s.load(*st)
            s.step(nb.LEAPFROG, 1e-3, 4)
            s.step(nb.LEAPFROG, 2e-3, 3)
            s.step(nb.VELOCITY_VERLET, 2e-3, 3)
            s.load(*st2)
            s.step(nb.VELOCITY_VERLET, 2e-3, 3)
            s.config = nb.Config(method=nb.DIRECT_FP64, G=2.0, softening=0.02)
            s.step(nb.VELOCITY_VERLET, 2e-3, 3)
            s.invalidate_forces()
            s.step(nb.VELOCITY_VERLET, 2e-3, 3)
            s.synchronize()
            return s.read_state()

    a, b = script(None), script(side.cuda_stream)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_bh_info_after_replays(nb):
    """The node count of a replayed build is read back, not a stale copy."""
    side = torch.cuda.Stream()
    n = 5000
    st = nb.disk_bulge(n, seed=2)
    cfg = nb.Config(method=nb.BARNES_HUT, G=1.0, softening=1e-3, theta=0.5)
    with nb.Sim(cfg, capacity=n, stream=side.cuda_stream) as s, \
            nb.Sim(cfg, capacity=n) as ref:
        s.load(*st)
        ref.load(*st)
        for _ in range(8):
            s.step(nb.LEAPFROG, 5e-3, 1)
            ref.step(nb.LEAPFROG, 5e-3, 1)
            assert s.bh_info()["num_nodes"] == ref.bh_info()["num_nodes"]
