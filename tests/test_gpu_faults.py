"""Failure handling without a GPU fault.

Allocation failures are injected on the host (nb_debug_fail_device_allocations:
the library's own allocator returns NB_ERR_OUT_OF_MEMORY before calling CUDA),
and serving jobs are cancelled through the API.  No CUDA call fails and the
device is never faulted.  Each case checks that the error is reported with its
status and message, and that the objects keep working afterwards: a retried
evaluation gives the same bits as a clean one, and the other jobs of a server
finish with the same bits as when run alone.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OOM, CANCELLED = 3, 9


@pytest.fixture(autouse=True)
def disarmed(nb):
    nb.debug_fail_device_allocations(-1)
    yield
    nb.debug_fail_device_allocations(-1)


def forces(nb, cfg, state):
    with nb.Sim(cfg, capacity=len(state[0])) as s:
        s.load(*state)
        s.compute_forces()
        return s.accelerations()


@pytest.mark.parametrize("method", ["barnes_hut", "mixed_sorted"])
def test_injected_allocation_failure_then_retry(nb, method):
    """Fail the k-th device allocation of create + load + evaluate, for every
    k until a run needs no more: each failure is NB_ERR_OUT_OF_MEMORY with the
    injected message, and the same simulation, retried, gives the clean bits."""
    n = 20000
    st = nb.disk_bulge(n, seed=7)
    if method == "barnes_hut":
        cfg = nb.Config(method=nb.BARNES_HUT, G=1.0, softening=1e-3, theta=0.5)
    else:
        cfg = nb.Config(method=nb.DIRECT_MIXED, G=1.0, softening=1e-3, flags=nb.MIXED_SORTED)
    ref = forces(nb, cfg, st)
    failures = 0
    for k in range(64):
        nb.debug_fail_device_allocations(k)
        sim, failed = None, False
        try:
            sim = nb.Sim(cfg, capacity=n)
            sim.load(*st)
            sim.compute_forces()
        except nb.NBodyError as e:
            failed = True
            assert e.status == OOM and "injected allocation failure" in str(e), str(e)
        finally:
            nb.debug_fail_device_allocations(-1)
        if failed:
            failures += 1
            if sim is None:
                continue                   # nb_create itself failed: nothing to retry
            sim.load(*st)
            sim.compute_forces()
        got = sim.accelerations()
        sim.close()
        for u, v in zip(got, ref):
            assert np.array_equal(u, v), (method, k)
        if not failed:
            break                          # k is past the run's last allocation
    assert failures >= 2


def run_alone(nb, state, steps):
    with nb.Server() as s:
        jid = s.submit(state, steps)
        s.run_until_idle()
        return s.result(jid)


def same(r1, r2):
    return all(np.array_equal(r1[k], r2[k]) for k in r1)


@pytest.mark.parametrize("fail_at", [0, 1])
def test_server_isolates_a_failed_job(nb, fail_at):
    """The device allocation of a Barnes-Hut job fails (at its admission, or,
    with fail_at 1, possibly in its first step): that job ends with the error,
    the tick succeeds, and the other jobs give their alone results."""
    direct = nb.plummer(2000, seed=51)
    bad = nb.disk_bulge(20000, seed=52)
    later = nb.disk_bulge(18000, seed=53)
    alone_direct, alone_later = run_alone(nb, direct, 10), run_alone(nb, later, 10)
    with nb.Server() as s:
        jd = s.submit(direct, 10)
        s.tick()
        jbad = s.submit(bad, 10)           # the only Barnes-Hut job of the next tick
        nb.debug_fail_device_allocations(fail_at)
        s.tick()
        nb.debug_fail_device_allocations(-1)
        jl = s.submit(later, 10)
        s.run_until_idle()
        with pytest.raises(nb.NBodyError) as e:
            s.result(jbad)
        assert e.value.status == OOM and "injected allocation failure" in str(e.value)
        rd, rl = s.result(jd), s.result(jl)
        st = s.stats()
    assert st["jobs_failed"] == 1 and st["jobs_finished"] == 3
    assert same(rd, alone_direct) and same(rl, alone_later)


def test_cancel_queued_and_running_jobs(nb):
    """Cancelling frees a job's resources at once: a queued job leaves the
    queue, a running direct job gives its pool slot back (a job that needs it
    is admitted next tick), a running Barnes-Hut job its budget.  Cancelled
    results are NB_ERR_CANCELLED; the remaining job gives its alone bits."""
    keep = nb.plummer(3000, seed=61)
    alone_keep = run_alone(nb, keep, 20)
    with nb.Server(pool_bodies=10000) as s:
        a = s.submit(keep, 20)
        b = s.submit(nb.plummer(4000, seed=62), 20)
        c = s.submit(nb.disk_bulge(20000, seed=63), 20)
        s.tick()
        s.tick()
        d = s.submit(nb.plummer(6000, seed=64), 5)   # 3000 + 4000 + 6000 > 10000: waits
        running, queued = s.tick()
        assert (running, queued) == (3, 1)
        e = s.submit(nb.plummer(5000, seed=65), 5)
        s.cancel(e)                                  # queued
        s.cancel(c)                                  # running, Barnes-Hut
        s.cancel(b)                                  # running, direct: frees 4000 slots
        running, queued = s.tick()                   # d fits in [3000, 10000) now
        assert (running, queued) == (2, 0)
        with pytest.raises(nb.NBodyError) as err:
            s.cancel(12345)
        assert err.value.status == 1
        s.run_until_idle()
        with pytest.raises(nb.NBodyError) as err:
            s.cancel(a)                              # already finished
        assert err.value.status == 1
        for j in (b, c, e):
            with pytest.raises(nb.NBodyError) as err:
                s.result(j)
            assert err.value.status == CANCELLED
        ra = s.result(a)
        s.result(d)
        st = s.stats()
    assert st["jobs_cancelled"] == 3 and st["jobs_failed"] == 0
    assert same(ra, alone_keep)
