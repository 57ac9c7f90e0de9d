"""GPU serving loop (nb_server_*): continuous batching, admission by HBM
budget, and results that do not depend on the mix a job ran in.

"Same alone and in the mix" is checked bit for bit (the batched force kernel
sums each system alone, per-body updates are elementwise, Barnes-Hut jobs are
separate objects), which is stronger than the mixed-path tolerance.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 30


def run_alone(nb, state, steps=STEPS, **cfg):
    with nb.Server(**cfg) as s:
        jid = s.submit(state, steps)
        s.run_until_idle()
        return s.result(jid)


def test_same_alone_and_in_mix(nb):
    a = nb.plummer(3000, seed=21)          # direct job
    b = nb.disk_bulge(20000, seed=22)      # Barnes-Hut job
    others = [nb.plummer(1500, seed=23), nb.plummer(5000, seed=24), nb.disk_bulge(17000, seed=25),
              nb.plummer(700, seed=26)]
    ra, rb = run_alone(nb, a), run_alone(nb, b)
    with nb.Server() as s:
        ids = [s.submit(others[0], 40), s.submit(others[2], 25)]
        for _ in range(3):
            s.tick()
        ja = s.submit(a, STEPS)            # arrives while others are running
        ids.append(s.submit(others[1], 10))
        s.tick()
        jb = s.submit(b, STEPS)
        for _ in range(5):
            s.tick()
        ids.append(s.submit(others[3], 50))
        s.run_until_idle()
        ma, mb = s.result(ja), s.result(jb)
        st = s.stats()
    assert st["max_running"] >= 4
    for k in ra:
        assert np.array_equal(ra[k], ma[k]), ("direct", k)
        assert np.array_equal(rb[k], mb[k]), ("barnes-hut", k)


def test_direct_job_matches_oracle(nb, oracle):
    state = nb.plummer(1024, seed=30)
    r = run_alone(nb, state, steps=20, softening=0.01, dt=1e-3)
    ref = oracle.run(oracle.LEAPFROG, oracle.DIRECT, *state[:6], state[6], 1.0, 0.01, 1e-3, 20)
    for k, key in enumerate(["x", "y", "z"]):
        assert np.abs(r[key] - ref[k]).max() <= 1e-8 * np.abs(ref[k]).max()
    for k, key in enumerate(["vx", "vy", "vz"]):
        assert np.abs(r[key] - ref[3 + k]).max() <= 1e-6 * np.abs(ref[3 + k]).max()


def test_admission_by_hbm_budget(nb):
    pool = 65536
    pool_bytes = pool * (10 * 8 + 2 * 16)
    bh_bytes = 320 * 20000
    budget = pool_bytes + bh_bytes + bh_bytes // 2   # room for one Barnes-Hut job at a time
    jobs = [nb.disk_bulge(20000, seed=40 + k) for k in range(3)]
    with nb.Server(pool_bodies=pool, hbm_budget_bytes=budget) as s:
        ids = [s.submit(j, 5) for j in jobs]
        running, queued = s.tick()
        assert running == 1 and queued == 2
        s.run_until_idle()
        st = s.stats()
        for j in ids:
            s.result(j)
    assert st["jobs_finished"] == 3
    assert st["peak_device_bytes"] <= budget
    assert st["max_running"] == 1


def test_stats_and_errors(nb):
    with nb.Server(pool_bodies=4096) as s:
        with pytest.raises(nb.NBodyError) as e:
            s.submit(nb.plummer(5000, seed=1), 3)     # direct job larger than the pool
        assert e.value.status == 4
        jid = s.submit(nb.plummer(2000, seed=2), 3)
        with pytest.raises(nb.NBodyError):
            s.result(jid)                              # not finished
        s.run_until_idle()
        st = s.stats()
        assert st["steps_done"] == 3 and st["jobs_finished"] == 1
        assert st["interactions"] == pytest.approx(3 * 2000 * 1999)
        assert st["step_ms_p99"] >= st["step_ms_p50"] > 0
