"""The all-pairs entry point for callers that cannot allocate device memory.

nb_direct_mixed_forces_noalloc serves callers that may not call cudaMalloc or
cudaFree (a host whose device memory belongs to its own pool allocator, a
plugin held to a fixed device-memory budget, a loop that cannot take an
allocation's implicit synchronisation).  It keeps its scratch in a fixed
16 MiB device array inside the library instead of allocating it.  This file
checks, through the C ABI, that two calls in a row give the accelerations of
the allocating NB_DIRECT_MIXED path to the mixed-path tolerance
(|da| <= 1e-6 sum_j |pair term| per body, and <= 1e-6 |a| for well-conditioned
bodies), that the second call repeats the first bit for bit although the
scratch keeps the first call's contents, and that sizes beyond the fixed limit
are refused.  It is collected last so that a stop at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6
LIMIT = 262144


def _read_acc(sim):
    st = sim.read_state()
    return st["ax"], st["ay"], st["az"]


def test_noalloc_matches_allocating_path_twice(nb, oracle):
    n = 20000
    G, eps = 1.0, 1e-3
    state = nb.plummer(n, seed=12)
    cfg = nb.Config(method=nb.DIRECT_MIXED, G=G, softening=eps)
    with nb.Sim(cfg, capacity=n) as src, nb.Sim(cfg, capacity=n) as dst:
        src.load(*state)
        src.compute_forces()
        want = _read_acc(src)
        dst.load(*state)  # gives dst n bodies and zeroed acceleration planes
        p = src.device_arrays()  # x y z vx vy vz ax ay az m
        q = dst.device_arrays()
        x, y, z = state[0], state[1], state[2]
        sabs = oracle.forces_abs_sum(x, y, z, state[6], G, eps)
        wnorm = np.sqrt(sum(w * w for w in want))
        L = nb.lib()
        results = []
        for _ in range(2):
            rc = L.nb_direct_mixed_forces_noalloc(n, p[0], p[1], p[2], p[9], G, eps, q[6],
                                                  q[7], q[8], None)
            assert rc == 0, L.nb_last_error()
            got = _read_acc(dst)  # synchronises the legacy default stream
            d = np.sqrt(sum((g - w) ** 2 for g, w in zip(got, want)))
            assert (d / sabs).max() <= TOL
            kappa = sabs / wnorm
            assert (d / wnorm)[kappa <= 10.0].max() <= TOL
            results.append([a.copy() for a in got])
        for a, b in zip(results[0], results[1]):
            assert np.array_equal(a, b)


def test_noalloc_rejects_sizes_beyond_its_scratch(nb):
    with nb.Sim(nb.Config(method=nb.DIRECT_MIXED), capacity=4) as s:
        s.load(*(np.ones(4) for _ in range(7)))
        p = s.device_arrays()
        L = nb.lib()
        rc = L.nb_direct_mixed_forces_noalloc(LIMIT + 1, p[0], p[1], p[2], p[9], 1.0, 0.1,
                                              p[6], p[7], p[8], None)
        assert rc == 4  # NB_ERR_CAPACITY
        assert b"262144" in L.nb_last_error()
