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
scratch keeps the first call's contents, that near and at the size limit (where
the j-split is cut to fit the scratch) the results stay within the mixed-path
tolerance of the allocating all-pairs kernel and nothing is written past n,
and that sizes beyond the fixed limit are refused.  It is collected last so
that a stop at the first failure has already run every other test.
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


def _abs_sums(torch, x, y, z, m, eps, tile=256):
    """S_i = sum_j |pair term| in FP64 on the GPU."""
    p = torch.from_numpy(np.stack([x, y, z], 1)).cuda()
    mm = torch.from_numpy(np.ascontiguousarray(m)).cuda()
    out = torch.empty(p.shape[0], dtype=torch.float64, device="cuda")
    for i0 in range(0, p.shape[0], tile):
        d = p[None, :, :] - p[i0:i0 + tile, None, :]
        r2 = (d * d).sum(-1)
        out[i0:i0 + tile] = (mm[None, :] * torch.sqrt(r2) / (r2 + eps * eps) ** 1.5).sum(1)
    return out.cpu().numpy()


@pytest.mark.parametrize("n", [200000, LIMIT])
def test_noalloc_near_its_size_limit(nb, n):
    """From about 150,000 bodies the j-split is cut to fit the 16 MiB scratch
    (one segment at the limit), a summation order the allocating path never
    uses.  Against the allocating all-pairs kernel (NB_FLAG_MIXED_UNSORTED) on
    the same bodies: both are within 1e-6 S_i of the exact sum, so they differ
    by at most 2e-6 S_i, and by 2e-6 |a| where the sum is well conditioned;
    every output is finite and the 1024 doubles after each output array are
    left untouched."""
    torch = pytest.importorskip("torch")
    G, eps = 1.0, 1e-3
    state = nb.plummer(n, seed=21)
    cfg = nb.Config(method=nb.DIRECT_MIXED, G=G, softening=eps, flags=nb.MIXED_UNSORTED)
    with nb.Sim(cfg, capacity=n) as src:
        src.load(*state)
        src.compute_forces()
        want = _read_acc(src)
        p = src.device_arrays()
        pad = 1024
        outs = [torch.zeros(n + pad, dtype=torch.float64, device="cuda") for _ in range(3)]
        torch.cuda.synchronize()
        L = nb.lib()
        rc = L.nb_direct_mixed_forces_noalloc(n, p[0], p[1], p[2], p[9], G, eps,
                                              outs[0].data_ptr(), outs[1].data_ptr(),
                                              outs[2].data_ptr(), None)
        assert rc == 0, L.nb_last_error()
        torch.cuda.synchronize()
        got = [o.cpu().numpy() for o in outs]
    for g in got:
        assert np.isfinite(g[:n]).all()
        assert not g[n:].any()
    got = [g[:n] for g in got]
    sabs = _abs_sums(torch, state[0], state[1], state[2], state[6], eps)
    d = np.sqrt(sum((u - v) ** 2 for u, v in zip(got, want)))
    wnorm = np.sqrt(sum(w * w for w in want))
    assert (d / sabs).max() <= 2 * TOL
    assert (d / wnorm)[sabs / wnorm <= 10.0].max() <= 2 * TOL
