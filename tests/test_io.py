"""Particle files (the reference's format, CUDA/tests/test3_correctness.cu:16-38):
host-side reading and writing through the C ABI, no GPU needed."""
import os

import numpy as np
import pytest

from conftest import ref_root

REF_PARTICLES = os.path.join(ref_root() or "", "particles_100.txt")


def test_particles_round_trip_bit_exact(nb, tmp_path):
    rng = np.random.default_rng(7)
    n = 257
    cols = [rng.normal(size=n) * 10.0 ** rng.integers(-12, 12, size=n) for _ in range(7)]
    cols[6] = np.abs(cols[6])
    p = str(tmp_path / "bodies.txt")
    nb.write_particles(p, *cols)
    back = nb.read_particles(p)
    for a, b in zip(cols, back):
        assert np.array_equal(a, b)
    with open(p) as f:
        assert f.readline().strip() == str(n)


def test_particles_empty_file_has_zero_bodies(nb, tmp_path):
    p = tmp_path / "empty.txt"
    p.write_text("0\n")
    out = nb.read_particles(str(p))
    assert all(len(v) == 0 for v in out)


@pytest.mark.parametrize("text", ["", "abc\n", "3\n1 2 3 4 5 6 7\n1 2 3\n", "-2\n", "2.5\n",
                                  "1e30\n", "nan\n", "inf\n"])
def test_particles_malformed_is_io_error(nb, tmp_path, text):
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(nb.NBodyError) as e:
        nb.read_particles(str(p))
    assert e.value.status == 8


def test_particles_missing_file_is_io_error(nb, tmp_path):
    with pytest.raises(nb.NBodyError) as e:
        nb.read_particles(str(tmp_path / "nope.txt"))
    assert e.value.status == 8
    assert "nope.txt" in nb.lib().nb_last_error().decode()


def test_particles_capacity_error(nb, tmp_path):
    import ctypes as C
    p = tmp_path / "three.txt"
    p.write_text("3\n" + "1 0 0 0 0 0 0\n" * 3)
    bufs = [np.empty(2) for _ in range(7)]
    n = C.c_size_t()
    st = nb.lib().nb_particles_read(os.fsencode(str(p)), 2, C.byref(n),
                                    *[b.ctypes.data_as(C.c_void_p) for b in bufs])
    assert st == 4 and n.value == 3


@pytest.mark.skipif(not ref_root() or not os.path.exists(REF_PARTICLES),
                    reason="reference checkout not located (REF_ROOT)")
def test_reads_reference_fixture_like_its_loader(nb):
    """Same values as a whitespace-split parse (the reference's `file >> ...`)."""
    tok = open(REF_PARTICLES).read().split()
    n = int(tok[0])
    rec = np.array([float(t) for t in tok[1:1 + 7 * n]]).reshape(n, 7)
    x, y, z, vx, vy, vz, m = nb.read_particles(REF_PARTICLES)
    assert len(x) == n == 100
    for k, col in enumerate((m, x, y, z, vx, vy, vz)):
        assert np.array_equal(col, rec[:, k])
