"""Shared test set-up: import paths, the `gpu` marker, oracle/engine handles."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(REPO, "n-body-gravity-simulation_gb300")
ORACLE_DIR = os.path.join(REPO, "oracle")
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (REPO, PKG_DIR, ORACLE_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)


def ref_root():
    """Where the reference checkout lies, or None: $REF_ROOT, else the location
    oracle/build_ref.sh recorded when it compiled the reference here
    (oracle/_ref/ref_root.txt).  Tests that read reference files skip without it."""
    env = os.environ.get("REF_ROOT")
    if env:
        return env if os.path.isdir(env) else None
    rec = os.path.join(ORACLE_DIR, "_ref", "ref_root.txt")
    if os.path.exists(rec):
        path = open(rec).read().strip()
        return path if os.path.isdir(path) else None
    return None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    if not os.path.exists(O.LIB_PATH):
        O.build(with_ref=False)
    return O


@pytest.fixture(scope="session")
def nb():
    """The engine's Python front end; on a GPU run the library must exist."""
    import nbody_gb300
    if not os.path.exists(nbody_gb300.LIB_PATH):
        import build as pkg_build  # n-body-gravity-simulation_gb300/build.py
        pkg_build.build()
    nbody_gb300.lib()
    return nbody_gb300
