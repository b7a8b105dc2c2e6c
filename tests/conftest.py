"""Test configuration: the `gpu` marker, import paths and shared fixtures.

-m "not gpu" tests run anywhere (oracle, host logic, C-ABI loading); -m gpu tests need a CUDA
device and call the CUDA library through its C ABI.
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "rb-thermoparticles_gb300")
for p in (PKG, os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and librbtp.so")


@pytest.fixture(scope="session")
def lib_built():
    """Build librbtp.so in-tree (no-op when up to date) and return its path."""
    import rbtp_build  # rb-thermoparticles_gb300/rbtp_build.py
    return rbtp_build.build(host=False)


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle_py
    oracle_py.build()
    return oracle_py


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


@pytest.fixture(scope="session")
def ref_driver(lib_built, oracle_mod):
    """The reference-pin driver (oracle/ref_pin/ref_driver.cpp), built once per session; skips
    where the reference's cubins were not built (they exist only where its sources are)."""
    import refpin
    if not refpin.have_cubins():
        pytest.skip("reference pin cubins are built only where the reference sources exist")
    return refpin.build_driver()
