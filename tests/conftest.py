"""Shared test setup.

``-m "not gpu"`` runs everywhere (the CPU oracle, the generator, the host-side
library and CLI paths); ``-m gpu`` needs a CUDA device (a GB300) and calls the
library through its C ABI.  The session builds the library, the CLI and the oracle
once (incremental: nothing is recompiled when up to date).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    from warp_reactor_gb300 import build
    return build.build_all()


@pytest.fixture(scope="session")
def wr(built):
    import warp_reactor_gb300
    return warp_reactor_gb300


@pytest.fixture(scope="session")
def oracle_port(built):
    from oracle import oracle
    return oracle.load("port")


@pytest.fixture(scope="session")
def oracle_prec(built):
    from oracle import oracle
    return oracle.load("prec")


@pytest.fixture(scope="session")
def oracle_libm(built):
    from oracle import oracle
    return oracle.load("libm")


@pytest.fixture(scope="session")
def gpu():
    """Skip unless a CUDA device is present (the GPU tests are marked gpu)."""
    import ctypes
    try:
        cudart = ctypes.CDLL("libcudart.so")
    except OSError:
        from warp_reactor_gb300 import build
        cudart = ctypes.CDLL(os.path.join(build._cuda_home(), "lib64", "libcudart.so"))
    n = ctypes.c_int(0)
    if cudart.cudaGetDeviceCount(ctypes.byref(n)) != 0 or n.value < 1:
        pytest.fail("no CUDA device: the gpu tests need a GB300")
    return n.value
