"""Shared fixtures: package import, built libraries, the CPU oracle."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import __graft_entry__ as graft  # noqa: E402

PKG = graft.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def pkg():
    return PKG


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle library (test infrastructure), built on demand."""
    from pdesolver_gb300 import build
    path = build.build_oracle()
    lib = C.CDLL(path)
    lib.oracle_pressure.restype = C.c_double
    lib.oracle_calc_norm.restype = C.c_double
    lib.oracle_logavg.restype = C.c_double
    lib.oracle_logavg.argtypes = [C.c_double, C.c_double]
    return lib


@pytest.fixture(scope="session")
def gpu_lib():
    """libeulergpu.so, built on demand (nvcc cross-compiles without a GPU)."""
    from pdesolver_gb300 import build
    build.build_library()
    from pdesolver_gb300 import eulergpu
    return eulergpu.library()


def oracle_residual(oracle, desc, params, q):
    from pdesolver_gb300 import abi
    res = np.zeros_like(q)
    st = oracle.oracle_eval_residual(C.byref(desc.desc), C.byref(params), abi.dptr(q), abi.dptr(res))
    assert st == 0, st
    return res
