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
    lib.oracle_functional_pressure.restype = C.c_double
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


def oracle_jacobian(oracle, desc, params, ms, q):
    """element blocks [E][n][n] and coupling blocks [I][2][nb][nb] (FP64)."""
    from pdesolver_gb300 import abi
    nv = ms.numDofPerNode
    n = ms.sbp.numnodes * nv
    nb = ms.sbp.stencilsize * nv
    diag = np.zeros((ms.numEl, n, n))
    cpl = np.zeros((max(ms.numInterfaces, 1), 2, nb, nb))
    st = oracle.oracle_eval_jacobian(C.byref(desc.desc), C.byref(params), abi.dptr(q),
                                     abi.dptr(diag), abi.dptr(cpl))
    assert st == 0, st
    return diag, cpl[:ms.numInterfaces]


def oracle_jvp(oracle, desc, params, q, v):
    from pdesolver_gb300 import abi
    res = np.zeros_like(q)
    jv = np.zeros_like(q)
    st = oracle.oracle_residual_jvp(C.byref(desc.desc), C.byref(params), abi.dptr(q),
                                    abi.dptr(np.ascontiguousarray(v)), abi.dptr(res), abi.dptr(jv))
    assert st == 0, st
    return jv


def block_apply(ms, diag, cpl, x):
    """y = J x for the element-block storage (host, numpy)."""
    E, n = diag.shape[0], diag.shape[1]
    op = ms.sbp
    nv = ms.numDofPerNode
    xe = x.reshape(E, n)
    # diag[e][c][r]: column-major -> y_r = sum_c D[c][r] x_c
    y = np.einsum("ecr,ec->er", diag, xe)
    for k, (eL, eR, fL, fR, o) in enumerate(ms.interfaces):
        iL = (op.perm[fL][:, None] * nv + np.arange(nv)[None]).ravel()
        iR = (op.perm[fR][:, None] * nv + np.arange(nv)[None]).ravel()
        y[eL, iL] += cpl[k, 0].T @ xe[eR, iR]
        y[eR, iR] += cpl[k, 1].T @ xe[eL, iL]
    return y.reshape(x.shape)


def block_apply_t(ms, diag, cpl, x):
    """y = J^T x for the element-block storage (host, numpy)."""
    E, n = diag.shape[0], diag.shape[1]
    op = ms.sbp
    nv = ms.numDofPerNode
    xe = x.reshape(E, n)
    y = np.einsum("ecr,er->ec", diag, xe)
    for k, (eL, eR, fL, fR, o) in enumerate(ms.interfaces):
        iL = (op.perm[fL][:, None] * nv + np.arange(nv)[None]).ravel()
        iR = (op.perm[fR][:, None] * nv + np.arange(nv)[None]).ravel()
        y[eR, iR] += cpl[k, 0] @ xe[eL, iL]
        y[eL, iL] += cpl[k, 1] @ xe[eR, iR]
    return y.reshape(x.shape)
