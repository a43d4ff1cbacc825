"""CPU oracle of the steady solve with p-continuation (test infrastructure).

Only the tests and bench.py's CPU legs use this module, as the checker and
the CPU baseline; nothing in the package imports it.

The steady solve of the bench workload runs Newton on the lowest degree,
prolongs the result to the next degree and runs Newton again
(`pdesolver.jl_gb300/eulergpu.py` `solve_steady` on the device).  Here the
same sequence runs on the host: `oracle_newton` (oracle/euler_oracle.cpp,
the restatement of newton / newtonInner, reference
src/NonlinearSolvers/newton.jl:137-304, with pseudo-transient continuation,
globalization.jl:165-320, and GMRES with the element block-Jacobi
preconditioner, ls_standard.jl:321-371, preconditioning.jl:62-139) per
level, and the degree prolongation q_hi[e] = T q_lo[e] with the same T as
the device path (`eulergpu.prolongation_matrix`), applied in numpy.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")


def load(path=LIB):
    """The oracle shared library with the return types of its scalar functions."""
    lib = C.CDLL(path)
    lib.oracle_set_threads.restype = C.c_int
    lib.oracle_pressure.restype = C.c_double
    lib.oracle_calc_norm.restype = C.c_double
    lib.oracle_logavg.restype = C.c_double
    lib.oracle_logavg.argtypes = [C.c_double, C.c_double]
    lib.oracle_functional_pressure.restype = C.c_double
    return lib


def newton(lib, ms, opts, q, newton_opts):
    """oracle_newton on the host state q (in place).  Returns (status, stats)."""
    from pdesolver_gb300 import abi, eulergpu
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    o = eulergpu.NewtonOpts.from_opts(newton_opts, 0)
    st = eulergpu.NewtonStats()
    rc = lib.oracle_newton(C.byref(desc.desc), C.byref(P), abi.dptr(q), C.byref(o), C.byref(st))
    return rc, st


def solve_steady(lib, levels, q_lo, newton_opts, level_tol=None):
    """Steady solve with p-continuation on the host: `levels` is a list of
    (mesh, opts) of increasing degree on the same elements, q_lo the start
    state of levels[0].  Intermediate levels stop at level_tol.  Returns
    (q of the last level, [stats per level], seconds)."""
    from pdesolver_gb300 import eulergpu
    t0 = time.perf_counter()
    q = np.ascontiguousarray(q_lo, dtype=np.float64).copy()
    stats = []
    for k, (ms, opts) in enumerate(levels):
        if k > 0:
            ms_lo = levels[k - 1][0]
            T = eulergpu.prolongation_matrix(ms_lo.sbp, ms.sbp, ms.numDofPerNode)
            E = ms.numEl
            q = np.ascontiguousarray((q.reshape(E, -1) @ T.T).reshape(
                E, ms.numNodesPerElement, ms.numDofPerNode))
        o = dict(newton_opts)
        if k < len(levels) - 1 and level_tol is not None:
            o["res_abstol"] = level_tol
        rc, st = newton(lib, ms, opts, q, o)
        if rc != 0:
            raise RuntimeError(f"oracle Newton failed on level {k}: status {rc}, {st.asdict()}")
        stats.append(st)
    return q, stats, time.perf_counter() - t0


# (the MeshDesc objects below stay referenced for the duration of each call:
# they own the contiguous arrays the descriptor points into)

def residual(lib, ms, opts, q):
    from pdesolver_gb300 import abi, eulergpu
    res = np.zeros_like(q)
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    rc = lib.oracle_eval_residual(C.byref(desc.desc), C.byref(P), abi.dptr(q), abi.dptr(res))
    if rc != 0:
        raise RuntimeError(f"oracle residual failed: status {rc}")
    return res


def strong_norm(lib, ms, r):
    """calcNorm with M^-1 weights (reference Utils.jl:427-449)."""
    from pdesolver_gb300 import abi
    desc = abi.MeshDesc(ms)
    r = np.ascontiguousarray(r)
    return lib.oracle_calc_norm(C.byref(desc.desc), abi.dptr(r), 1)


def functional_pressure(lib, ms, opts, q, group=0):
    from pdesolver_gb300 import abi, eulergpu
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    q = np.ascontiguousarray(q)
    return lib.oracle_functional_pressure(C.byref(desc.desc), C.byref(P), abi.dptr(q), group)


def rk4(lib, ms, opts, q, h, nsteps):
    """oracle_rk4 for nsteps steps of size h on q (in place); returns stats."""
    from pdesolver_gb300 import abi, eulergpu
    st = eulergpu.Rk4Stats()
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    rc = lib.oracle_rk4(C.byref(desc.desc), C.byref(P), abi.dptr(q), C.c_double(h),
                        C.c_double(nsteps * h), 0, C.c_double(-1.0), C.byref(st))
    if rc != 0:
        raise RuntimeError(f"oracle rk4 failed: status {rc}")
    return st
