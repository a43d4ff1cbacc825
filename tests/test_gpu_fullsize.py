"""Parity at the full sizes of the benchmark workloads (device path through
the C ABI against the CPU oracle on the same inputs).

  * 64x64 quarter annulus (8,192 triangles), SBP-Gamma p=3, Roe faces,
    vortex Dirichlet data: the whole steady solve (Newton p=1 to 1e-4,
    prolongation, Newton p=3 to |R|_{M^-1} < 1e-10) in FP64 and in mixed
    precision against the oracle's own solve from the same start.
    Reference: test/euler/newton/serial (full solves compared with stored
    results) and test_jac.jl:2370-2465.
  * 24^3 x 6 warped tets (82,944 elements), diagonal-E p=2, Ismail-Roe split
    form: the residual at 1e-12 and 5 RK4 steps at 1e-11 at full size, and
    50 RK4 steps at 1e-11 on the 8^3 x 6 cube.

Tolerances (written in each assertion):
  residual: max |R_gpu - R_oracle| <= 1e-12 max |R_oracle|
  RK4 state: max |q_gpu - q_oracle| <= 1e-11 max |q_oracle|
  Newton: |R| < 1e-10 on both; the oracle's own residual at the device's
  FP64 and mixed states < 1e-10 (each device state is a converged solution of
  the oracle's discretisation); integral of p along r = 1 within 1e-10 (FP64)
  and 1e-8 (mixed); the FP64 and mixed states within 1e-10 relative of the
  oracle's (measured on a GB300: 6e-13 and 4e-13).
"""
import os
import sys

import numpy as np
import pytest

from pdesolver_gb300 import eulergpu, problems

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import steady  # noqa: E402  (the oracle's steady-solve driver)

pytestmark = pytest.mark.gpu

NEWTON_OPTS = {"res_abstol": 1e-10, "res_reltol": 1e-14, "itermax": 200, "krylov_reltol": 1e-2,
               "newton_globalize_euler": True, "euler_tau": 5.0}
LEVEL_TOL = 1e-4


@pytest.fixture(scope="module")
def olib(oracle):
    lib = steady.load()
    lib.oracle_set_threads(os.cpu_count() or 1)
    return lib


def test_c2_steady_solve_full_size_matches_oracle(gpu_lib, olib):
    levels, q0 = [], None
    for p in (1, 3):
        ms, opts, q = problems.config2(p=p)
        levels.append((ms, opts))
        if q0 is None:
            q0 = q
    qo, so, _ = steady.solve_steady(olib, levels, q0, NEWTON_OPTS, LEVEL_TOL)
    ms3, opts3 = levels[-1]
    assert so[-1].converged == 1 and so[-1].res_norm < 1e-10
    fo = steady.functional_pressure(olib, ms3, opts3, qo)
    gl = [eulergpu.GPUMesh(ms, opts) for ms, opts in levels]
    for prec, ftol in ((0, 1e-10), (1, 1e-8)):
        qg, sg = eulergpu.solve_steady(gl, q0.copy(), NEWTON_OPTS, precision=prec, level_tol=LEVEL_TOL)
        assert sg[-1].converged == 1 and sg[-1].res_norm < 1e-10, prec
        r = steady.residual(olib, ms3, opts3, qg)
        assert steady.strong_norm(olib, ms3, r) < 1e-10, prec
        fg = gl[-1].functional_pressure(qg, 0)
        assert abs(fg - fo) <= ftol * abs(fo), (prec, fg, fo)
        assert np.abs(qg - qo).max() <= 1e-10 * np.abs(qo).max(), prec


def test_c3_residual_and_rk4_full_size_match_oracle(gpu_lib, olib):
    ms, opts, q = problems.config3()
    assert ms.numEl == 82944
    g = eulergpu.GPUMesh(ms, opts)
    rg = np.zeros_like(q)
    g.eval_residual(q, rg)
    ro = steady.residual(olib, ms, opts, q)
    assert np.abs(rg - ro).max() <= 1e-12 * np.abs(ro).max()
    h = 1e-3
    qg = q.copy()
    st = g.rk4(qg, h, 5 * h)
    assert st.steps == 5
    qo = q.copy()
    assert steady.rk4(olib, ms, opts, qo, h, 5).steps == 5
    assert np.abs(qg - qo).max() <= 1e-11 * np.abs(qo).max()
    assert np.abs(qg - q).max() > 1e-6      # the state moved


def test_c3_fifty_rk4_steps_match_oracle(gpu_lib, olib):
    ms, opts, q = problems.config3(n=8)
    g = eulergpu.GPUMesh(ms, opts)
    h = 1e-3
    qg = q.copy()
    assert g.rk4(qg, h, 50 * h).steps == 50
    qo = q.copy()
    assert steady.rk4(olib, ms, opts, qo, h, 50).steps == 50
    assert np.abs(qg - qo).max() <= 1e-11 * np.abs(qo).max()
