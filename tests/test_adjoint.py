"""Steady adjoint pieces on the CPU: the right-preconditioned GMRES used for
the transposed solve, the functional derivative against finite differences
of the oracle functional, and calcAdjoint with the oracle's Jacobian blocks
standing in for the device operator (transposed applies as in the library)
against a dense solve.  The device run is tests/test_zzz_adjoint.py."""
import ctypes as C
from types import SimpleNamespace

import numpy as np
import pytest

from conftest import block_apply, block_apply_t, oracle_jacobian
from pdesolver_gb300 import abi, adjoint, eulergpu, problems

torch = pytest.importorskip("torch")


def _dense_system(n=60, seed=0):
    rng = np.random.default_rng(seed)
    A = np.eye(n) * 4 + rng.normal(size=(n, n)) / np.sqrt(n)
    return A, rng.normal(size=n)


@pytest.mark.parametrize("restart", [5, 30])
def test_gmres_solves_and_restarts(restart):
    A, b = _dense_system()
    At = torch.from_numpy(A)
    Minv = torch.from_numpy(np.diag(1.0 / np.diag(A)))
    x = torch.zeros(len(b), dtype=torch.float64)
    st = adjoint.gmres(lambda v, o: o.copy_(At @ v), lambda v, o: o.copy_(Minv @ v),
                       torch.from_numpy(b), x, restart=restart, reltol=1e-12)
    assert st["converged"] and st["res_final"] <= 1e-12 * np.linalg.norm(b)
    np.testing.assert_allclose(x.numpy(), np.linalg.solve(A, b), rtol=0, atol=1e-10)
    assert (st["restarts"] > 0) == (restart == 5)
    # itermax stops early; a zero right-hand side takes no iteration
    x2 = torch.zeros(len(b), dtype=torch.float64)
    st2 = adjoint.gmres(lambda v, o: o.copy_(At @ v), lambda v, o: o.copy_(v),
                        torch.from_numpy(b), x2, restart=restart, reltol=1e-14, itermax=3)
    assert st2["iters"] == 3 and not st2["converged"]
    x3 = torch.zeros(len(b), dtype=torch.float64)
    st3 = adjoint.gmres(lambda v, o: o.copy_(At @ v), lambda v, o: o.copy_(v),
                        torch.zeros(len(b), dtype=torch.float64), x3)
    assert st3["iters"] == 0 and st3["converged"] and float(x3.abs().max()) == 0.0


def _functional(oracle, desc, P, q, group):
    oracle.oracle_functional_pressure.restype = C.c_double
    return oracle.oracle_functional_pressure(C.byref(desc.desc), C.byref(P),
                                             abi.dptr(np.ascontiguousarray(q)), group)


@pytest.mark.parametrize("case", ["gamma3", "tet2"])
def test_functional_derivative_vs_finite_differences(oracle, case):
    """evalFunctionalDeriv_q . v = central difference of the oracle's
    boundary functional (boundary_functional.jl:82-126) along v."""
    if case == "tet2":
        ms, opts, q = problems.config3(n=2, p=2, seed=7)
        group = 1
    else:
        ms, opts, q = problems.config1(n=4, p=3, family="gamma", seed=8)
        group = 0
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    eqn = SimpleNamespace(q=q)
    fn = adjoint.PressureFunctional(group)
    dj = adjoint.evalFunctionalDeriv_q(ms, ms.sbp, eqn, opts, fn)
    assert np.abs(dj).max() > 0
    rng = np.random.default_rng(3)
    h = 1e-4            # central differences: O(h^2) error, round-off eps J / h
    for _ in range(3):
        v = rng.normal(size=q.shape) * np.abs(q).max() * 1e-2
        fd = (_functional(oracle, desc, P, q + h * v, group)
              - _functional(oracle, desc, P, q - h * v, group)) / (2 * h)
        assert (dj * v).sum() == pytest.approx(fd, rel=1e-7)
    # only the nodes of the group's faces are touched
    touched = np.zeros(ms.numEl, dtype=bool)
    lo, hi = ms.bndry_offsets[group], ms.bndry_offsets[group + 1]
    touched[ms.bndryfaces[lo:hi, 0]] = True
    assert np.abs(dj[~touched]).max(initial=0.0) == 0.0


class _OracleLO:
    """the oracle's Jacobian blocks behind the library's transposed-apply
    interface (numpy or CPU torch arrays)."""

    def __init__(self, ms, diag, cpl):
        self.ms, self.diag, self.cpl = ms, diag, cpl
        self.shape = (ms.numEl, ms.sbp.numnodes, ms.numDofPerNode)

    def apply_transpose(self, x, y):
        xn = x.numpy() if hasattr(x, "numpy") else x
        out = block_apply_t(self.ms, self.diag, self.cpl, xn.reshape(self.shape))
        (y.copy_(torch.from_numpy(out.reshape(-1))) if hasattr(y, "copy_") else np.copyto(y, out))


class _OraclePC:
    def __init__(self, lo):
        self.lo = lo

    def apply_transpose(self, x, y):
        xn = (x.numpy() if hasattr(x, "numpy") else x).reshape(self.lo.diag.shape[0], -1)
        # M^-T x per element: J_e = diag[e]^T in the column-major block storage
        out = np.stack([np.linalg.solve(d, xe) for d, xe in zip(self.lo.diag, xn)]).reshape(-1)
        (y.copy_(torch.from_numpy(out)) if hasattr(y, "copy_") else np.copyto(y, out))


def test_calc_adjoint_against_dense_solve(oracle):
    """(dR/dq)^T psi = -dJ/dq by the transposed GMRES equals the dense solve
    at 1e-9, and psi^T (dR/dq) v = -dJ/dq . v for random v."""
    ms, opts, q = problems.config1(n=3, p=2, family="omega", seed=9)
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    diag, cpl = oracle_jacobian(oracle, desc, P, ms, q)
    lo = _OracleLO(ms, diag, cpl)
    ls = SimpleNamespace(lo=lo, pc=_OraclePC(lo), restart=30, reltol=1e-12, abstol=-1.0, itermax=-1)
    eqn = SimpleNamespace(q=q)
    fn = adjoint.PressureFunctional(0)
    psi = np.zeros_like(q)
    st = adjoint.calcAdjoint(ms, ms.sbp, eqn, opts, ls, fn, psi, device="cpu")
    assert st["converged"]
    N = q.size
    J = np.stack([block_apply(ms, diag, cpl, np.eye(N)[i].reshape(q.shape)).reshape(-1)
                  for i in range(N)], axis=1)
    dj = adjoint.evalFunctionalDeriv_q(ms, ms.sbp, eqn, opts, fn).reshape(-1)
    ref = np.linalg.solve(J.T, -dj)
    np.testing.assert_allclose(psi.reshape(-1), ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    v = np.random.default_rng(4).normal(size=N)
    assert psi.reshape(-1) @ (J @ v) == pytest.approx(-(dj @ v), rel=1e-9)


def test_eval_residual_revq_with_the_oracle_blocks(oracle):
    """evalResidual_revq: q_bar = (dR/dq)^T res_bar, overwritten or summed
    into (zero_output), against the oracle's directional derivative:
    res_bar . (J v) = q_bar . v."""
    from conftest import oracle_jvp

    class LO:
        def __init__(self, ms, diag, cpl):
            self.ms, self.diag, self.cpl = ms, diag, cpl

        def calc(self, q):
            self.q = q

        def apply_transpose(self, x, y):
            y[...] = block_apply_t(self.ms, self.diag, self.cpl, x)
            return y

    ms, opts, q = problems.config1(n=3, p=2, family="gamma", seed=10)
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    lo = LO(ms, *oracle_jacobian(oracle, desc, P, ms, q))
    eqn = SimpleNamespace(q=q)
    rng = np.random.default_rng(6)
    rb, v = rng.normal(size=q.shape), rng.normal(size=q.shape)
    qb = np.full(q.size, 7.0)
    adjoint.evalResidual_revq(ms, ms.sbp, eqn, opts, rb.reshape(-1), qb, lo=lo)
    assert lo.q is q
    jv = oracle_jvp(oracle, desc, P, q, v)
    assert (rb * jv).sum() == pytest.approx(qb @ v.reshape(-1), rel=1e-11)
    qb2 = np.ones(q.size)
    adjoint.evalResidual_revq(ms, ms.sbp, eqn, opts, rb.reshape(-1), qb2, lo=lo, zero_output=False)
    np.testing.assert_allclose(qb2, qb + 1.0, rtol=0, atol=1e-14 * np.abs(qb).max())
