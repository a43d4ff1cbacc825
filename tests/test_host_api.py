"""The reference-named host functions over the C ABI (physicsRhs,
evalJacobian, calcMaxWaveSpeed, newton, rk4) pass the reference's arguments
through to the device calls; checked here with a stand-in for the device mesh
(no GPU).  The device calls themselves are covered by the GPU tests."""
import numpy as np
import pytest

from pdesolver_gb300 import eulergpu


class FakeGPU:
    def __init__(self):
        self.calls = []

    def eval_residual(self, q, res, t=0.0):
        self.calls.append(("res", t))
        res[...] = 2.0 * q
        return res

    def calc_norm(self, r, strongres=True):
        self.calls.append(("norm", strongres))
        return float(np.sqrt((r * r).sum()))

    def max_wave_speed(self, q):
        return 3.5

    def newton(self, q, opts, precision=0):
        self.calls.append(("newton", dict(opts), precision))
        q += 1.0
        return "stats"

    def rk4(self, q, h, t_max, itermax=0, res_tol=-1.0):
        self.calls.append(("rk4", h, t_max, itermax, res_tol))
        return "rk4stats"


def eqn_with(q):
    eqn = object.__new__(eulergpu.EulerData)
    eqn.q = q
    eqn.res = np.zeros_like(q)
    eqn.gpu = FakeGPU()
    return eqn


def test_physics_rhs_and_norm():
    q = np.arange(24.0).reshape(2, 3, 4)
    eqn = eqn_with(q.copy())
    out = np.zeros(q.size)
    nrm = eulergpu.physicsRhs(None, None, eqn, {}, out, t=0.5)
    assert np.array_equal(out, 2.0 * q.ravel())
    assert nrm == pytest.approx(np.sqrt(((2 * q) ** 2).sum()))
    assert eqn.gpu.calls == [("res", 0.5), ("norm", True)]
    # rhs_vec may alias eqn.res_vec
    assert eulergpu.physicsRhs(None, None, eqn, {}, eqn.res_vec) == pytest.approx(nrm)


def test_drivers_pass_options_and_refuse_other_residuals():
    q = np.zeros((1, 3, 4))
    eqn = eqn_with(q)
    opts = {"res_abstol": 1e-9, "euler_tau": 2.0}
    assert eulergpu.newton(eulergpu.physicsRhs, None, None, eqn, opts, precision=1) == "stats"
    assert np.all(eqn.q == 1.0)
    assert eulergpu.rk4(eulergpu.evalResidual, 0.1, 1.0, None, None, eqn, opts, res_tol=1e-6) == "rk4stats"
    assert eqn.gpu.calls == [("newton", opts, 1), ("rk4", 0.1, 1.0, 0, 1e-6)]
    assert eulergpu.calcMaxWaveSpeed(None, None, eqn, opts) == 3.5
    with pytest.raises(NotImplementedError):
        eulergpu.newton(lambda *a: None, None, None, eqn, opts)
    with pytest.raises(NotImplementedError):
        eulergpu.rk4(lambda *a: None, 0.1, 1.0, None, None, eqn, opts)


def test_eval_jacobian_fills_the_operator():
    class FakeLO:
        def calc(self, q):
            self.q = q

    q = np.ones((1, 3, 4))
    eqn = eqn_with(q)
    lo = FakeLO()
    assert eulergpu.evalJacobian(None, None, eqn, {}, lo) is lo
    assert lo.q is q
