"""eg_rk4_static (RK4 with its work vectors in a static device array, no
allocation in the call) against eg_rk4 through the C ABI.  Collected last so
that it also runs after every other GPU test in the same process."""
import ctypes as C

import numpy as np
import pytest

from pdesolver_gb300 import abi, eulergpu, problems

pytestmark = pytest.mark.gpu

# the two entry points launch the same kernels in the same order on the same
# inputs; the bar is the RK4 parity tolerance of the other GPU tests
RTOL = 1e-13


def _rk4(lib, fn, g, q, h, nsteps, res_tol=-1.0):
    st = eulergpu.Rk4Stats()
    rc = getattr(lib, fn)(g.handle, abi.dptr(q), h, nsteps * h, 0, res_tol,
                          abi.EG_MEM_HOST, C.byref(st))
    return rc, st


def test_rk4_static_matches_rk4_two_calls(gpu_lib):
    lib = eulergpu.library()
    ms, opts, q0 = problems.config1(n=6, p=2, seed=5)
    assert ms.numDof <= 524288
    g = eulergpu.GPUMesh(ms, opts)
    h, nsteps = 2e-3, 6
    ref = q0.copy()
    rc, st_ref = _rk4(lib, "eg_rk4", g, ref, h, nsteps)
    assert rc == 0 and st_ref.steps == nsteps
    scale = np.abs(ref).max()
    for call in range(2):  # two calls in a row reuse the same scratch
        q = q0.copy()
        rc, st = _rk4(lib, "eg_rk4_static", g, q, h, nsteps)
        assert rc == 0, lib.eg_last_error()
        assert st.steps == st_ref.steps and st.t == st_ref.t
        assert np.abs(q - ref).max() <= RTOL * scale, call
        assert np.abs(q - q0).max() > 0.0


def test_rk4_static_device_state_and_norm(gpu_lib):
    """device-resident state and the per-step norm (res_tol) path."""
    torch = pytest.importorskip("torch")
    lib = eulergpu.library()
    ms, opts, q0 = problems.config1(n=4, p=1, seed=6)
    g = eulergpu.GPUMesh(ms, opts)
    h, nsteps = 2e-3, 4
    outs = []
    for fn in ("eg_rk4", "eg_rk4_static", "eg_rk4_static"):
        qd = torch.from_numpy(q0.copy()).cuda()
        st = eulergpu.Rk4Stats()
        rc = getattr(lib, fn)(g.handle, C.c_void_p(qd.data_ptr()), h, nsteps * h, 0, 1e-30,
                              abi.EG_MEM_DEVICE, C.byref(st))
        assert rc == 0, lib.eg_last_error()
        outs.append((qd.cpu().numpy(), st.steps, st.res_norm))
    ref = outs[0]
    for q, steps, nrm in outs[1:]:
        assert steps == ref[1]
        assert abs(nrm - ref[2]) <= RTOL * abs(ref[2])
        assert np.abs(q - ref[0]).max() <= RTOL * np.abs(ref[0]).max()


def test_rk4_static_rejects_oversized_mesh_and_timers(gpu_lib):
    lib = eulergpu.library()
    lib.eg_last_error.restype = C.c_char_p
    ms, opts, q = problems.config3(n=6)   # 1,296 tets x 23 nodes x 5 = 149,040 unknowns
    g = eulergpu.GPUMesh(ms, opts)
    g.set_timing(True)
    rc, _ = _rk4(lib, "eg_rk4_static", g, q.copy(), 1e-3, 1)
    assert rc == abi.EG_ERR_INVALID and b"timers" in lib.eg_last_error()
    g.set_timing(False)
    ms2, opts2, q2 = problems.config3(n=10)  # 6,000 tets: 690,000 unknowns
    assert ms2.numDof > 524288
    g2 = eulergpu.GPUMesh(ms2, opts2)
    before = q2.copy()
    rc, _ = _rk4(lib, "eg_rk4_static", g2, q2, 1e-3, 1)
    assert rc == abi.EG_ERR_INVALID
    assert b"static scratch limit" in lib.eg_last_error()
    assert np.array_equal(q2, before)
