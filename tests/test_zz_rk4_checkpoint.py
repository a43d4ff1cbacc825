"""RK4 with checkpointing through the reference-named driver
(eulergpu.rk4 with opts["use_checkpointing"], rk4.jl:165-229) on the device:
the checkpointed run, and a restart from its last checkpoint, end where one
uninterrupted eg_rk4 call ends.  The host side (checkpoint files, step
bookkeeping, kill and restart) is covered on the CPU by test_checkpoint.py."""
import numpy as np
import pytest

from pdesolver_gb300 import checkpoint, eulergpu, problems

pytestmark = pytest.mark.gpu

# the segments launch the same kernels in the same order on the same states
RTOL = 1e-13


def test_rk4_checkpointed_on_device_equals_uninterrupted(gpu_lib, tmp_path):
    ms, opts, q0 = problems.config1(n=6, p=2, seed=8)
    _, _, eqn, _ = eulergpu.createObjects(ms, opts)
    h = 2e-3
    t_max = 12 * h
    ref = q0.copy()
    st_ref = eqn.gpu.rk4(ref, h, t_max)
    assert st_ref.steps == 12
    scale = np.abs(ref).max()

    eqn.q[...] = q0
    ck_opts = dict(opts, use_checkpointing=True, checkpoint_freq=5, ncheckpoints=2,
                   checkpoint_dir=str(tmp_path))
    st = eulergpu.rk4(eulergpu.evalResidual, h, t_max, ms, ms.sbp, eqn, ck_opts)
    assert st.steps == 12 and st.t == pytest.approx(t_max)
    assert np.abs(eqn.q - ref).max() <= RTOL * scale

    # restart from the last checkpoint (step index 10, 8 steps done)
    restart = checkpoint.read_restart_opts(tmp_path)
    eqn.q[...] = 0.0
    checkpoint.loadRestartState(eqn.q, restart)
    assert np.abs(eqn.q - q0).max() > 0.0
    st2 = eulergpu.rk4(eulergpu.evalResidual, h, t_max, ms, ms.sbp, eqn, restart)
    assert st2.steps == 4
    assert np.abs(eqn.q - ref).max() <= RTOL * scale
