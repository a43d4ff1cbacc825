"""Checkpoint / restart (the reference's src/Utils/checkpoint.jl and the
checkpointing in rk4.jl), host side, CPU only.

The API sequence restates test/euler/test_checkpoint.jl:9-104.  The RK4
driver is checked with a host stand-in for the device stepper (same stage
order and stopping tests as the device RK4), so that a checkpointed run, a
run killed and restarted, and a run restarted after a checkpoint that was
cut off while being written all end bit-for-bit where an uninterrupted run
ends."""
import os

import numpy as np
import pytest

from pdesolver_gb300 import checkpoint as ck


def test_checkpointer_api(tmp_path):
    """test/euler/test_checkpoint.jl:9-104."""
    rng = np.random.default_rng(0)
    q = rng.random(40)
    opts = {"ncheckpoints": 2}
    chk = ck.Checkpointer.new(0, 2, "abc", root=tmp_path)
    data = {"a": 42, "b": rng.random(10)}

    assert chk.ncheckpoints == 2
    assert chk.paths[1] == os.path.join(str(tmp_path), "abc_checkpoint2")
    assert os.path.isdir(chk.paths[1])
    assert chk.status == [ck.CheckpointFree] * 2 and chk.history == [-1, -1]
    assert ck.countFreeCheckpoints(chk) == 2
    assert ck.getNextFreeCheckpoint(chk) == 1

    assert ck.saveNextFreeCheckpoint(chk, q, opts, data) == 1
    assert ck.countFreeCheckpoints(chk) == 1
    assert ck.getNextFreeCheckpoint(chk) == 2
    assert ck.getOldestCheckpoint(chk) == 1
    assert ck.getLastCheckpoint(chk) == 1
    assert chk.status[0] == ck.CheckpointUsed and chk.history[0] == 1

    q *= 2
    q2 = q.copy()
    assert ck.saveNextFreeCheckpoint(chk, q, opts, data) == 2
    assert ck.countFreeCheckpoints(chk) == 0
    assert chk.status[1] == ck.CheckpointUsed
    assert ck.getOldestCheckpoint(chk) == 1
    with pytest.raises(RuntimeError):
        ck.saveNextFreeCheckpoint(chk, q, opts, data)

    q *= 2
    assert ck.loadLastCheckpoint(chk, q) == 2
    np.testing.assert_array_equal(q, q2)

    chk2 = ck.Checkpointer.from_opts(opts, 0)
    assert chk2.ncheckpoints == chk.ncheckpoints
    assert chk2.history == chk.history and chk2.status == chk.status and chk2.paths == chk.paths

    data2 = ck.readCheckpointData(chk, ck.getLastCheckpoint(chk))
    assert data2["a"] == 42
    np.testing.assert_array_equal(data2["b"], data["b"])

    # a checkpoint cut off while being written: the older one is loaded
    ck.deleteFlagFile(chk, ck.getLastCheckpoint(chk))
    opts["most_recent_checkpoint"] = 1
    opts["most_recent_checkpoint_path"] = chk.paths[0]
    chk2 = ck.Checkpointer.from_opts(opts, 0)
    assert ck.countFreeCheckpoints(chk2) == 1
    assert ck.getLastCheckpoint(chk2) == 1

    # more checkpoints
    chk = ck.Checkpointer.new(0, 5, root=tmp_path)
    for _ in range(4):
        ck.saveNextFreeCheckpoint(chk, q, opts, data)
    ck.freeCheckpoint(chk, 2)
    assert ck.countFreeCheckpoints(chk) == 2
    assert ck.getNextFreeCheckpoint(chk) == 2
    assert ck.getLastCheckpoint(chk) == 4
    assert ck.getOldestCheckpoint(chk) == 1
    ck.saveNextFreeCheckpoint(chk, q, opts, data)
    assert ck.countFreeCheckpoints(chk) == 1
    assert ck.getNextFreeCheckpoint(chk) == 5
    assert ck.getLastCheckpoint(chk) == 2
    assert ck.getOldestCheckpoint(chk) == 1


def test_free_and_load_rules(tmp_path):
    chk = ck.Checkpointer.new(0, 3, root=tmp_path)
    q = np.arange(6.0)
    ck.freeCheckpoint(chk, 2)                       # freeing a free one is allowed
    assert ck.freeOldestCheckpoint(chk) == -1       # nothing to free
    with pytest.raises(RuntimeError):
        ck.loadCheckpoint(chk, 1, q)                # unused
    with pytest.raises(IndexError):
        ck.saveCheckpoint(chk, 4, q, {}, {})
    opts = {}
    ck.saveCheckpoint(chk, 3, q, opts, {"i": 7})
    assert opts["most_recent_checkpoint"] == 3 and ck.checkFlagFile(chk, 3)
    with pytest.raises(RuntimeError):
        ck.saveCheckpoint(chk, 3, q, opts, {})      # not free
    with pytest.raises(ValueError):
        ck.loadCheckpoint(chk, 3, np.zeros(5))      # wrong size
    assert ck.freeOldestCheckpoint(chk) == 3
    assert chk.history == [-1, -1, -1] and ck.countFreeCheckpoints(chk) == 3
    # the restart options name the checkpoint and set is_restart
    ro = ck.read_restart_opts(tmp_path)
    assert ro["is_restart"] is True and ro["writing_checkpoint"] == 3
    with pytest.raises(RuntimeError):
        ck.Checkpointer.from_opts({"writing_checkpoint_path": "", "most_recent_checkpoint_path": ""})


class _Stepper:
    """host stand-in for the device RK4 (same stage order and stopping tests:
    the stage-1 norm test and itermax break after the stage-1 update)."""

    def __init__(self, q, A, h, res_tol=-1.0, die_after=None):
        self.q, self.A, self.h, self.res_tol = q, A, h, res_tol
        self.die_after = die_after
        self.total = 0

    def __call__(self, n, itermax_local):
        q, A, h = self.q, self.A, self.h
        xold = q.copy()
        steps = 0
        for i in range(2, n + 2):
            if self.die_after is not None and self.total == self.die_after:
                raise KeyboardInterrupt("killed")
            k1 = A @ q
            q[:] = xold + (h / 2) * k1
            if self.res_tol > 0 and np.linalg.norm(k1) < self.res_tol:
                break
            if itermax_local > 0 and i > itermax_local:
                break
            k2 = A @ q
            q[:] = xold + (h / 2) * k2
            k3 = A @ q
            q[:] = xold + h * k3
            k4 = A @ q
            xold = xold + (h / 6) * (k1 + 2 * k2 + 2 * k3 + k4)
            q[:] = xold
            steps += 1
            self.total += 1
        return steps


def _problem(n=12):
    rng = np.random.default_rng(5)
    A = -np.eye(n) + 0.2 * rng.normal(size=(n, n))
    return A, rng.random(n)


@pytest.mark.parametrize("itermax,res_tol", [(0, -1.0), (23, -1.0), (0, 2.2)])
def test_rk4_checkpointed_equals_uninterrupted(tmp_path, itermax, res_tol):
    A, q0 = _problem()
    h, t_max = 0.01, 0.37                           # 37 steps, i = 2 .. 38
    ref = q0.copy()
    ref_steps = _Stepper(ref, A, h, res_tol)(int(round(t_max / h)), itermax)
    q = q0.copy()
    opts = {"use_checkpointing": True, "checkpoint_freq": 5, "ncheckpoints": 2}
    steps, t, _ = ck.rk4_checkpointed(_Stepper(q, A, h, res_tol), q, h, t_max, opts,
                                      itermax=itermax, root=tmp_path)
    assert steps == ref_steps
    np.testing.assert_array_equal(q, ref)
    if itermax == 0 and res_tol < 0:
        assert steps == 37 and t == pytest.approx(t_max)
    else:
        assert steps < 37


@pytest.mark.parametrize("lose_last", [False, True])
def test_rk4_killed_and_restarted(tmp_path, lose_last):
    """a run killed at step 27 restarts from its last complete checkpoint
    (i = 25, or i = 20 when the i = 25 checkpoint lost its flag file) and
    ends where the uninterrupted run ends."""
    A, q0 = _problem()
    h, t_max = 0.01, 0.37
    ref = q0.copy()
    _Stepper(ref, A, h)(37, 0)

    q = q0.copy()
    opts = {"use_checkpointing": True, "checkpoint_freq": 5, "ncheckpoints": 2}
    with pytest.raises(KeyboardInterrupt):
        ck.rk4_checkpointed(_Stepper(q, A, h, die_after=25), q, h, t_max, opts, root=tmp_path)
    restart = ck.read_restart_opts(tmp_path)
    assert restart["is_restart"] and restart["writing_checkpoint_path"].endswith("checkpoint1")
    if lose_last:
        os.remove(os.path.join(restart["writing_checkpoint_path"], ck.FlagFile_fname))
    q2 = np.zeros_like(q0)
    ck.loadRestartState(q2, restart)
    chk = ck.Checkpointer.from_opts(restart)
    assert ck.readLastCheckpointData(chk)["i"] == (20 if lose_last else 25)
    steps, t, i = ck.rk4_checkpointed(_Stepper(q2, A, h), q2, h, t_max, restart, root=tmp_path)
    assert steps == (19 if lose_last else 14) and i == 39
    assert t == pytest.approx(t_max)
    np.testing.assert_array_equal(q2, ref)


def test_rk4_checkpoint_rotation(tmp_path):
    """with more checkpoint steps than checkpoints the oldest is freed first;
    the history names the most recent steps."""
    A, q0 = _problem()
    q = q0.copy()
    opts = {"use_checkpointing": True, "checkpoint_freq": 4, "ncheckpoints": 3}
    ck.rk4_checkpointed(_Stepper(q, A, 0.01), q, 0.01, 0.30, opts, root=tmp_path)
    chk = ck.Checkpointer.from_opts(opts)
    steps_saved = [ck.readCheckpointData(chk, c)["i"] for c in chk.history]
    assert steps_saved == [28, 24, 20]
    with pytest.raises(ValueError):
        ck.rk4_checkpointed(_Stepper(q, A, 0.01), q, 0.01, 0.3,
                            {"checkpoint_freq": 0}, root=tmp_path)


class _FakeDevice:
    """stands in for GPUMesh.rk4 (host state, same semantics) so that the
    reference-named driver eulergpu.rk4 is checked here without a GPU."""

    def __init__(self, A):
        self.A = A

    def rk4(self, q, h, t_max, itermax=0, res_tol=-1.0):
        from pdesolver_gb300 import eulergpu
        flat = q.reshape(-1)
        n = int(round(t_max / h))
        st = eulergpu.Rk4Stats()
        st.steps = _Stepper(flat, self.A, h, res_tol)(n, itermax)
        st.t = h * max(st.steps, 1)
        return st


def test_eulergpu_rk4_checkpointing_glue(tmp_path):
    from types import SimpleNamespace
    from pdesolver_gb300 import eulergpu
    A, q0 = _problem()
    h, t_max = 0.01, 0.22
    ref = SimpleNamespace(q=q0.reshape(3, 4).copy(), gpu=_FakeDevice(A))
    st_ref = eulergpu.rk4(eulergpu.evalResidual, h, t_max, None, None, ref, {})
    eqn = SimpleNamespace(q=q0.reshape(3, 4).copy(), gpu=_FakeDevice(A))
    opts = {"use_checkpointing": True, "checkpoint_freq": 4, "ncheckpoints": 2,
            "checkpoint_dir": str(tmp_path)}
    st = eulergpu.rk4(eulergpu.evalResidual, h, t_max, None, None, eqn, opts)
    assert st.steps == st_ref.steps == 22 and st.t == pytest.approx(t_max)
    np.testing.assert_array_equal(eqn.q, ref.q)
    # restart from the last checkpoint (i = 20) and finish again
    restart = ck.read_restart_opts(tmp_path)
    again = SimpleNamespace(q=np.zeros((3, 4)), gpu=_FakeDevice(A))
    ck.loadRestartState(again.q, restart)
    st2 = eulergpu.rk4(eulergpu.evalResidual, h, t_max, None, None, again, restart)
    assert st2.steps == 4
    np.testing.assert_array_equal(again.q, ref.q)
    with pytest.raises(NotImplementedError):
        eulergpu.rk4(lambda *a: None, h, t_max, None, None, eqn, opts)
