"""Checkpoint / restart of explicit time marching (the reference's
src/Utils/checkpoint.jl, used by rk4.jl:60-88, 165-229 and the restart in
solver/common.jl:502-509).

A ``Checkpointer`` owns ``ncheckpoints`` directories ``<prefix>_checkpoint<i>``
(1-based indices, as in the reference) and records which are in use and the
order they were written in (``history``, most recent first, -1 = unused).  A
checkpoint holds the solution vector, the solver's own restart data and the
options for a restart.  Completion is marked by a flag file written last, and
the options carry two checkpoints (``writing_checkpoint`` and
``most_recent_checkpoint``), so a run killed while writing restarts from the
older, complete one.

The names and the semantics follow the reference's API; the on-disk formats
are this package's own (JSON for the checkpointer and the options, ``.npy``
for the solution, ``.npz`` for the solver data).  The reference writes its
shared files from MPI rank 0 between barriers; here every process solves its
own problems, so each process checkpoints on its own (one ``Checkpointer``
per problem, told apart by ``prefix``), and ``myrank`` only names the
per-rank files.

``rk4_checkpointed`` is the time loop of rk4.jl with checkpointing: the device
advances the state in segments between checkpoint steps, and the host writes
the state at each checkpoint step.
"""
from __future__ import annotations

import json
import os

import numpy as np

CheckpointFree = 1
CheckpointUsed = 2

Checkpointer_fname = "checkpointer.json"
Solution_fname = "qvec"
Input_fname = "input_vals_restart.json"
CheckpointData_fname = "checkpointdata"
FlagFile_fname = "flagfile.dat"
FlagFile_val = 42


def _rank_fname(stem, rank, ext):
    return f"{stem}_{rank}{ext}"


class Checkpointer:
    """Which checkpoints are used and in which order they were written
    (checkpoint.jl:66-80).  Indices are 1-based."""

    def __init__(self, ncheckpoints, paths, status, history):
        self.ncheckpoints = int(ncheckpoints)
        self.paths = list(paths)
        self.status = list(status)
        self.history = list(history)

    @classmethod
    def new(cls, myrank=0, ncheckpoints=2, prefix="", root=None):
        """all checkpoints free, their directories created under `root`
        (default: the current directory) and stale flag files removed
        (checkpoint.jl:103-147)."""
        if ncheckpoints < 0:
            raise ValueError("ncheckpoints must be >= 0")
        root = os.path.abspath(root or os.getcwd())
        pre = f"{prefix}_" if prefix else ""
        paths = [os.path.join(root, f"{pre}checkpoint{i}") for i in range(1, ncheckpoints + 1)]
        for p in paths:
            os.makedirs(p, exist_ok=True)
        chk = cls(ncheckpoints, paths, [CheckpointFree] * ncheckpoints, [-1] * ncheckpoints)
        for i in range(1, ncheckpoints + 1):
            deleteFlagFile(chk, i)
        return chk

    @classmethod
    def from_opts(cls, opts, myrank=0):
        """the checkpointer of the most recent complete checkpoint named in
        the options (checkpoint.jl:183-216): the one being written if its
        flag file is there, else the one before it."""
        path = opts.get("writing_checkpoint_path", "")
        if not (path and checkFlagFile(path)):
            path = opts.get("most_recent_checkpoint_path", "")
            if not (path and checkFlagFile(path)):
                raise RuntimeError("no complete checkpoint to restart from")
        with open(os.path.join(path, Checkpointer_fname)) as f:
            d = json.load(f)
        return cls(d["ncheckpoints"], d["paths"], d["status"], d["history"])

    def to_dict(self):
        return {"ncheckpoints": self.ncheckpoints, "paths": self.paths,
                "status": self.status, "history": self.history}

    def copy(self):
        return Checkpointer(self.ncheckpoints, self.paths, self.status, self.history)

    def _check_index(self, checkpoint):
        if not 1 <= checkpoint <= self.ncheckpoints:
            raise IndexError(f"checkpoint {checkpoint} not in 1..{self.ncheckpoints}")


# ---------------------------------------------------------------- internals

def writeCheckpointer(chk, checkpoint):
    """the checkpointer, into checkpoint `checkpoint` (checkpoint.jl:265-274)."""
    with open(os.path.join(chk.paths[checkpoint - 1], Checkpointer_fname), "w") as f:
        json.dump(chk.to_dict(), f)


def writeFlagFile(chk, checkpoint):
    """marks the checkpoint complete (checkpoint.jl:455-463)."""
    with open(os.path.join(chk.paths[checkpoint - 1], FlagFile_fname), "wb") as f:
        f.write(np.int64(FlagFile_val).tobytes())
        f.flush()
        os.fsync(f.fileno())


def checkFlagFile(chk_or_path, checkpoint=None):
    """True if the checkpoint's flag file exists and holds the flag value
    (checkpoint.jl:474-503); takes (checkpointer, index) or a directory."""
    path = chk_or_path.paths[checkpoint - 1] if checkpoint is not None else chk_or_path
    fpath = os.path.join(path, FlagFile_fname)
    if not os.path.isfile(fpath):
        return False
    with open(fpath, "rb") as f:
        raw = f.read()
    return len(raw) == 8 and int(np.frombuffer(raw, dtype=np.int64)[0]) == FlagFile_val


def deleteFlagFile(chk, checkpoint):
    """removes the flag file if there is one (checkpoint.jl:516-523)."""
    fpath = os.path.join(chk.paths[checkpoint - 1], FlagFile_fname)
    if os.path.isfile(fpath):
        os.remove(fpath)


def writeCheckpointData(chk, checkpoint, data, comm_rank=0):
    """the solver's restart data (a mapping of names to numbers or arrays)
    into the checkpoint (checkpoint.jl:537-548)."""
    fpath = os.path.join(chk.paths[checkpoint - 1], _rank_fname(CheckpointData_fname, comm_rank, ".npz"))
    np.savez(fpath, **{k: np.asarray(v) for k, v in dict(data).items()})


def markCheckpointUsed(chk, checkpoint):
    """status -> used, and the checkpoint goes to the head of the history
    (checkpoint.jl:558-583)."""
    if chk.status[checkpoint - 1] != CheckpointFree:
        raise RuntimeError(f"checkpoint {checkpoint} is not free")
    if chk.history[-1] != -1:
        raise RuntimeError("checkpoint history is full")
    chk.status[checkpoint - 1] = CheckpointUsed
    chk.history = [checkpoint] + chk.history[:-1]


def _json_default(x):
    if isinstance(x, np.generic):
        return x.item()
    if isinstance(x, np.ndarray):
        return x.tolist()
    raise TypeError(f"option value of type {type(x).__name__} cannot be written to a restart file")


def _write_restart_opts(chk, checkpoint, opts):
    """the options with is_restart = true, in the checkpoint, and a link to
    them in the checkpoints' parent directory (checkpoint.jl:355-369)."""
    opts_restart = dict(opts)
    opts_restart["is_restart"] = True
    fname = os.path.join(chk.paths[checkpoint - 1], Input_fname)
    with open(fname, "w") as f:
        json.dump(opts_restart, f, default=_json_default, indent=1, sort_keys=True)
    link = os.path.join(os.path.dirname(chk.paths[checkpoint - 1]), Input_fname)
    tmp = link + ".tmp"
    if os.path.lexists(tmp):
        os.remove(tmp)
    os.symlink(fname, tmp)
    os.replace(tmp, link)


def read_restart_opts(root=None):
    """the options of the most recently started checkpoint under `root` (the
    reference restarts by reading the linked input file)."""
    with open(os.path.join(os.path.abspath(root or os.getcwd()), Input_fname)) as f:
        return json.load(f)


# ---------------------------------------------------------------- API

def saveCheckpoint(chk, checkpoint, q_vec, opts, checkpoint_data, comm_rank=0):
    """q_vec, the solver data, the restart options and the checkpointer into
    a free checkpoint; the flag file last (checkpoint.jl:308-384).  The
    checkpoint is marked used, and the options name it as being written,
    before anything is written."""
    chk._check_index(checkpoint)
    if chk.status[checkpoint - 1] != CheckpointFree:
        raise RuntimeError(f"Cannot save to non-free checkpoint number {checkpoint}")
    deleteFlagFile(chk, checkpoint)
    markCheckpointUsed(chk, checkpoint)
    opts["writing_checkpoint"] = checkpoint
    opts["writing_checkpoint_path"] = chk.paths[checkpoint - 1]
    np.save(os.path.join(chk.paths[checkpoint - 1], _rank_fname(Solution_fname, comm_rank, ".npy")),
            np.ascontiguousarray(np.asarray(q_vec, dtype=np.float64).reshape(-1)))
    writeCheckpointData(chk, checkpoint, checkpoint_data, comm_rank)
    _write_restart_opts(chk, checkpoint, opts)
    writeCheckpointer(chk, checkpoint)
    writeFlagFile(chk, checkpoint)
    opts["most_recent_checkpoint"] = checkpoint
    opts["most_recent_checkpoint_path"] = chk.paths[checkpoint - 1]


def loadCheckpoint(chk, checkpoint, q_vec, comm_rank=0):
    """q_vec <- the solution saved in a used checkpoint (checkpoint.jl:
    419-434).  Loading does not free the checkpoint."""
    chk._check_index(checkpoint)
    if chk.status[checkpoint - 1] != CheckpointUsed:
        raise RuntimeError(f"Cannot load unused checkpoint number {checkpoint}")
    saved = np.load(os.path.join(chk.paths[checkpoint - 1], _rank_fname(Solution_fname, comm_rank, ".npy")))
    flat = q_vec.reshape(-1)
    if saved.shape != flat.shape:
        raise ValueError(f"checkpoint holds {saved.size} values, the state has {flat.size}")
    flat[...] = saved


def readCheckpointData(chk, checkpoint, comm_rank=0):
    """the solver data saved in a checkpoint, as a dict (checkpoint.jl:606-619);
    0-d arrays come back as Python scalars."""
    chk._check_index(checkpoint)
    fpath = os.path.join(chk.paths[checkpoint - 1], _rank_fname(CheckpointData_fname, comm_rank, ".npz"))
    with np.load(fpath, allow_pickle=False) as z:
        return {k: (z[k].item() if z[k].ndim == 0 else z[k].copy()) for k in z.files}


def readLastCheckpointData(chk, comm_rank=0):
    """readCheckpointData of the most recent checkpoint (checkpoint.jl:631-637)."""
    return readCheckpointData(chk, getLastCheckpoint(chk), comm_rank)


def saveNextFreeCheckpoint(chk, q_vec, opts, checkpoint_data, comm_rank=0):
    """saveCheckpoint into the lowest free checkpoint; returns its index
    (checkpoint.jl:659-667).  Raises when none is free."""
    checkpoint = getNextFreeCheckpoint(chk)
    if checkpoint == 0:
        raise RuntimeError("no free checkpoint")
    saveCheckpoint(chk, checkpoint, q_vec, opts, checkpoint_data, comm_rank)
    return checkpoint


def loadLastCheckpoint(chk, q_vec, comm_rank=0):
    """loadCheckpoint of the most recent checkpoint; returns its index
    (checkpoint.jl:689-697)."""
    checkpoint = getLastCheckpoint(chk)
    loadCheckpoint(chk, checkpoint, q_vec, comm_rank)
    return checkpoint


def countFreeCheckpoints(chk):
    return sum(1 for s in chk.status if s == CheckpointFree)


def getNextFreeCheckpoint(chk):
    """the lowest free index, or 0 when all are used."""
    for i, s in enumerate(chk.status, start=1):
        if s == CheckpointFree:
            return i
    return 0


def getLastCheckpoint(chk):
    """the most recently written checkpoint (-1: none)."""
    return chk.history[0] if chk.ncheckpoints else -1


def getOldestCheckpoint(chk):
    """the least recently written checkpoint still in use (-1: none)."""
    used = [h for h in chk.history if h != -1]
    return used[-1] if used else -1


def freeOldestCheckpoint(chk):
    """frees the least recently written checkpoint; returns it (-1: all were
    free) (checkpoint.jl:791-799)."""
    checkpoint = getOldestCheckpoint(chk)
    if checkpoint != -1:
        freeCheckpoint(chk, checkpoint)
    return checkpoint


def freeCheckpoint(chk, checkpoint):
    """marks a checkpoint free and removes it from the history; freeing a
    free checkpoint is allowed (checkpoint.jl:816-858)."""
    chk._check_index(checkpoint)
    if chk.status[checkpoint - 1] == CheckpointFree:
        return
    chk.history = [h for h in chk.history if h != checkpoint] + [-1]
    chk.status[checkpoint - 1] = CheckpointFree


def loadRestartState(q_vec, opts, comm_rank=0):
    """q_vec <- the state of the most recent complete checkpoint the options
    name (solver/common.jl:502-509); returns the checkpointer."""
    chk = Checkpointer.from_opts(opts, comm_rank)
    loadLastCheckpoint(chk, q_vec, comm_rank)
    return chk


# ---------------------------------------------------------------- RK4 driver

def explicit_checkpoint_setup(opts, myrank=0, root=None):
    """(checkpointer, data, skip_checkpoint) for a self-starting explicit
    method (rk4.jl:68-88).  A new run starts at step index i = 2 with fresh
    checkpoints; a restart reads both from the most recent complete
    checkpoint and skips the checkpoint due at its first step."""
    if not opts.get("is_restart", False):
        chk = Checkpointer.new(myrank, int(opts.get("ncheckpoints", 2)),
                               prefix=opts.get("checkpoint_prefix", ""), root=root)
        return chk, {"i": 2}, False
    chk = Checkpointer.from_opts(opts, myrank)
    return chk, readLastCheckpointData(chk, myrank), True


def rk4_checkpointed(advance, q_vec, h, t_max, opts, itermax=0, myrank=0, root=None):
    """The rk4.jl time loop (rk4.jl:195-336) with checkpointing.

    Step indices run i = 2 .. round(t_max/h) + 1 as in the reference.  Before
    step i, when i is a multiple of opts["checkpoint_freq"], the state is
    saved with i (the oldest checkpoint is freed first when none is free).
    Between checkpoint steps the state is advanced by
    ``advance(n, itermax_local)``, which takes n full RK4 steps in place on
    q_vec and returns the steps taken; fewer than n means a stopping test
    ended the run (the device driver's res_tol, or itermax, which the local
    count `itermax_local` places at the same global step as the reference's
    ``i > itermax``).

    Returns (steps taken in this call, final time, last step index)."""
    freq = int(opts.get("checkpoint_freq", 200))
    if freq < 1:
        raise ValueError("checkpoint_freq must be >= 1")
    if int(opts.get("ncheckpoints", 2)) < 1:
        raise ValueError("checkpointing needs at least one checkpoint")
    t_steps = int(round(t_max / h))
    chk, data, skip = explicit_checkpoint_setup(opts, myrank, root)
    i = int(data["i"])
    taken_total = 0
    stopped = False
    while i <= t_steps + 1:
        if i % freq == 0:
            if skip:
                skip = False
            else:
                if countFreeCheckpoints(chk) == 0:
                    freeOldestCheckpoint(chk)
                saveNextFreeCheckpoint(chk, q_vec, opts, {"i": i}, myrank)
        end = min((i // freq + 1) * freq, t_steps + 2)
        n = end - i
        itl = max(1, itermax - (i - 2)) if itermax > 0 else 0
        taken = int(advance(n, itl))
        taken_total += taken
        i += taken
        if taken < n:
            stopped = True
            break
    # the reference's t after the loop: the start of the last step taken
    # (or stopped in) plus h
    t = (i - 2) * h + h if stopped else max(t_steps, 1) * h
    return taken_total, t, i
