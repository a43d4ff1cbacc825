"""Batches of independent steady solves on one GPU.

The reference solves one problem per process (`solvePDE`, startup_func.jl:
122-275); a batch of independent problems has no exchange step, so on one
GB300 the problems share the device through concurrent CUDA streams:

* `workers` host threads each own a stream and take the next problem from a
  queue ordered largest first (longest-processing-time order);
* the library calls release the GIL (ctypes), so the threads drive the GPU
  at the same time; each problem's meshes run on the thread's stream;
* a problem's Newton work objects (Jacobian, preconditioner, Krylov basis)
  stay allocated between solves (`eg_newton_solve`), so a warm batch
  allocates nothing and no `cudaFree` serialises the streams;
* small Krylov solves run as one-block persistent kernels side by side;
  larger ones take the GPU one grid at a time (eg_arnoldi.cu), or, with
  batch_gmres, share cooperative launches (eg_arnoldi_batch.cu).

A problem that does not converge, or whose pseudo-time steps keep hitting a
non-physical state, is retried from its initial state with the initial
pseudo-time step divided by 4 (at most `retries` times).
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field

from .eulergpu import EulerGPUError, solve_steady


@dataclass
class SteadyProblem:
    """One steady solve: meshes of the continuation levels (lowest degree
    first), the initial state of levels[0] (a float64 CUDA tensor), Newton
    options and the tolerance of the intermediate levels."""
    levels: list
    q0: object
    opts: dict
    level_tol: float | None = None
    tag: object = None
    work: float = 0.0  # scheduling estimate (larger first)


@dataclass
class SteadyResult:
    tag: object
    q: object = None
    stats: list = field(default_factory=list)
    t_start: float = 0.0
    t_end: float = 0.0
    retries: int = 0
    error: str | None = None

    @property
    def seconds(self):
        return self.t_end - self.t_start


def solve_one(pr: SteadyProblem, precision=1, retries=2, stream=None) -> SteadyResult:
    """Solve one problem (on `stream`, a torch CUDA stream, when given)."""
    if stream is not None:
        for g in pr.levels:
            g.set_stream(stream.cuda_stream)
    res = SteadyResult(tag=pr.tag, t_start=time.perf_counter())
    opts = dict(pr.opts)
    for attempt in range(retries + 1):
        q = pr.q0.copy() if hasattr(pr.q0, "copy") and not hasattr(pr.q0, "clone") else pr.q0.clone()
        try:
            res.q, res.stats = solve_steady(pr.levels, q, opts, precision=precision,
                                            level_tol=pr.level_tol)
            res.error = None
            break
        except EulerGPUError as e:
            res.error = str(e)
            res.retries = attempt + 1
            opts["euler_tau"] = opts.get("euler_tau", 1.0) * 0.25
    res.t_end = time.perf_counter()
    return res


def solve_batch(problems, workers=8, precision=1, retries=2, batch_gmres=False):
    """Solve every problem; returns one SteadyResult per problem (in input
    order).  Each worker thread owns one CUDA stream.  With batch_gmres the
    workers' multi-block Krylov solves that meet in time run in shared
    cooperative launches (eg_set_gmres_batching); each result is the same bits
    as alone.  Off by default: on the batched workload a shared launch lasts as
    long as its longest solve, and the waiting of the shorter ones outweighs
    the sharing (2.96 against 3.10 solves/s)."""
    import torch

    from .eulergpu import set_gmres_batching
    set_gmres_batching(bool(batch_gmres))
    try:
        return _solve_batch(problems, workers, precision, retries)
    finally:
        set_gmres_batching(False)


def _solve_batch(problems, workers, precision, retries):
    import torch
    order = sorted(range(len(problems)), key=lambda i: -problems[i].work)
    lock = threading.Lock()
    pos = [0]
    results = [None] * len(problems)
    errors = []

    def worker():
        stream = torch.cuda.Stream()
        try:
            with torch.cuda.stream(stream):
                while True:
                    with lock:
                        if pos[0] >= len(order):
                            return
                        i = order[pos[0]]
                        pos[0] += 1
                    results[i] = solve_one(problems[i], precision, retries, stream)
        except Exception as e:  # surfaced to the caller below
            errors.append(e)

    threads = [threading.Thread(target=worker, daemon=True) for _ in range(max(1, workers))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return results
