"""Steady-solve serving loop: continuous batching of requests on one GPU.

The reference runs one steady solve per process (`solvePDE`,
startup_func.jl:122-275) and sizes its memory offline with estimateMem.jl.
Here a server takes requests (mesh levels, degree, free stream, initial
state) as they arrive and keeps up to `slots` of them on the device at once:

* admission: a request enters when a slot is free and its device footprint
  (``eg_estimate_mem``: mesh, state, explicit Jacobian, block-Jacobi
  inverses, Krylov basis and Newton vectors of every continuation level)
  fits the HBM budget next to the requests in flight and the idle meshes
  kept for reuse.  Requests are taken in arrival order; when the oldest one
  waits for memory, later ones that fit may pass it, at most `max_bypass`
  times, after which nothing passes it until it is admitted;
* overlap: each slot is a host thread with its own CUDA stream; the library
  calls release the GIL, so the admitted requests' Newton iterations
  (residual, Jacobian, block inverse, one-block Krylov solves) run on the
  device side by side, multi-block Krylov solves take the GPU in turn (or,
  with batch_gmres, share cooperative launches, each on its own SMs); a
  request that arrives while others run starts as soon as a slot and memory
  free up, not when a batch ends;
* residency: a request's meshes, state, Jacobian and preconditioner stay on
  the device for its whole solve; afterwards its meshes (with the Newton work
  objects they keep) go to an idle pool keyed by geometry, so a later request
  on the same geometry allocates nothing.  Idle meshes are destroyed, least
  recently used first, when an admission needs their memory;
* each request's arithmetic does not depend on what else runs: its kernels
  see only its own arrays, and the block counts of its launches depend only
  on its own sizes, so a result is the same alone and in the mix;
* preemption (the serving counterpart of the reference's checkpoint/restart,
  src/Utils/checkpoint.jl): `preempt(rid)` stops a running request at its
  next continuation-level boundary.  Its state at that point (the converged
  state of the finished level, the Newton options of the current attempt, the
  statistics so far) is copied to host memory as a RequestSnapshot, its
  device slot and memory budget are released (its meshes, with their Newton
  work objects, go to the idle pool like a finished request's, where an
  admission that needs the memory evicts them), and the request goes to the
  back of the queue.  When it is admitted again it resumes from the snapshot
  on any slot: the prolongation and the next level's Newton solve start from
  the same bits, so the result is bitwise the one of an uninterrupted solve.

`SteadySolveServer.serve(requests)` replays the requests' arrival times in
real time and returns one result per request with its latency (completion
minus arrival) and queueing delay.
"""
from __future__ import annotations

import collections
import threading
import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class RequestSnapshot:
    """Host copy of a request's progress at a continuation-level boundary:
    `level` is the next level to solve, q the converged state of level
    `level - 1`, opts the Newton options of the current attempt (the
    pseudo-time step after retries), stats the finished levels' statistics."""
    level: int
    q: np.ndarray
    opts: dict
    attempt: int
    stats: list


@dataclass
class SolveRequest:
    """One steady solve.  levels: [(host Mesh, opts)] of the continuation
    levels, lowest degree first; q0: host initial state of levels[0]; key:
    geometry key (requests with equal keys share device meshes); arrival:
    seconds after the stream starts."""
    rid: int
    levels: list
    q0: np.ndarray
    opts: dict
    key: tuple = None
    arrival: float = 0.0
    level_tol: float | None = None
    functional_group: int | None = 0
    footprint: int = 0
    snapshot: RequestSnapshot | None = None   # set when the request was preempted


@dataclass
class RequestResult:
    rid: int
    q: np.ndarray | None = None      # final state (host)
    functional: float | None = None  # integral of p over the request's BC group
    stats: list = field(default_factory=list)
    arrival: float = 0.0             # host clock, seconds
    admitted: float = 0.0
    done: float = 0.0
    footprint: int = 0
    retries: int = 0
    launches: int = 0                # library kernel launches of the request
    preemptions: int = 0             # times the request was stopped and resumed
    error: str | None = None

    @property
    def latency(self):
        return self.done - self.arrival

    @property
    def queued(self):
        return self.admitted - self.arrival


def request_footprint(levels, precision, restart=30):
    """Estimated device bytes of a request: every level's mesh, state and
    Newton work objects (eg_estimate_mem), the prolongation matrix of each
    finer level, plus one level-0 state the server uploads."""
    from .eulergpu import estimate_mem
    total, prev = 0, None
    for ms, _ in levels:
        total += estimate_mem(ms, precision=precision, restart=restart, prolong_from=prev).total
        prev = ms.sbp
    ms0 = levels[0][0]
    return int(total + 8 * ms0.numEl * ms0.sbp.numnodes * ms0.numDofPerNode)


class MeshPool:
    """Idle device meshes by geometry key, least recently used first."""

    def __init__(self):
        self._idle = collections.OrderedDict()   # key -> list of (meshes, bytes)
        self.bytes = 0

    def has(self, key):
        return bool(self._idle.get(key))

    def take(self, key):
        lst = self._idle.get(key)
        if not lst:
            return None
        meshes, nbytes = lst.pop()
        if not lst:
            del self._idle[key]
        self.bytes -= nbytes
        return meshes, nbytes

    def give(self, key, meshes, nbytes):
        self._idle.setdefault(key, []).append((meshes, nbytes))
        self._idle.move_to_end(key)
        self.bytes += nbytes

    def evict(self):
        """remove the least recently used idle entry; returns (meshes, bytes)
        or None.  The caller destroys the meshes."""
        for key in list(self._idle):
            meshes, nbytes = self._idle[key].pop(0)
            if not self._idle[key]:
                del self._idle[key]
            self.bytes -= nbytes
            return meshes, nbytes
        return None

    def drain(self):
        out = [m for lst in self._idle.values() for m, _ in lst]
        self._idle.clear()
        self.bytes = 0
        return out


class SteadySolveServer:
    """Continuous-batching server of steady solves on the current GPU.

    hbm_budget: device bytes the requests (in flight + idle pool) may hold.
    slots: requests on the device at once (one host thread and CUDA stream
    each).  precision: 1 mixed (FP32 Jacobian, PC, Krylov), 0 plain FP64.

    run_request / make_meshes / close_meshes / make_stream are the device
    hooks; tests replace them to check the scheduling on the CPU.
    """

    def __init__(self, hbm_budget, slots=8, precision=1, retries=2, max_bypass=8,
                 run_request=None, make_meshes=None, close_meshes=None, make_stream=None,
                 clock=time.perf_counter, batch_gmres=False):
        self.budget = int(hbm_budget)
        self.slots = int(slots)
        self.precision = int(precision)
        self.retries = int(retries)
        self.max_bypass = int(max_bypass)
        self.clock = clock
        self.batch_gmres = bool(batch_gmres) and run_request is None
        self._run_request = run_request or self._gpu_run_request
        self._make_meshes = make_meshes or self._gpu_make_meshes
        self._close_meshes = close_meshes or self._gpu_close_meshes
        self._make_stream = make_stream or self._gpu_make_stream
        self.pool = MeshPool()
        self._cv = threading.Condition()
        self._pending = collections.deque()
        self._in_flight = 0          # bytes of admitted requests
        self._running = 0
        self._head_bypassed = 0
        self._closed = False
        self._results = {}
        self._preempt = set()        # rids to stop at their next level boundary
        self._threads = []
        self.peak_bytes = 0
        self.peak_running = 0
        self.admission_log = []      # (time, rid, bytes in flight after, pool bytes)

    # ---- device hooks ----------------------------------------------------
    @staticmethod
    def _gpu_make_stream():
        import torch
        return torch.cuda.Stream()

    @staticmethod
    def _gpu_make_meshes(req):
        from .eulergpu import GPUMesh
        return [GPUMesh(ms, opts) for ms, opts in req.levels]

    @staticmethod
    def _gpu_close_meshes(meshes):
        for g in meshes:
            g.close()

    def _gpu_run_request(self, req, meshes, stream, res):
        """Run (or resume) a request; returns a RequestSnapshot when it was
        preempted at a level boundary, else None."""
        for g, (_, opts) in zip(meshes, req.levels):
            g.set_stream(stream.cuda_stream)
            if g.opts != opts:
                g.set_params(opts)
        l0 = sum(g.timings().launches for g in meshes)
        try:
            return self._gpu_solve(req, meshes, stream, res)
        finally:
            res.launches += sum(g.timings().launches for g in meshes) - l0

    def _gpu_solve(self, req, meshes, stream, res):
        """The p-continuation solve of eulergpu.solve_steady level by level,
        with the retry rule of batch.solve_one (from the initial state, the
        initial pseudo-time step divided by 4), resumable from a snapshot and
        stoppable at a level boundary."""
        import torch

        from .eulergpu import EulerGPUError, prolong
        snap = req.snapshot
        attempt = snap.attempt if snap else 0
        opts = dict(snap.opts) if snap else dict(req.opts)
        with torch.cuda.stream(stream):
            while True:
                try:
                    if snap is not None:
                        start, stats = snap.level, list(snap.stats)
                        q = torch.from_numpy(np.ascontiguousarray(snap.q)).to("cuda")
                    else:
                        start, stats = 0, []
                        q = torch.from_numpy(np.ascontiguousarray(req.q0)).to("cuda")
                    snap = None
                    for k in range(start, len(meshes)):
                        g = meshes[k]
                        if k > 0:
                            ms = g.mesh
                            qn = q.new_zeros((ms.numEl, ms.numNodesPerElement, ms.numDofPerNode))
                            prolong(meshes[k - 1], q, g, qn)
                            q = qn
                        o = dict(opts)
                        if k < len(meshes) - 1 and req.level_tol is not None:
                            o["res_abstol"] = req.level_tol
                        stats.append(g.newton(q, o, precision=self.precision).asdict())
                        if k < len(meshes) - 1 and req.rid in self._preempt:
                            self._preempt.discard(req.rid)
                            return RequestSnapshot(level=k + 1, q=q.cpu().numpy(), opts=opts,
                                                   attempt=attempt, stats=stats)
                    break
                except EulerGPUError as e:
                    attempt += 1
                    res.retries = attempt
                    if attempt > self.retries:
                        res.error = str(e)
                        res.stats = stats
                        return None
                    opts["euler_tau"] = opts.get("euler_tau", 1.0) * 0.25
            res.stats = stats
            if req.functional_group is not None:
                res.functional = meshes[-1].functional_pressure(q, req.functional_group)
            res.q = q.cpu().numpy()
        return None

    # ---- scheduling ------------------------------------------------------
    def _pick(self):
        """index in _pending of the request to admit now, or None; called
        with the lock held and a free slot.  A request fits when its
        footprint fits next to the requests in flight: idle pooled meshes
        are evicted to make room (a pooled entry of its own key is reused)."""
        for k, req in enumerate(self._pending):
            if k > 0 and self._head_bypassed >= self.max_bypass:
                return None
            if self._in_flight + req.footprint <= self.budget:
                return k
        return None

    def _admit(self):
        """called with the lock held: admit one request if possible; returns
        (req, meshes or None, evicted list) or None."""
        if self._running >= self.slots or not self._pending:
            return None
        k = self._pick()
        if k is None:
            return None
        req = self._pending[k]
        del self._pending[k]
        if k > 0:
            self._head_bypassed += 1
        else:
            self._head_bypassed = 0
        taken = self.pool.take(req.key) if req.key is not None else None
        evicted = []
        while self._in_flight + self.pool.bytes + req.footprint > self.budget:
            ev = self.pool.evict()
            if ev is None:
                break
            evicted.append(ev[0])
        self._in_flight += req.footprint
        self._running += 1
        self.peak_bytes = max(self.peak_bytes, self._in_flight + self.pool.bytes)
        self.peak_running = max(self.peak_running, self._running)
        self.admission_log.append((self.clock(), req.rid, self._in_flight, self.pool.bytes))
        return req, (taken[0] if taken else None), evicted

    def _worker(self):
        stream = self._make_stream()
        while True:
            with self._cv:
                while True:
                    if self._closed and not self._pending:
                        return
                    got = self._admit()
                    if got is not None:
                        break
                    self._cv.wait(0.05)
            req, meshes, evicted = got
            for m in evicted:
                self._close_meshes(m)
            res = self._results[req.rid]
            if req.snapshot is None:
                res.admitted = self.clock()
            res.footprint = req.footprint
            snap = None
            try:
                if meshes is None:
                    meshes = self._make_meshes(req)
                snap = self._run_request(req, meshes, stream, res)
            except Exception as e:  # reported per request
                res.error = f"{type(e).__name__}: {e}"
            stopped = isinstance(snap, RequestSnapshot) and res.error is None
            if not stopped:
                res.done = self.clock()
            with self._cv:
                self._in_flight -= req.footprint
                self._running -= 1
                if stopped:
                    # the request leaves the device: state on the host, back
                    # of the queue, resumed from the snapshot when admitted
                    req.snapshot = snap
                    res.preemptions += 1
                    self._pending.append(req)
                else:
                    req.snapshot = None
                    self._preempt.discard(req.rid)
                if meshes is not None and req.key is not None and res.error is None:
                    self.pool.give(req.key, meshes, req.footprint)
                    meshes = None
                self._cv.notify_all()
            if meshes is not None:
                self._close_meshes(meshes)

    def start(self):
        if self.batch_gmres:
            from .eulergpu import set_gmres_batching
            set_gmres_batching(True)
        self._closed = False
        self._threads = [threading.Thread(target=self._worker, daemon=True)
                         for _ in range(self.slots)]
        for t in self._threads:
            t.start()

    def preempt(self, rid):
        """Stop request `rid` at its next continuation-level boundary (see the
        module docstring): its state moves to host memory, its slot and
        memory are released, and it resumes later from there.  A request
        that has no level boundary left finishes normally."""
        with self._cv:
            self._preempt.add(rid)

    def submit(self, req: SolveRequest):
        """queue a request now (its arrival is the current clock)."""
        res = RequestResult(rid=req.rid, arrival=self.clock())
        if req.footprint > self.budget:
            res.error = f"footprint {req.footprint} B exceeds the HBM budget {self.budget} B"
            res.admitted = res.done = res.arrival
            with self._cv:
                self._results[req.rid] = res
                self._cv.notify_all()
            return res
        with self._cv:
            self._results[req.rid] = res
            self._pending.append(req)
            self._cv.notify_all()
        return res

    def finish(self):
        """wait until every submitted request is done; stop the workers."""
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()
        self._threads = []
        if self.batch_gmres:
            from .eulergpu import set_gmres_batching
            set_gmres_batching(False)

    def close(self):
        """destroy the idle device meshes."""
        for m in self.pool.drain():
            self._close_meshes(m)

    def serve(self, requests, footprint=None):
        """Replay `requests` at their arrival times (seconds after the call)
        and return their results in input order.  footprint(req) sets
        req.footprint when given (default: request_footprint of its levels)."""
        for r in requests:
            if footprint is not None:
                r.footprint = int(footprint(r))
            elif not r.footprint:
                r.footprint = request_footprint(r.levels, self.precision)
        order = sorted(range(len(requests)), key=lambda i: requests[i].arrival)
        self.start()
        t0 = self.clock()
        out = {}
        for i in order:
            req = requests[i]
            delay = t0 + req.arrival - self.clock()
            if delay > 0:
                time.sleep(delay)
            out[i] = self.submit(req)
        self.finish()
        return [out[i] for i in range(len(requests))]


def latency_summary(results):
    """p50 / p99 latency and queueing delay, solves/s over the stream."""
    ok = [r for r in results if r.error is None]
    if not ok:
        return {"completed": 0, "failed": len(results)}
    lat = np.array([r.latency for r in ok])
    que = np.array([r.queued for r in ok])
    span = max(r.done for r in ok) - min(r.arrival for r in results)
    return {"completed": len(ok), "failed": len(results) - len(ok),
            "solves_per_s": len(ok) / span if span > 0 else float("inf"),
            "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_max_s": float(lat.max()),
            "queued_p50_s": float(np.percentile(que, 50)),
            "queued_p99_s": float(np.percentile(que, 99)),
            "span_s": span}
