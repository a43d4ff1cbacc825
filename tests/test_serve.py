"""Serving loop scheduling on the CPU (no GPU work): admission against the
HBM budget and the slot count, arrival-order admission with a bounded
bypass, reuse and eviction of idle device meshes, and the footprint model
(eg_estimate_mem, the counterpart of the reference's src/estimateMem.jl).

The device hooks of SteadySolveServer are replaced by fakes that sleep, so
these tests exercise exactly the host logic the GPU server runs."""
import threading
import time

import numpy as np
import pytest

from pdesolver_gb300 import eulergpu, problems, serve


class FakeDevice:
    """Stands in for the device hooks: records meshes made and closed and
    the requests running at each moment."""

    def __init__(self, seconds=0.02):
        self.seconds = seconds
        self.lock = threading.Lock()
        self.made = []
        self.closed = []
        self.running = set()
        self.max_running = 0
        self.order = []

    def make_meshes(self, req):
        with self.lock:
            self.made.append(req.rid)
        return [("mesh", req.rid)]

    def close_meshes(self, meshes):
        with self.lock:
            self.closed.append(meshes)

    def run(self, req, meshes, stream, res):
        with self.lock:
            self.running.add(req.rid)
            self.max_running = max(self.max_running, len(self.running))
            self.order.append(req.rid)
        time.sleep(req.opts.get("seconds", self.seconds))
        res.q = np.full(3, float(req.rid))
        with self.lock:
            self.running.discard(req.rid)


def make_server(dev, budget, slots, **kw):
    return serve.SteadySolveServer(budget, slots=slots, run_request=dev.run,
                                   make_meshes=dev.make_meshes, close_meshes=dev.close_meshes,
                                   make_stream=lambda: None, **kw)


def req(rid, fp, arrival=0.0, key=None, seconds=None):
    opts = {} if seconds is None else {"seconds": seconds}
    return serve.SolveRequest(rid=rid, levels=[], q0=np.zeros(1), opts=opts, key=key,
                              arrival=arrival, footprint=fp)


def test_budget_and_slots_are_never_exceeded():
    rng = np.random.default_rng(0)
    dev = FakeDevice(0.01)
    budget = 100
    srv = make_server(dev, budget, slots=4)
    reqs = [req(i, int(rng.integers(5, 60)), arrival=0.002 * i) for i in range(40)]
    out = srv.serve(reqs)
    assert all(r.error is None for r in out)
    assert [r.q[0] for r in out] == list(range(40))
    assert srv.peak_running <= 4 and dev.max_running <= 4
    assert srv.peak_bytes <= budget
    assert all(inflight <= budget for _, _, inflight, _ in srv.admission_log)
    s = serve.latency_summary(out)
    assert s["completed"] == 40 and s["latency_p99_s"] >= s["latency_p50_s"] > 0


def test_later_arrivals_start_while_earlier_ones_run():
    """continuous batching: a request that arrives while another runs is
    admitted into a free slot at once, not after the running one ends."""
    dev = FakeDevice()
    srv = make_server(dev, 100, slots=2)
    out = srv.serve([req(0, 10, 0.0, seconds=0.6), req(1, 10, 0.05, seconds=0.05)])
    assert out[1].admitted < out[0].done
    assert out[1].done < out[0].done
    assert out[1].queued < 0.2


def test_oversized_request_is_refused():
    dev = FakeDevice()
    srv = make_server(dev, 50, slots=2)
    out = srv.serve([req(0, 10), req(1, 51), req(2, 10)])
    assert out[1].error and "exceeds the HBM budget" in out[1].error
    assert out[0].error is None and out[2].error is None
    assert 1 not in dev.made


def test_bypass_of_a_waiting_request_is_bounded():
    """a request waiting for memory is passed by smaller later ones at most
    max_bypass times."""
    dev = FakeDevice()
    srv = make_server(dev, 100, slots=8, max_bypass=2)
    reqs = [req(0, 60, 0.0, seconds=0.6), req(1, 50, 0.01, seconds=0.05)]
    reqs += [req(2 + k, 10, 0.02 + 0.001 * k, seconds=0.3) for k in range(5)]
    out = srv.serve(reqs)
    assert all(r.error is None for r in out)
    bypassers = [r for r in out[2:] if r.admitted < out[1].admitted]
    assert len(bypassers) == 2
    # the waiting request enters once the first one has finished
    assert out[1].admitted >= out[0].done - 1e-3


def test_idle_meshes_are_reused_and_evicted_lru():
    dev = FakeDevice(0.005)
    srv = make_server(dev, 100, slots=1)
    # same key twice: the second request reuses the first one's meshes
    out = srv.serve([req(0, 40, 0.0, key="a"), req(1, 40, 0.05, key="a")])
    assert all(r.error is None for r in out)
    assert dev.made == [0] and srv.pool.bytes == 40
    # a new key that needs the pooled memory evicts it
    out = srv.serve([req(2, 70, 0.0, key="b")])
    assert out[0].error is None
    assert dev.closed == [[("mesh", 0)]]
    assert srv.pool.bytes == 70
    srv.close()
    assert srv.pool.bytes == 0 and len(dev.closed) == 2


def test_failed_request_is_reported_and_not_pooled():
    dev = FakeDevice()

    def run(r, meshes, stream, res):
        if r.rid == 1:
            raise RuntimeError("negative density")
        dev.run(r, meshes, stream, res)

    srv = serve.SteadySolveServer(100, slots=2, run_request=run, make_meshes=dev.make_meshes,
                                  close_meshes=dev.close_meshes, make_stream=lambda: None)
    out = srv.serve([req(0, 10, key="a"), req(1, 10, key="b")])
    assert out[0].error is None and "negative density" in out[1].error
    assert srv.pool.has("a") and not srv.pool.has("b")
    assert [("mesh", 1)] in dev.closed


def test_preempted_request_leaves_the_device_and_resumes_last():
    """preempt(rid): the request stops at its level boundary (the fake device
    returns a snapshot), releases its slot and memory, goes to the back of
    the queue, later resumes from its snapshot once, and completes with one
    result; the request waiting behind it runs in between."""
    dev = FakeDevice(seconds=0.03)
    seen = []

    def run(req, meshes, stream, res):
        seen.append((req.rid, None if req.snapshot is None else req.snapshot.level))
        dev.run(req, meshes, stream, res)
        if req.rid == 0 and req.snapshot is None:
            return serve.RequestSnapshot(level=1, q=np.zeros(3), opts={}, attempt=0, stats=[])
        assert req.rid != 0 or req.snapshot.level == 1
        return None

    srv = serve.SteadySolveServer(100, slots=1, run_request=run, make_meshes=dev.make_meshes,
                                  close_meshes=dev.close_meshes, make_stream=lambda: None)
    out = srv.serve([req(0, 50), req(1, 50, arrival=0.005)])
    assert [r.error for r in out] == [None, None]
    assert seen == [(0, None), (1, None), (0, 1)]
    assert out[0].preemptions == 1 and out[1].preemptions == 0
    assert out[0].done > out[1].done
    assert srv._in_flight == 0 and srv._running == 0


def test_estimate_mem_counts_the_newton_objects(gpu_lib):
    """eg_estimate_mem (loads the library, no device work): the Jacobian,
    inverse blocks and Krylov basis have the sizes the solver allocates."""
    ms, _, _ = problems.config2(n=16, p=3)
    nv, n, N = ms.numDofPerNode, ms.sbp.numnodes * ms.numDofPerNode, ms.numDof
    e32 = eulergpu.estimate_mem(ms, precision=1)
    e64 = eulergpu.estimate_mem(ms, precision=0)
    e0 = eulergpu.estimate_mem(ms)
    assert e0.jacobian == e0.pc == e0.krylov == e0.newton == 0
    assert e0.mesh == e32.mesh and e0.eqn == 2 * 8 * N
    assert e32.pc == -(-4 * ms.numEl * n * n // 512) * 512
    assert e64.pc == 2 * e32.pc
    assert e32.krylov >= 31 * N * 4 and e64.krylov >= 31 * N * 8
    assert e32.total == e32.mesh + e32.eqn + e32.jacobian + e32.pc + e32.krylov + e32.newton
    assert e64.total > e32.total
    # the mesh part holds at least the metric terms, state staging and face fluxes
    d = ms.dim
    assert e0.mesh >= 8 * ms.numEl * ms.sbp.numnodes * (d * d + 2) + 2 * 8 * N
    assert e32.allocations > e0.allocations > 20
    # a request's footprint: both continuation levels
    spec = {"n": 16, "p": 3, "M_in": 0.5, "seed": 1}
    levels, _ = problems.config4_problem(spec)
    fp = serve.request_footprint(levels, precision=1)
    assert fp > eulergpu.estimate_mem(levels[1][0], precision=1).total
    assert eulergpu.library().eg_estimate_mem(None, None) == 1   # EG_ERR_INVALID


def test_serving_stream_specs():
    specs = problems.config5_specs(count=400, seed=6)
    d3 = [s for s in specs if s["dim"] == 3]
    assert 0.12 < len(d3) / len(specs) < 0.28
    assert all(8 <= s["n"] <= 24 and s["p"] in (1, 2) for s in d3)
    d2 = [s for s in specs if s["dim"] == 2]
    assert all(8 <= s["n"] <= 96 and 1 <= s["p"] <= 4 for s in d2)
    assert all(0.3 <= s["M_in"] <= 0.7 and s["gap"] >= 0 for s in specs)
    assert problems.config5_specs(count=400, seed=6) == specs


def test_estimate_mem_face_diagonal_coupling(gpu_lib):
    """diagonal-E tets keep one nv x nv coupling block per stencil node: the
    estimate's Jacobian part drops by the dense blocks' share."""
    ms = problems.request_meshes((3, 4, 2))[-1]
    q = eulergpu.mem_query(ms, precision=1)
    assert q.face_diagonal == 1
    e_diag = eulergpu.estimate_mem(ms, precision=1)
    q.face_diagonal = 0
    e_dense = abi_estimate(q)
    nv, S, I = ms.numDofPerNode, ms.sbp.stencilsize, ms.numInterfaces
    dense_cpl = 4 * I * 2 * (S * nv) ** 2
    diag_cpl = 4 * I * 2 * S * nv * nv
    assert e_dense.jacobian - e_diag.jacobian == pytest.approx(dense_cpl - diag_cpl, abs=1024)
    assert eulergpu.mem_query(problems.request_meshes((2, 8, 3))[-1], 1).face_diagonal == 0


def abi_estimate(q):
    import ctypes as C
    from pdesolver_gb300 import abi
    out = abi.EgMemEstimate()
    eulergpu.check(eulergpu.library().eg_estimate_mem(C.byref(q), C.byref(out)))
    return out
