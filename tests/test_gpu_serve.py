"""3-D Newton solves, new parameters on an existing device mesh, the
device-memory estimate, and the serving loop on the GPU.

Tolerances: Newton (FP64) state 1e-9 relative to max|q| and functional
1e-10; mixed functional 1e-8 (as for the 2-D solves).  Served results are
compared with the same requests solved alone: state 1e-10 relative to
max|q|, functional 1e-8 (a request's arithmetic does not depend on the mix,
so they agree to the last bit in practice).
"""
import ctypes as C

import numpy as np
import pytest

from pdesolver_gb300 import abi, eulergpu, problems, serve

pytestmark = pytest.mark.gpu

NEWTON_OPTS = {"res_abstol": 1e-10, "res_reltol": 1e-14, "itermax": 60, "krylov_reltol": 1e-2,
               "newton_globalize_euler": True, "euler_tau": 5.0}


def _cube(n, p, M=0.45, seed=11):
    levels, q0 = problems.cube_problem({"n": n, "p": p, "M_in": M, "seed": seed})
    return levels[-1][0], levels[-1][1], levels, q0


@pytest.mark.parametrize("p", [1, 2])
def test_newton_3d_matches_oracle(gpu_lib, oracle, p):
    """Newton-GMRES with pseudo-transient continuation on the warped cube
    (2^3 hexes -> 48 tets, diagonal-E tets, Roe faces, free-stream data)
    from the perturbed free stream, against the oracle's Newton."""
    ms, opts, _, _ = _cube(2, p)
    rng = np.random.default_rng(5)
    q0 = problems.free_stream(3, ms.coords.shape[:2], Ma=opts["Ma"])
    q0 = np.ascontiguousarray(q0 * (1 + rng.uniform(-0.01, 0.01, size=q0.shape)))
    g = eulergpu.GPUMesh(ms, opts)
    qo = q0.copy()
    o = eulergpu.NewtonOpts.from_opts(NEWTON_OPTS, 0)
    st = eulergpu.NewtonStats()
    assert oracle.oracle_newton(C.byref(g.desc.desc), C.byref(g.params), abi.dptr(qo), C.byref(o),
                                C.byref(st)) == 0
    fo = oracle.oracle_functional_pressure(C.byref(g.desc.desc), C.byref(g.params), abi.dptr(qo), 0)
    q64 = q0.copy()
    st = g.newton(q64, NEWTON_OPTS, precision=0)
    assert st.converged == 1 and st.res_norm < 1e-10
    assert np.abs(q64 - qo).max() <= 1e-9 * np.abs(qo).max()
    assert abs(g.functional_pressure(q64, 0) - fo) <= 1e-10 * abs(fo)
    q32 = q0.copy()
    st = g.newton(q32, NEWTON_OPTS, precision=1)
    assert st.converged == 1 and st.res_norm < 1e-10
    assert abs(g.functional_pressure(q32, 0) - fo) <= 1e-8 * abs(fo)


def test_set_params_equals_fresh_mesh(gpu_lib):
    """eg_mesh_set_params (new vortex Mach number) gives the residual of a
    mesh created with those parameters, bit for bit."""
    ms, opts, q = problems.config1(n=6, p=2)
    o2 = dict(opts, Ma=0.35, vortex_M_in=0.35)
    g = eulergpu.GPUMesh(ms, opts)
    g.set_params(o2)
    r1 = g.eval_residual(q, np.zeros_like(q))
    r2 = eulergpu.GPUMesh(ms, o2).eval_residual(q, np.zeros_like(q))
    r0 = eulergpu.GPUMesh(ms, opts).eval_residual(q, np.zeros_like(q))
    assert np.array_equal(r1, r2)
    assert not np.array_equal(r1, r0)


@pytest.mark.parametrize("case", ["annulus48_p3", "cube10_p2"])
def test_estimate_mem_bounds_what_the_library_takes(gpu_lib, case):
    """eg_estimate_mem against the device memory a mesh and its mixed-
    precision Newton work objects take (cudaMemGetInfo before and after);
    the cube's diagonal-E operator stores face-diagonal coupling blocks."""
    import torch
    torch.cuda.init()
    # load the kernels once (lazy module loading takes device memory too)
    ms_s, opts_s, q_s = problems.config2(n=4, p=3)
    gs = eulergpu.GPUMesh(ms_s, opts_s)
    gs.newton(q_s.copy(), dict(NEWTON_OPTS, itermax=200), precision=1)
    gs.close()
    if case == "annulus48_p3":
        ms, opts, q = problems.config2(n=48, p=3)
    else:
        ms = problems.request_meshes((3, 10, 2))[-1]
        levels, q = problems.request_problem({"dim": 3, "n": 10, "p": 2, "M_in": 0.5, "seed": 2},
                                             [ms])
        opts = levels[0][1]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    g = eulergpu.GPUMesh(ms, opts)
    try:
        g.newton(q.copy(), dict(NEWTON_OPTS, itermax=1), precision=1)
    except eulergpu.EulerGPUError:
        pass   # one iteration does not converge; the work objects exist
    torch.cuda.synchronize()
    taken = free0 - torch.cuda.mem_get_info()[0]
    est = eulergpu.estimate_mem(ms, precision=1)
    lib_bytes = est.total - est.eqn     # q and res are the caller's (host here)
    slack = est.allocations * (2 << 20)
    assert 0.9 * lib_bytes - slack <= taken <= 1.1 * lib_bytes + slack, (taken, lib_bytes)
    g.close()


def _requests():
    """a small 2-D / 3-D mix; two requests share a geometry with different
    Mach numbers (the second reuses the first one's device meshes)."""
    specs = [{"dim": 2, "n": 6, "p": 3, "M_in": 0.5},
             {"dim": 3, "n": 2, "p": 2, "M_in": 0.4},
             {"dim": 2, "n": 8, "p": 2, "M_in": 0.35},
             {"dim": 2, "n": 6, "p": 3, "M_in": 0.62},
             {"dim": 3, "n": 3, "p": 1, "M_in": 0.55},
             {"dim": 2, "n": 10, "p": 1, "M_in": 0.45}]
    reqs = []
    for k, sp in enumerate(specs):
        sp["seed"] = 100 + k
        levels, q0 = problems.request_problem(sp)
        reqs.append(serve.SolveRequest(rid=k, levels=levels, q0=q0, opts=NEWTON_OPTS,
                                       key=problems.geometry_key(sp), arrival=0.02 * k,
                                       level_tol=1e-4))
    return reqs


def test_served_results_equal_alone(gpu_lib):
    """continuous batching: six requests arriving 20 ms apart, up to four on
    the device at once, give the results of the same requests solved one at
    a time on a fresh server."""
    mix = serve.SteadySolveServer(8 << 30, slots=4, precision=1, batch_gmres=True)
    out = mix.serve(_requests())
    mix.close()
    assert all(r.error is None for r in out), [r.error for r in out]
    assert mix.peak_running >= 2
    for r in _requests():
        alone = serve.SteadySolveServer(8 << 30, slots=1, precision=1)
        a = alone.serve([serve.SolveRequest(rid=r.rid, levels=r.levels, q0=r.q0, opts=r.opts,
                                            key=r.key, level_tol=r.level_tol)])[0]
        alone.close()
        m = out[r.rid]
        assert a.error is None
        assert all(s["converged"] == 1 and s["res_norm"] < 1e-10 for s in m.stats[-1:])
        assert np.abs(m.q - a.q).max() <= 1e-10 * np.abs(a.q).max()
        assert abs(m.functional - a.functional) <= 1e-8 * abs(a.functional)


def test_batched_gmres_gives_the_same_bits_as_alone(gpu_lib):
    """eight steady solves of mixed sizes (one- and multi-block Krylov solves,
    2-D and 3-D) on eight threads with batched GMRES (several solves per
    cooperative launch, barriers over each solve's own blocks) give the
    states and iteration counts of the same solves run one at a time without
    batching."""
    import torch
    from pdesolver_gb300 import batch
    specs = [{"dim": 2, "n": 6, "p": 3}, {"dim": 2, "n": 10, "p": 2}, {"dim": 2, "n": 12, "p": 1},
             {"dim": 2, "n": 20, "p": 4}, {"dim": 3, "n": 3, "p": 2}, {"dim": 3, "n": 2, "p": 1},
             {"dim": 2, "n": 16, "p": 3}, {"dim": 2, "n": 24, "p": 2}]
    probs = []
    for k, sp in enumerate(specs):
        sp.update(M_in=0.35 + 0.04 * k, seed=200 + k)
        levels, q0 = problems.request_problem(sp)
        gl = [eulergpu.GPUMesh(ms, o) for ms, o in levels]
        probs.append(batch.SteadyProblem(levels=gl, q0=torch.from_numpy(q0).cuda(), opts=NEWTON_OPTS,
                                         level_tol=1e-4, tag=k, work=float(q0.size)))
    alone = [batch.solve_one(pr, precision=1) for pr in probs]
    mixed = batch.solve_batch(probs, workers=8, precision=1, batch_gmres=True)
    for a, b in zip(alone, mixed):
        assert a.error is None and b.error is None, (a.error, b.error)
        assert [s.krylov_iters for s in a.stats] == [s.krylov_iters for s in b.stats]
        assert torch.equal(a.q, b.q)


def test_preempted_request_resumes_bitwise(gpu_lib):
    """preemption at a continuation-level boundary: request 0 (2-D, p=1 then
    p=3) is stopped after its p=1 level, its state goes to host memory, the
    other requests run on the single slot, and it resumes from the snapshot;
    its final state and functional are bitwise those of the same request
    solved without interruption.  All three arrive at once, so request 0
    re-enters the queue behind the other two and finishes last."""
    reqs = _requests()[:3]
    for r in reqs:
        r.arrival = 0.0    # all queued when request 0 stops
    srv = serve.SteadySolveServer(8 << 30, slots=1, precision=1)
    srv.preempt(0)
    out = srv.serve(reqs)
    srv.close()
    assert all(r.error is None for r in out), [r.error for r in out]
    assert out[0].preemptions == 1 and len(out[0].stats) == 2
    assert out[0].done > out[1].done
    ref_srv = serve.SteadySolveServer(8 << 30, slots=1, precision=1)
    r0 = _requests()[0]
    ref = ref_srv.serve([serve.SolveRequest(rid=0, levels=r0.levels, q0=r0.q0, opts=r0.opts,
                                            key=r0.key, level_tol=r0.level_tol)])[0]
    ref_srv.close()
    assert ref.preemptions == 0
    assert np.array_equal(out[0].q, ref.q)
    assert out[0].functional == ref.functional
    assert [s["krylov_iters"] for s in out[0].stats] == [s["krylov_iters"] for s in ref.stats]
