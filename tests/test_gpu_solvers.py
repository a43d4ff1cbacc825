"""GPU Jacobian, block-Jacobi preconditioner, GMRES, Newton, RK4 and the
boundary functional against the CPU oracle (through the C ABI).

Tolerances: Jacobian (FP64) 1e-10 relative to the largest entry; block
inverse 1e-12; Newton (FP64) converged state and functional 1e-10, mixed
(FP32 Jacobian/PC/Krylov) functional 1e-8; RK4 1e-11.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import block_apply, block_apply_t, oracle_jacobian, oracle_jvp
from pdesolver_gb300 import abi, eulergpu, problems

pytestmark = pytest.mark.gpu


def setup(fam="gamma", p=3, n=4, flux="RoeFlux", seed=51):
    ms, opts, q = problems.config1(n=n, p=p, family=fam, seed=seed)
    opts = dict(opts, Flux_name=flux)
    g = eulergpu.GPUMesh(ms, opts)
    return ms, opts, q, g


@pytest.mark.parametrize("fam,p,flux", [("omega", 2, "RoeFlux"), ("gamma", 3, "RoeFlux"),
                                        ("gamma", 2, "IRFlux"), ("gamma", 4, "RoeFlux")])
def test_jacobian_blocks_fp64(gpu_lib, oracle, fam, p, flux):
    ms, opts, q, g = setup(fam, p, flux=flux)
    lo = eulergpu.LinearOperator(g, precision=0)
    lo.calc(q)
    d, c = lo.blocks()
    rd, rc = oracle_jacobian(oracle, g.desc, g.params, ms, q)
    scale = max(np.abs(rd).max(), np.abs(rc).max())
    assert np.abs(d - rd).max() <= 1e-10 * scale
    assert np.abs(c - rc).max() <= 1e-10 * scale


@pytest.mark.parametrize("p,flux", [(1, "RoeFlux"), (2, "RoeFlux"), (2, "IRFlux"), (3, "RoeFlux")])
def test_jacobian_blocks_tet(gpu_lib, oracle, p, flux):
    """warped cube (2^3 x 6 tets), diagonal-E tets (face nodes are volume
    nodes: the element face terms and coupling blocks take the one-term path),
    weak-form volume, at a perturbed free stream: FP64 blocks 1e-10, FP32
    1e-5 relative to the largest entry."""
    ms, opts, q = problems.config3(n=2, p=p, seed=71)
    opts = dict(opts, Flux_name=flux, volume_integral_type=1)
    g = eulergpu.GPUMesh(ms, opts)
    rd, rc = oracle_jacobian(oracle, g.desc, g.params, ms, q)
    scale = max(np.abs(rd).max(), np.abs(rc).max())
    v = np.random.default_rng(8).normal(size=q.shape)
    jv = oracle_jvp(oracle, g.desc, g.params, q, v)
    for prec, tol in ((0, 1e-10), (1, 1e-5)):
        lo = eulergpu.LinearOperator(g, precision=prec)
        lo.calc(q)
        d, c = lo.blocks()
        assert np.abs(d - rd).max() <= tol * scale
        assert np.abs(c - rc).max() <= tol * scale
        # operator apply (face-diagonal coupling rows) == J v
        y = lo.apply(np.ascontiguousarray(v), np.zeros_like(v))
        assert np.abs(y - jv).max() <= tol * np.abs(jv).max()


def test_jacobian_fp32_and_apply(gpu_lib, oracle):
    ms, opts, q, g = setup()
    rd, rc = oracle_jacobian(oracle, g.desc, g.params, ms, q)
    scale = max(np.abs(rd).max(), np.abs(rc).max())
    lo32 = eulergpu.LinearOperator(g, precision=1)
    lo32.calc(q)
    d, c = lo32.blocks()
    assert np.abs(d - rd).max() <= 1e-5 * scale
    # FP64 operator apply == dual-number directional derivative of the residual
    lo = eulergpu.LinearOperator(g, precision=0)
    lo.calc(q)
    rng = np.random.default_rng(9)
    for _ in range(3):
        v = rng.normal(size=q.shape)
        y = lo.apply(np.ascontiguousarray(v), np.zeros_like(v))
        jv = oracle_jvp(oracle, g.desc, g.params, q, v)
        assert np.abs(y - jv).max() <= 1e-10 * np.abs(jv).max()
        y32 = lo32.apply(np.ascontiguousarray(v), np.zeros_like(v))
        assert np.abs(y32 - jv).max() <= 1e-5 * np.abs(jv).max()


def test_block_jacobi_inverse(gpu_lib, oracle):
    """test/euler/test_jac.jl:3073-3140: the element block-Jacobi
    preconditioner inverts the element blocks (1e-12)."""
    ms, opts, q, g = setup()
    lo = eulergpu.LinearOperator(g, precision=0)
    lo.calc(q)
    pc = eulergpu.BlockJacobiPC(lo)
    pc.calc()
    d, _ = lo.blocks()
    x = np.random.default_rng(3).normal(size=q.shape)
    b = np.einsum("ecr,ec->er", d, x.reshape(d.shape[0], -1)).reshape(q.shape)
    y = pc.apply(np.ascontiguousarray(b), np.zeros_like(b))
    assert np.abs(y - x).max() <= 1e-12 * np.abs(x).max() * 10


@pytest.mark.parametrize("case", ["gamma1", "gamma2", "gamma4", "omega4", "tet1", "tet2"])
@pytest.mark.parametrize("precision", [0, 1])
def test_block_inverse_every_block_size(gpu_lib, case, precision):
    """block inverses of 12 .. 115 unknowns (shared-memory Gauss-Jordan up to
    32 unknowns, register-tiled above): M^-1 (D x) = x for the element blocks
    D at a perturbed state; FP64 1e-12, FP32 1e-4 relative (times 10)."""
    if case.startswith("tet"):
        levels, q = problems.cube_problem({"n": 2, "p": int(case[-1]), "M_in": 0.5, "seed": 9})
        ms, opts = levels[-1]
        if len(levels) > 1:
            q = problems.free_stream(3, ms.coords.shape[:2], Ma=0.5)
            q = np.ascontiguousarray(q * (1 + np.random.default_rng(9).uniform(-0.01, 0.01, q.shape)))
    else:
        ms, opts, q = problems.config1(n=4, p=int(case[-1]), family=case[:-1], seed=61)
    g = eulergpu.GPUMesh(ms, opts)
    lo = eulergpu.LinearOperator(g, precision=precision)
    lo.calc(q)
    pc = eulergpu.BlockJacobiPC(lo)
    pc.calc()
    d, _ = lo.blocks()
    x = np.random.default_rng(4).normal(size=q.shape)
    b = np.einsum("ecr,ec->er", d, x.reshape(d.shape[0], -1)).reshape(q.shape)
    y = pc.apply(np.ascontiguousarray(b), np.zeros_like(b))
    tol = 1e-12 if precision == 0 else 1e-4
    assert np.abs(y - x).max() <= tol * np.abs(x).max() * 10


@pytest.mark.parametrize("precision,tol", [(0, 1e-8), (1, 1e-4)])
def test_gmres_solves(gpu_lib, precision, tol):
    ms, opts, q, g = setup(n=6)
    lo = eulergpu.LinearOperator(g, precision=precision)
    lo.calc(q)
    pc = eulergpu.BlockJacobiPC(lo)
    pc.calc()
    ls = eulergpu.LinearSolver(pc, lo, restart=30)
    ls.set_tolerances(reltol=tol, abstol=0.0, itermax=3000)
    b = np.random.default_rng(7).normal(size=q.shape)
    x = np.zeros_like(b)
    st = ls.solve(b, x)
    assert st.converged == 1
    assert 0 <= st.reorth <= st.iters
    lo64 = eulergpu.LinearOperator(g, precision=0)
    lo64.calc(q)
    r = b - lo64.apply(x, np.zeros_like(x))
    assert np.linalg.norm(r) <= 3 * tol * np.linalg.norm(b)


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-5)])
def test_gmres_cluster_matches_grid_solves(gpu_lib, precision, tol):
    """A small system (operator well under 2 MB) is solved by one 16-block
    thread-block cluster by default; the same system on a one-block and on a
    12-block cooperative grid (eg_ls_set_grid) reaches the same true residual
    tolerance in about the same number of Krylov iterations (the block
    partition changes only the order of the reductions).  Two default solves
    give the same bits."""
    ms, opts, q, g = setup(n=8, p=2, fam="gamma")
    lo = eulergpu.LinearOperator(g, precision=precision)
    lo.calc(q)
    pc = eulergpu.BlockJacobiPC(lo)
    pc.calc()
    ls = eulergpu.LinearSolver(pc, lo, restart=30)
    ls.set_tolerances(reltol=tol, abstol=0.0, itermax=3000)
    b = np.random.default_rng(23).normal(size=q.shape)
    lo64 = eulergpu.LinearOperator(g, precision=0)
    lo64.calc(q)
    xs, its = [], []
    for grid in (0, 0, 1, 12):
        ls.set_grid(grid)
        x = np.zeros_like(b)
        st = ls.solve(b, x)
        assert st.converged == 1
        r = b - lo64.apply(x, np.zeros_like(x))
        assert np.linalg.norm(r) <= 3 * tol * np.linalg.norm(b), grid
        xs.append(x)
        its.append(st.iters)
    ls.set_grid(0)
    assert np.array_equal(xs[0], xs[1])          # the cluster solve is deterministic
    assert max(its) <= 1.1 * min(its) + 3, its


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-5)])
def test_gmres_transpose_solves(gpu_lib, precision, tol):
    """linearSolveTranspose in the library (eg_ls_solve_transpose): J^T x = b
    against the dense solve of the transposed FP64 blocks (FP64 to 1e-10
    relative residual; FP32 operator and Krylov to 1e-5), host and device
    arrays, and the forward solve on the same solver object still works."""
    torch = pytest.importorskip("torch")
    ms, opts, q, g = setup(n=4, p=2, fam="gamma")
    lo = eulergpu.LinearOperator(g, precision=precision)
    lo.calc(q)
    pc = eulergpu.BlockJacobiPC(lo)
    pc.calc()
    ls = eulergpu.LinearSolver(pc, lo, restart=30)
    ls.set_tolerances(reltol=tol, abstol=0.0, itermax=2000)
    b = np.random.default_rng(17).normal(size=q.shape)
    x = np.zeros_like(b)
    st = ls.solve_transpose(b, x)
    assert st.converged == 1 and st.iters > 0
    lo64 = eulergpu.LinearOperator(g, precision=0)
    lo64.calc(q)
    r = b - lo64.apply_transpose(x, np.zeros_like(x))
    assert np.linalg.norm(r) <= 3 * tol * np.linalg.norm(b)
    xd = torch.zeros(ms.numDof, dtype=torch.float64, device="cuda")
    bd = torch.from_numpy(b.reshape(-1)).cuda()
    st2 = ls.solve_transpose(bd, xd)
    assert st2.iters == st.iters
    assert np.abs(xd.cpu().numpy().reshape(x.shape) - x).max() <= 1e-12 * np.abs(x).max()
    # the forward solve of the same solver is untouched by the transposed one
    y = np.zeros_like(b)
    assert ls.solve(b, y).converged == 1
    rf = b - lo64.apply(y, np.zeros_like(y))
    assert np.linalg.norm(rf) <= 3 * tol * np.linalg.norm(b)


NEWTON_OPTS = {"res_abstol": 1e-10, "res_reltol": 1e-14, "itermax": 150,
               "newton_globalize_euler": True, "euler_tau": 0.5, "krylov_reltol": 1e-2}


def _oracle_newton(oracle, g, q):
    o = eulergpu.NewtonOpts.from_opts(NEWTON_OPTS, 0)
    st = eulergpu.NewtonStats()
    rc = oracle.oracle_newton(C.byref(g.desc.desc), C.byref(g.params), abi.dptr(q), C.byref(o),
                              C.byref(st))
    assert rc == 0, (rc, st.asdict())
    return st


def test_newton_fp64_and_mixed_match_oracle(gpu_lib, oracle):
    """Newton-GMRES with pseudo-transient continuation from the perturbed free
    stream to |R| < 1e-10 (8x8 annulus, SBP-Gamma p=3).  FP64: state and
    integral of p along r = 1 agree with the oracle's Newton to 1e-10;
    mixed (FP32 Jacobian, PC, Krylov): functional within 1e-8."""
    ms, opts, q0 = problems.config2(n=8)
    g = eulergpu.GPUMesh(ms, opts)
    qo = q0.copy()
    _oracle_newton(oracle, g, qo)
    fo = oracle.oracle_functional_pressure(C.byref(g.desc.desc), C.byref(g.params), abi.dptr(qo), 0)
    q64 = q0.copy()
    st = g.newton(q64, NEWTON_OPTS, precision=0)
    assert st.converged == 1 and st.res_norm < 1e-10
    assert np.abs(q64 - qo).max() <= 1e-9 * np.abs(qo).max()
    f64 = g.functional_pressure(q64, 0)
    assert abs(f64 - fo) <= 1e-10 * abs(fo)
    q32 = q0.copy()
    st = g.newton(q32, NEWTON_OPTS, precision=1)
    assert st.converged == 1 and st.res_norm < 1e-10
    f32 = g.functional_pressure(q32, 0)
    assert abs(f32 - fo) <= 1e-8 * abs(fo)


def test_rk4_matches_oracle(gpu_lib, oracle):
    ms, opts, q0 = problems.config1()
    g = eulergpu.GPUMesh(ms, opts)
    h = 1e-3
    qg = q0.copy()
    g.rk4(qg, h, 10 * h)
    qo = q0.copy()
    st = eulergpu.Rk4Stats()
    assert oracle.oracle_rk4(C.byref(g.desc.desc), C.byref(g.params), abi.dptr(qo), C.c_double(h),
                             C.c_double(10 * h), 0, C.c_double(-1.0), C.byref(st)) == 0
    assert st.steps == 10
    assert np.abs(qg - qo).max() <= 1e-11 * np.abs(qo).max()


def test_rk4_graph_path_equals_eager_path(gpu_lib):
    """eg_rk4 replays each step as a CUDA graph when the timers are off and
    launches the same kernels one by one when they are on: the states, step
    counts and norms are bitwise equal, for whole steps, for the per-step
    norm test (res_tol) and for the itermax stop after stage 1."""
    ms, opts, q0 = problems.config1(n=6, p=2, seed=12)
    g = eulergpu.GPUMesh(ms, opts)
    h = 2e-3
    for itermax, res_tol in ((0, -1.0), (0, 1e-30), (4, -1.0)):
        out = []
        for timers in (False, True, False):
            g.set_timing(timers)
            q = q0.copy()
            st = g.rk4(q, h, 7 * h, itermax=itermax, res_tol=res_tol)
            out.append((q, st.steps, st.t, st.res_norm))
        g.set_timing(False)
        for q, steps, t, nrm in out[1:]:
            assert np.array_equal(q, out[0][0])
            assert (steps, t, nrm) == out[0][1:]
    # one device step of the graph path counts its kernels like the eager path
    l0 = g.timings().launches
    g.rk4(q0.copy(), h, 3 * h)
    l1 = g.timings().launches
    g.set_timing(True)
    g.rk4(q0.copy(), h, 3 * h)
    g.set_timing(False)
    assert g.timings().launches - l1 == l1 - l0


def test_wrong_sized_state_is_refused(gpu_lib):
    """a state of another degree's mesh is refused before any device work."""
    import torch
    ms, opts, q = problems.config1(n=3, p=1, seed=3)
    ms3, opts3, _ = problems.config1(n=3, p=3, seed=3)
    g3 = eulergpu.GPUMesh(ms3, opts3)
    with pytest.raises(ValueError):
        g3.functional_pressure(q, 0)
    with pytest.raises(ValueError):
        g3.functional_pressure(torch.from_numpy(q).cuda(), 0)


def test_functional_matches_oracle(gpu_lib, oracle):
    ms, opts, q = problems.config1()
    g = eulergpu.GPUMesh(ms, opts)
    for grp in range(len(ms.bc_types)):
        fo = oracle.oracle_functional_pressure(C.byref(g.desc.desc), C.byref(g.params), abi.dptr(q), grp)
        assert abs(g.functional_pressure(q, grp) - fo) <= 1e-13 * abs(fo)


@pytest.mark.parametrize("precision", [0, 1])
def test_newton_single_block_gmres_with_large_chunk(gpu_lib, precision):
    """a small p=1 system (16x16 annulus, 512 elements) runs its GMRES as one
    persistent block whose element chunk takes 40 KB of dynamic shared memory
    next to the kernel's static shared memory (FP64: above the default 48 KB
    per-block limit unless the kernel opts in)."""
    ms, opts, q0 = problems.config2(n=16, p=1)
    g = eulergpu.GPUMesh(ms, opts)
    q = q0.copy()
    st = g.newton(q, NEWTON_OPTS, precision=precision)
    assert st.converged == 1 and st.res_norm < 1e-10


@pytest.mark.parametrize("device_state", [False, True])
def test_newton_graph_path_equals_eager_path(gpu_lib, device_state):
    """one Newton iteration as three CUDA graphs around the persistent GMRES
    launch gives the eagerly launched iteration's result bit for bit (phase
    timers force the eager path)."""
    import torch
    ms, opts, q0 = problems.config2(n=8, p=2)
    g = eulergpu.GPUMesh(ms, opts)
    qa = torch.from_numpy(q0).cuda() if device_state else q0.copy()
    st = g.newton(qa, NEWTON_OPTS, precision=1)
    assert st.converged == 1 and st.graph_iters == st.iters > 0
    g.set_timing(True)
    qb = torch.from_numpy(q0).cuda() if device_state else q0.copy()
    st2 = g.newton(qb, NEWTON_OPTS, precision=1)
    g.set_timing(False)
    assert st2.converged == 1 and st2.graph_iters == 0 and st2.iters == st.iters
    a = qa.cpu().numpy() if device_state else qa
    b = qb.cpu().numpy() if device_state else qb
    assert np.array_equal(a, b)
    # a second graph solve reuses the captured graphs
    qc = q0.copy()
    st3 = g.newton(qc, NEWTON_OPTS, precision=1)
    assert st3.graph_iters == st3.iters and np.array_equal(qc, a)


@pytest.mark.parametrize("case", ["gamma3", "tet2"])
def test_transposed_operator_and_preconditioner(gpu_lib, oracle, case):
    """applyLinearOperatorTranspose / applyPCTranspose: y = J^T x against the
    oracle's blocks (dense coupling for SBP-Gamma, face-diagonal for the
    diagonal-E tets), and M^-T (D^T x) = x; FP64 1e-12, FP32 1e-5."""
    if case == "tet2":
        ms, opts, q = problems.config3(n=2, p=2, seed=81)
        opts = dict(opts, Flux_name="RoeFlux", volume_integral_type=1)
    else:
        ms, opts, q = problems.config1(n=4, p=3, family="gamma", seed=82)
    g = eulergpu.GPUMesh(ms, opts)
    rd, rc = oracle_jacobian(oracle, g.desc, g.params, ms, q)
    x = np.random.default_rng(12).normal(size=q.shape)
    ref = block_apply_t(ms, rd, rc, x)
    for prec, tol in ((0, 1e-12), (1, 1e-5)):
        lo = eulergpu.LinearOperator(g, precision=prec)
        lo.calc(q)
        y = lo.apply_transpose(np.ascontiguousarray(x), np.zeros_like(x))
        assert np.abs(y - ref).max() <= tol * np.abs(ref).max() * 10
        pc = eulergpu.BlockJacobiPC(lo)
        pc.calc()
        d, _ = lo.blocks()
        b = np.einsum("ecr,er->ec", d, x.reshape(d.shape[0], -1)).reshape(q.shape)
        z = pc.apply_transpose(np.ascontiguousarray(b), np.zeros_like(b))
        assert np.abs(z - x).max() <= (1e-11 if prec == 0 else 1e-4) * np.abs(x).max()


@pytest.mark.parametrize("case", ["tet1", "tet2", "tet3", "gamma2"])
def test_split_form_jacobian_blocks(gpu_lib, oracle, case):
    """element blocks of the entropy-stable split form (Hadamard pair terms
    differentiated pair by pair) with IR faces against the oracle: FP64 1e-10,
    FP32 1e-5 relative to the largest entry; the operator apply equals the
    residual's directional derivative.  tet3 (diagonal-E p=3, 45 nodes, 225
    unknowns per element) accumulates its blocks in place in device memory."""
    if case.startswith("tet"):
        ms, opts, q = problems.config3(n=2, p=int(case[-1]), seed=91)
    else:
        ms, opts, q = problems.config1(n=4, p=2, family="gamma", seed=92)
        opts = dict(opts, Flux_name="IRFlux", volume_integral_type=2, Volume_flux_name="IRFlux")
    g = eulergpu.GPUMesh(ms, opts)
    rd, rc = oracle_jacobian(oracle, g.desc, g.params, ms, q)
    scale = max(np.abs(rd).max(), np.abs(rc).max())
    v = np.random.default_rng(13).normal(size=q.shape)
    jv = oracle_jvp(oracle, g.desc, g.params, q, v)
    for prec, tol in ((0, 1e-10), (1, 1e-5)):
        lo = eulergpu.LinearOperator(g, precision=prec)
        lo.calc(q)
        d, c = lo.blocks()
        assert np.abs(d - rd).max() <= tol * scale, (prec, np.abs(d - rd).max() / scale)
        assert np.abs(c - rc).max() <= tol * scale
        y = lo.apply(np.ascontiguousarray(v), np.zeros_like(v))
        assert np.abs(y - jv).max() <= tol * np.abs(jv).max() * 10


def test_newton_entropy_stable_3d_matches_oracle(gpu_lib, oracle):
    """steady Newton solve of the entropy-stable discretisation (split-form
    volume, IR faces) on the warped 2^3 x 6 cube from a perturbed free
    stream: FP64 state 1e-9 and functional 1e-10 against the oracle's Newton,
    mixed functional 1e-8."""
    ms, opts, q0 = problems.config3(n=2, p=1, seed=93)
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


@pytest.mark.parametrize("case", ["annulus_wall", "cube_wall"])
def test_wall_residual_and_jacobian_match_oracle(gpu_lib, oracle, case):
    """the entropy-stable no-penetration wall (noPenetrationESBC, bc.jl:
    767-795): residual 1e-12 and Jacobian blocks (FP64) 1e-10 against the
    oracle, weak form with Roe faces (annulus, inner arc a wall) and split
    form with IR faces (warped cube, face z = 0 a wall)."""
    from conftest import oracle_residual
    ms, opts, q = getattr(problems, case)()
    g = eulergpu.GPUMesh(ms, opts)
    r = np.zeros_like(q)
    g.eval_residual(q, r)
    ro = oracle_residual(oracle, g.desc, g.params, q)
    assert np.abs(r - ro).max() <= 1e-12 * np.abs(ro).max()
    lo = eulergpu.LinearOperator(g, precision=0)
    lo.calc(q)
    d, c = lo.blocks()
    rd, rc = oracle_jacobian(oracle, g.desc, g.params, ms, q)
    scale = max(np.abs(rd).max(), np.abs(rc).max())
    assert np.abs(d - rd).max() <= 1e-10 * scale
    assert np.abs(c - rc).max() <= 1e-10 * scale


def test_newton_entropy_stable_wall_matches_oracle(gpu_lib, oracle):
    """steady Newton solve of the entropy-stable discretisation with a wall
    (split form, IR faces, noPenetrationESBC on z = 0, free stream elsewhere)
    on the warped 2^3 x 6 cube, diagonal-E p=1: FP64 state 1e-9 and the
    pressure integral over the wall 1e-10 against the oracle's Newton, mixed
    precision 1e-8.  (At p=2 the entropy-conservative interior fluxes leave
    the Newton iteration stagnating near |R| = 3e-4, in the oracle as on the
    device.)"""
    ms, opts, q0 = problems.cube_wall(n=2, p=1)
    wall = int(np.nonzero(ms.bc_types == 2)[0][0])
    g = eulergpu.GPUMesh(ms, opts)
    qo = q0.copy()
    o = eulergpu.NewtonOpts.from_opts(NEWTON_OPTS, 0)
    st = eulergpu.NewtonStats()
    assert oracle.oracle_newton(C.byref(g.desc.desc), C.byref(g.params), abi.dptr(qo), C.byref(o),
                                C.byref(st)) == 0
    fo = oracle.oracle_functional_pressure(C.byref(g.desc.desc), C.byref(g.params), abi.dptr(qo), wall)
    q64 = q0.copy()
    st = g.newton(q64, NEWTON_OPTS, precision=0)
    assert st.converged == 1 and st.res_norm < 1e-10
    assert np.abs(q64 - qo).max() <= 1e-9 * np.abs(qo).max()
    assert abs(g.functional_pressure(q64, wall) - fo) <= 1e-10 * abs(fo)
    q32 = q0.copy()
    st = g.newton(q32, NEWTON_OPTS, precision=1)
    assert st.converged == 1 and st.res_norm < 1e-10
    assert abs(g.functional_pressure(q32, wall) - fo) <= 1e-8 * abs(fo)


def test_config1_rk4_at_cfl(gpu_lib, oracle):
    """Config 1 (b): 100 RK4 steps of the 512-triangle vortex annulus at CFL
    0.4, delta_t = CFL min_el_size / max wave speed (startup_func.jl:241-247,
    calcMaxWaveSpeed euler_funcs.jl:1810-1834), against the oracle's RK4 at
    1e-11; the wave speed against numpy at 1e-14."""
    ms, opts, q0 = problems.config1()
    g = eulergpu.GPUMesh(ms, opts)
    rho = q0[..., 0]
    u = q0[..., 1:3] / rho[..., None]
    p = 0.4 * (q0[..., 3] - 0.5 * rho * (u ** 2).sum(-1))
    ref = (np.sqrt(1.4 * p / rho) + np.sqrt((u ** 2).sum(-1))).max()
    assert abs(g.max_wave_speed(q0) - ref) <= 1e-14 * ref
    h = g.cfl_time_step(q0, 0.4)
    assert h == pytest.approx(0.4 * ms.min_el_size / ref, rel=1e-14)
    qg = q0.copy()
    st = g.rk4(qg, h, 100 * h)
    assert st.steps == 100
    qo = q0.copy()
    sto = eulergpu.Rk4Stats()
    assert oracle.oracle_rk4(C.byref(g.desc.desc), C.byref(g.params), abi.dptr(qo), C.c_double(h),
                             C.c_double(100 * h), 0, C.c_double(-1.0), C.byref(sto)) == 0
    assert sto.steps == 100
    assert np.abs(qg - qo).max() <= 1e-11 * np.abs(qo).max()
