#!/usr/bin/env python3
"""Benchmark of the GB300 Euler SBP hot path.

Headline workload (one step = one steady solve): the 64x64 quarter annulus
(8192 triangles), SBP-Gamma p=3, Roe faces, isentropic-vortex Dirichlet data
(M_in 0.5), started from the free stream (rho 1, Ma 0.5, aoa 0) times
(1 + U(-0.01, 0.01)) with seed 2, solved by Newton-GMRES(30) with the element
block-Jacobi preconditioner and pseudo-transient continuation to
calcNorm(R, M^-1) < 1e-10, with p-continuation (p = 1 to 1e-4, prolonged to
p = 3).  `value` is mixed-precision solves/s (FP64 residual and update, FP32
Jacobian / preconditioner / Krylov); the plain-FP64 solve rate is reported
beside it.  A second section measures FP64 residual evaluations/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c1|c2|c3|c4|c5|tune|gmres-grid] [--only KERNELS]

Other workloads: c1 (512-triangle vortex, RK4 at CFL 0.4, residual evals/s),
c3 (82,944-tet entropy-stable RK4), c4 (batch of 96 uneven steady solves),
c5 (served Poisson stream of steady solves, mixed against FP64), tune (the
element-kernel autotuner sweep), gmres-grid (persistent GMRES grid sizes);
--only runs isolated kernels for profiler captures.

--impl reference times the CPU restatement of the reference algorithm (the
oracle port; Julia, SummationByParts.jl, PUMI and PETSc are not available)
on the host cores with all threads.

Multi-GPU: independent problems have no exchange step: N ranks solve N
replicas of one mesh (c2, c3) or shards of the batch (c4), with no collective
on the data path.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as graft  # noqa: E402

graft.load_package()
from pdesolver_gb300 import abi, problems  # noqa: E402

WORKLOAD = ("steady Euler solve: annulus 64x64 (8192 triangles), SBP-Gamma p=3, Roe, isentropic "
            "vortex Dirichlet data (M_in 0.5), start free stream * (1 + U(-0.01,0.01)) seed 2, "
            "Newton-GMRES(30) + element block-Jacobi + pseudo-transient continuation to "
            "|R|_{M^-1} < 1e-10, p-continuation 1 -> 3")
NEWTON_OPTS = {"res_abstol": 1e-10, "res_reltol": 1e-14, "itermax": 200, "krylov_reltol": 1e-2,
               "newton_globalize_euler": True, "euler_tau": 5.0}
LEVEL_TOL = 1e-4
LEVELS = (1, 3)


def residual_model(ms):
    """Algorithmic bytes and FP64 flops of one residual evaluation.

    bytes: 8 [Ndof (q read + res write) + E Np (d^2 + 1) (dxidx, jac) +
    I Nf d (nrm_face) + B Nf 2d (coords_bndry, nrm_bndry)] + 4 (5 I + 2 B)
    (index ints); every array counted once.
    flops (FP64): per node d Euler fluxes (14 flops in 2D, 20 in 3D); Q^T F
    contraction 2 d Np^2 nv per element; per face node interpolation of both
    sides 2*2 S nv and a Roe flux (~130 flops); face lifting 2 F S Nf nv per
    element (S = face stencil size).
    """
    op = ms.sbp
    d, E, Np, Nf, S = ms.dim, ms.numEl, op.numnodes, op.numfacenodes, op.stencilsize
    I, B, nv = ms.numInterfaces, ms.numBoundaryFaces, d + 2
    ndof = E * Np * nv
    nbytes = 8 * (2 * ndof + E * Np * (d * d + 1) + I * Nf * d + B * Nf * 2 * d) + 4 * (5 * I + 2 * B)
    fl_node = 14 if d == 2 else 20
    flops = (E * Np * d * fl_node + 2 * d * Np * Np * nv * E
             + (I + B) * Nf * (2 * 2 * S * nv + 130) + 2 * (d + 1) * S * Nf * nv * E)
    return nbytes, flops


def krylov_kernel_bytes(ms, es):
    """Algorithmic bytes of one operator apply (element blocks + coupling
    blocks + x + y) and one block-Jacobi apply (inverse blocks + x + y), es
    bytes per value."""
    nv = ms.numDofPerNode
    n = ms.sbp.numnodes * nv
    nb = ms.sbp.stencilsize * nv
    ndof = ms.numDof
    spmv = es * (ms.numEl * n * n + ms.numInterfaces * 2 * nb * nb + 2 * ndof)
    pc = es * (ms.numEl * n * n + 2 * ndof)
    return spmv, pc


def gmres_bytes(ms, its, m, es):
    """Algorithmic bytes of one GMRES(m) solve in the persistent kernel with
    `its` Arnoldi iterations (full cycles but the last), es bytes per value.
    Arnoldi iteration j (basis v_0..v_j): the inverse blocks and the coupling
    blocks once (the operator I + C D^-1), v_j read and w written by the
    operator, one Gram-Schmidt pass (dots: v_0..v_j and w read; update:
    v_0..v_j and w read, v_{j+1} written), i.e. (2 j + 7) vectors.  Per cycle:
    the residual b - J x (element and coupling blocks, x, b, r and v_0: 5
    vectors) and the update x += D^-1 V y (jdone + 3 vectors and the inverse
    blocks); one more residual ends the solve.  No cache reuse is credited,
    and the second Gram-Schmidt passes are not counted."""
    nv = ms.numDofPerNode
    n = ms.sbp.numnodes * nv
    nb = ms.sbp.stencilsize * nv
    N = ms.numDof
    blocks = ms.numEl * n * n
    cpl = 2 * ms.numInterfaces * nb * nb
    total, left = 0, its
    while left > 0:
        jd = min(m, left)
        total += sum(blocks + cpl + (2 * j + 7) * N for j in range(jd))
        total += blocks + cpl + 5 * N            # residual at the cycle start
        total += blocks + (jd + 3) * N           # x += D^-1 V y
        left -= jd
    total += blocks + cpl + 5 * N                # final residual
    return es * total


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for s in self.samples for n, v in zip(names, s[3:7]) if v == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def measure_fp64_peak(torch):
    """FP64 throughput of a cuBLAS DGEMM (TFLOP/s): the FP64 denominator."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def _oracle():
    from pdesolver_gb300 import build
    lib = C.CDLL(build.build_oracle())
    lib.oracle_set_threads.restype = C.c_int
    return lib


def _oracle_steady():
    """oracle/steady.py: the host steady solve with p-continuation (the
    oracle, used by the CPU legs only)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import steady
    from pdesolver_gb300 import build
    build.build_oracle()
    return steady


def c2_levels():
    """(mesh, opts) per continuation level and the start state of the
    headline workload."""
    levels, q0 = [], None
    for p in LEVELS:
        ms, opts, q = problems.config2(p=p)
        levels.append((ms, opts))
        if q0 is None:
            q0 = q
    return levels, q0


def cpu_solve(threads, levels=None, q0=None):
    """One full steady solve of the headline workload by the CPU oracle (the
    restatement of the reference's Newton-GMRES path), timed end to end on
    `threads` host threads: Newton p=1 to 1e-4, prolongation, Newton p=3 to
    |R| < 1e-10.  Returns (seconds, threads used, converged state, per-level
    stats, functional)."""
    steady = _oracle_steady()
    lib = steady.load()
    used = lib.oracle_set_threads(int(threads))
    if levels is None:
        levels, q0 = c2_levels()
    q, st, sec = steady.solve_steady(lib, levels, q0, NEWTON_OPTS, LEVEL_TOL)
    f = steady.functional_pressure(lib, levels[-1][0], levels[-1][1], q)
    return sec, used, q, st, f


def cpu_residual_rate(ms, opts, q, budget_s=5.0, threads=1):
    from pdesolver_gb300 import eulergpu
    lib = _oracle()
    used = lib.oracle_set_threads(int(threads))
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    res = np.zeros_like(q)
    lib.oracle_eval_residual(C.byref(desc.desc), C.byref(P), abi.dptr(q), abi.dptr(res))
    n, t0 = 0, time.perf_counter()
    while True:
        lib.oracle_eval_residual(C.byref(desc.desc), C.byref(P), abi.dptr(q), abi.dptr(res))
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s:
            break
    return n / el, used, n, el


# wall-clock budget of the reference arm's timed solves (each a full solve of
# about 40 s on 16 Arm cores); fewer than --steps solves run when it is spent
REFERENCE_BUDGET_S = 480.0


def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # one step = one complete steady solve by the oracle on all host threads
    # (measured, not extrapolated); one untimed warm-up solve, then timed
    # solves until --steps are done or the budget is spent
    levels, q0 = c2_levels()
    warm = min(1, max(0, args.warmup))
    for _ in range(warm):
        cpu_solve(threads, levels, q0)
    secs, used, st, f = [], threads, None, None
    t_start = time.perf_counter()
    while len(secs) < max(1, args.steps):
        sec, used, _, st, f = cpu_solve(threads, levels, q0)
        secs.append(sec)
        if time.perf_counter() - t_start + sec > REFERENCE_BUDGET_S:
            break
    rate = len(secs) / sum(secs)
    sample = ("%d complete steady solves (Newton p=1 to 1e-4, prolongation, Newton p=3 to "
              "|R| < 1e-10) of the full 8192-triangle problem, each timed end to end; %d untimed "
              "warm-up solve(s); solve times %s s" % (len(secs), warm, [round(x, 2) for x in secs]))
    line = {
        "metric": "steady solves/s", "value": rate, "unit": "solves/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": len(secs), "warmup": warm, "steps_requested": args.steps,
        "warmup_requested": args.warmup, "ms_per_step": 1e3 / rate,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD},
        "cpu_baseline": {"value": rate, "unit": "solves/s", "cores": used, "kind": "port",
                         "sample": sample},
        "e2e": {"value": rate, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "newton": [{"p": p, "newton_its": s.iters, "krylov_its": s.krylov_iters,
                    "res_norm": s.res_norm} for p, s in zip(LEVELS, st)],
        "functional_r1": f,
        "note": "CPU restatement of the reference Newton-GMRES path (oracle port, OpenMP, all host "
                "threads), FP64 throughout as the reference's PETSc solve; the Julia reference "
                "cannot run here (no Julia, SummationByParts.jl, PUMI, PETSc). Steps beyond the "
                "%.0f s budget are not run (steps < steps_requested)" % REFERENCE_BUDGET_S,
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, dist):
    import torch
    from pdesolver_gb300 import eulergpu
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    levels, level_opts, q_init = [], [], None
    for p in LEVELS:
        ms, opts, q = problems.config2(p=p)
        g = eulergpu.GPUMesh(ms, opts)
        g.set_stream(stream.cuda_stream)
        levels.append(g)
        level_opts.append(opts)
        if q_init is None:
            q_init = q
    ms3 = levels[-1].mesh
    q0 = torch.from_numpy(q_init).cuda()
    qwork = torch.empty_like(q0)

    def solve(prec):
        qwork.copy_(q0)
        return eulergpu.solve_steady(levels, qwork, NEWTON_OPTS, precision=prec, level_tol=LEVEL_TOL)

    def launches():
        return sum(g.timings().launches for g in levels)

    for _ in range(args.warmup):
        solve(1)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = launches()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    stats_mixed = None
    with ClockSampler(dev) as clk:
        for k in range(args.steps):
            evs[k][0].record()
            q3, stats_mixed = solve(1)
            evs[k][1].record()
        torch.cuda.synchronize()
    n_launch = launches() - l0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = sum(step_ms)
    if dist:
        t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * args.steps / (total_ms * 1e-3)
    f_mixed = levels[-1].functional_pressure(q3, 0)
    q_mixed = q3.clone()

    # plain FP64 solves
    n64 = max(1, args.steps // 3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(n64):
        q64, stats64 = solve(0)
    e1.record()
    torch.cuda.synchronize()
    fp64_rate = n64 / (e0.elapsed_time(e1) * 1e-3)
    f64 = levels[-1].functional_pressure(q64, 0)

    # end to end through the public API with host buffers
    qh = q_init.copy()
    t0 = time.perf_counter()
    n_e2e = max(1, args.steps // 3)
    for _ in range(n_e2e):
        qh[...] = q_init
        eulergpu.solve_steady(levels, qh, NEWTON_OPTS, precision=1, level_tol=LEVEL_TOL)
    e2e_rate = world * n_e2e / (time.perf_counter() - t0)
    nb1 = q_init.nbytes
    nb3 = ms3.numDof * 8
    h2d = nb1 + nb1 + nb3        # Newton p=1 in, prolongation input, Newton p=3 in
    d2h = nb1 + nb3 + nb3        # Newton p=1 out, prolongation output, Newton p=3 out

    # the Krylov kernels of the mixed solve, timed alone (FP32 operator at the
    # converged state), L2 flushed before each launch
    lo = eulergpu.LinearOperator(levels[-1], precision=1)
    lo.calc(q_mixed)
    pc = eulergpu.BlockJacobiPC(lo)
    pc.calc()
    x = torch.randn(ms3.numDof, dtype=torch.float32, device="cuda")
    y = torch.empty_like(x)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    reps = 20
    t_spmv = t_pc = 0.0
    for _ in range(reps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        lo.apply_native(x, y)
        b.record()
        flush.zero_()
        c, d = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c.record()
        pc.apply_native(x, y)
        d.record()
        torch.cuda.synchronize()
        t_spmv += a.elapsed_time(b) / reps
        t_pc += c.elapsed_time(d) / reps
    b_spmv, b_pc = krylov_kernel_bytes(ms3, 4)

    # the persistent GMRES kernel (one launch per linear solve) on the same
    # system: 300 iterations (10 full cycles), L2 flushed before each solve
    ls = eulergpu.LinearSolver(pc, lo, restart=30)
    gm_its = 300
    ls.set_tolerances(reltol=1e-30, abstol=0.0, itermax=gm_its)
    bvec = torch.randn(ms3.numDof, dtype=torch.float64, device="cuda")
    xvec = torch.zeros_like(bvec)
    ls.solve(bvec, xvec)
    gm_ms = []
    for _ in range(3):
        xvec.zero_()
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        st_gm = ls.solve(bvec, xvec)
        b.record()
        torch.cuda.synchronize()
        gm_ms.append(a.elapsed_time(b))
    t_gm = statistics.median(gm_ms)
    b_gm = gmres_bytes(ms3, st_gm.iters, 30, 4)

    # FP64 residual evaluations/s (L2 flushed between evaluations)
    ms2, opts2, qr = problems.config2()
    gres = eulergpu.GPUMesh(ms2, opts2)
    gres.set_stream(stream.cuda_stream)
    qd = torch.from_numpy(qr).cuda()
    rd = torch.zeros_like(qd)
    for _ in range(3):
        gres.eval_residual_async(qd, rd)
    # launch shape of the element kernel picked by the autotuner
    res_tune = gres.autotune(qd, reps=10)
    res_cfg = gres.launch_config()
    for _ in range(3):
        gres.eval_residual_async(qd, rd)
    gres.set_timing(True)
    gres.reset_timings()
    nres = 30
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nres)]
    for k in range(nres):
        flush.zero_()
        ev[k][0].record()
        gres.eval_residual_async(qd, rd)
        ev[k][1].record()
    torch.cuda.synchronize()
    tm = gres.timings()
    gres.set_timing(False)
    res_ms = sum(a.elapsed_time(b) for a, b in ev) / nres
    rbytes, rflops = residual_model(ms2)
    t_face = tm.t_face_flux / nres
    t_elem = tm.t_element / nres

    if rank != 0:
        return
    peaks, src = measured_peaks()
    fp64_peak = measure_fp64_peak(torch)
    dom_name, dom_ms, dom_bytes = "k_gmres_coop", t_gm, b_gm
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic = None
    traffic_source = None
    try:
        # DRAM bytes per Arnoldi iteration from an ncu capture of the same
        # kernel on the same system (profiles/), scaled to this launch
        with open(os.path.join(ROOT, "profiles", "krylov_c2_traffic.json")) as f:
            rec = json.load(f)
        per_it = rec.get("k_gmres_coop_bytes_per_iteration")
        if per_it:
            traffic = per_it * st_gm.iters
            traffic_source = ("profiles/krylov_c2_traffic.json (captured %s): %s; DRAM bytes per "
                              "iteration x %d iterations" % (rec.get("captured", "?"), rec.get("source", ""),
                                                              st_gm.iters))
    except (OSError, ValueError, AttributeError):
        pass
    # the CPU oracle: one complete solve on all host threads (the CPU
    # baseline, measured end to end), whose converged state and functional
    # are also the reference values of the errors below
    cpu_levels = [(g.mesh, o) for g, o in zip(levels, level_opts)]
    cpu_sec, cpu_threads, q_orc, st_orc, f_orc = cpu_solve(os.cpu_count() or 1, cpu_levels, q_init)
    steady = _oracle_steady()
    olib = steady.load()
    olib.oracle_set_threads(os.cpu_count() or 1)
    ms3_, opts3_ = cpu_levels[-1]
    qm_h = q_mixed.cpu().numpy()
    q64_h = q64.cpu().numpy()
    res_orc = steady.residual(olib, ms2, opts2, qr)
    res_gpu = rd.cpu().numpy()
    err = {
        "residual_fp64": float(np.abs(res_gpu - res_orc).max() / np.abs(res_orc).max()),
        "state_fp64": float(np.abs(q64_h - q_orc).max() / np.abs(q_orc).max()),
        "state_mixed": float(np.abs(qm_h - q_orc).max() / np.abs(q_orc).max()),
        "functional_fp64": abs(f64 - f_orc) / abs(f_orc),
        "functional_mixed": abs(f_mixed - f_orc) / abs(f_orc),
        "oracle_residual_at_state_fp64": steady.strong_norm(
            olib, ms3_, steady.residual(olib, ms3_, opts3_, q64_h)),
        "oracle_residual_at_state_mixed": steady.strong_norm(
            olib, ms3_, steady.residual(olib, ms3_, opts3_, qm_h)),
        "oracle_res_norm": st_orc[-1].res_norm,
        "what": "max-norm relative errors against the CPU oracle on the same inputs: the FP64 "
                "residual at the start state; the converged states and the integral of p along "
                "r=1 of the FP64 and mixed solves against the oracle's own FP64 solve; and "
                "|R|_{M^-1} of the oracle's residual at each device state",
    }
    r_cpu, _, r_n, r_el = cpu_residual_rate(ms2, opts2, qr, budget_s=3.0, threads=1)
    line = {
        "metric": "steady solves/s", "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "elements": ms3.numEl, "ndof": ms3.numDof,
                   "precision": "mixed: FP64 residual/norm/update, FP32 Jacobian/PC/Krylov",
                   "l2": "working set (FP32 Jacobian 100 MB + inverse blocks 75 MB + Krylov basis "
                         "47 MB) exceeds the 129 MB L2",
                   "parallelism": f"replicas x{world}"},
        "newton": {"levels": [{"p": p, "newton_its": s.iters, "krylov_its": s.krylov_iters,
                               "res_norm": s.res_norm, "t_residual_ms": s.t_residual,
                               "t_jacobian_ms": s.t_jacobian, "t_pc_ms": s.t_pc,
                               "t_krylov_ms": s.t_krylov} for p, s in zip(LEVELS, stats_mixed)],
                   "fp64_solves_per_s": fp64_rate, "mixed_over_fp64": value / world / fp64_rate,
                   "fp64_counts": {str(p): [s.iters, s.krylov_iters] for p, s in zip(LEVELS, stats64)},
                   "functional_r1_mixed": f_mixed, "functional_r1_fp64": f64,
                   "functional_rel_diff": abs(f_mixed - f64) / abs(f64)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                     "traffic_source": traffic_source, "peak_source": src,
                     "kernel": dom_name + " (FP32: one launch = one GMRES(30) solve of the p=3 "
                               "Newton system at the converged state, %d iterations)" % st_gm.iters,
                     "algorithmic_bytes_per_launch": dom_bytes, "kernel_ms": dom_ms,
                     "us_per_iteration": 1e3 * dom_ms / max(st_gm.iters, 1)},
        "krylov_kernels_ms": {"k_spmv (stream path)": t_spmv, "k_block_apply (stream path)": t_pc,
                              "k_spmv_GBs": b_spmv / (t_spmv * 1e-3) / 1e9},
        "residual": {"evals_per_s": 1e3 / res_ms, "ms_per_eval": res_ms,
                     "phases_ms": {"k_face_flux": t_face, "k_element": t_elem},
                     "element_launch_config": res_cfg,
                     "autotune_ms": [[c["elements_per_cta"], int(c["volume_mma"]), ms]
                                     for c, ms in res_tune],
                     "hbm_frac": rbytes / ((t_face + t_elem) * 1e-3) / 1e9 / peaks["hbm_gbs"],
                     "fp64_tflops": rflops / ((t_face + t_elem) * 1e-3) / 1e12,
                     "fp64_frac_of_dgemm": rflops / ((t_face + t_elem) * 1e-3) / 1e12 / fp64_peak,
                     "dgemm_fp64_tflops": fp64_peak,
                     "cpu_evals_per_s_1core": r_cpu},
        "cpu_baseline": {"value": 1.0 / cpu_sec, "unit": "solves/s", "cores": cpu_threads,
                         "kind": "port",
                         "sample": "one complete steady solve of this workload by the oracle (FP64, "
                                   "all host threads), timed end to end: %.1f s, Newton/Krylov "
                                   "iterations %s" % (cpu_sec, [[s.iters, s.krylov_iters]
                                                                for s in st_orc])},
        "error_vs_oracle": err,
        "e2e": {"value": e2e_rate, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(n_launch),
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


C3_WORKLOAD = ("explicit RK4: unit cube 24^3 hexes -> 6 tets (82,944 elements), warped (0.05 sin, "
               "seeded phase, quadratic geometry), diagonal-E p=2 (23 nodes), Ismail-Roe split-form "
               "volume + IR faces, free-stream boundaries, Mach 0.5 free stream with density * "
               "(1 + N(0, 0.01)) seed 4; one step = one RK4 time step (4 FP64 residuals), dt 1e-3")


def split_model(ms):
    """FP64 flops of one split-form residual: per node pair one direction
    n_jk (2 d^2 flops), one Ismail-Roe average from per-node quantities
    (~40 flops + 8 divisions, a division counted as 1) and one projection
    (~4 nv flops), plus the per-node square roots / logarithms (counted 4 +
    2) and the IR face flux per face node (~70 flops) with face lifting."""
    op = ms.sbp
    d, E, Np, Nf = ms.dim, ms.numEl, op.numnodes, op.numfacenodes
    nv = d + 2
    P = Np * (Np - 1) // 2
    pair = 2 * d * d + 48 + 4 * nv + 2 * nv
    flops = E * P * pair + E * Np * 12 + (ms.numInterfaces + ms.numBoundaryFaces) * Nf * 90 \
        + 2 * (d + 1) * Nf * nv * E
    nbytes = 8 * (2 * ms.numDof + E * Np * (d * d + 1)) + 8 * ms.numInterfaces * Nf * d
    return nbytes, flops


def run_c3(args, rank, world):
    """3-D entropy-stable explicit workload (one step = one RK4 step)."""
    import torch
    from pdesolver_gb300 import eulergpu
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    t0 = time.perf_counter()
    ms, opts, q = problems.config3()
    t_mesh = time.perf_counter() - t0
    g = eulergpu.GPUMesh(ms, opts)
    g.set_stream(stream.cuda_stream)
    qd = torch.from_numpy(q).cuda()
    # elements per CTA of the split-form kernel picked by the autotuner
    tune = g.autotune(qd, reps=5)
    cfg = g.launch_config()
    h = 1e-3   # the oracle is unstable at 2e-3 on this mesh, stable at 1.5e-3 on 12^3
    nsteps = max(args.steps, 1)
    for _ in range(args.warmup):
        g.rk4(qd, h, h)
    qd.copy_(torch.from_numpy(q))
    torch.cuda.synchronize()
    l0 = g.timings().launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        e0.record()
        st = g.rk4(qd, h, nsteps * h)
        e1.record()
        torch.cuda.synchronize()
    n_launch = g.timings().launches - l0
    total_ms = e0.elapsed_time(e1)
    value = world * st.steps / (total_ms * 1e-3)
    # residual phase times (L2 flushed; inputs > L2 anyway)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    rd = torch.zeros_like(qd)
    g.set_timing(True)
    g.reset_timings()
    nres = 5
    for _ in range(nres):
        flush.zero_()
        g.eval_residual_async(qd, rd)
    tm = g.timings()
    g.set_timing(False)
    t_face, t_elem = tm.t_face_flux / nres, tm.t_element / nres
    # end to end with host buffers
    qh = q.copy()
    t1 = time.perf_counter()
    g.set_stream(None)
    st2 = g.rk4(qh, h, nsteps * h)
    e2e = world * st2.steps / (time.perf_counter() - t1)
    if rank != 0:
        return
    peaks, src = measured_peaks()
    fp64_peak = measure_fp64_peak(torch)
    nbytes, flops = split_model(ms)
    t_res = (t_face + t_elem) * 1e-3
    lib = _oracle()
    used = lib.oracle_set_threads(1)
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    res = np.zeros_like(q)
    tc = time.perf_counter()
    lib.oracle_eval_residual(C.byref(desc.desc), C.byref(P), abi.dptr(q), abi.dptr(res))
    t_cpu_res = time.perf_counter() - tc
    # errors against the oracle on the same inputs: the residual at the start
    # state, and 5 RK4 steps (the oracle on all host threads)
    rg = np.zeros_like(q)
    g.eval_residual(q, rg)
    qg5 = q.copy()
    g.rk4(qg5, h, 5 * h)
    steady = _oracle_steady()
    olib = steady.load()
    olib.oracle_set_threads(os.cpu_count() or 1)
    qo5 = q.copy()
    steady.rk4(olib, ms, opts, qo5, h, 5)
    err = {"residual": float(np.abs(rg - res).max() / np.abs(res).max()),
           "rk4_5_steps_state": float(np.abs(qg5 - qo5).max() / np.abs(qo5).max()),
           "what": "max-norm relative errors against the CPU oracle on the same inputs (full mesh)"}
    line = {
        "metric": "RK4 steps/s", "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": st.steps, "warmup": args.warmup, "ms_per_step": total_ms / max(st.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": C3_WORKLOAD, "elements": ms.numEl, "ndof": ms.numDof,
                   "res_tol": "off (no per-step norm readback)",
                   "l2": "inputs (q 76 MB, metrics 137 MB) exceed the 129 MB L2",
                   "mesh_setup_s": t_mesh},
        "roofline": {"bound": "fp64", "achieved": flops / t_res / 1e12, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": flops / t_res / 1e12 / fp64_peak,
                     "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                     "kernel": "residual (k_face_flux IR + k_split_element)",
                     "algorithmic_flops_per_eval": flops, "traffic": None},
        "roofline_hbm": {"achieved": nbytes / t_res / 1e9, "peak": peaks["hbm_gbs"],
                         "frac": nbytes / t_res / 1e9 / peaks["hbm_gbs"]},
        "phases_ms": {"k_face_flux": t_face, "k_split_element": t_elem},
        "element_launch_config": cfg,
        "autotune_ms": [[c["elements_per_cta"], ms_] for c, ms_ in tune],
        "cpu_baseline": {"value": 1.0 / (4 * t_cpu_res), "unit": "steps/s", "cores": used,
                         "kind": "port", "sample": "one full split-form residual on 1 core "
                                                   "(%.1f s), 4 per RK4 step" % t_cpu_res},
        "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": int(q.nbytes / nsteps),
                "d2h_bytes_per_step": int(q.nbytes / nsteps)},
        "error_vs_oracle": err,
        "gpu_launches": int(n_launch),
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


C1_WORKLOAD = ("isentropic vortex (rho_in 2, M_in 0.5) on the quarter annulus r in [1,3], 16x16 "
               "quads -> 512 triangles, SBP-Omega p=2, Roe faces, vortex Dirichlet data; state = "
               "vortex * (1 + N(0, 1e-3)) seed 1; one step = one RK4 step at CFL 0.4 "
               "(delta_t = CFL min_el_size / max wave speed)")


def run_c1(args, rank, world):
    """Config 1: the small FP64 case.  value = RK4 steps/s (100 steps at CFL
    0.4 per timed step); the residual section gives evaluations/s.  The mesh
    is 12,288 unknowns, so both are launch- and latency-bound."""
    import torch
    from pdesolver_gb300 import eulergpu
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ms, opts, q = problems.config1()
    g = eulergpu.GPUMesh(ms, opts)
    g.set_stream(stream.cuda_stream)
    qd = torch.from_numpy(q).cuda()
    h = g.cfl_time_step(qd, 0.4)
    # launch shape of the element kernel for this mesh (the RK4 step graphs
    # are captured with it)
    tune = g.autotune(qd, reps=10)
    nsteps = 100
    qw = torch.empty_like(qd)
    for _ in range(args.warmup):
        qw.copy_(qd)
        g.rk4(qw, h, nsteps * h)
    torch.cuda.synchronize()
    l0 = g.timings().launches
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    with ClockSampler(dev) as clk:
        for k in range(args.steps):
            qw.copy_(qd)
            evs[k][0].record()
            st = g.rk4(qw, h, nsteps * h)
            evs[k][1].record()
        torch.cuda.synchronize()
    n_launch = g.timings().launches - l0
    total_ms = sum(a.elapsed_time(b) for a, b in evs)
    value = world * args.steps * nsteps / (total_ms * 1e-3)
    # residual evaluations/s (inputs are L2-resident: 98 KB state)
    rd = torch.zeros_like(qd)
    for _ in range(10):
        g.eval_residual_async(qd, rd)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nres = 1000
    e0.record()
    for _ in range(nres):
        g.eval_residual_async(qd, rd)
    e1.record()
    torch.cuda.synchronize()
    res_us = 1e3 * e0.elapsed_time(e1) / nres
    # end to end with host arrays: 100 steps per call
    qh = q.copy()
    g.set_stream(None)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        qh[...] = q
        g.rk4(qh, h, nsteps * h)
    e2e = world * args.steps * nsteps / (time.perf_counter() - t0)
    if rank != 0:
        return
    lib = _oracle()
    used = lib.oracle_set_threads(1)
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    res = np.zeros_like(q)
    lib.oracle_eval_residual(C.byref(desc.desc), C.byref(P), abi.dptr(q), abi.dptr(res))
    # the CPU baseline: the oracle's own RK4, the same 100 steps, timed (1 core)
    steady = _oracle_steady()
    olib = steady.load()
    olib.oracle_set_threads(1)
    qo = q.copy()
    tc = time.perf_counter()
    sto = steady.rk4(olib, ms, opts, qo, h, nsteps)
    t_cpu_steps = time.perf_counter() - tc
    qg = q.copy()
    g.rk4(qg, h, nsteps * h)
    rg = np.zeros_like(q)
    g.eval_residual(q, rg)
    err = {"residual": float(np.abs(rg - res).max() / np.abs(res).max()),
           "rk4_100_steps_state": float(np.abs(qg - qo).max() / np.abs(qo).max()),
           "what": "max-norm relative errors against the CPU oracle on the same inputs"}
    rbytes, rflops = residual_model(ms)
    peaks, src = measured_peaks()
    line = {
        "metric": "RK4 steps/s", "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps / nsteps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": C1_WORKLOAD, "elements": ms.numEl, "ndof": ms.numDof,
                   "delta_t": h, "rk4_steps_per_timed_step": nsteps,
                   "l2": "the 98 KB state is L2-resident: this case is launch-bound by design",
                   "parallelism": f"replicas x{world}"},
        "residual": {"evals_per_s": 1e6 / res_us, "us_per_eval": res_us,
                     "algorithmic_bytes": rbytes, "fp64_flops": rflops,
                     "element_launch_config": g.launch_config(),
                     "autotune_ms": [[c["elements_per_cta"], int(c["volume_mma"]), ms_]
                                     for c, ms_ in tune]},
        "roofline": {"bound": "latency", "achieved": rbytes / (res_us * 1e-6) / 1e9,
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": rbytes / (res_us * 1e-6) / 1e9 / peaks["hbm_gbs"], "peak_source": src,
                     "traffic": None,
                     "kernel": "residual (k_face_flux + k_element): 0.35 MB per evaluation, far "
                               "below the launch floor; the fraction is not meaningful"},
        "cpu_baseline": {"value": sto.steps / t_cpu_steps, "unit": "steps/s", "cores": 1,
                         "kind": "port",
                         "sample": "the oracle's RK4, %d steps of this workload on 1 core, timed "
                                   "(%.3f s)" % (sto.steps, t_cpu_steps)},
        "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": int(q.nbytes / nsteps),
                "d2h_bytes_per_step": int(q.nbytes / nsteps)},
        "error_vs_oracle": err,
        "gpu_launches": int(n_launch),
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


C4_WORKLOAD = ("batch of 96 steady Euler solves: quarter annuli n x n with n ~ logU(8, 96) "
               "(E = 2 n^2 triangles), SBP-Gamma p ~ U{1,2,3,4}, Roe, isentropic vortex Dirichlet "
               "data with M_in ~ U(0.3, 0.7), each from the free stream * (1 + U(-0.01, 0.01)), "
               "seed 5; Newton-GMRES(30) + block-Jacobi + pseudo-transient continuation to "
               "|R| < 1e-10 with p-continuation from p=1; mixed precision; one step = the whole "
               "batch")


def c4_cpu_rates(threads=1, n_gmres=20):
    """Oracle phase times per element for each degree (a 32 x 32 annulus per
    degree): residual, Jacobian, block LU, one GMRES iteration."""
    from pdesolver_gb300 import eulergpu
    lib = _oracle()
    used = lib.oracle_set_threads(int(threads))
    rates = {}
    for p in (1, 2, 3, 4):
        ms, opts, q = problems.config2(n=32, p=p, seed=1)
        desc = abi.MeshDesc(ms)
        P = eulergpu.params_from_opts(opts)
        out = np.zeros(4)
        st = lib.oracle_newton_phase_times(C.byref(desc.desc), C.byref(P), abi.dptr(q), n_gmres,
                                           abi.dptr(out))
        assert st == 0, st
        rates[p] = [x / ms.numEl for x in out]
    return rates, used


def _init_dist(world):
    """torch.distributed over NCCL for N > 1 ranks (host-side timing only),
    else None."""
    if world <= 1:
        return None
    import torch.distributed as td
    if not td.is_initialized():
        td.init_process_group("nccl")
    return td


def run_c4(args, rank, world):
    """Batched steady solves on concurrent streams (one step = the batch)."""
    import torch
    from pdesolver_gb300 import batch, eulergpu
    from pdesolver_gb300 import replicas
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    dist = _init_dist(world)
    specs = problems.config4_specs()
    if world > 1:
        # the problems are sharded over the ranks (no exchange between them)
        work = [2 * sp["n"] ** 2 * ((3, 7, 12, 18)[sp["p"] - 1] * 4) ** 2 for sp in specs]
        specs = [specs[i] for i in replicas.shard(work, world)[rank]]
    t0 = time.perf_counter()
    probs = []
    for k, sp in enumerate(specs):
        lv, q0 = problems.config4_problem(sp)
        gl = [eulergpu.GPUMesh(ms, opts) for ms, opts in lv]
        ms_f = lv[-1][0]
        n_f = ms_f.sbp.numnodes * ms_f.numDofPerNode
        probs.append(batch.SteadyProblem(levels=gl, q0=torch.from_numpy(q0).cuda(), opts=NEWTON_OPTS,
                                         level_tol=LEVEL_TOL, tag=k, work=ms_f.numEl * n_f * n_f))
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    workers = args.workers
    batched = args.gmres_batching == "on"
    for _ in range(max(1, args.warmup)):
        batch.solve_batch(probs, workers=workers, batch_gmres=batched)
    torch.cuda.synchronize()
    l0 = sum(g.timings().launches for pr in probs for g in pr.levels)
    # several streams driven by host threads: the host clock between two
    # device-wide synchronisations times the batch
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t1 = time.perf_counter()
        for _ in range(args.steps):
            results = batch.solve_batch(probs, workers=workers, batch_gmres=batched)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t1
        if dist:
            dist.barrier()
    n_launch = sum(g.timings().launches for pr in probs for g in pr.levels) - l0
    nsolve = len(probs) * args.steps
    # whole job: every rank's solves over the slowest rank's time
    value, _, wall = replicas.job_rate(nsolve, wall, dist)
    total_ms = 1e3 * wall
    failed = [r.tag for r in results if r.error]
    retried = sum(1 for r in results if r.retries)
    # algorithmic bytes: the persistent GMRES solves (gmres_bytes per level)
    abytes = 0
    counts = []
    for pr, r in zip(probs, results):
        lv = []
        for g, st in zip(pr.levels, r.stats):
            abytes += gmres_bytes(g.mesh, st.krylov_iters, 30, 4)
            lv.append((g.mesh.sbp.p, g.mesh.numEl, st.iters, st.krylov_iters))
        counts.append(lv)
    # end to end: the batch through the public API with host arrays
    hprobs = [batch.SteadyProblem(levels=pr.levels, q0=pr.q0.cpu().numpy(), opts=pr.opts,
                                  level_tol=pr.level_tol, tag=pr.tag, work=pr.work) for pr in probs]
    t2 = time.perf_counter()
    batch.solve_batch(hprobs, workers=workers, batch_gmres=batched)
    e2e, _, _ = replicas.job_rate(len(probs), time.perf_counter() - t2, dist)
    # the same batch with the other Krylov launch mode, for comparison
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    batch.solve_batch(probs, workers=workers, batch_gmres=not batched)
    torch.cuda.synchronize()
    other_rate = len(probs) / (time.perf_counter() - t3)
    # the plain FP64 path on the same batch (FP64 Jacobian, preconditioner and
    # Krylov), and how far the two precisions' converged states lie apart
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    res64 = batch.solve_batch(probs, workers=workers, precision=0, batch_gmres=False)
    torch.cuda.synchronize()
    fp64_wall = time.perf_counter() - t4
    fp64_rate, _, _ = replicas.job_rate(len(probs), fp64_wall, dist)
    sdiff = []
    for a, b in zip(results, res64):
        if a.error is None and b.error is None:
            qa, qb = np.asarray(a.q.cpu() if hasattr(a.q, "cpu") else a.q), \
                np.asarray(b.q.cpu() if hasattr(b.q, "cpu") else b.q)
            sdiff.append(float(np.abs(qa - qb).max() / np.abs(qb).max()))
    h2d = sum(pr.q0.numel() * 8 + sum(g.ndof * 8 for g in pr.levels[1:]) for pr in probs)
    d2h = sum(sum(g.ndof * 8 for g in pr.levels) + sum(g.ndof * 8 for g in pr.levels[1:])
              for pr in probs)
    if rank != 0:
        return
    peaks, src = measured_peaks()
    rates, used = c4_cpu_rates(1)
    cpu_t = 0.0
    for lv in counts:
        for p, E, its, kits in lv:
            r = rates[p]
            cpu_t += E * (its * (r[0] + r[1] + r[2]) + r[0] + kits * r[3])
    line = {
        "metric": "steady solves/s", "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic",
        "config": {"workload": C4_WORKLOAD, "problems": len(probs), "workers": workers,
                   "total_elements": sum(pr.levels[-1].mesh.numEl for pr in probs),
                   "total_ndof_final": sum(pr.levels[-1].ndof for pr in probs),
                   "timing": "host clock between device synchronisations (threads x streams)",
                   "setup_s": t_setup, "l2": "per-problem working sets up to 1.2 GB; the batch "
                                             "exceeds the 129 MB L2",
                   "parallelism": f"{workers} host threads x 1 stream each; problems sharded over "
                                  f"{world} rank(s), no collective on the data path",
                   "gmres_batching": args.gmres_batching},
        "batch": {"failed": failed, "retried": retried,
                  ("solves_per_s_gmres_batching_off" if batched else "solves_per_s_gmres_batching_on"):
                      other_rate,
                  "fp64_solves_per_s": fp64_rate, "mixed_over_fp64": value / fp64_rate,
                  "fp64_failed": [r.tag for r in res64 if r.error],
                  "state_rel_diff_mixed_vs_fp64_max": max(sdiff) if sdiff else None,
                  "krylov_its": sum(l[3] for lv in counts for l in lv),
                  "newton_its": sum(l[2] for lv in counts for l in lv),
                  "solve_s_p50": statistics.median(r.seconds for r in results),
                  "solve_s_max": max(r.seconds for r in results)},
        "roofline": {"bound": "hbm", "achieved": abytes / (total_ms * 1e-3 / args.steps) / 1e9,
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": abytes / (total_ms * 1e-3 / args.steps) / 1e9 / peaks["hbm_gbs"],
                     "peak_source": src, "traffic": None,
                     "kernel": "sum of the batch's persistent GMRES solves (gmres_bytes) over the "
                               "batch time (all phases)",
                     "algorithmic_bytes_per_step": abytes},
        "cpu_baseline": {"value": len(probs) / cpu_t, "unit": "solves/s", "cores": used,
                         "kind": "port",
                         "sample": "oracle phase times (residual, Jacobian, block LU, 20 GMRES "
                                   "iterations) on a 32x32 annulus per degree, per element, "
                                   "scaled by each problem's elements and this run's "
                                   "Newton/GMRES counts"},
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(n_launch),
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


C5_WORKLOAD = ("serving: Poisson arrivals of steady-solve requests at 0.8 x the measured "
               "capacity, 80% 2-D annuli from the batched distribution (n ~ logU(8, 96), "
               "SBP-Gamma p ~ U{1..4}, vortex M_in ~ U(0.3, 0.7)), 20% 3-D warped cubes "
               "(n ~ U{8..24}, 6 n^3 diagonal-E tets, p ~ U{1, 2}, free stream Mach ~ U(0.3, 0.7)); "
               "Roe, free stream * (1 + U(-0.01, 0.01)) starts, Newton-GMRES(30) + block-Jacobi + "
               "pseudo-transient continuation to |R| < 1e-10 with p-continuation; 150 GB HBM "
               "budget; seed 6")


def _c5_build_meshes(keys, workers):
    """Host meshes of every geometry key, built by a spawn process pool (the
    client side of the stream: requests arrive with their meshes)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    keys = sorted(set(keys), key=lambda k: -(k[1] ** k[0]) * k[2])
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        built = list(ex.map(problems.request_meshes, keys, chunksize=1))
    return dict(zip(keys, built))


def _c5_requests(specs, meshes, rate, arrivals=True):
    from pdesolver_gb300 import serve
    t, out = 0.0, []
    for k, sp in enumerate(specs):
        key = problems.geometry_key(sp)
        levels, q0 = problems.request_problem(sp, meshes[key])
        if arrivals:
            t += sp["gap"] / rate
        out.append(serve.SolveRequest(rid=k, levels=levels, q0=q0, opts=NEWTON_OPTS, key=key,
                                      arrival=t if arrivals else 0.0, level_tol=LEVEL_TOL))
    return out


def c5_cpu_rates(threads=1, n_gmres=20):
    """Oracle phase times per element (residual, Jacobian, block LU, one
    GMRES iteration) for the 2-D degrees (32 x 32 annulus) and the 3-D
    degrees (4^3 x 6 warped cube)."""
    from pdesolver_gb300 import eulergpu
    lib = _oracle()
    used = lib.oracle_set_threads(int(threads))
    rates = {}
    for key in [(2, 32, p) for p in (1, 2, 3, 4)] + [(3, 4, p) for p in (1, 2)]:
        ms = problems.request_meshes(key)[-1]
        lv, q = problems.request_problem({"dim": key[0], "n": key[1], "p": key[2], "M_in": 0.5,
                                          "seed": 1}, [ms])
        desc = abi.MeshDesc(ms)
        P = eulergpu.params_from_opts(lv[0][1])
        out = np.zeros(4)
        assert lib.oracle_newton_phase_times(C.byref(desc.desc), C.byref(P), abi.dptr(q), n_gmres,
                                             abi.dptr(out)) == 0
        rates[(key[0], key[2])] = [x / ms.numEl for x in out]
    return rates, used


def run_c5(args, rank, world):
    """Serving: a Poisson stream of steady-solve requests (one step = the
    stream); mixed precision, and the plain FP64 path on the same arrivals."""
    import torch
    from pdesolver_gb300 import serve
    dev = int(os.environ.get("LOCAL_RANK", 0))
    budget = int(150e9)
    all_specs = problems.config5_specs(count=2000, seed=6)
    specs = all_specs[:args.requests]
    probe_specs = problems.config5_specs(count=args.probe, seed=7)
    t0 = time.perf_counter()
    meshes = _c5_build_meshes([problems.geometry_key(s) for s in specs + probe_specs],
                              max(1, min(16, os.cpu_count() or 1)))
    t_build = time.perf_counter() - t0
    torch.cuda.set_device(dev)
    torch.cuda.init()
    summaries, results, servers = {}, {}, {}
    # capacity: the probe requests all queued at once (closed loop), mixed precision
    probe = _c5_requests(probe_specs, meshes, 1.0, arrivals=False)
    srv = serve.SteadySolveServer(budget, slots=args.workers, precision=1,
                                  batch_gmres=args.gmres_batching == "on")
    pres = srv.serve(probe)
    srv.close()
    capacity = serve.latency_summary(pres)["solves_per_s"]
    # the plain FP64 server's capacity on the same probe requests
    probe64 = _c5_requests(probe_specs, meshes, 1.0, arrivals=False)
    srv = serve.SteadySolveServer(budget, slots=args.workers, precision=0,
                                  batch_gmres=args.gmres_batching == "on")
    pres64 = srv.serve(probe64)
    srv.close()
    capacity64 = serve.latency_summary(pres64)["solves_per_s"]
    rate = 0.8 * capacity
    fp64_stream = args.fp64_stream == "on" or (args.fp64_stream == "auto" and len(specs) <= 300)
    arms = (("mixed", 1), ("fp64", 0)) if fp64_stream else (("mixed", 1),)
    with ClockSampler(dev) as clk:
        for name, prec in arms:
            reqs = _c5_requests(specs, meshes, rate)
            srv = serve.SteadySolveServer(budget, slots=args.workers, precision=prec,
                                          batch_gmres=args.gmres_batching == "on")
            torch.cuda.synchronize()
            res = srv.serve(reqs)
            torch.cuda.synchronize()
            srv.close()
            s = serve.latency_summary(res)
            s.update(peak_bytes_estimated=srv.peak_bytes, peak_requests_on_device=srv.peak_running,
                     retried=sum(1 for r in res if r.retries),
                     errors=sorted({r.error[:200] for r in res if r.error})[:4])
            summaries[name] = s
            results[name] = res
    mixed = summaries["mixed"]
    # the two precisions agree on every request's functional
    fdiff = [abs(a.functional - b.functional) / abs(b.functional)
             for a, b in zip(results["mixed"], results.get("fp64", []))
             if a.error is None and b.error is None and b.functional]
    if rank != 0:
        return
    rates, used = c5_cpu_rates(1)
    cpu_t, n_ok = 0.0, 0
    for sp, r in zip(specs, results["mixed"]):
        if r.error is not None:
            continue
        n_ok += 1
        levels = meshes[problems.geometry_key(sp)]
        for ms, st in zip(levels, r.stats):
            rr = rates[(ms.dim, ms.sbp.p)]
            cpu_t += ms.numEl * (st["iters"] * (rr[0] + rr[1] + rr[2]) + rr[0] + st["krylov_iters"] * rr[3])
    h2d = sum(r.q0.nbytes for r in _c5_requests(specs, meshes, rate))
    d2h = sum(r.q.nbytes for r in results["mixed"] if r.q is not None)
    # the mixed stream's persistent GMRES solves (gmres_bytes per level) over its span
    abytes = 0
    for sp, r in zip(specs, results["mixed"]):
        for ms, st in zip(meshes[problems.geometry_key(sp)], r.stats):
            abytes += gmres_bytes(ms, st["krylov_iters"], 30, 4)
    peaks, src = measured_peaks()
    n_launch = sum(r.launches for r in results["mixed"])
    line = {
        "metric": "served steady solves/s (p50/p99 latency)", "value": mixed["solves_per_s"] * world,
        "unit": "solves/s", "n_gpus": world, "steps": 1, "warmup": 1,
        "ms_per_step": 1e3 * mixed["span_s"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
        "config": {"workload": C5_WORKLOAD, "requests": len(specs),
                   "sample": f"the first {len(specs)} of the 2000-request stream",
                   "requests_3d": sum(1 for s in specs if s["dim"] == 3),
                   "slots": args.workers, "hbm_budget_bytes": budget,
                   "capacity_probe": {"requests": len(probe), "solves_per_s": capacity,
                                      "fp64_solves_per_s": capacity64,
                                      "mixed_over_fp64": capacity / capacity64 if capacity64 else None,
                                      "seed": 7},
                   "arrival_rate_per_s": rate, "host_mesh_build_s": t_build,
                   "timing": "host clock: completion minus arrival per request; solves/s = "
                             "completed / (last completion - first arrival)",
                   "l2": "per-request working sets up to 14 GB; inputs exceed the 129 MB L2",
                   "parallelism": f"{args.workers} slots (host threads x streams), replicas x{world}",
                   "gmres_batching": args.gmres_batching},
        "serving": {"mixed": mixed,
                    "fp64": summaries.get("fp64", "not run: the FP64 server on the same arrivals "
                                                  "(0.8x the mixed capacity) is overloaded; its "
                                                  "capacity is the probe's fp64_solves_per_s"),
                    "functional_rel_diff_mixed_vs_fp64_max": max(fdiff) if fdiff else None},
        "cpu_baseline": {"value": n_ok / cpu_t if cpu_t else None, "unit": "solves/s", "cores": used,
                         "kind": "port",
                         "sample": "oracle phase times per element (32x32 annulus per 2-D degree, "
                                   "4^3x6 cube per 3-D degree) scaled by each request's elements "
                                   "and this run's Newton/GMRES counts, no queueing"},
        "e2e": {"value": mixed["solves_per_s"] * world, "unit": "solves/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "hbm", "achieved": abytes / mixed["span_s"] / 1e9,
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": abytes / mixed["span_s"] / 1e9 / peaks["hbm_gbs"], "peak_source": src,
                     "traffic": None,
                     "kernel": "sum of the mixed stream's persistent GMRES solves (gmres_bytes) over "
                               "the stream span; arrivals, not the GPU, set the pace at 0.8x capacity"},
        "gpu_launches": int(n_launch),
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_tune(args):
    """Autotuner sweep of the element kernel per operator and degree: weak
    form (Roe) on the 64 x 64 annulus with SBP-Gamma p = 1..4 and on the
    warped 24^3 x 6 cube with diagonal-E tets p = 1, 2, 3; split form (IR) on
    the same cubes.  Prints one JSON line with every candidate's time."""
    import torch
    from pdesolver_gb300 import eulergpu
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    cases = [("2d weak gamma", p, problems.config2(p=p)) for p in (1, 2, 3, 4)]
    for p in (1, 2, 3):
        ms, opts, q = problems.config3(n=24, p=p)
        cases.append(("3d split diage", p, (ms, opts, q)))
        cases.append(("3d weak diage", p, (ms, dict(opts, Flux_name="RoeFlux", volume_integral_type=1), q)))
    out = []
    for name, p, (ms, opts, q) in cases:
        g = eulergpu.GPUMesh(ms, opts)
        qd = torch.from_numpy(q).cuda()
        table = g.autotune(qd, reps=10)
        best = g.launch_config()
        default = [ms_ for c, ms_ in table if c["elements_per_cta"] == max(1, 256 // ms.sbp.numnodes)
                   and not c["volume_mma"]]
        cpu_core = [ms_ for c, ms_ in table if not c["volume_mma"]]
        mma = [ms_ for c, ms_ in table if c["volume_mma"]]
        out.append({"operator": name, "p": p, "Np": ms.sbp.numnodes, "elements": ms.numEl,
                    "best": best, "best_ms": min(ms_ for _, ms_ in table),
                    "builtin_ms": default[0] if default else None,
                    "best_cuda_core_ms": min(cpu_core) if cpu_core else None,
                    "best_mma_ms": min(mma) if mma else None,
                    "table": [[c["elements_per_cta"], int(c["volume_mma"]), ms_] for c, ms_ in table]})
        g.close()
    print(json.dumps({"autotune": out}), flush=True)


def run_gmres_grid(args):
    """Microseconds per Arnoldi iteration of the persistent GMRES kernel
    against its grid size (eg_ls_set_grid; 0 = automatic), FP32 operator and
    block-Jacobi inverses at a perturbed free stream, GMRES(30), 120
    iterations, L2 flushed, best of 3.  One JSON line per operator."""
    import torch
    from pdesolver_gb300 import eulergpu
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    cases = [("c2 p1", (2, 64, 1)), ("c2 p3", (2, 64, 3)), ("n32 p3", (2, 32, 3)),
             ("n16 p2", (2, 16, 2)), ("n24 p1", (2, 24, 1)), ("n96 p4", (2, 96, 4)),
             ("cube4 p1", (3, 4, 1)), ("cube16 p2", (3, 16, 2)), ("cube24 p2", (3, 24, 2))]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for name, key in cases:
        ms = problems.request_meshes(key)[-1]
        lv, q = problems.request_problem({"dim": key[0], "n": key[1], "p": key[2], "M_in": 0.5,
                                          "seed": 1}, [ms])
        gm = eulergpu.GPUMesh(ms, lv[0][1])
        gm.set_stream(stream.cuda_stream)
        lo = eulergpu.LinearOperator(gm, precision=1)
        lo.calc(q)
        pc = eulergpu.BlockJacobiPC(lo)
        pc.calc()
        ls = eulergpu.LinearSolver(pc, lo, restart=30)
        ls.set_tolerances(reltol=1e-30, abstol=0.0, itermax=120)
        b = torch.randn(ms.numDof, dtype=torch.float64, device="cuda")
        x = torch.zeros_like(b)
        row = {"case": name, "E": ms.numEl, "n": ms.sbp.numnodes * ms.numDofPerNode}
        for nb in [0, 1, 4, 8, 16, 32, 64, 96, 152]:
            if nb == 1 and ms.numEl > 20000:
                continue
            ls.set_grid(nb)
            x.zero_()
            ls.solve(b, x)
            ts = []
            for _ in range(3):
                x.zero_()
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                st = ls.solve(b, x)
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1) / max(st.iters, 1) * 1e3)
            row[str(nb)] = round(min(ts), 2)
        print(json.dumps(row), flush=True)
        for o in (ls, pc, lo, gm):
            o.close()


def run_kernels_only(args, which):
    """Short run of the isolated kernels for profiling captures: the FP32
    operator / block-Jacobi applies of the C2 problem (p=3, initial state), or
    the FP64 residual kernels; `args.steps` launches of each."""
    import torch
    from pdesolver_gb300 import eulergpu
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ms, opts, q = problems.config2(p=3)
    g = eulergpu.GPUMesh(ms, opts)
    g.set_stream(stream.cuda_stream)
    out = {}
    if which == "split":
        ms, opts, q = problems.config3(n=8)
        g = eulergpu.GPUMesh(ms, opts)
        g.set_stream(stream.cuda_stream)
        qd = torch.from_numpy(q).cuda()
        rd = torch.zeros_like(qd)
        for _ in range(args.steps):
            g.eval_residual_async(qd, rd)
        torch.cuda.synchronize()
        out["kernels"] = ["k_face_flux<3>", "k_split_element<3>"]
        out["launches_each"] = args.steps
        print(json.dumps(out), flush=True)
        return
    if which == "cluster":
        # a small system's GMRES (16 x 16 annulus, SBP-Gamma p=2, 1.6 MB of
        # FP32 element blocks): one solve of `steps` iterations on the default
        # launch, a thread-block cluster
        ms_k = problems.request_meshes((2, 16, 2))[-1]
        lv_k, q_k = problems.request_problem({"dim": 2, "n": 16, "p": 2, "M_in": 0.5, "seed": 1},
                                             [ms_k])
        gk = eulergpu.GPUMesh(ms_k, lv_k[0][1])
        gk.set_stream(stream.cuda_stream)
        lo = eulergpu.LinearOperator(gk, precision=1)
        lo.calc(q_k)
        pc = eulergpu.BlockJacobiPC(lo)
        pc.calc()
        ls = eulergpu.LinearSolver(pc, lo, restart=30)
        ls.set_tolerances(reltol=1e-30, abstol=0.0, itermax=args.steps)
        b = torch.randn(ms_k.numDof, dtype=torch.float64, device="cuda",
                        generator=torch.Generator("cuda").manual_seed(1))
        x = torch.zeros_like(b)
        st = ls.solve(b, x)
        torch.cuda.synchronize()
        out["kernels"] = ["k_gmres_cluster<2,28,float>"]
        out["iterations"] = st.iters
        print(json.dumps(out), flush=True)
        return
    if which == "flux":
        # the flux kernels' instruction counts: a small C2 weak-form case
        # (Roe, 32 x 32 annulus, SBP-Gamma p=3) and a small C3 split-form case
        # (IR, 8^3 x 6 warped tets, diagonal-E p=2), default launch shapes
        for ms_k, opts_k, q_k in (problems.config2(n=32, p=3), problems.config3(n=8)):
            gk = eulergpu.GPUMesh(ms_k, opts_k)
            gk.set_stream(stream.cuda_stream)
            qd = torch.from_numpy(q_k).cuda()
            rd = torch.zeros_like(qd)
            for _ in range(args.steps):
                gk.eval_residual_async(qd, rd)
            torch.cuda.synchronize()
        out["kernels"] = ["k_face_flux<2>", "k_element<2,0>", "k_face_flux<3>", "k_split_element<3>"]
        out["launches_each"] = args.steps
        print(json.dumps(out), flush=True)
        return
    if which == "blockinv":
        # block-Jacobi inverses: the C2 p=3 operator (48 unknowns per block) and
        # the warped 8^3 x 6 cube with diagonal-E p=2 tets (115 unknowns)
        for key in ((2, 64, 3), (3, 8, 2)):
            msk = problems.request_meshes(key)[-1]
            lvk, qk = problems.request_problem({"dim": key[0], "n": key[1], "p": key[2],
                                                "M_in": 0.5, "seed": 1}, [msk])
            gk = eulergpu.GPUMesh(msk, lvk[0][1])
            gk.set_stream(stream.cuda_stream)
            lo = eulergpu.LinearOperator(gk, precision=1)
            lo.calc(qk)
            pc = eulergpu.BlockJacobiPC(lo)
            for _ in range(args.steps):
                pc.calc()
            torch.cuda.synchronize()
        out["kernels"] = ["k_block_inverse_reg<float,2,8,8>", "k_block_inverse_reg<float,4,8,16>"]
        out["launches_each"] = args.steps
        print(json.dumps(out), flush=True)
        return
    if which == "gmres":
        # one Newton linear system: FP32 Jacobian + block-Jacobi at the initial
        # state, GMRES(30) for `steps` iterations (one restart cycle per 30)
        lo = eulergpu.LinearOperator(g, precision=1)
        lo.calc(q)
        pc = eulergpu.BlockJacobiPC(lo)
        pc.calc()
        ls = eulergpu.LinearSolver(pc, lo, restart=30)
        ls.set_tolerances(reltol=1e-12, abstol=0.0, itermax=args.steps)
        b = np.random.default_rng(0).normal(size=q.shape)
        x = np.zeros_like(b)
        ls.solve(b, x)                       # capture + warm
        x[...] = 0
        t0 = time.perf_counter()
        st = ls.solve(b, x)
        out["gmres_its"] = st.iters
        out["ms_per_iteration_wall"] = 1e3 * (time.perf_counter() - t0) / max(st.iters, 1)
        out["kernels"] = ["GMRES cycle"]
    elif which == "krylov":
        lo = eulergpu.LinearOperator(g, precision=1)
        lo.calc(q)
        pc = eulergpu.BlockJacobiPC(lo)
        pc.calc()
        x = torch.randn(ms.numDof, dtype=torch.float32, device="cuda")
        y = torch.empty_like(x)
        for _ in range(args.steps):
            lo.apply_native(x, y)
            pc.apply_native(x, y)
        out["kernels"] = ["k_spmv<2,float>", "k_block_apply<float>"]
    else:
        qd = torch.from_numpy(q).cuda()
        rd = torch.zeros_like(qd)
        for _ in range(args.steps):
            g.eval_residual_async(qd, rd)
        out["kernels"] = ["k_face_flux<2>", "k_element<2>"]
    torch.cuda.synchronize()
    out["launches_each"] = args.steps
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "tune", "gmres-grid"],
                    help="c2: steady Newton solves (headline); c3: 3-D entropy-stable RK4; "
                         "c4: batch of 96 steady solves; c5: served stream of steady solves")
    ap.add_argument("--workers", type=int, default=8,
                    help="host threads of the c4 batch / serving slots of c5")
    ap.add_argument("--requests", type=int, default=2000, help="c5: requests of the stream served")
    ap.add_argument("--gmres-batching", default="off", choices=["on", "off"],
                    help="c4/c5: Krylov solves of concurrent problems in shared cooperative launches")
    ap.add_argument("--probe", type=int, default=32, help="c5: requests of the capacity probe")
    ap.add_argument("--fp64-stream", default="auto", choices=["auto", "on", "off"],
                    help="c5: also serve the stream with the FP64 server (auto: up to 300 requests)")
    ap.add_argument("--only", default=None, choices=["krylov", "residual", "gmres", "split", "blockinv",
                                                     "flux", "cluster"],
                    help="run only the isolated kernels (for profiler captures)")
    args = ap.parse_args()
    if args.only:
        run_kernels_only(args, args.only)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.workload == "c1" and args.impl == "ours":
        run_c1(args, rank, world)
        return
    if args.workload == "c3" and args.impl == "ours":
        run_c3(args, rank, world)
        return
    if args.workload == "c4" and args.impl == "ours":
        run_c4(args, rank, world)
        return
    if args.workload == "gmres-grid" and args.impl == "ours":
        run_gmres_grid(args)
        return
    if args.workload == "tune" and args.impl == "ours":
        run_tune(args)
        return
    if args.workload == "c5" and args.impl == "ours":
        run_c5(args, rank, world)
        return
    dist = None
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        td.init_process_group("nccl")
        dist = td
    run_ours(args, rank, world, dist)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
