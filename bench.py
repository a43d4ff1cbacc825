#!/usr/bin/env python3
"""Benchmark of the GB300 Euler SBP hot path.

Default workload: FP64 residual evaluation (evalResidual) on the 64x64
quarter-annulus, 8192 triangles, SBP-Gamma p=3, Roe faces, vortex Dirichlet
data, perturbed free-stream state (seed 2).  One step = one residual
evaluation.  Prints one JSON line (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference's evalResidual
(the oracle port: Julia, SummationByParts.jl and PUMI are not available) on
the host cores with all threads, same workload and metric.

Multi-GPU: the path has no exchange step between independent problems, so
N ranks run N independent replicas (weak scaling, no collective on the
data path); value = evaluations of all ranks / max-over-ranks time.
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

WORKLOAD = ("annulus 64x64 (8192 triangles), SBP-Gamma p=3, Roe, isentropic-vortex "
            "Dirichlet data, free stream * (1 + U(-0.01, 0.01)) seed 2; one step = one FP64 "
            "evalResidual")


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
                 "--format=csv,noheader,nounits", "-lms", "100"],
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


def cpu_residual_baseline(ms, opts, q, budget_s=10.0, threads=1, max_steps=None):
    """Oracle residual (port of the reference) timed on the host."""
    from pdesolver_gb300 import build, eulergpu
    lib = C.CDLL(build.build_oracle())
    lib.oracle_set_threads.restype = C.c_int
    used = lib.oracle_set_threads(int(threads))
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    res = np.zeros_like(q)
    lib.oracle_eval_residual(C.byref(desc.desc), C.byref(P), abi.dptr(q), abi.dptr(res))  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        lib.oracle_eval_residual(C.byref(desc.desc), C.byref(P), abi.dptr(q), abi.dptr(res))
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s or (max_steps and n >= max_steps):
            break
    return n / el, used, n, el


def run_reference(args, rank, world):
    if rank != 0:
        return
    ms, opts, q = problems.config2()
    steps = max(args.steps, 1)
    threads = os.cpu_count() or 1
    rate, used, n, el = cpu_residual_baseline(ms, opts, q, budget_s=60.0, threads=threads,
                                              max_steps=steps)
    line = {
        "metric": "residual evals/s", "value": rate, "unit": "evals/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": n, "warmup": 1, "ms_per_step": 1e3 * el / n,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD},
        "cpu_baseline": {"value": rate, "unit": "evals/s", "cores": used, "kind": "port",
                         "sample": f"{n} residual evaluations of the full workload"},
        "e2e": {"value": rate, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference evalResidual (oracle port, OpenMP); the "
                "Julia reference cannot run here (no Julia, SummationByParts.jl, PUMI)",
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, dist):
    import torch
    from pdesolver_gb300 import eulergpu
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ms, opts, q = problems.config2()
    g = eulergpu.GPUMesh(ms, opts)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    g.set_stream(stream.cuda_stream)
    qd = torch.from_numpy(q).cuda()
    rd = torch.zeros_like(qd)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    nbytes, flops = residual_model(ms)

    for _ in range(args.warmup):
        flush.zero_()
        g.eval_residual_async(qd, rd)
    g.sync()
    torch.cuda.synchronize()
    l0 = g.timings().launches

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for k in range(args.steps):
            flush.zero_()                      # L2 flush, outside the timed bracket
            evs[k][0].record()
            g.eval_residual_async(qd, rd)
            evs[k][1].record()
        torch.cuda.synchronize()
        launches = g.timings().launches - l0
        # keep the GPU busy long enough for the clock sampler to see it
        t_end = time.perf_counter() + 0.5
        while time.perf_counter() < t_end:
            for _ in range(20):
                g.eval_residual_async(qd, rd)
            torch.cuda.synchronize()
    g.sync()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = sum(step_ms)
    if dist:
        t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * args.steps / (total_ms * 1e-3)

    # per-phase device times (CUDA events around each launch)
    g.set_timing(True)
    g.reset_timings()
    for _ in range(args.steps):
        flush.zero_()
        g.eval_residual_async(qd, rd)
    tm = g.timings()
    g.set_timing(False)
    t_face = tm.t_face_flux / args.steps
    t_elem = tm.t_element / args.steps

    # end to end through the public API with host buffers (pinned)
    qh = torch.from_numpy(q).pin_memory()
    rh = torch.zeros_like(qh).pin_memory()
    qn, rn = qh.numpy(), rh.numpy()
    g.set_stream(None)
    g.eval_residual(qn, rn)
    e2e_t = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.eval_residual(qn, rn)
        e2e_t += time.perf_counter() - t0
    e2e_val = world * args.steps / e2e_t if not dist else None
    if dist:
        t = torch.tensor([e2e_t], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_val = world * args.steps / float(t.item())

    if rank != 0:
        return
    peaks, src = measured_peaks()
    fp64 = measure_fp64_peak(torch)
    t_res = (t_face + t_elem) * 1e-3
    achieved_gbs = nbytes / t_res / 1e9
    achieved_tf = flops / t_res / 1e12
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "residual_c2_traffic.json")) as f:
            traffic = json.load(f).get("bytes_per_eval")
    except (OSError, ValueError):
        pass
    cpu_rate, cpu_threads, cpu_n, cpu_el = cpu_residual_baseline(ms, opts, q, budget_s=10.0, threads=1)
    line = {
        "metric": "residual evals/s", "value": value, "unit": "evals/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "elements": ms.numEl, "ndof": int(q.size),
                   "l2": "flushed between steps (256 MB write outside the timed bracket)",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved_gbs / peaks["hbm_gbs"], "traffic": traffic,
                     "peak_source": src, "kernel": "residual (k_face_flux + k_element)",
                     "algorithmic_bytes_per_eval": nbytes},
        "roofline_fp64": {"bound": "fp64", "achieved": achieved_tf, "peak": fp64,
                          "unit": "TFLOP/s", "frac": achieved_tf / fp64,
                          "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                          "algorithmic_flops_per_eval": flops},
        "phases_ms": {"k_face_flux": t_face, "k_element": t_elem},
        "cpu_baseline": {"value": cpu_rate, "unit": "evals/s", "cores": cpu_threads, "kind": "port",
                         "sample": f"{cpu_n} full residual evaluations in {cpu_el:.1f} s"},
        "e2e": {"value": e2e_val, "unit": "evals/s", "h2d_bytes_per_step": int(q.nbytes),
                "d2h_bytes_per_step": int(q.nbytes)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch.distributed as td
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        td.init_process_group("nccl")
        dist = td
    run_ours(args, rank, world, dist)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
