"""GPU residual parity with the CPU oracle (through the C ABI).

Bar: max-norm relative error <= 1e-12 (FP64 residual), i.e.
max|R_gpu - R_oracle| <= 1e-12 * max|R_oracle|.
"""
import os

import numpy as np
import pytest

from conftest import oracle_residual
from pdesolver_gb300 import abi, eulergpu, mesh, problems, sbp

pytestmark = pytest.mark.gpu
TOL = 1e-12
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel_err(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def gpu_residual(ms, opts, q):
    g = eulergpu.GPUMesh(ms, opts)
    res = np.zeros_like(q)
    g.eval_residual(q, res)
    return res, g


@pytest.mark.parametrize("name", ["c1", "gamma3", "tet2", "tet3", "wall3", "annwall"])
def test_residual_matches_golden(gpu_lib, name):
    """GPU residual on the fixture's bit-exact inputs vs the committed oracle
    residual (weak and split forms, diagonal-E p=2 and p=3, and the
    entropy-stable wall in 2-D and 3-D)."""
    from test_golden import GEN
    ms, opts, q, gold = GEN.load(name)
    res, _ = gpu_residual(ms, opts, np.ascontiguousarray(q))
    assert rel_err(res, gold) <= TOL


@pytest.mark.parametrize("fam,p", [("omega", 1), ("omega", 2), ("omega", 3), ("omega", 4),
                                   ("gamma", 1), ("gamma", 2), ("gamma", 3), ("gamma", 4)])
def test_residual_tri_operators(gpu_lib, oracle, fam, p):
    ms, opts, q = problems.config1(n=6, p=p, family=fam, seed=100 + p)
    res, g = gpu_residual(ms, opts, q)
    ref = oracle_residual(oracle, g.desc, g.params, q)
    assert rel_err(res, ref) <= TOL


@pytest.mark.parametrize("p,flux", [(1, "IRFlux"), (2, "IRFlux"), (2, "RoeFlux"), (3, "IRFlux"),
                                    (3, "RoeFlux")])
def test_residual_tet_split_form(gpu_lib, oracle, p, flux):
    ms, opts, q = problems.config3(n=3, p=p, seed=20 + p)
    opts = dict(opts, Flux_name=flux)
    res, g = gpu_residual(ms, opts, q)
    ref = oracle_residual(oracle, g.desc, g.params, q)
    assert rel_err(res, ref) <= TOL


def test_residual_config2_full_size(gpu_lib, oracle):
    """64x64 annulus (8192 triangles), SBP-Gamma p=3, Roe, perturbed free stream."""
    ms, opts, q = problems.config2()
    res, g = gpu_residual(ms, opts, q)
    ref = oracle_residual(oracle, g.desc, g.params, q)
    assert rel_err(res, ref) <= TOL


def test_device_pointers_match_host_path(gpu_lib):
    torch = pytest.importorskip("torch")
    ms, opts, q = problems.config1()
    res_h, g = gpu_residual(ms, opts, q)
    qd = torch.from_numpy(q).cuda()
    rd = torch.zeros_like(qd)
    g.eval_residual(qd, rd)
    assert np.array_equal(rd.cpu().numpy(), res_h)   # same kernels: bitwise
    # asynchronous entry on the caller's stream
    s = torch.cuda.current_stream()
    g.set_stream(s.cuda_stream)
    rd.zero_()
    g.eval_residual_async(qd, rd)
    g.sync()
    assert np.array_equal(rd.cpu().numpy(), res_h)
    g.set_stream(None)


def test_negative_density_reports_status(gpu_lib):
    ms, opts, q = problems.config1()
    q = q.copy()
    q[7, 2, 0] = -1.0
    g = eulergpu.GPUMesh(ms, opts)
    res = np.zeros_like(q)
    with pytest.raises(eulergpu.EulerGPUError) as ei:
        g.eval_residual(q, res)
    assert ei.value.status == abi.EG_ERR_NEG_DENSITY
    # the mesh object stays usable after the error
    q[7, 2, 0] = 1.0
    g.eval_residual(np.ascontiguousarray(problems.config1()[2]), res)


def test_freestream_preserved_full_size_cube(gpu_lib):
    """Size-independent property at the full 3D size (82,944 warped tets):
    a uniform flow has zero residual (metric identities + consistency)."""
    op = sbp.get_operator(3, "diage", 2)
    ms = mesh.cube(op, 24, warp=0.05, seed=3, bc=mesh.BC_FREESTREAM)
    opts = {"Ma": 0.5, "aoa": 3.0, "Flux_name": "IRFlux", "volume_integral_type": 2}
    q = problems.free_stream(3, ms.coords.shape[:2], Ma=0.5, aoa=np.deg2rad(3.0))
    res, _ = gpu_residual(ms, opts, np.ascontiguousarray(q))
    assert np.abs(res).max() < 1e-12


def test_norm_matches_oracle(gpu_lib, oracle):
    import ctypes as C
    ms, opts, q = problems.config1()
    g = eulergpu.GPUMesh(ms, opts)
    r = np.random.default_rng(5).normal(size=q.shape)
    for strong in (0, 1):
        ref = oracle.oracle_calc_norm(C.byref(g.desc.desc), abi.dptr(r), strong)
        assert abs(g.calc_norm(r, strong) - ref) <= 1e-13 * ref


@pytest.mark.parametrize("fam,p", [("omega", 2), ("gamma", 3), ("gamma", 4)])
def test_residual_every_launch_config(gpu_lib, oracle, fam, p):
    """every elements-per-CTA choice, with the CUDA-core and the FP64
    tensor-core (mma.sync m8n8k4) volume contraction, meets the residual bar."""
    ms, opts, q = problems.config1(n=7, p=p, family=fam, seed=300 + p)
    g = eulergpu.GPUMesh(ms, opts)
    ref = oracle_residual(oracle, g.desc, g.params, q)
    np_ = ms.sbp.numnodes
    for mma in (False, True):
        epb = 1
        while (epb - 1) * np_ < 1024 and epb <= 128:
            g.set_launch_config(epb, mma)
            res = g.eval_residual(q, np.zeros_like(q))
            assert rel_err(res, ref) <= TOL, (epb, mma, rel_err(res, ref))
            epb *= 2


def test_split_form_launch_configs(gpu_lib, oracle):
    ms, opts, q = problems.config3(n=3, p=2, seed=41)
    g = eulergpu.GPUMesh(ms, opts)
    ref = oracle_residual(oracle, g.desc, g.params, q)
    for epb in (1, 2, 4, 8):
        g.set_launch_config(epb, False)
        res = g.eval_residual(q, np.zeros_like(q))
        assert rel_err(res, ref) <= TOL, epb
    with pytest.raises(eulergpu.EulerGPUError):
        g.set_launch_config(2, True)       # no tensor-core split form
    with pytest.raises(eulergpu.EulerGPUError):
        g.set_launch_config(512, False)    # more threads than a CTA holds


def test_autotune_keeps_the_fastest_and_stays_exact(gpu_lib, oracle):
    import torch
    ms, opts, q = problems.config2(n=32, p=3)
    g = eulergpu.GPUMesh(ms, opts)
    table = g.autotune(torch.from_numpy(q).cuda(), reps=5)
    assert len(table) >= 4 and any(c["volume_mma"] for c, _ in table)
    best = min(table, key=lambda t: t[1])[0]
    assert g.launch_config() == best
    ref = oracle_residual(oracle, g.desc, g.params, q)
    assert rel_err(g.eval_residual(q, np.zeros_like(q)), ref) <= TOL
