"""Python mirror of the reference's physics-module interface over the C ABI.

The reference's Euler module is driven through

* ``evalResidual(mesh, sbp, eqn, opts, t)``  (src/solver/euler/euler.jl:111)
* ``evalJacobian(mesh, sbp, eqn, opts, assembler, t)`` (evalJacobian.jl:6)
* ``calcNorm(eqn, res_vec; strongres)``      (src/Utils/Utils.jl:427)

Here ``mesh`` is a :class:`pdesolver_gb300.mesh.Mesh`, ``sbp`` its operator,
``eqn`` an :class:`EulerData` holding ``q``/``res`` in the reference layout
(``q[E, Np, nv]`` row-major == Julia ``q[nv, Np, E]``) and ``opts`` a dict with
the reference's option keys.  Every call goes to libeulergpu.so; there is no
CPU fallback: if the library is missing or no GPU is visible the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

_LIB = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libeulergpu.so")


class EulerGPUError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def library():
    """Load the in-tree libeulergpu.so (built by build.py); raise if absent."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libeulergpu.so not built ({LIB_PATH}); run the build step")
        lib = C.CDLL(LIB_PATH)
        _declare(lib)
        _LIB = lib
    return _LIB


def _declare(lib):
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    lib.eg_version.restype = C.c_int
    lib.eg_last_error.restype = C.c_char_p
    lib.eg_mesh_create.argtypes = [C.POINTER(abi.EgMeshDesc), C.POINTER(abi.EgParams), C.POINTER(vp)]
    lib.eg_mesh_destroy.argtypes = [vp]
    lib.eg_mesh_num_dof.argtypes = [vp]
    lib.eg_mesh_num_dof.restype = C.c_int64
    lib.eg_eval_residual.argtypes = [vp, vp, vp, C.c_double, C.c_int32]
    lib.eg_calc_norm.argtypes = [vp, vp, C.c_int32, C.c_int32, dp]
    lib.eg_mesh_set_stream.argtypes = [vp, vp, C.c_int32]
    lib.eg_eval_residual_async.argtypes = [vp, vp, vp]
    lib.eg_sync.argtypes = [vp]
    lib.eg_set_timing.argtypes = [vp, C.c_int32]
    lib.eg_get_timings.argtypes = [vp, C.POINTER(Timings)]
    lib.eg_reset_timings.argtypes = [vp]
    lib.eg_calc_functional.argtypes = [vp, vp, C.c_int32, C.c_int32, dp]
    lib.eg_calc_max_wave_speed.argtypes = [vp, vp, C.c_int32, dp]
    lib.eg_prolong.argtypes = [vp, vp, vp, vp, vp, C.c_int32]
    lib.eg_lo_create.argtypes = [vp, C.c_int32, C.POINTER(vp)]
    lib.eg_lo_destroy.argtypes = [vp]
    lib.eg_lo_calc.argtypes = [vp, vp, C.c_int32]
    lib.eg_lo_apply.argtypes = [vp, vp, vp, C.c_int32]
    lib.eg_lo_get_blocks.argtypes = [vp, vp, vp]
    lib.eg_lo_apply_native.argtypes = [vp, vp, vp]
    lib.eg_pc_apply_native.argtypes = [vp, vp, vp]
    lib.eg_pc_create.argtypes = [vp, C.POINTER(vp)]
    lib.eg_pc_destroy.argtypes = [vp]
    lib.eg_pc_calc.argtypes = [vp]
    lib.eg_pc_apply.argtypes = [vp, vp, vp, C.c_int32]
    lib.eg_lo_apply_transpose.argtypes = [vp, vp, vp, C.c_int32]
    lib.eg_pc_apply_transpose.argtypes = [vp, vp, vp, C.c_int32]
    lib.eg_ls_create.argtypes = [vp, vp, C.c_int32, C.POINTER(vp)]
    lib.eg_ls_destroy.argtypes = [vp]
    lib.eg_ls_set_tolerances.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_int32]
    lib.eg_ls_solve.argtypes = [vp, vp, vp, C.c_int32, C.POINTER(LsStats)]
    lib.eg_ls_solve_transpose.argtypes = [vp, vp, vp, C.c_int32, C.POINTER(LsStats)]
    lib.eg_ls_set_grid.argtypes = [vp, C.c_int32]
    lib.eg_set_gmres_batching.argtypes = [C.c_int32, C.c_double]
    lib.eg_newton_solve.argtypes = [vp, vp, C.c_int32, C.POINTER(NewtonOpts), C.POINTER(NewtonStats)]
    lib.eg_rk4.argtypes = [vp, vp, C.c_double, C.c_double, C.c_int32, C.c_double, C.c_int32,
                           C.POINTER(Rk4Stats)]
    lib.eg_rk4_static.argtypes = lib.eg_rk4.argtypes
    lib.eg_newton_release.argtypes = [vp]
    lib.eg_mesh_set_params.argtypes = [vp, C.POINTER(abi.EgParams)]
    lib.eg_estimate_mem.argtypes = [C.POINTER(abi.EgMemQuery), C.POINTER(abi.EgMemEstimate)]
    lib.eg_set_launch_config.argtypes = [vp, C.POINTER(abi.EgLaunchConfig)]
    lib.eg_get_launch_config.argtypes = [vp, C.POINTER(abi.EgLaunchConfig)]
    lib.eg_autotune.argtypes = [vp, vp, C.c_int32, C.POINTER(abi.EgTuneEntry), C.c_int32,
                                C.POINTER(C.c_int32)]


class LsStats(C.Structure):
    _fields_ = [("iters", C.c_int32), ("restarts", C.c_int32), ("converged", C.c_int32),
                ("reorth", C.c_int32), ("res0", C.c_double), ("res_final", C.c_double)]


class NewtonOpts(C.Structure):
    _fields_ = [("res_abstol", C.c_double), ("res_reltol", C.c_double), ("step_tol", C.c_double),
                ("krylov_reltol", C.c_double), ("itermax", C.c_int32),
                ("krylov_itermax", C.c_int32), ("gmres_restart", C.c_int32), ("precision", C.c_int32),
                ("globalize_euler", C.c_int32), ("euler_tau", C.c_double)]

    @classmethod
    def from_opts(cls, opts=None, precision=0):
        """Reference option keys (read_input.jl:414-496) with their defaults."""
        o = dict(opts or {})
        return cls(o.get("res_abstol", 1e-6), o.get("res_reltol", 1e-6), o.get("step_tol", 0.0),
                   o.get("krylov_reltol", 1e-2), o.get("itermax", 50),
                   o.get("krylov_itermax", 1000), o.get("gmres_restart", 30), precision,
                   int(o.get("newton_globalize_euler", False)), o.get("euler_tau", 1.0))


class NewtonStats(C.Structure):
    _fields_ = [("iters", C.c_int32), ("krylov_iters", C.c_int32), ("converged", C.c_int32),
                ("graph_iters", C.c_int32), ("res_norm0", C.c_double), ("res_norm", C.c_double),
                ("step_norm", C.c_double), ("t_residual", C.c_double), ("t_jacobian", C.c_double),
                ("t_pc", C.c_double), ("t_krylov", C.c_double)]

    def asdict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class Rk4Stats(C.Structure):
    _fields_ = [("steps", C.c_int32), ("reserved", C.c_int32), ("t", C.c_double),
                ("res_norm", C.c_double)]


class Timings(C.Structure):
    """eg_timings: per-phase device milliseconds (reference Timings buckets)."""
    _fields_ = [("t_face_flux", C.c_double), ("t_element", C.c_double), ("t_norm", C.c_double),
                ("t_other", C.c_double), ("launches", C.c_int64), ("timed", C.c_int64)]


def check(status):
    if status != abi.EG_OK:
        raise EulerGPUError(status, library().eg_last_error().decode())


FLUX_NAMES = {"RoeFlux": abi.EG_FLUX_ROE, "IRFlux": abi.EG_FLUX_IR}


def params_from_opts(opts: dict) -> abi.EgParams:
    """Translate reference option keys (read_input.jl) into eg_params."""
    return abi.EgParams.make(
        gamma=opts.get("gamma", 1.4), Ma=opts.get("Ma", 0.5), aoa_deg=opts.get("aoa", 0.0),
        M_in=opts.get("vortex_M_in", 0.5),
        face_flux=FLUX_NAMES[opts.get("Flux_name", "RoeFlux")],
        volume_integral_type=opts.get("volume_integral_type", 1),
        volume_flux=FLUX_NAMES[opts.get("Volume_flux_name", "IRFlux")],
        p_free=opts.get("p_free"))


def mem_query(mesh, precision=None, restart=30, prolong_from=None):
    """eg_mem_query of a host Mesh: precision None (mesh and state only),
    0 (FP64 Newton) or 1 (mixed); prolong_from = the coarser level's operator."""
    op = mesh.sbp
    ident = np.broadcast_to(np.eye(op.numfacenodes), op.interp.shape)
    face_diag = op.stencilsize == op.numfacenodes and bool(np.array_equal(op.interp, ident))
    return abi.EgMemQuery(
        mesh.dim, mesh.numEl, op.numnodes, op.numfacenodes, op.stencilsize, mesh.numInterfaces,
        mesh.numBoundaryFaces, mesh.nbrperm.shape[0], -1 if precision is None else int(precision),
        int(restart), 0 if prolong_from is None else prolong_from.numnodes, int(face_diag))


def estimate_mem(mesh, precision=None, restart=30, prolong_from=None):
    """Device bytes the library takes for `mesh` (and, with a precision, its
    Newton work objects) plus the caller's q and res (reference estimateMem.jl)."""
    out = abi.EgMemEstimate()
    qy = mem_query(mesh, precision, restart, prolong_from)
    check(library().eg_estimate_mem(C.byref(qy), C.byref(out)))
    return out


def set_gmres_batching(enable=True, window_us=50.0):
    """run the Krylov solves of concurrent Newton solves (one thread per mesh)
    in shared cooperative launches (process-wide switch)."""
    check(library().eg_set_gmres_batching(int(bool(enable)), float(window_us)))


class GPUMesh:
    """Owner of one eg_mesh (device copy of mesh + operator + parameters)."""

    def __init__(self, mesh, opts: dict):
        self.lib = library()
        self.mesh = mesh
        self.opts = dict(opts)
        self.desc = abi.MeshDesc(mesh)
        self.params = params_from_opts(opts)
        h = C.c_void_p()
        check(self.lib.eg_mesh_create(C.byref(self.desc.desc), C.byref(self.params), C.byref(h)))
        self.handle = h
        self.ndof = int(self.lib.eg_mesh_num_dof(h))

    def set_params(self, opts: dict):
        """new physics options (Mach numbers, fluxes) for this device mesh; the
        boundary Dirichlet states are re-evaluated on the host and uploaded."""
        params = params_from_opts(opts)
        check(self.lib.eg_mesh_set_params(self.handle, C.byref(params)))
        self.params = params
        self.opts = dict(opts)

    def set_launch_config(self, elements_per_cta=0, volume_mma=False):
        """element-kernel launch shape: elements per CTA (0: built-in) and the
        FP64 tensor-core volume contraction (weak form only)."""
        c = abi.EgLaunchConfig(int(elements_per_cta), int(bool(volume_mma)))
        check(self.lib.eg_set_launch_config(self.handle, C.byref(c)))

    def launch_config(self):
        c = abi.EgLaunchConfig()
        check(self.lib.eg_get_launch_config(self.handle, C.byref(c)))
        return {"elements_per_cta": c.elements_per_cta, "volume_mma": bool(c.volume_mma)}

    def autotune(self, q_dev, reps=20):
        """time every admissible element-kernel configuration on the device
        state q_dev and keep the fastest; returns [(config dict, ms)]."""
        table = (abi.EgTuneEntry * 64)()
        n = C.c_int32(0)
        check(self.lib.eg_autotune(self.handle, self._dev(q_dev, self.ndof, "torch.float64"),
                                   int(reps), table, 64, C.byref(n)))
        return [({"elements_per_cta": t.config.elements_per_cta,
                  "volume_mma": bool(t.config.volume_mma)}, t.ms) for t in table[:n.value]]

    def close(self):
        if getattr(self, "handle", None):
            self.lib.eg_mesh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- array helpers -----------------------------------------------------
    @staticmethod
    def _ptr(a, n):
        """(pointer, mem flag) of a numpy array (host) or a CUDA tensor of n
        float64 values; the library sees raw pointers, so the size is
        checked here."""
        if isinstance(a, np.ndarray):
            if not (a.flags.c_contiguous and a.dtype == np.float64):
                raise ValueError("expected a C-contiguous float64 array")
            if a.size != n:
                raise ValueError(f"expected {n} values, got an array of {a.size}")
            return C.c_void_p(a.ctypes.data), abi.EG_MEM_HOST
        # torch tensor on the device
        if a.dtype.__repr__() != "torch.float64" or not a.is_contiguous():
            raise ValueError("expected a contiguous float64 tensor")
        if a.numel() != n:
            raise ValueError(f"expected {n} values, got a tensor of {a.numel()}")
        if a.device.type != "cuda":
            return C.c_void_p(a.data_ptr()), abi.EG_MEM_HOST
        return C.c_void_p(a.data_ptr()), abi.EG_MEM_DEVICE

    @staticmethod
    def _dev(t, n, dtype_name):
        """device pointer of a contiguous CUDA tensor of n values of dtype_name."""
        if getattr(t, "device", None) is None or t.device.type != "cuda":
            raise ValueError("expected a CUDA tensor")
        if t.dtype.__repr__() != dtype_name or not t.is_contiguous() or t.numel() != n:
            raise ValueError(f"expected a contiguous {dtype_name} tensor of {n} values")
        return C.c_void_p(t.data_ptr())

    def eval_residual(self, q, res, t=0.0):
        pq, mq = self._ptr(q, self.ndof)
        pr, mr = self._ptr(res, self.ndof)
        if mq != mr:
            raise ValueError("q and res must both be host or both be device arrays")
        check(self.lib.eg_eval_residual(self.handle, pq, pr, t, mq))
        return res

    def set_stream(self, stream_handle):
        """run this mesh's work on a caller's CUDA stream (an int handle, 0 =
        CUDA's default stream), or on the library's own stream with None."""
        if stream_handle is None:
            check(self.lib.eg_mesh_set_stream(self.handle, None, 1))
        else:
            check(self.lib.eg_mesh_set_stream(self.handle, C.c_void_p(stream_handle), 0))

    def eval_residual_async(self, q_dev, res_dev):
        """enqueue R(q) with device tensors, no host synchronisation."""
        check(self.lib.eg_eval_residual_async(self.handle, self._dev(q_dev, self.ndof, "torch.float64"),
                                              self._dev(res_dev, self.ndof, "torch.float64")))

    def sync(self):
        check(self.lib.eg_sync(self.handle))

    def set_timing(self, on=True):
        check(self.lib.eg_set_timing(self.handle, int(on)))

    def timings(self):
        t = Timings()
        check(self.lib.eg_get_timings(self.handle, C.byref(t)))
        return t

    def reset_timings(self):
        check(self.lib.eg_reset_timings(self.handle))

    def functional_pressure(self, q, bc_group=0):
        """integral of p over the faces of a boundary-condition group."""
        pq, mq = self._ptr(q, self.ndof)
        out = C.c_double()
        check(self.lib.eg_calc_functional(self.handle, pq, bc_group, mq, C.byref(out)))
        return out.value

    def max_wave_speed(self, q):
        """calcMaxWaveSpeed: max over the nodes of a + |u| (euler_funcs.jl:1810)."""
        pq, mq = self._ptr(q, self.ndof)
        out = C.c_double()
        check(self.lib.eg_calc_max_wave_speed(self.handle, pq, mq, C.byref(out)))
        return out.value

    def cfl_time_step(self, q, cfl):
        """delta_t = CFL * min_el_size / wave_speed (startup_func.jl:241-247);
        min_el_size is the smallest node spacing of an element (mesh.py)."""
        return cfl * self.mesh.min_el_size / self.max_wave_speed(q)

    def newton(self, q, opts=None, precision=0):
        """steady Newton solve in place (reference newton.jl:54); returns stats.
        Raises EulerGPUError(EG_ERR_NOT_CONVERGED) if the tolerances are not met."""
        pq, mq = self._ptr(q, self.ndof)
        o = NewtonOpts.from_opts(opts, precision)
        st = NewtonStats()
        rc = self.lib.eg_newton_solve(self.handle, pq, mq, C.byref(o), C.byref(st))
        self.last_newton = st
        check(rc)
        return st

    def release_newton(self):
        """free the Newton work objects the mesh keeps between solves."""
        check(self.lib.eg_newton_release(self.handle))

    def rk4(self, q, h, t_max, itermax=0, res_tol=-1.0):
        """classical RK4 in place (reference rk4.jl:404); returns stats."""
        pq, mq = self._ptr(q, self.ndof)
        st = Rk4Stats()
        check(self.lib.eg_rk4(self.handle, pq, h, t_max, itermax, res_tol, mq, C.byref(st)))
        return st

    def calc_norm(self, r, strongres=True):
        pr, mr = self._ptr(r, self.ndof)
        out = C.c_double()
        check(self.lib.eg_calc_norm(self.handle, pr, int(strongres), mr, C.byref(out)))
        return out.value


class EulerData:
    """The fields of the reference's EulerData the hot path touches."""

    def __init__(self, mesh, opts):
        self.q = np.zeros((mesh.numEl, mesh.numNodesPerElement, mesh.numDofPerNode))
        self.res = np.zeros_like(self.q)
        self.M = np.repeat(mesh.M[:, :, None], mesh.numDofPerNode, axis=2)
        self.Minv = 1.0 / self.M
        self.gpu = GPUMesh(mesh, opts)

    @property
    def q_vec(self):
        return self.q.reshape(-1)

    @property
    def res_vec(self):
        return self.res.reshape(-1)


def createObjects(mesh, opts):
    """(mesh, sbp, eqn, opts) tuple as the reference's createObjects returns."""
    return mesh, mesh.sbp, EulerData(mesh, opts), opts


def evalResidual(mesh, sbp, eqn, opts, t=0.0):
    """eqn.res <- R(eqn.q) on the GPU (weak form; reference euler.jl:111)."""
    eqn.gpu.eval_residual(eqn.q, eqn.res, t)


def calcNorm(eqn, res_vec, strongres=False):
    """SBP norm of a residual vector (reference Utils.jl:427)."""
    r = np.ascontiguousarray(np.asarray(res_vec, dtype=np.float64).reshape(eqn.q.shape))
    return eqn.gpu.calc_norm(r, strongres)


def physicsRhs(mesh, sbp, eqn, opts, rhs_vec=None, t=0.0):
    """physicsRhs (reference src/jacobian/residual_evaluation.jl:64-84): R(eqn.q)
    into eqn.res (and rhs_vec when given, which may alias eqn.res_vec); returns
    calcNorm(R, strongres=true), the M^-1-weighted norm Newton tests."""
    evalResidual(mesh, sbp, eqn, opts, t)
    if rhs_vec is not None and rhs_vec is not eqn.res_vec:
        rhs_vec[...] = eqn.res_vec
    return calcNorm(eqn, eqn.res_vec, strongres=True)


def evalJacobian(mesh, sbp, eqn, opts, assembler, t=0.0):
    """evalJacobian (reference src/solver/euler/evalJacobian.jl:6-72): the
    explicit Jacobian at eqn.q into `assembler`, a LinearOperator of this
    mesh.  Its blocks are overwritten (the reference adds into a matrix its
    caller zeroed first, jacobian.jl:118-121)."""
    assembler.calc(eqn.q)
    return assembler


def calcMaxWaveSpeed(mesh, sbp, eqn, opts):
    """calcMaxWaveSpeed (reference euler_funcs.jl:1810-1834) of eqn.q."""
    return eqn.gpu.max_wave_speed(eqn.q)


def _euler_rhs_only(func):
    if func is not None and func is not evalResidual and func is not physicsRhs:
        raise NotImplementedError("the device drivers evaluate the Euler residual only")


def newton(func, mesh, sbp, eqn, opts, pmesh=None, precision=0):
    """newton (reference src/NonlinearSolvers/newton.jl:54): eqn.q is driven
    to the steady state in place with the options' res_abstol / res_reltol /
    step_tol / krylov_reltol / newton_globalize_euler / euler_tau; func must be
    the Euler residual (evalResidual or physicsRhs).  precision 1 runs the
    Jacobian, preconditioner and Krylov solve in FP32.  Raises EulerGPUError
    (EG_ERR_NOT_CONVERGED) when the tolerances are not met."""
    _euler_rhs_only(func)
    return eqn.gpu.newton(eqn.q, opts, precision=precision)


def rk4(func, h, t_max, mesh, sbp, eqn, opts, res_tol=-1.0, real_time=False, itermax=0):
    """rk4 (reference src/NonlinearSolvers/rk4.jl:404): eqn.q advanced in
    place by round(t_max / h) classical RK4 steps (fewer when itermax > 0 or
    the stage-1 norm drops below res_tol > 0); func must be the Euler
    residual.  real_time is accepted for the signature (the residual is
    time-independent).

    With opts["use_checkpointing"] the state is saved every
    opts["checkpoint_freq"] steps into opts["ncheckpoints"] rotating
    checkpoints under opts.get("checkpoint_dir", cwd) (rk4.jl:165-229); with
    opts["is_restart"] the run continues from the step of the most recent
    complete checkpoint, whose state the caller loads first with
    checkpoint.loadRestartState (as the reference's startup does).  The device
    advances the state between checkpoint steps; the results equal an
    uninterrupted run's."""
    _euler_rhs_only(func)
    opts = {} if opts is None else opts
    if not opts.get("use_checkpointing", False):
        return eqn.gpu.rk4(eqn.q, h, t_max, itermax=itermax, res_tol=res_tol)
    from . import checkpoint

    last = [0.0]

    def advance(n, itermax_local):
        st = eqn.gpu.rk4(eqn.q, h, n * h, itermax=itermax_local, res_tol=res_tol)
        last[0] = st.res_norm
        return st.steps

    steps, t, _ = checkpoint.rk4_checkpointed(advance, eqn.q, h, t_max, opts, itermax=itermax,
                                              root=opts.get("checkpoint_dir"))
    st = Rk4Stats()
    st.steps, st.t, st.res_norm = steps, t, last[0]
    return st


class LinearOperator:
    """Explicit Jacobian (reference AbstractLO: calcLinearOperator /
    applyLinearOperator), element-block sparse on the device."""

    def __init__(self, gmesh: GPUMesh, precision=0):
        self.g = gmesh
        self.lib = gmesh.lib
        self.precision = precision
        h = C.c_void_p()
        check(self.lib.eg_lo_create(gmesh.handle, precision, C.byref(h)))
        self.handle = h
        op = gmesh.mesh.sbp
        self.n = op.numnodes * gmesh.mesh.numDofPerNode
        self.nb = op.stencilsize * gmesh.mesh.numDofPerNode

    def calc(self, q):
        pq, mq = GPUMesh._ptr(q, self.g.ndof)
        check(self.lib.eg_lo_calc(self.handle, pq, mq))

    def apply(self, x, y):
        px, mx = GPUMesh._ptr(x, self.g.ndof)
        py, my = GPUMesh._ptr(y, self.g.ndof)
        if mx != my:
            raise ValueError("x and y must both be host or both be device arrays")
        check(self.lib.eg_lo_apply(self.handle, px, py, mx))
        return y

    def apply_transpose(self, x, y):
        """y = J^T x (reference applyLinearOperatorTranspose)."""
        px, mx = GPUMesh._ptr(x, self.g.ndof)
        py, my = GPUMesh._ptr(y, self.g.ndof)
        if mx != my:
            raise ValueError("x and y must both be host or both be device arrays")
        check(self.lib.eg_lo_apply_transpose(self.handle, px, py, mx))
        return y

    @property
    def native_dtype(self):
        return "torch.float32" if self.precision == 1 else "torch.float64"

    def apply_native(self, x_dev, y_dev):
        """y = J x on device tensors of the operator's precision (enqueued)."""
        n, dt = self.g.ndof, self.native_dtype
        check(self.lib.eg_lo_apply_native(self.handle, GPUMesh._dev(x_dev, n, dt),
                                          GPUMesh._dev(y_dev, n, dt)))

    def blocks(self):
        ms = self.g.mesh
        diag = np.zeros((ms.numEl, self.n, self.n))
        cpl = np.zeros((max(ms.numInterfaces, 1), 2, self.nb, self.nb))
        check(self.lib.eg_lo_get_blocks(self.handle, C.c_void_p(diag.ctypes.data),
                                        C.c_void_p(cpl.ctypes.data)))
        return diag, cpl[:ms.numInterfaces]

    def close(self):
        if getattr(self, "handle", None):
            self.lib.eg_lo_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BlockJacobiPC:
    """Element block-Jacobi preconditioner (reference NewtonBDiagPC)."""

    def __init__(self, lo: LinearOperator):
        self.lo = lo
        self.lib = lo.lib
        h = C.c_void_p()
        check(self.lib.eg_pc_create(lo.handle, C.byref(h)))
        self.handle = h

    def calc(self):
        check(self.lib.eg_pc_calc(self.handle))

    def apply(self, x, y):
        px, mx = GPUMesh._ptr(x, self.lo.g.ndof)
        py, my = GPUMesh._ptr(y, self.lo.g.ndof)
        if mx != my:
            raise ValueError("x and y must both be host or both be device arrays")
        check(self.lib.eg_pc_apply(self.handle, px, py, mx))
        return y

    def apply_transpose(self, x, y):
        """y = M^-T x (reference applyPCTranspose)."""
        px, mx = GPUMesh._ptr(x, self.lo.g.ndof)
        py, my = GPUMesh._ptr(y, self.lo.g.ndof)
        if mx != my:
            raise ValueError("x and y must both be host or both be device arrays")
        check(self.lib.eg_pc_apply_transpose(self.handle, px, py, mx))
        return y

    def apply_native(self, x_dev, y_dev):
        """y = M^-1 x on device tensors of the operator's precision (enqueued)."""
        n, dt = self.lo.g.ndof, self.lo.native_dtype
        check(self.lib.eg_pc_apply_native(self.handle, GPUMesh._dev(x_dev, n, dt),
                                          GPUMesh._dev(y_dev, n, dt)))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.eg_pc_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LinearSolver:
    """GMRES(restart) with right block-Jacobi preconditioning (reference
    StandardLinearSolver: linearSolve / setTolerances)."""

    def __init__(self, pc: BlockJacobiPC, lo: LinearOperator, restart=30):
        self.pc, self.lo, self.lib = pc, lo, lo.lib
        h = C.c_void_p()
        check(self.lib.eg_ls_create(lo.handle, pc.handle, restart, C.byref(h)))
        self.handle = h
        self.restart = restart
        self.reltol, self.abstol, self.itermax = -1.0, -1.0, -1

    def set_tolerances(self, reltol=-1.0, abstol=-1.0, dtol=-1.0, itermax=-1):
        """setTolerances (reference ls_standard.jl): negative values keep the
        current setting.  The values are also kept here for the transposed
        solve (adjoint.linearSolveTranspose)."""
        check(self.lib.eg_ls_set_tolerances(self.handle, reltol, abstol, dtol, itermax))
        if reltol >= 0:
            self.reltol = reltol
        if abstol >= 0:
            self.abstol = abstol
        if itermax > 0:
            self.itermax = itermax

    def set_grid(self, blocks=0):
        """blocks of the persistent GMRES kernel (0: automatic)."""
        check(self.lib.eg_ls_set_grid(self.handle, int(blocks)))

    def solve(self, b, x):
        pb, mb = GPUMesh._ptr(b, self.lo.g.ndof)
        px, mx = GPUMesh._ptr(x, self.lo.g.ndof)
        if mb != mx:
            raise ValueError("b and x must both be host or both be device arrays")
        st = LsStats()
        check(self.lib.eg_ls_solve(self.handle, pb, px, mb, C.byref(st)))
        return st

    def solve_transpose(self, b, x):
        """linearSolveTranspose (reference ls_standard.jl:230-244): x <- the
        solution of J^T x = b (x is also the initial guess), on the device."""
        pb, mb = GPUMesh._ptr(b, self.lo.g.ndof)
        px, mx = GPUMesh._ptr(x, self.lo.g.ndof)
        if mb != mx:
            raise ValueError("b and x must both be host or both be device arrays")
        st = LsStats()
        check(self.lib.eg_ls_solve_transpose(self.handle, pb, px, mb, C.byref(st)))
        return st

    def close(self):
        if getattr(self, "handle", None):
            self.lib.eg_ls_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def prolongation_matrix(op_lo, op_hi, nv):
    """T[(j,a)][(m,b)] = delta_ab P[j][m] with P the degree-p_lo interpolation
    from op_lo's nodes to op_hi's nodes (least squares where op_lo has more
    nodes than degree-p_lo polynomials, as SBP-Gamma does)."""
    from . import sbp as _sbp
    V_lo, _ = _sbp.vandermonde(op_lo.nodes, op_lo.p)
    V_hi, _ = _sbp.vandermonde(op_hi.nodes, op_lo.p)
    P = V_hi @ np.linalg.pinv(V_lo)
    return np.ascontiguousarray(np.kron(P, np.eye(nv)))


def prolong(g_lo: GPUMesh, q_lo, g_hi: GPUMesh, q_hi):
    """q_hi <- degree prolongation of q_lo (same elements, on the device)."""
    T = prolongation_matrix(g_lo.mesh.sbp, g_hi.mesh.sbp, g_lo.mesh.numDofPerNode)
    pl, ml = GPUMesh._ptr(q_lo, g_lo.ndof)
    ph, mh = GPUMesh._ptr(q_hi, g_hi.ndof)
    if ml != mh:
        raise ValueError("q_lo and q_hi must both be host or both be device arrays")
    check(g_lo.lib.eg_prolong(g_lo.handle, pl, g_hi.handle, ph, C.c_void_p(T.ctypes.data), ml))
    return q_hi


def solve_steady(levels, q_lo, opts=None, precision=0, level_tol=None, level_opts=None):
    """Steady solve with p-continuation: Newton on levels[0] (a GPUMesh of the
    lowest degree) from q_lo, prolong the result to the next level, Newton
    again, up to levels[-1].  Intermediate levels stop at level_tol (default:
    the final tolerance); level_opts[k] (a dict) overrides options of level k.
    Returns (q of the last level, list of stats)."""
    opts = dict(opts or {})
    stats = []
    q = q_lo
    for k, g in enumerate(levels):
        if k > 0:
            qn = np.zeros((g.mesh.numEl, g.mesh.numNodesPerElement, g.mesh.numDofPerNode)) \
                if isinstance(q, np.ndarray) else q.new_zeros(
                    (g.mesh.numEl, g.mesh.numNodesPerElement, g.mesh.numDofPerNode))
            prolong(levels[k - 1], q, g, qn)
            q = qn
        o = dict(opts)
        if k < len(levels) - 1 and level_tol is not None:
            o["res_abstol"] = level_tol
        if level_opts is not None and level_opts[k]:
            o.update(level_opts[k])
        stats.append(g.newton(q, o, precision=precision))
    return q, stats
