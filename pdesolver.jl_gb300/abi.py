"""ctypes declarations of the C ABI in include/eulergpu.h.

``MeshDesc.from_mesh`` fills an ``eg_mesh_desc`` from a host ``Mesh`` (the
arrays are kept alive by the returned object).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

EG_OK = 0
EG_ERR_INVALID = 1
EG_ERR_CUDA = 2
EG_ERR_OOM = 3
EG_ERR_NEG_DENSITY = 4
EG_ERR_NEG_PRESSURE = 5
EG_ERR_NONFINITE = 6
EG_ERR_LU_PIVOT = 7
EG_ERR_KRYLOV = 8
EG_ERR_NOT_CONVERGED = 9
EG_ERR_TIMEOUT = 10
EG_ERR_UNSUPPORTED = 11

STATUS_NAMES = {v: k for k, v in list(globals().items()) if k.startswith("EG_") and isinstance(v, int)}

EG_MEM_HOST = 0
EG_MEM_DEVICE = 1
EG_FLUX_ROE = 0
EG_FLUX_IR = 1
EG_BC_VORTEX = 0
EG_BC_FREESTREAM = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class EgParams(C.Structure):
    _fields_ = [
        ("gamma", C.c_double), ("Ma", C.c_double), ("aoa", C.c_double),
        ("rho_free", C.c_double), ("p_free", C.c_double),
        ("vortex_r_in", C.c_double), ("vortex_rho_in", C.c_double), ("vortex_M_in", C.c_double),
        ("face_flux", C.c_int32), ("volume_integral_type", C.c_int32),
        ("volume_flux", C.c_int32), ("reserved", C.c_int32),
    ]

    @classmethod
    def make(cls, gamma=1.4, Ma=0.5, aoa_deg=0.0, M_in=0.5, face_flux=EG_FLUX_ROE,
             volume_integral_type=1, volume_flux=EG_FLUX_IR, p_free=None):
        """Defaults follow read_input.jl (gamma 1.4, p_free = 1/gamma,
        rho_free = 1) and the vortex of common_funcs.jl:25-79 (r_in = 1,
        rho_in = 2) with the inner Mach number M_in as a parameter."""
        return cls(gamma, Ma, aoa_deg * math.pi / 180.0, 1.0,
                   (1.0 / gamma) if p_free is None else p_free,
                   1.0, 2.0, M_in, face_flux, volume_integral_type, volume_flux, 0)


class EgMeshDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("num_el", C.c_int32), ("nodes_per_el", C.c_int32),
        ("nodes_per_face", C.c_int32), ("stencil_size", C.c_int32),
        ("num_interfaces", C.c_int32), ("num_bndry", C.c_int32), ("num_bc", C.c_int32),
        ("num_orient", C.c_int32), ("reserved", C.c_int32),
        ("Q", _dp), ("w", _dp), ("interp", _dp), ("perm", _ip), ("nbrperm", _ip),
        ("wface", _dp), ("dxidx", _dp), ("jac", _dp), ("coords", _dp),
        ("interfaces", _ip), ("nrm_face", _dp), ("bndryfaces", _ip),
        ("bndry_offsets", _ip), ("bc_types", _ip), ("coords_bndry", _dp), ("nrm_bndry", _dp),
    ]


class EgMemQuery(C.Structure):
    """eg_mem_query: the mesh counts eg_estimate_mem reads."""
    _fields_ = [(k, C.c_int32) for k in (
        "dim", "num_el", "nodes_per_el", "nodes_per_face", "stencil_size", "num_interfaces",
        "num_bndry", "num_orient", "newton_precision", "gmres_restart", "prolong_from_nodes",
        "face_diagonal")]


class EgMemEstimate(C.Structure):
    _fields_ = [("mesh", C.c_uint64), ("eqn", C.c_uint64), ("jacobian", C.c_uint64),
                ("pc", C.c_uint64), ("krylov", C.c_uint64), ("newton", C.c_uint64),
                ("total", C.c_uint64), ("allocations", C.c_int64)]

    def asdict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class EgLaunchConfig(C.Structure):
    _fields_ = [("elements_per_cta", C.c_int32), ("volume_mma", C.c_int32),
                ("reserved", C.c_int32 * 2)]


class EgTuneEntry(C.Structure):
    _fields_ = [("config", EgLaunchConfig), ("ms", C.c_double)]


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class MeshDesc:
    """Owns the contiguous arrays behind an ``EgMeshDesc``."""

    def __init__(self, mesh):
        op = mesh.sbp
        self.mesh = mesh
        # Q[k][j][i] = Q_k(i, j)  (Julia sbp.Q memory order)
        self._arr = dict(
            Q=_f64(np.transpose(op.Q, (0, 2, 1))), w=_f64(op.w), interp=_f64(op.interp),
            perm=_i32(op.perm), nbrperm=_i32(mesh.nbrperm), wface=_f64(op.wface),
            dxidx=_f64(mesh.dxidx), jac=_f64(mesh.jac), coords=_f64(mesh.coords),
            interfaces=_i32(mesh.interfaces if mesh.numInterfaces else np.zeros((0, 5))),
            nrm_face=_f64(mesh.nrm_face), bndryfaces=_i32(mesh.bndryfaces.reshape(-1, 2)),
            bndry_offsets=_i32(mesh.bndry_offsets), bc_types=_i32(mesh.bc_types),
            coords_bndry=_f64(mesh.coords_bndry), nrm_bndry=_f64(mesh.nrm_bndry),
        )
        d = EgMeshDesc()
        d.dim = mesh.dim
        d.num_el = mesh.numEl
        d.nodes_per_el = op.numnodes
        d.nodes_per_face = op.numfacenodes
        d.stencil_size = op.stencilsize
        d.num_interfaces = mesh.numInterfaces
        d.num_bndry = mesh.numBoundaryFaces
        d.num_bc = len(mesh.bc_types)
        d.num_orient = mesh.nbrperm.shape[0]
        for k, a in self._arr.items():
            ptr_t = _ip if a.dtype == np.int32 else _dp
            setattr(d, k, a.ctypes.data_as(ptr_t))
        self.desc = d

    @property
    def ptr(self):
        return C.byref(self.desc)


def dptr(a):
    return a.ctypes.data_as(_dp)
