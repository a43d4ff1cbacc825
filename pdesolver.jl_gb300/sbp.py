"""Summation-by-parts operators on simplices (host-side set-up data).

The reference takes its volume operator (``sbp.Q``, ``sbp.w``,
``sbp.numnodes``) and face operator (``sbpface.interp``, ``perm``,
``nbrperm``, ``wface``, ``normal``) from SummationByParts.jl, constructed at
src/solver/common.jl:276-390.  That package is not vendored, so this module
builds operators with the same structure from the committed cubature rules
(``cubature_tables.py``) and the SBP definition:

* ``H = diag(w)`` with ``w`` the cubature weights (positive, exact to degree
  >= 2p-1);
* ``E_k = sum_f R_f^T B_f N_{f,k} R_f`` with ``R_f`` interpolation from the
  volume nodes to the face cubature nodes (exact for degree p), ``B_f`` the
  face cubature weights (exact for degree 2p) and ``N_{f,k}`` the k-th
  component of the reference outward normal of face f scaled to the face's
  measure over the measure of the reference face;
* ``Q_k = S_k + E_k / 2`` with ``S_k`` antisymmetric, the minimum-norm
  solution of the accuracy conditions ``Q_k V = H dV/dxi_k`` for the degree-p
  polynomial basis ``V``;
* ``D_k = H^{-1} Q_k``.

The same arrays feed the GPU library and the CPU oracle, so GPU-vs-oracle
parity is defined on them; entry-wise agreement with SummationByParts.jl is
not claimed (that package is absent).
"""
from __future__ import annotations

import dataclasses
import functools
import itertools

import numpy as np

from . import cubature_tables as _tab

TRI_VERTS = np.array([[-1.0, -1.0], [1.0, -1.0], [-1.0, 1.0]])
TET_VERTS = np.array([[-1.0, -1.0, -1.0], [1.0, -1.0, -1.0],
                      [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]])
# local faces as vertex index lists (0-based), outward normals follow
TRI_FACES = [(0, 1), (1, 2), (2, 0)]
TET_FACES = [(0, 1, 2), (0, 1, 3), (1, 2, 3), (0, 2, 3)]


def _tri_ref_normals():
    out = []
    for a, b in TRI_FACES:
        t = (TRI_VERTS[b] - TRI_VERTS[a]) / 2.0      # d x / d t on [-1, 1]
        out.append(np.array([t[1], -t[0]]))          # outward for CCW vertices
    return np.array(out)


def _tet_ref_normals():
    out = []
    cen = TET_VERTS.mean(axis=0)
    for a, b, c in TET_FACES:
        u = (TET_VERTS[b] - TET_VERTS[a]) / 2.0
        v = (TET_VERTS[c] - TET_VERTS[a]) / 2.0
        n = np.cross(u, v)                            # |n| = face area / 2
        if np.dot(n, TET_VERTS[a] - cen) < 0:
            n = -n
        out.append(n)
    return np.array(out)


def _poly_basis(dim, p):
    if dim == 2:
        return [(i, d - i) for d in range(p + 1) for i in range(d + 1)]
    return [(i, j, d - i - j) for d in range(p + 1) for i in range(d + 1) for j in range(d - i + 1)]


def vandermonde(x, p):
    """monomial Vandermonde V[n, m] and its derivatives dV[k][n, m]."""
    dim = x.shape[1]
    mono = _poly_basis(dim, p)
    V = np.zeros((x.shape[0], len(mono)))
    dV = np.zeros((dim, x.shape[0], len(mono)))
    for m, e in enumerate(mono):
        V[:, m] = np.prod(x ** np.array(e), axis=1)
        for k in range(dim):
            if e[k] == 0:
                continue
            e2 = list(e)
            e2[k] -= 1
            dV[k, :, m] = e[k] * np.prod(x ** np.array(e2), axis=1)
    return V, dV


@dataclasses.dataclass
class SBPOperator:
    """Volume + face SBP operator on the reference simplex.

    Mirrors the fields the reference reads from ``sbp`` and ``sbpface``
    (docs/src/interfaces.md; src/solver/euler/flux.jl:613-646;
    src/solver/euler/faceElementIntegrals.jl:75-109).
    """
    dim: int
    p: int
    family: str
    nodes: np.ndarray        # [Np, dim] reference coordinates
    w: np.ndarray            # [Np] cubature weights (diag of H)
    Q: np.ndarray            # [dim, Np, Np], Q[k][i, j]
    E: np.ndarray            # [dim, Np, Np]
    S: np.ndarray            # [dim, Np, Np] antisymmetric part
    D: np.ndarray            # [dim, Np, Np]
    wface: np.ndarray        # [Nf] face cubature weights
    face_ref: np.ndarray     # [Nf, dim-1] face cubature points in face coordinates
    R: np.ndarray            # [F, Nf, Np] dense interpolation volume -> face f
    perm: np.ndarray         # [F, S] stencil volume nodes of face f (int32)
    interp: np.ndarray       # [F, Nf, S] interpolation from the stencil of face f
    normals: np.ndarray      # [F, dim] scaled reference outward normals
    face_xi: np.ndarray      # [F, Nf, dim] reference coordinates of face nodes
    sparse_face: bool        # True: face nodes are volume nodes (diagonal E)

    @property
    def numnodes(self):
        return self.nodes.shape[0]

    @property
    def numfacenodes(self):
        return self.wface.shape[0]

    @property
    def numfaces(self):
        return self.dim + 1

    @property
    def stencilsize(self):
        return self.perm.shape[1]

    @property
    def numorient(self):
        return 1 if self.dim == 2 else 6


def _face_points_tri(f, t):
    a, b = TRI_FACES[f]
    return np.outer((1 - t) / 2, TRI_VERTS[a]) + np.outer((1 + t) / 2, TRI_VERTS[b])


def _face_points_tet(f, st):
    a, b, c = TET_FACES[f]
    l2 = (st[:, 0] + 1) / 2
    l3 = (st[:, 1] + 1) / 2
    l1 = 1 - l2 - l3
    return (np.outer(l1, TET_VERTS[a]) + np.outer(l2, TET_VERTS[b]) + np.outer(l3, TET_VERTS[c]))


def _solve_S(V, HdV, EV):
    """antisymmetric S (min-norm) with S V = HdV - EV/2."""
    n, m = V.shape
    B = HdV - 0.5 * EV
    pairs = [(i, j) for i in range(n) for j in range(i + 1, n)]
    A = np.zeros((n * m, len(pairs)))
    for c, (i, j) in enumerate(pairs):
        # S[i, j] = s, S[j, i] = -s ; (S V)[r, col] = sum_j S[r, j] V[j, col]
        for col in range(m):
            A[i * m + col, c] += V[j, col]
            A[j * m + col, c] -= V[i, col]
    s, *_ = np.linalg.lstsq(A, B.reshape(-1), rcond=None)
    S = np.zeros((n, n))
    for c, (i, j) in enumerate(pairs):
        S[i, j] = s[c]
        S[j, i] = -s[c]
    resid = np.max(np.abs(S @ V - B))
    if resid > 1e-11:
        raise RuntimeError(f"SBP accuracy conditions not solvable: {resid}")
    return S


def _lagrange_1d(xn, t):
    """1-D Lagrange interpolation matrix from nodes xn to points t."""
    L = np.ones((len(t), len(xn)))
    for j in range(len(xn)):
        for m in range(len(xn)):
            if m != j:
                L[:, j] *= (t - xn[m]) / (xn[j] - xn[m])
    return L


def _finish(dim, p, family, x, w, face_ref, wface, R, perm, interp, sparse):
    normals = _tri_ref_normals() if dim == 2 else _tet_ref_normals()
    F = dim + 1
    Np = x.shape[0]
    E = np.zeros((dim, Np, Np))
    for f in range(F):
        for k in range(dim):
            E[k] += normals[f, k] * (R[f].T * wface) @ R[f]
    V, dV = vandermonde(x, p)
    H = np.diag(w)
    Q = np.zeros((dim, Np, Np))
    S = np.zeros((dim, Np, Np))
    for k in range(dim):
        S[k] = _solve_S(V, H @ dV[k], E[k] @ V)
        Q[k] = S[k] + 0.5 * E[k]
    D = Q / w[None, :, None]
    face_xi = np.zeros((F, wface.shape[0], dim))
    for f in range(F):
        face_xi[f] = (_face_points_tri(f, face_ref[:, 0]) if dim == 2
                      else _face_points_tet(f, face_ref))
    return SBPOperator(dim=dim, p=p, family=family, nodes=x, w=w, Q=Q, E=E, S=S, D=D,
                       wface=wface, face_ref=face_ref, R=R, perm=perm.astype(np.int32),
                       interp=interp, normals=normals, face_xi=face_xi, sparse_face=sparse)


@functools.lru_cache(maxsize=None)
def tri_operator(family: str, p: int) -> SBPOperator:
    """Triangle SBP-Omega (all nodes interior) or SBP-Gamma (p+1 nodes on
    every edge) operator of degree p (reference: getTriSBPOmega /
    getTriSBPGamma, called at src/solver/common.jl:276-390)."""
    ent = _tab.TRI[(family, p)]
    x = np.array(ent["points"]).reshape(-1, 2)
    w = np.array(ent["weights"])
    Np = x.shape[0]
    t, wface = np.polynomial.legendre.leggauss(p + 1)
    Nf = t.shape[0]
    R = np.zeros((3, Nf, Np))
    if family == "omega":
        V, _ = vandermonde(x, p)
        Vinv = np.linalg.inv(V)
        perm = np.tile(np.arange(Np), (3, 1))
        interp = np.zeros((3, Nf, Np))
        for f in range(3):
            Vf, _ = vandermonde(_face_points_tri(f, t), p)
            R[f] = Vf @ Vinv
            interp[f] = R[f]
    elif family == "gamma":
        perm = np.zeros((3, p + 1), dtype=np.int64)
        interp = np.zeros((3, Nf, p + 1))
        for f, (a, b) in enumerate(TRI_FACES):
            va, vb = TRI_VERTS[a], TRI_VERTS[b]
            L = np.linalg.norm(vb - va)
            on = []
            for n in range(Np):
                d = np.linalg.norm(x[n] - va) + np.linalg.norm(x[n] - vb) - L
                if abs(d) < 1e-12:
                    on.append((2 * np.linalg.norm(x[n] - va) / L - 1, n))
            on.sort()
            if len(on) != p + 1:
                raise RuntimeError("gamma operator: wrong node count on an edge")
            tn = np.array([o[0] for o in on])
            perm[f] = [o[1] for o in on]
            interp[f] = _lagrange_1d(tn, t)
            R[f][:, perm[f]] = interp[f]
    else:
        raise ValueError(family)
    return _finish(2, p, family, x, w, t[:, None], wface, R, perm, interp, False)


@functools.lru_cache(maxsize=None)
def tet_operator_diage(p: int) -> SBPOperator:
    """Tetrahedral diagonal-E SBP operator (face nodes are volume nodes), the
    kind the reference gets from getTetSBPDiagE (src/solver/common.jl:276-390)."""
    ent = _tab.TET_DIAGE[p]
    x = np.array(ent["points"]).reshape(-1, 3)
    w = np.array(ent["weights"])
    fpts = np.array(ent["face_points"]).reshape(-1, 2)
    wface = np.array(ent["face_weights"])
    Np, Nf = x.shape[0], fpts.shape[0]
    R = np.zeros((4, Nf, Np))
    perm = np.zeros((4, Nf), dtype=np.int64)
    for f in range(4):
        phys = _face_points_tet(f, fpts)
        for i in range(Nf):
            d = np.linalg.norm(x - phys[i], axis=1)
            n = int(np.argmin(d))
            if d[n] > 1e-12:
                raise RuntimeError("diagonal-E operator: face node is not a volume node")
            perm[f, i] = n
            R[f, i, n] = 1.0
    interp = np.tile(np.eye(Nf), (4, 1, 1))
    return _finish(3, p, "diage", x, w, fpts, wface, R, perm, interp, True)


def get_operator(dim: int, family: str, p: int) -> SBPOperator:
    if dim == 2:
        return tri_operator(family, p)
    if family != "diage":
        raise ValueError("3-D operators: diagonal-E only")
    return tet_operator_diage(p)


def tet_orientations():
    """The 6 vertex permutations of a triangular face (for nbrperm tables)."""
    return list(itertools.permutations(range(3)))
