"""Structured simplex meshes with SBP node data (host-side set-up).

Stands in for the PUMI mesh object of the reference (PumiInterface.jl, not
vendored).  It produces the fields the reference's Euler path reads from
``mesh`` (docs/src/interfaces.md:210-470):

* ``coords[E, Np, d]``                     node coordinates
* ``dxidx[E, Np, d(x), d(xi)]``            ``|dx/dxi| * dxi_k/dx_p`` (reference
                                           ``dxidx[k, p, node, el]``)
* ``jac[E, Np]``                           ``det(dxi/dx)``
* ``interfaces[I, 5]``                     (elementL, elementR, faceL, faceR, orient)
* ``nbrperm[n_orient, Nf]``                face-node permutation for elementR
* ``nrm_face[I, Nf, d]``                   scaled normal, outward from elementL
* ``bndryfaces[B, 2]``                     (element, face)
* ``bndry_offsets[numBC + 1]``             BC groups
* ``coords_bndry, nrm_bndry[B, Nf, d]``

All indices are 0-based.  Memory layouts are the reference's column-major
arrays read in reverse index order, so a Julia caller can pass its own
arrays without copies.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .sbp import SBPOperator, TET_FACES, TRI_FACES, TET_VERTS, TRI_VERTS

BC_VORTEX = 0      # isentropicVortexBC (src/solver/euler/bc.jl:542-568)
BC_FREESTREAM = 1  # FreeStreamBC (src/solver/euler/bc.jl:1562-1647)


@dataclasses.dataclass
class Mesh:
    dim: int
    sbp: SBPOperator
    coords: np.ndarray
    dxidx: np.ndarray
    jac: np.ndarray
    interfaces: np.ndarray
    nbrperm: np.ndarray
    nrm_face: np.ndarray
    coords_face: np.ndarray
    bndryfaces: np.ndarray
    bndry_offsets: np.ndarray
    bc_types: np.ndarray
    coords_bndry: np.ndarray
    nrm_bndry: np.ndarray
    bndry_tag: np.ndarray         # geometric boundary id of each boundary face
    name: str = ""

    @property
    def numEl(self):
        return self.coords.shape[0]

    @property
    def numNodesPerElement(self):
        return self.coords.shape[1]

    @property
    def numDofPerNode(self):
        return self.dim + 2

    @property
    def numDof(self):
        return self.numEl * self.numNodesPerElement * self.numDofPerNode

    @property
    def numInterfaces(self):
        return self.interfaces.shape[0]

    @property
    def numBoundaryFaces(self):
        return self.bndryfaces.shape[0]

    @property
    def M(self):
        """diagonal mass matrix per node, w / jac (src/Utils/mass_matrix.jl:20-61)."""
        return self.sbp.w[None, :] / self.jac


def _metrics_from_jacobian(J):
    """J[..., p, k] = dx_p/dxi_k -> (dxidx[..., p(x), k(xi)], jac)."""
    det = np.linalg.det(J)
    if np.any(det <= 0):
        raise RuntimeError("mesh: non-positive mapping Jacobian")
    inv = np.linalg.inv(J)                    # inv[..., k, p] = dxi_k/dx_p
    dxidx = det[..., None, None] * np.swapaxes(inv, -1, -2)
    return dxidx, 1.0 / det


def _face_key(verts):
    return tuple(sorted(int(v) for v in verts))


def _connect(elverts, faces_local, sbp, coords_node_fn, face_points_fn, tag_fn,
             bc_of_tag):
    """Build interfaces / boundary faces and the geometric node matchings."""
    E = elverts.shape[0]
    table = {}
    ifaces, bfaces = [], []
    for e in range(E):
        for f, lv in enumerate(faces_local):
            key = _face_key(elverts[e, list(lv)])
            if key in table:
                eo, fo = table.pop(key)
                ifaces.append((eo, e, fo, f))
            else:
                table[key] = (e, f)
    for key, (e, f) in sorted(table.items(), key=lambda kv: kv[1]):
        bfaces.append((e, f))
    Nf = sbp.numfacenodes
    perms = []
    iface = np.zeros((len(ifaces), 5), dtype=np.int32)
    for n, (eL, eR, fL, fR) in enumerate(ifaces):
        xL = face_points_fn(eL, fL)
        xR = face_points_fn(eR, fR)
        perm = []
        for i in range(Nf):
            d = np.linalg.norm(xR - xL[i], axis=1)
            j = int(np.argmin(d))
            if d[j] > 1e-9 * max(1.0, np.abs(xL).max()):
                raise RuntimeError("mesh: face nodes of neighbours do not match")
            perm.append(j)
        perm = tuple(perm)
        if perm not in perms:
            perms.append(perm)
        iface[n] = (eL, eR, fL, fR, perms.index(perm))
    nbrperm = np.array(perms if perms else [tuple(range(Nf))], dtype=np.int32)
    tags = np.array([tag_fn(face_points_fn(e, f)) for e, f in bfaces], dtype=np.int32)
    bc = np.array([bc_of_tag(t) for t in tags], dtype=np.int32)
    order = np.lexsort((np.arange(len(bfaces)), tags, bc))
    bfaces = np.array(bfaces, dtype=np.int32).reshape(-1, 2)[order]
    tags = tags[order]
    bc = bc[order]
    bc_types = np.unique(bc).astype(np.int32)
    offsets = np.searchsorted(bc, bc_types).tolist() + [len(bc)]
    return iface, nbrperm, bfaces, np.array(offsets, dtype=np.int32), bc_types, tags


def _face_geometry(sbp, dxidx_face_fn, faces, coords_fn):
    """scaled normals and coordinates at the face nodes of (element, face)."""
    Nf, d = sbp.numfacenodes, sbp.dim
    nrm = np.zeros((len(faces), Nf, d))
    crd = np.zeros((len(faces), Nf, d))
    for n, (e, f) in enumerate(faces):
        Dx = dxidx_face_fn(e, f)          # [Nf, d(x), d(xi)]
        nrm[n] = np.einsum("k,ipk->ip", sbp.normals[f], Dx)
        crd[n] = coords_fn(e, f)
    return nrm, crd


def annulus(sbp: SBPOperator, nr: int, ntheta: int, r_in=1.0, r_out=3.0,
            bc=BC_VORTEX) -> Mesh:
    """Quarter annulus r in [r_in, r_out], theta in [0, pi/2] on nr x ntheta
    (r, theta) quads, each split along the diagonal from (r_i, theta_j) to
    (r_{i+1}, theta_{j+1}) into 2 straight-sided triangles (2 nr ntheta
    elements).  Boundary tags: 0 r = r_in, 1 r = r_out, 2 theta = 0,
    3 theta = pi/2."""
    assert sbp.dim == 2
    r = np.linspace(r_in, r_out, nr + 1)
    th = np.linspace(0.0, np.pi / 2, ntheta + 1)
    R, T = np.meshgrid(r, th, indexing="ij")
    vx = np.stack([(R * np.cos(T)).ravel(), (R * np.sin(T)).ravel()], axis=1)
    vid = lambda i, j: i * (ntheta + 1) + j  # noqa: E731
    els = []
    for i in range(nr):
        for j in range(ntheta):
            a, b, c, d = vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)
            els.append((a, b, c))
            els.append((a, c, d))
    elverts = np.array(els, dtype=np.int64)
    X = vx[elverts]                                  # [E, 3, 2]
    # affine map from the reference triangle: x = X0 + (X1-X0)(xi+1)/2 + (X2-X0)(eta+1)/2
    J = np.stack([(X[:, 1] - X[:, 0]) / 2, (X[:, 2] - X[:, 0]) / 2], axis=2)  # [E, p, k]
    dx, jac_e = _metrics_from_jacobian(J)
    Np = sbp.numnodes
    lam = _bary_tri(sbp.nodes)
    coords = np.einsum("nv,evp->enp", lam, X)
    dxidx = np.repeat(dx[:, None], Np, axis=1)
    jac = np.repeat(jac_e[:, None], Np, axis=1)

    def face_pts(e, f):
        return np.einsum("nv,vp->np", _bary_tri(sbp.face_xi[f]), X[e])

    def tag_fn(pts):
        rr = np.linalg.norm(pts, axis=1)
        if np.allclose(rr, r_in, atol=1e-9 * r_out) or np.all(rr < r_in + 1e-9):
            return 0
        if np.all(np.abs(pts[:, 1]) < 1e-12):
            return 2
        if np.all(np.abs(pts[:, 0]) < 1e-12):
            return 3
        return 1

    iface, nbrperm, bfaces, offs, bct, tags = _connect(
        elverts, TRI_FACES, sbp, None, face_pts, tag_fn, lambda t: bc)
    nrm_f, crd_f = _face_geometry(sbp, lambda e, f: np.repeat(dx[e][None], sbp.numfacenodes, 0),
                                  iface[:, [0, 2]], face_pts)
    nrm_b, crd_b = _face_geometry(sbp, lambda e, f: np.repeat(dx[e][None], sbp.numfacenodes, 0),
                                  bfaces, face_pts)
    return Mesh(2, sbp, coords, dxidx, jac, iface, nbrperm, nrm_f, crd_f, bfaces, offs,
                bct, crd_b, nrm_b, tags, name=f"annulus{nr}x{ntheta}")


def _bary_tri(xi):
    l2 = (xi[:, 0] + 1) / 2
    l3 = (xi[:, 1] + 1) / 2
    return np.stack([1 - l2 - l3, l2, l3], axis=1)


def _bary_tet(xi):
    l2 = (xi[:, 0] + 1) / 2
    l3 = (xi[:, 1] + 1) / 2
    l4 = (xi[:, 2] + 1) / 2
    return np.stack([1 - l2 - l3 - l4, l2, l3, l4], axis=1)


# P2 Lagrange geometry on the tetrahedron: vertex and edge-midpoint nodes
_TET_EDGES = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]


def _p2_tet_shape(lam):
    """quadratic Lagrange shape functions [n, 10] and their barycentric
    derivatives [n, 10, 4]."""
    n = lam.shape[0]
    N = np.zeros((n, 10))
    dN = np.zeros((n, 10, 4))
    for v in range(4):
        N[:, v] = lam[:, v] * (2 * lam[:, v] - 1)
        dN[:, v, v] = 4 * lam[:, v] - 1
    for m, (a, b) in enumerate(_TET_EDGES):
        N[:, 4 + m] = 4 * lam[:, a] * lam[:, b]
        dN[:, 4 + m, a] = 4 * lam[:, b]
        dN[:, 4 + m, b] = 4 * lam[:, a]
    return N, dN


def cube(sbp: SBPOperator, n: int, warp=0.05, seed=3, bc=BC_FREESTREAM) -> Mesh:
    """Unit cube of n^3 hexes, each split into 6 tetrahedra around the main
    diagonal (6 n^3 elements).  With ``warp`` != 0 every node is moved by
    x_i += warp * sin(pi x + phi) sin(pi y + phi) sin(pi z + phi) (same shift
    on each axis), phi drawn from ``seed``.  The warp is applied to the
    quadratic (P2) geometry nodes of each tetrahedron and the SBP node
    coordinates are interpolated from them, so neighbouring elements share
    their faces exactly and the metric terms, computed analytically from the
    P2 map, vary from node to node.  Boundary tags 0..5: x=0, x=1, y=0, y=1,
    z=0, z=1 of the unwarped cube."""
    assert sbp.dim == 3
    phi = float(np.random.default_rng(seed).uniform(0.0, 2 * np.pi)) if warp else 0.0
    g = np.linspace(0.0, 1.0, n + 1)
    Xg, Yg, Zg = np.meshgrid(g, g, g, indexing="ij")
    vx = np.stack([Xg.ravel(), Yg.ravel(), Zg.ravel()], axis=1)
    vid = lambda i, j, k: (i * (n + 1) + j) * (n + 1) + k  # noqa: E731
    # Kuhn split: the 6 monotone paths from corner 000 to 111
    paths = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    els = []
    for i in range(n):
        for j in range(n):
            for k in range(n):
                for pth in paths:
                    c = [i, j, k]
                    vs = [vid(*c)]
                    for ax in pth:
                        c[ax] += 1
                        vs.append(vid(*c))
                    els.append(vs)
    elverts = np.array(els, dtype=np.int64)
    X = vx[elverts]
    # orient positively
    J0 = np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]], axis=2)
    neg = np.linalg.det(J0) < 0
    elverts[neg, 2], elverts[neg, 3] = elverts[neg, 3].copy(), elverts[neg, 2].copy()
    X = vx[elverts]                                  # [E, 4, 3] unwarped vertices

    def warpfn(p):
        if not warp:
            return p
        s = (np.sin(np.pi * p[..., 0] + phi) * np.sin(np.pi * p[..., 1] + phi)
             * np.sin(np.pi * p[..., 2] + phi))
        return p + warp * s[..., None]

    # P2 geometry nodes of every element (unwarped positions, then warped)
    G = np.concatenate([X, np.stack([(X[:, a] + X[:, b]) / 2 for a, b in _TET_EDGES], 1)], 1)
    G = warpfn(G)                                    # [E, 10, 3]

    def geom(e_idx, xi):
        lam = _bary_tet(xi)
        N, dN = _p2_tet_shape(lam)
        # d lam / d xi: lam2 = (xi+1)/2 ... lam1 = 1 - sum
        dlam = np.array([[-0.5, -0.5, -0.5], [0.5, 0, 0], [0, 0.5, 0], [0, 0, 0.5]])
        dNdxi = np.einsum("nmv,vk->nmk", dN, dlam)
        x = np.einsum("nm,emp->enp", N, G[e_idx])
        Jm = np.einsum("nmk,emp->enpk", dNdxi, G[e_idx])
        return x, Jm

    allE = np.arange(X.shape[0])
    coords, Jn = geom(allE, sbp.nodes)
    dxidx, jac = _metrics_from_jacobian(Jn)

    def face_pts(e, f):
        x, _ = geom(np.array([e]), sbp.face_xi[f])
        return x[0]

    def face_dx(e, f):
        _, Jf = geom(np.array([e]), sbp.face_xi[f])
        d, _ = _metrics_from_jacobian(Jf[0])
        return d

    def tag_fn(pts):
        # classify by the unwarped face: use the face centroid of the
        # element's vertices instead (robust to the warp)
        return -1

    iface, nbrperm, bfaces, offs, bct, tags = _connect(
        elverts, TET_FACES, sbp, None, face_pts, tag_fn, lambda t: bc)
    # geometric tags from the unwarped vertex positions
    for n_, (e, f) in enumerate(bfaces):
        c = X[e, list(TET_FACES[f])].mean(axis=0)
        ax = int(np.argmin(np.minimum(np.abs(c), np.abs(1 - c))))
        tags[n_] = 2 * ax + (1 if abs(1 - c[ax]) < abs(c[ax]) else 0)
    nrm_f, crd_f = _face_geometry(sbp, face_dx, iface[:, [0, 2]], face_pts)
    nrm_b, crd_b = _face_geometry(sbp, face_dx, bfaces, face_pts)
    return Mesh(3, sbp, coords, dxidx, jac, iface, nbrperm, nrm_f, crd_f, bfaces, offs,
                bct, crd_b, nrm_b, tags, name=f"cube{n}")
