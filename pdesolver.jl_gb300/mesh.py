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

from .sbp import SBPOperator, TET_FACES, TRI_FACES

BC_VORTEX = 0      # isentropicVortexBC (src/solver/euler/bc.jl:542-568)
BC_FREESTREAM = 1  # FreeStreamBC (src/solver/euler/bc.jl:1562-1647)
BC_NOPENETRATION_ES = 2  # noPenetrationESBC (src/solver/euler/bc.jl:767-795)


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
    min_el_size: float = 0.0      # smallest node spacing in an element (CFL length)

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


def save_npz(path, ms, **extra):
    """Write a mesh and its SBP operator (all arrays, bit-exact) to an npz."""
    op = ms.sbp
    arrs = {f"mesh_{f.name}": getattr(ms, f.name) for f in dataclasses.fields(ms)
            if isinstance(getattr(ms, f.name), np.ndarray)}
    arrs.update({f"sbp_{f.name}": getattr(op, f.name) for f in dataclasses.fields(op)
                 if isinstance(getattr(op, f.name), np.ndarray)})
    meta = np.array([ms.dim, op.p, int(op.sparse_face)], dtype=np.int64)
    np.savez_compressed(path, meta=meta, meta_family=np.array(op.family),
                        meta_name=np.array(ms.name), **arrs, **extra)


def load_npz(path):
    """Inverse of save_npz: (mesh, other arrays)."""
    z = np.load(path)
    dim, p, sparse = (int(v) for v in z["meta"])
    opf = {f.name: z[f"sbp_{f.name}"] for f in dataclasses.fields(SBPOperator)
           if f"sbp_{f.name}" in z}
    op = SBPOperator(dim=dim, p=p, family=str(z["meta_family"]), sparse_face=bool(sparse), **opf)
    mf = {f.name: z[f"mesh_{f.name}"] for f in dataclasses.fields(Mesh) if f"mesh_{f.name}" in z}
    ms = Mesh(dim=dim, sbp=op, name=str(z["meta_name"]), **mf)
    extra = {k: z[k] for k in z.files if not k.startswith(("mesh_", "sbp_", "meta"))}
    return ms, extra


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


def _connect(elverts, faces_local, sbp, face_pts_all, tags_of_faces, bc_of_tag):
    """Interfaces, boundary faces and the geometric face-node matchings.

    face_pts_all[e, f, i, :] are the physical coordinates of face node i of
    local face f of element e.  Vectorised over all faces.
    """
    E, F = elverts.shape[0], len(faces_local)
    Nf = sbp.numfacenodes
    keys = np.sort(np.stack([elverts[:, list(lv)] for lv in faces_local], axis=1), axis=2)
    keys = keys.reshape(E * F, -1)
    order = np.lexsort(keys.T[::-1])
    ks = keys[order]
    same = np.all(ks[1:] == ks[:-1], axis=1)
    if np.any(same[1:] & same[:-1]):
        # a run of three or more equal keys: a face shared by more than two
        # elements (non-manifold or duplicated elements) would become two
        # overlapping interfaces and be integrated twice
        nbad = int(np.count_nonzero(same[1:] & same[:-1]))
        raise ValueError(f"mesh: {nbad} faces are shared by more than two elements "
                         "(non-manifold mesh or duplicated elements)")
    first = np.nonzero(same)[0]
    a, b = order[first], order[first + 1]          # element-face ids sharing a face
    pair_lo = np.minimum(a, b)
    pair_hi = np.maximum(a, b)
    srt = np.argsort(pair_lo, kind="stable")
    pair_lo, pair_hi = pair_lo[srt], pair_hi[srt]
    matched = np.zeros(E * F, dtype=bool)
    matched[pair_lo] = True
    matched[pair_hi] = True
    bids = np.nonzero(~matched)[0]
    eL, fL = pair_lo // F, pair_lo % F
    eR, fR = pair_hi // F, pair_hi % F
    xL = face_pts_all[eL, fL]                      # [I, Nf, d]
    xR = face_pts_all[eR, fR]
    dist = np.linalg.norm(xL[:, :, None, :] - xR[:, None, :, :], axis=3)   # [I, Nf, Nf]
    perm = np.argmin(dist, axis=2)
    scale = max(1.0, float(np.abs(face_pts_all).max()))
    if np.any(np.take_along_axis(dist, perm[:, :, None], 2) > 1e-9 * scale):
        raise RuntimeError("mesh: face nodes of neighbours do not match")
    uperm, orient = np.unique(perm, axis=0, return_inverse=True)
    iface = np.stack([eL, eR, fL, fR, orient.reshape(-1)], axis=1).astype(np.int32)
    nbrperm = uperm.astype(np.int32) if len(uperm) else np.arange(Nf, dtype=np.int32)[None]
    be, bf = bids // F, bids % F
    tags = np.asarray(tags_of_faces(be, bf), dtype=np.int32)
    # one boundary-condition group per geometric boundary (reference BC1..BCn
    # with bndry_offsets), ordered by tag, faces in element order within it
    o = np.lexsort((np.arange(len(bids)), tags))
    bfaces = np.stack([be, bf], axis=1).astype(np.int32)[o]
    tags = tags[o]
    gtags = np.unique(tags)
    bc_types = np.array([bc_of_tag(int(t)) for t in gtags], dtype=np.int32)
    offsets = np.searchsorted(tags, gtags).tolist() + [len(tags)]
    return iface, nbrperm, bfaces, np.array(offsets, dtype=np.int32), bc_types, tags


def _face_normals(sbp, dxidx_face_all, faces):
    """scaled normals n_f . dxidx at the face nodes of (element, face) rows."""
    e, f = faces[:, 0], faces[:, 1]
    Dx = dxidx_face_all[e, f]                      # [n, Nf, d(x), d(xi)]
    return np.einsum("nk,nipk->nip", sbp.normals[f], Dx)


def annulus(sbp: SBPOperator, nr: int, ntheta: int, r_in=1.0, r_out=3.0,
            bc=BC_VORTEX, bc_of_tag=None) -> Mesh:
    """Quarter annulus r in [r_in, r_out], theta in [0, pi/2] on nr x ntheta
    (r, theta) quads, each split along the diagonal from (r_i, theta_j) to
    (r_{i+1}, theta_{j+1}) into 2 straight-sided triangles (2 nr ntheta
    elements).  Boundary tags: 0 r = r_in, 1 r = r_out, 2 theta = 0,
    3 theta = pi/2; each tag gets `bc`, or bc_of_tag[tag] (a mapping or a
    callable) when given."""
    assert sbp.dim == 2
    vx, elverts, _ = annulus_grid(nr, ntheta, r_in, r_out)
    X = vx[elverts]                                  # [E, 3, 2]
    # affine map from the reference triangle: x = X0 + (X1-X0)(xi+1)/2 + (X2-X0)(eta+1)/2
    J = np.stack([(X[:, 1] - X[:, 0]) / 2, (X[:, 2] - X[:, 0]) / 2], axis=2)  # [E, p, k]
    dx, jac_e = _metrics_from_jacobian(J)
    Np = sbp.numnodes
    lam = _bary_tri(sbp.nodes)
    coords = np.einsum("nv,evp->enp", lam, X)
    dxidx = np.repeat(dx[:, None], Np, axis=1)
    jac = np.repeat(jac_e[:, None], Np, axis=1)

    Nf = sbp.numfacenodes
    fpts = np.stack([np.einsum("nv,evp->enp", _bary_tri(sbp.face_xi[f]), X) for f in range(3)], 1)

    def tags_of(be, bf):
        pts = fpts[be, bf]                          # [nb, Nf, 2]
        rr = np.linalg.norm(pts, axis=2)
        t = np.ones(len(be), dtype=np.int32)
        t[np.all(np.abs(pts[:, :, 0]) < 1e-12, axis=1)] = 3
        t[np.all(np.abs(pts[:, :, 1]) < 1e-12, axis=1)] = 2
        t[np.all(rr < r_in + 1e-9 * r_out, axis=1)] = 0
        return t

    iface, nbrperm, bfaces, offs, bct, tags = _connect(elverts, TRI_FACES, sbp, fpts, tags_of,
                                                       _bc_lookup(bc_of_tag, bc))
    dxf = np.repeat(np.repeat(dx[:, None, None], 3, axis=1), Nf, axis=2)   # [E, F, Nf, 2, 2]
    nrm_f = _face_normals(sbp, dxf, iface[:, [0, 2]])
    crd_f = fpts[iface[:, 0], iface[:, 2]]
    nrm_b = _face_normals(sbp, dxf, bfaces)
    crd_b = fpts[bfaces[:, 0], bfaces[:, 1]]
    return Mesh(2, sbp, coords, dxidx, jac, iface, nbrperm, nrm_f, crd_f, bfaces, offs,
                bct, crd_b, nrm_b, tags, name=f"annulus{nr}x{ntheta}",
                min_el_size=_min_node_spacing(coords))


def _min_node_spacing(coords):
    """smallest distance between two SBP nodes of one element, over the mesh
    (coords [E, Np, d]).  The reference takes mesh.min_el_size from
    PumiInterface, which is absent; for high-order SBP elements the node
    spacing is the length that bounds the explicit time step: on the
    512-triangle SBP-Omega p=2 vortex, RK4 at CFL 0.4 is stable with it and
    blows up within 5 steps with the element edge (3x longer)."""
    Np = coords.shape[1]
    best = np.inf
    for i in range(Np):
        for j in range(i):
            best = min(best, float(np.linalg.norm(coords[:, i] - coords[:, j], axis=1).min()))
    return best


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


def cube(sbp: SBPOperator, n: int, warp=0.05, seed=3, bc=BC_FREESTREAM, bc_of_tag=None) -> Mesh:
    """Unit cube of n^3 hexes, each split into 6 tetrahedra around the main
    diagonal (6 n^3 elements).  With ``warp`` != 0 every node is moved by
    x_i += warp * sin(pi x + phi) sin(pi y + phi) sin(pi z + phi) (same shift
    on each axis), phi drawn from ``seed``.  The warp is applied to the
    quadratic (P2) geometry nodes of each tetrahedron and the SBP node
    coordinates are interpolated from them, so neighbouring elements share
    their faces exactly and the metric terms, computed analytically from the
    P2 map, vary from node to node.  Boundary tags 0..5: x=0, x=1, y=0, y=1,
    z=0, z=1 of the unwarped cube; each tag gets `bc`, or bc_of_tag[tag]
    (a mapping or a callable) when given."""
    assert sbp.dim == 3
    phi = float(np.random.default_rng(seed).uniform(0.0, 2 * np.pi)) if warp else 0.0
    vx, elverts, _ = cube_grid(n, with_tags=False)
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

    fpts, fdx = [], []
    for f in range(4):
        xf, Jf = geom(allE, sbp.face_xi[f])
        fpts.append(xf)
        fdx.append(_metrics_from_jacobian(Jf)[0])
    fpts = np.stack(fpts, 1)                        # [E, 4, Nf, 3]
    fdx = np.stack(fdx, 1)                          # [E, 4, Nf, 3, 3]

    def tags_of(be, bf):
        # classify by the unwarped face (centroid of the element's vertices)
        fv = np.array(TET_FACES)[bf]                # [nb, 3]
        c = X[be[:, None], fv].mean(axis=1)         # [nb, 3]
        dist = np.minimum(np.abs(c), np.abs(1 - c))
        ax = np.argmin(dist, axis=1)
        hi = np.abs(1 - c[np.arange(len(be)), ax]) < np.abs(c[np.arange(len(be)), ax])
        return 2 * ax + hi.astype(np.int32)

    iface, nbrperm, bfaces, offs, bct, tags = _connect(elverts, TET_FACES, sbp, fpts, tags_of,
                                                       _bc_lookup(bc_of_tag, bc))
    nrm_f = _face_normals(sbp, fdx, iface[:, [0, 2]])
    crd_f = fpts[iface[:, 0], iface[:, 2]]
    nrm_b = _face_normals(sbp, fdx, bfaces)
    crd_b = fpts[bfaces[:, 0], bfaces[:, 1]]
    return Mesh(3, sbp, coords, dxidx, jac, iface, nbrperm, nrm_f, crd_f, bfaces, offs,
                bct, crd_b, nrm_b, tags, name=f"cube{n}",
                min_el_size=_min_node_spacing(coords))


# ---------------------------------------------------------------- any simplex mesh

def _bc_lookup(bc_of_tag, bc):
    if bc_of_tag is None:
        return lambda t: bc
    if callable(bc_of_tag):
        return bc_of_tag

    def look(t):
        if t not in bc_of_tag:
            raise ValueError(f"mesh: no boundary condition for boundary tag {t}")
        return bc_of_tag[t]
    return look


def from_elements(sbp: SBPOperator, vertices, elements, boundary_tags, bc_of_tag=None,
                  bc=BC_FREESTREAM, default_tag=None, name="mesh") -> Mesh:
    """Mesh of straight-sided simplices from a neutral description: vertex
    coordinates [nv, d] (a third column of zeros is accepted in 2-D),
    elements [E, d+1] (0-based vertex ids, either orientation; negatively
    oriented ones are reordered), and the tag of every boundary face as a
    mapping {sorted tuple of its vertex ids: tag}.  Boundary faces missing
    from the mapping get `default_tag`, or raise when it is None.  Each tag
    is one boundary-condition group (the reference's BC1..BCn over
    geometric edges); its condition is bc_of_tag[tag] (a mapping or a
    callable), or `bc` for every tag.  This is the role PUMI's mesh reader
    plays for the reference (PumiInterface.jl, not vendored); the node
    placement, metrics and face matching are those of the structured
    generators, so a structured mesh described this way gives the same
    arrays."""
    d = sbp.dim
    vx = np.asarray(vertices, dtype=np.float64)
    if vx.ndim != 2 or vx.shape[1] < d:
        raise ValueError(f"mesh: vertices must be [nv, {d}]")
    if vx.shape[1] > d:
        if np.abs(vx[:, d:]).max(initial=0.0) > 0.0:
            raise ValueError(f"mesh: vertices of a {d}-D mesh have non-zero extra coordinates")
        vx = vx[:, :d]
    vx = np.ascontiguousarray(vx)
    elverts = np.array(elements, dtype=np.int64)
    if elverts.ndim != 2 or elverts.shape[1] != d + 1 or len(elverts) == 0:
        raise ValueError(f"mesh: elements must be a non-empty [E, {d + 1}] array")
    if elverts.min() < 0 or elverts.max() >= len(vx):
        raise ValueError("mesh: element vertex id out of range")
    X = vx[elverts]
    J0 = np.stack([X[:, k + 1] - X[:, 0] for k in range(d)], axis=2)
    det0 = np.linalg.det(J0)
    # zero-volume elements (repeated or collinear/coplanar vertices) have no
    # metric terms: refuse them instead of dividing by zero later
    edge = np.linalg.norm(J0, axis=1).max(axis=1)
    flat = np.abs(det0) <= 64 * np.finfo(np.float64).eps * edge ** d
    if np.any(flat):
        raise ValueError(f"mesh: {int(np.count_nonzero(flat))} elements are degenerate "
                         f"(zero volume; first: element {int(np.nonzero(flat)[0][0])})")
    neg = det0 < 0
    elverts[neg, d - 1], elverts[neg, d] = elverts[neg, d].copy(), elverts[neg, d - 1].copy()
    X = vx[elverts]                                  # [E, d+1, d]
    # affine map from the reference simplex: x = X0 + sum_k (X_{k+1} - X0)(xi_k + 1)/2
    J = np.stack([(X[:, k + 1] - X[:, 0]) / 2 for k in range(d)], axis=2)   # [E, p, k]
    dx, jac_e = _metrics_from_jacobian(J)
    Np, Nf = sbp.numnodes, sbp.numfacenodes
    bary = _bary_tri if d == 2 else _bary_tet
    faces_local = TRI_FACES if d == 2 else TET_FACES
    F = len(faces_local)
    coords = np.einsum("nv,evp->enp", bary(sbp.nodes), X)
    dxidx = np.repeat(dx[:, None], Np, axis=1)
    jac = np.repeat(jac_e[:, None], Np, axis=1)
    fpts = np.stack([np.einsum("nv,evp->enp", bary(sbp.face_xi[f]), X) for f in range(F)], 1)
    tagmap = {tuple(sorted(int(v) for v in k)): int(t) for k, t in dict(boundary_tags).items()}
    fl = np.array(faces_local)

    def tags_of(be, bf):
        keys = np.sort(elverts[be[:, None], fl[bf]], axis=1)
        out = np.empty(len(be), dtype=np.int32)
        missing = 0
        for n, k in enumerate(map(tuple, keys.tolist())):
            t = tagmap.get(k, default_tag)
            if t is None:
                missing += 1
                t = -1
            out[n] = t
        if missing:
            raise ValueError(f"mesh: {missing} boundary faces have no tag (and no default_tag)")
        return out

    iface, nbrperm, bfaces, offs, bct, tags = _connect(elverts, faces_local, sbp, fpts, tags_of,
                                                       _bc_lookup(bc_of_tag, bc))
    dxf = np.repeat(np.repeat(dx[:, None, None], F, axis=1), Nf, axis=2)   # [E, F, Nf, d, d]
    nrm_f = _face_normals(sbp, dxf, iface[:, [0, 2]])
    crd_f = fpts[iface[:, 0], iface[:, 2]]
    nrm_b = _face_normals(sbp, dxf, bfaces)
    crd_b = fpts[bfaces[:, 0], bfaces[:, 1]]
    return Mesh(d, sbp, coords, dxidx, jac, iface, nbrperm, nrm_f, crd_f, bfaces, offs,
                bct, crd_b, nrm_b, tags, name=name, min_el_size=_min_node_spacing(coords))


def annulus_grid(nr, ntheta, r_in=1.0, r_out=3.0):
    """the vertices [nv, 2] and triangles [E, 3] of ``annulus`` and the tag
    of each boundary edge ({sorted vertex pair: tag}, tags as in annulus),
    as a neutral description for ``from_elements``."""
    r = np.linspace(r_in, r_out, nr + 1)
    th = np.linspace(0.0, np.pi / 2, ntheta + 1)
    R, T = np.meshgrid(r, th, indexing="ij")
    vx = np.stack([(R * np.cos(T)).ravel(), (R * np.sin(T)).ravel()], axis=1)
    vid = lambda i, j: i * (ntheta + 1) + j  # noqa: E731
    els = []
    for i in range(nr):
        for j in range(ntheta):
            a, b, c, dd = vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)
            els.append((a, b, c))
            els.append((a, c, dd))
    tags = {}
    for j in range(ntheta):
        tags[tuple(sorted((vid(0, j), vid(0, j + 1))))] = 0
        tags[tuple(sorted((vid(nr, j), vid(nr, j + 1))))] = 1
    for i in range(nr):
        tags[tuple(sorted((vid(i, 0), vid(i + 1, 0))))] = 2
        tags[tuple(sorted((vid(i, ntheta), vid(i + 1, ntheta))))] = 3
    return vx, np.array(els, dtype=np.int64), tags


def cube_grid(n, with_tags=True):
    """the vertices [nv, 3] and tetrahedra [6 n^3, 4] of ``cube`` before its
    warp (the Kuhn split of each hex: the 6 monotone vertex paths from its
    corner 000 to 111; orientation as generated) and, with `with_tags`, the
    tag of every boundary triangle ({sorted vertex triple: tag}, tags as in
    cube; else None)."""
    g = np.linspace(0.0, 1.0, n + 1)
    Xg, Yg, Zg = np.meshgrid(g, g, g, indexing="ij")
    vx = np.stack([Xg.ravel(), Yg.ravel(), Zg.ravel()], axis=1)
    vid = lambda i, j, k: (i * (n + 1) + j) * (n + 1) + k  # noqa: E731
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
    if not with_tags:
        return vx, elverts, None
    tris = elverts[:, np.array(TET_FACES)].reshape(-1, 3)          # every local face
    P = vx[tris]                                                     # [F, 3 vertices, 3]
    tags = {}
    for ax in range(3):
        for side in (0, 1):
            on = np.all(P[:, :, ax] == float(side), axis=1)
            for tri in np.sort(tris[on], axis=1).tolist():
                tags[tuple(tri)] = 2 * ax + side
    return vx, elverts, tags


# ---------------------------------------------------------------- on-disk form
# A neutral description of a Mesh: every array the hot path reads (the fields
# of the reference's AbstractMesh that evalResidual / evalJacobian touch,
# docs/src/interfaces.md), the boundary tags and the operator's identity
# (dimension, family, degree; the operator is rebuilt, not stored).  The
# reference reads PUMI .smb files, which need PUMI; this is the stand-in for
# bringing a mesh from another tool.
_MESH_ARRAYS = ("coords", "dxidx", "jac", "interfaces", "nbrperm", "nrm_face", "coords_face",
                "bndryfaces", "bndry_offsets", "bc_types", "coords_bndry", "nrm_bndry", "bndry_tag")


def save_mesh(path, mesh: Mesh):
    """write `mesh` to an .npz file (see load_mesh)."""
    np.savez_compressed(path, **{k: getattr(mesh, k) for k in _MESH_ARRAYS},
                        dim=mesh.dim, sbp_family=mesh.sbp.family, sbp_p=mesh.sbp.p,
                        name=mesh.name, min_el_size=mesh.min_el_size)


def load_mesh(path) -> Mesh:
    """read a mesh written by save_mesh; the SBP operator is rebuilt from its
    family and degree, and the arrays are checked against its node counts."""
    from . import sbp as _sbp
    with np.load(path, allow_pickle=False) as z:
        dim = int(z["dim"])
        op = _sbp.get_operator(dim, str(z["sbp_family"]), int(z["sbp_p"]))
        arrs = {k: np.array(z[k]) for k in _MESH_ARRAYS}
        name, h = str(z["name"]), float(z["min_el_size"])
    E, Np = arrs["coords"].shape[:2]
    if Np != op.numnodes or arrs["coords"].shape[2] != dim:
        raise ValueError(f"coords {arrs['coords'].shape} do not match the {op.family} p={op.p} operator")
    if arrs["dxidx"].shape != (E, Np, dim, dim) or arrs["jac"].shape != (E, Np):
        raise ValueError("metric arrays do not match the element and node counts")
    I = arrs["interfaces"].shape[0]
    if arrs["nrm_face"].shape != (I, op.numfacenodes, dim):
        raise ValueError("interface normals do not match the interfaces and face nodes")
    return Mesh(dim, op, arrs["coords"], arrs["dxidx"], arrs["jac"], arrs["interfaces"],
                arrs["nbrperm"], arrs["nrm_face"], arrs["coords_face"], arrs["bndryfaces"],
                arrs["bndry_offsets"], arrs["bc_types"], arrs["coords_bndry"], arrs["nrm_bndry"],
                arrs["bndry_tag"], name=name, min_el_size=h)
