"""SBP operator and mesh properties (the pins available for the missing
SummationByParts.jl / PUMI dependencies).  CPU only."""
import numpy as np
import pytest

from pdesolver_gb300 import cubature_tables, mesh, sbp

OPS = [(2, "omega", p) for p in (1, 2, 3, 4)] + [(2, "gamma", p) for p in (1, 2, 3, 4)] + \
      [(3, "diage", p) for p in (1, 2, 3)]


@pytest.mark.parametrize("dim,fam,p", OPS)
def test_sbp_properties(dim, fam, p):
    """Q + Q^T = E, H = diag(w) > 0, D = H^-1 Q exact for degree p,
    Q 1 = 0 (SBP definition; the reference pins operators only through
    these properties)."""
    op = sbp.get_operator(dim, fam, p)
    assert np.all(op.w > 0)
    V, dV = sbp.vandermonde(op.nodes, p)
    for k in range(dim):
        np.testing.assert_allclose(op.Q[k] + op.Q[k].T, op.E[k], atol=1e-13)
        np.testing.assert_allclose(op.D[k] @ V, dV[k], atol=5e-12)
        np.testing.assert_allclose(op.Q[k].sum(axis=1), 0.0, atol=1e-13)
        np.testing.assert_allclose(op.S[k], -op.S[k].T, atol=1e-15)
    # total volume of the reference element
    np.testing.assert_allclose(op.w.sum(), 2.0 if dim == 2 else 4.0 / 3.0, rtol=1e-14)


def test_node_counts_match_reference_dofcount():
    """src/dofcount.jl:21-88: tri Omega 3/6/10/15, tri Gamma 3/7/12/18."""
    assert [cubature_tables.TRI[("omega", p)]["n"] for p in (1, 2, 3, 4)] == [3, 6, 10, 15]
    assert [cubature_tables.TRI[("gamma", p)]["n"] for p in (1, 2, 3, 4)] == [3, 7, 12, 18]


@pytest.mark.parametrize("fam,p", [("omega", 1), ("omega", 2), ("gamma", 3), ("gamma", 4)])
def test_face_interp_exact(fam, p):
    """face interpolation is exact for degree-p polynomials on every face."""
    op = sbp.get_operator(2, fam, p)
    V, _ = sbp.vandermonde(op.nodes, p)
    for f in range(3):
        Vf, _ = sbp.vandermonde(op.face_xi[f], p)
        np.testing.assert_allclose(op.interp[f] @ V[op.perm[f]], Vf, atol=1e-12)


def test_annulus_counts():
    """mesh counts of the 16x16 and 64x64 annulus (E, I, B)."""
    op = sbp.get_operator(2, "omega", 2)
    m = mesh.annulus(op, 16, 16)
    assert (m.numEl, m.numInterfaces, m.numBoundaryFaces) == (512, 736, 64)
    assert np.all(m.jac > 0)
    # area of the polygonal annulus, and closed boundary: sum of normals = 0
    assert abs(m.M.sum() - np.pi / 4 * 8) < 2e-2
    tot = (op.wface[None, :, None] * m.nrm_bndry).sum(axis=(0, 1))
    np.testing.assert_allclose(tot, 0.0, atol=1e-13)


def test_cube_counts_and_watertight():
    op = sbp.get_operator(3, "diage", 2)
    m = mesh.cube(op, 3, warp=0.05, seed=3)
    n = 3
    assert m.numEl == 6 * n ** 3 and m.numBoundaryFaces == 12 * n ** 2
    assert m.numInterfaces == (4 * m.numEl - m.numBoundaryFaces) // 2
    tot = (op.wface[None, :, None] * m.nrm_bndry).sum(axis=(0, 1))
    np.testing.assert_allclose(tot, 0.0, atol=1e-13)
    # normals of matching interface nodes agree from both sides
    for (eL, eR, fL, fR, o) in m.interfaces[:50]:
        xl = m.coords_face
    assert np.all(m.jac > 0)


def test_nbrperm_matches_geometry():
    op = sbp.get_operator(2, "gamma", 3)
    m = mesh.annulus(op, 4, 4)
    for n, (eL, eR, fL, fR, o) in enumerate(m.interfaces):
        for i in range(op.numfacenodes):
            iR = m.nbrperm[o, i]
            xl = op.interp[fL, i] @ m.coords[eL, op.perm[fL]]
            xr = op.interp[fR, iR] @ m.coords[eR, op.perm[fR]]
            np.testing.assert_allclose(xl, xr, atol=1e-13)


@pytest.mark.parametrize("which", ["annulus", "cube"])
def test_mesh_file_round_trip(tmp_path, oracle, which):
    """save_mesh / load_mesh (the neutral on-disk mesh form): the arrays come
    back bit for bit, the operator is rebuilt, and the oracle residual on the
    loaded mesh equals the original's."""
    import ctypes as C
    from pdesolver_gb300 import abi, eulergpu, problems
    if which == "annulus":
        ms, opts, q = problems.config1(n=4, p=2)
    else:
        ms, opts, q = problems.config3(n=2, p=2)
    path = tmp_path / "mesh.npz"
    mesh.save_mesh(path, ms)
    ld = mesh.load_mesh(path)
    for k in mesh._MESH_ARRAYS:
        assert np.array_equal(getattr(ld, k), getattr(ms, k)), k
    assert ld.sbp.numnodes == ms.sbp.numnodes and np.array_equal(ld.sbp.Q, ms.sbp.Q)
    assert ld.min_el_size == ms.min_el_size
    P = eulergpu.params_from_opts(opts)
    r = [np.zeros_like(q), np.zeros_like(q)]
    for m_, out in zip((ms, ld), r):
        d = abi.MeshDesc(m_)
        assert oracle.oracle_eval_residual(C.byref(d.desc), C.byref(P), abi.dptr(q), abi.dptr(out)) == 0
    assert np.array_equal(r[0], r[1])
