"""Neutral mesh input (the role of PUMI's reader for the reference): any
straight-sided simplex mesh from vertices, elements and boundary tags
(mesh.from_elements), and Gmsh MSH 2.2 ASCII files (mesh_io).  CPU only."""
import numpy as np
import pytest

from conftest import oracle_residual
from pdesolver_gb300 import abi, mesh, mesh_io, problems, sbp


def _same(a, b, atol=0.0):
    for k in mesh._MESH_ARRAYS:
        x, y = getattr(a, k), getattr(b, k)
        assert x.shape == y.shape, k
        if x.dtype.kind in "iu" or atol == 0.0:
            assert np.array_equal(x, y), k
        else:
            np.testing.assert_allclose(x, y, rtol=1e-13, atol=atol, err_msg=k)


@pytest.mark.parametrize("fam,p", [("omega", 2), ("gamma", 3)])
def test_gmsh_annulus_round_trip_is_bit_exact(tmp_path, fam, p):
    op = sbp.get_operator(2, fam, p)
    ref = mesh.annulus(op, 4, 6)
    vx, el, tags = mesh.annulus_grid(4, 6)
    path = tmp_path / "annulus.msh"
    mesh_io.write_gmsh(path, vx, el, tags)
    got = mesh_io.read_gmsh(path, op, bc=mesh.BC_VORTEX)
    _same(got, ref)
    assert got.min_el_size == ref.min_el_size


@pytest.mark.parametrize("p", [1, 2])
def test_gmsh_cube_round_trip(tmp_path, p):
    op = sbp.get_operator(3, "diage", p)
    ref = mesh.cube(op, 2, warp=0.0)
    vx, el, tags = mesh.cube_grid(2)
    path = tmp_path / "cube.msh"
    mesh_io.write_gmsh(path, vx, el, tags)
    got = mesh_io.read_gmsh(path, op)
    # the generator maps through quadratic geometry nodes, the reader affinely
    _same(got, ref, atol=1e-12)
    assert got.min_el_size == pytest.approx(ref.min_el_size, rel=1e-14)


def test_boundary_conditions_by_physical_name(tmp_path, oracle):
    """physical names select the condition of each boundary group; the
    oracle residual on the file's mesh equals the one on the generated mesh."""
    op = sbp.get_operator(2, "omega", 2)
    vx, el, tags = mesh.annulus_grid(3, 3)
    path = tmp_path / "named.msh"
    mesh_io.write_gmsh(path, vx, el, tags, names={0: "inner", 1: "outer", 2: "bottom", 3: "left"})
    got = mesh_io.read_gmsh(path, op, bc_of_tag={"inner": mesh.BC_VORTEX, "outer": mesh.BC_VORTEX,
                                                 "bottom": mesh.BC_FREESTREAM, 3: mesh.BC_FREESTREAM})
    assert got.bc_types.tolist() == [mesh.BC_VORTEX, mesh.BC_VORTEX, mesh.BC_FREESTREAM,
                                     mesh.BC_FREESTREAM]
    ref = mesh.annulus(op, 3, 3)
    ref.bc_types = got.bc_types.copy()
    P = abi.EgParams.make(Ma=0.5, M_in=0.5)
    q = np.ascontiguousarray(problems.vortex_state(ref.coords, M_in=0.5) * 1.001)
    r1 = oracle_residual(oracle, abi.MeshDesc(got), P, q)
    r2 = oracle_residual(oracle, abi.MeshDesc(ref), P, q)
    assert np.array_equal(r1, r2)
    with pytest.raises(ValueError):
        mesh_io.read_gmsh(path, op, bc_of_tag={"inner": mesh.BC_VORTEX})


def test_element_orientation_is_normalised(oracle):
    """elements given clockwise are reordered; with a symmetric operator the
    residual is the same at every node (nodes permuted within elements)."""
    op = sbp.get_operator(2, "gamma", 2)
    vx, el, tags = mesh.annulus_grid(3, 4)
    flipped = el[:, [0, 2, 1]]
    a = mesh.from_elements(op, vx, el, tags, bc=mesh.BC_VORTEX)
    b = mesh.from_elements(op, vx, flipped, tags, bc=mesh.BC_VORTEX)
    assert (b.jac > 0).all()
    P = abi.EgParams.make(Ma=0.5, M_in=0.5)
    ra, rb = [], []
    for ms, out in ((a, ra), (b, rb)):
        q = problems.vortex_state(ms.coords, M_in=0.5)
        q = np.ascontiguousarray(q * (1 + 1e-3 * np.sin(7 * ms.coords[..., :1])))
        out.append(oracle_residual(oracle, abi.MeshDesc(ms), P, q))
    for e in range(a.numEl):
        ia = np.lexsort(a.coords[e].T)
        ib = np.lexsort(b.coords[e].T)
        np.testing.assert_allclose(a.coords[e, ia], b.coords[e, ib], atol=1e-14)
        np.testing.assert_allclose(ra[0][e, ia], rb[0][e, ib], atol=1e-12)


def test_reader_refusals(tmp_path):
    op = sbp.get_operator(2, "omega", 1)
    vx, el, tags = mesh.annulus_grid(2, 2)
    some = dict(list(tags.items())[:-1])               # one boundary edge untagged
    with pytest.raises(ValueError):
        mesh.from_elements(op, vx, el, some)
    m = mesh.from_elements(op, vx, el, some, default_tag=7)
    assert 7 in m.bndry_tag.tolist()
    with pytest.raises(ValueError):
        mesh.from_elements(op, vx, el[:, :2], tags)    # not triangles
    with pytest.raises(ValueError):
        mesh.from_elements(op, vx, el + len(vx), tags)  # vertex ids out of range
    with pytest.raises(ValueError):
        mesh.from_elements(op, np.c_[vx, np.ones(len(vx))], el, tags)   # not planar
    p4 = tmp_path / "v4.msh"
    p4.write_text("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n")
    with pytest.raises(ValueError, match="2.x ASCII"):
        mesh_io.read_gmsh(p4, op)
    p9 = tmp_path / "curved.msh"
    p9.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n1\n1 0 0 0\n$EndNodes\n"
                  "$Elements\n1\n1 9 2 0 1 1 1 1 1 1 1\n$EndElements\n")
    with pytest.raises(ValueError, match="not supported"):
        mesh_io.read_gmsh(p9, op)
    p3 = tmp_path / "only_lines.msh"
    mesh_io.write_gmsh(p3, vx, el, tags)
    with pytest.raises(ValueError, match="3-D"):
        mesh_io.read_gmsh(p3, sbp.get_operator(3, "diage", 1))


def test_degenerate_and_non_manifold_meshes_are_refused(tmp_path):
    """a flat triangle (zero volume, e.g. a bad Gmsh file) and a face shared
    by three elements are refused with a message, not turned into a
    non-finite residual or a doubly integrated interface."""
    op = sbp.get_operator(2, "omega", 1)
    vx, el, tags = mesh.annulus_grid(2, 2)
    flat = np.array([[0, 1, 1]] + el[1:].tolist())     # repeated vertex
    with pytest.raises(ValueError, match="degenerate"):
        mesh.from_elements(op, vx, flat, tags, default_tag=0)
    vx2 = np.r_[vx, [[(vx[el[0, 0]] + vx[el[0, 1]])[0] / 2, (vx[el[0, 0]] + vx[el[0, 1]])[1] / 2]]]
    collinear = np.r_[el, [[el[0, 0], el[0, 1], len(vx)]]]   # vertices on one line
    with pytest.raises(ValueError, match="degenerate"):
        mesh.from_elements(op, vx2, collinear, tags, default_tag=0)
    path = tmp_path / "flat.msh"
    mesh_io.write_gmsh(path, vx2, collinear, tags)
    with pytest.raises(ValueError, match="degenerate"):
        mesh_io.read_gmsh(path, op)
    # a third element on an interior edge (one two elements share), on a new vertex
    edges = {}
    for e in el.tolist():
        for a, b in ((0, 1), (1, 2), (0, 2)):
            k = tuple(sorted((e[a], e[b])))
            edges[k] = edges.get(k, 0) + 1
    inner = next(k for k, c in edges.items() if c == 2)
    vx3 = np.r_[vx, [[5.0, 5.0]]]
    third = np.r_[el, [[inner[0], inner[1], len(vx)]]]
    with pytest.raises(ValueError, match="more than two elements"):
        mesh.from_elements(op, vx3, third, tags, default_tag=0)


@pytest.mark.parametrize("fam,p", [("omega", 2), ("gamma", 3)])
def test_distorted_mesh_preserves_free_stream(oracle, fam, p):
    """a mesh of irregular straight-sided triangles (the annulus grid with its
    interior vertices moved at random) built by from_elements keeps a uniform
    flow at round-off, in the weak form with Roe fluxes and in the split form
    with Ismail-Roe fluxes: its metrics, normals and face matching agree."""
    op = sbp.get_operator(2, fam, p)
    vx, el, tags = mesh.annulus_grid(6, 6)
    boundary = np.unique(np.array(list(tags.keys())).ravel())
    interior = np.setdiff1d(np.arange(len(vx)), boundary)
    rng = np.random.default_rng(17)
    vx = vx.copy()
    vx[interior] += rng.uniform(-0.08, 0.08, size=(len(interior), 2))
    ms = mesh.from_elements(op, vx, el, tags)
    assert (ms.jac > 0).all()
    desc = abi.MeshDesc(ms)
    for P in (abi.EgParams.make(Ma=0.5, aoa_deg=20.0),
              abi.EgParams.make(Ma=0.5, aoa_deg=20.0, face_flux=abi.EG_FLUX_IR, volume_integral_type=2)):
        q = problems.free_stream(2, ms.coords.shape[:2], Ma=0.5, aoa=20.0 * np.pi / 180)
        res = oracle_residual(oracle, desc, P, np.ascontiguousarray(q))
        assert np.abs(res).max() < 1e-12
