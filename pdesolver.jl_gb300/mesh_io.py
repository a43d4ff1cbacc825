"""Mesh files from other tools: Gmsh's MSH 2.2 ASCII format.

The reference reads PUMI ``.smb`` meshes (PumiInterface.jl, not vendored);
those need PUMI.  A PUMI mesh of the reference's cases is typically made by
Gmsh first, so a Gmsh file is the neutral description this package reads:
straight-sided triangles (2-D) or tetrahedra (3-D) and the physical tags of
their boundary edges or triangles, which become the boundary-condition
groups (the reference's ``BC1 = [geometric edges]`` options).

Only what the Euler path needs is read: nodes, the elements of the mesh
dimension, and the boundary elements one dimension lower with their
physical tag; other element types (points, higher-order or mixed elements)
are refused or, for points and lower-dimensional elements without a
boundary role, ignored.  The format is written with ``write_gmsh`` in the
same subset (also used to export this package's generated meshes).
"""
from __future__ import annotations

import numpy as np

from . import mesh as _mesh

# MSH element type ids: 1 = 2-node line, 2 = 3-node triangle, 4 = 4-node
# tetrahedron, 15 = 1-node point
_LINE, _TRI, _TET, _POINT = 1, 2, 4, 15
_NODES_OF = {_LINE: 2, _TRI: 3, _TET: 4, _POINT: 1}
_DIM_OF = {_POINT: 0, _LINE: 1, _TRI: 2, _TET: 3}


def _sections(path):
    with open(path) as f:
        lines = [ln.strip() for ln in f]
    secs, i = {}, 0
    while i < len(lines):
        ln = lines[i]
        if ln.startswith("$") and not ln.startswith("$End"):
            name = ln[1:]
            j = i + 1
            while j < len(lines) and lines[j] != f"$End{name}":
                j += 1
            if j == len(lines):
                raise ValueError(f"gmsh: section ${name} is not closed")
            secs[name] = lines[i + 1:j]
            i = j + 1
        else:
            i += 1
    return secs


def read_gmsh_raw(path):
    """(vertices [nv, 3], elements by dimension {dim: (type, [n, k] 0-based
    vertex ids, physical tags [n])}, physical names {(dim, tag): name}) of a
    MSH 2.2 ASCII file."""
    secs = _sections(path)
    fmt = secs.get("MeshFormat")
    if not fmt:
        raise ValueError("gmsh: no $MeshFormat section")
    version, ftype = fmt[0].split()[:2]
    if not version.startswith("2.") or ftype != "0":
        raise ValueError(f"gmsh: only MSH 2.x ASCII is read (file: version {version}, type {ftype})")
    if "Nodes" not in secs or "Elements" not in secs:
        raise ValueError("gmsh: $Nodes and $Elements are required")
    nodes = secs["Nodes"]
    nn = int(nodes[0])
    ids = np.empty(nn, dtype=np.int64)
    vx = np.empty((nn, 3))
    for n, ln in enumerate(nodes[1:nn + 1]):
        tok = ln.split()
        ids[n] = int(tok[0])
        vx[n] = [float(t) for t in tok[1:4]]
    index = {int(v): n for n, v in enumerate(ids)}
    if len(index) != nn:
        raise ValueError("gmsh: repeated node ids")
    els = secs["Elements"]
    ne = int(els[0])
    by_type = {}
    for ln in els[1:ne + 1]:
        tok = [int(t) for t in ln.split()]
        etype, ntags = tok[1], tok[2]
        if etype not in _NODES_OF:
            raise ValueError(f"gmsh: element type {etype} is not supported "
                             "(straight-sided lines, triangles, tetrahedra and points only)")
        tags = tok[3:3 + ntags]
        verts = tok[3 + ntags:]
        if len(verts) != _NODES_OF[etype]:
            raise ValueError(f"gmsh: element of type {etype} with {len(verts)} nodes")
        try:
            vv = [index[v] for v in verts]
        except KeyError as e:
            raise ValueError(f"gmsh: element refers to unknown node {e.args[0]}") from None
        by_type.setdefault(etype, ([], []))
        by_type[etype][0].append(vv)
        by_type[etype][1].append(tags[0] if tags else 0)
    elements = {_DIM_OF[t]: (t, np.array(v, dtype=np.int64), np.array(p, dtype=np.int64))
                for t, (v, p) in by_type.items()}
    names = {}
    for ln in secs.get("PhysicalNames", [])[1:]:
        tok = ln.split(maxsplit=2)
        names[(int(tok[0]), int(tok[1]))] = tok[2].strip().strip('"')
    return vx, elements, names


def read_gmsh(path, sbp, bc_of_tag=None, bc=_mesh.BC_FREESTREAM, default_tag=None, name=None):
    """Mesh (see mesh.from_elements) of a MSH 2.2 ASCII file for operator
    `sbp`: the elements of dimension sbp.dim, boundary tags from the
    physical tags of the elements one dimension lower.  bc_of_tag maps a
    physical tag (int) or physical name (str) to a boundary condition
    (mesh.BC_VORTEX / mesh.BC_FREESTREAM); without it every boundary gets
    `bc`."""
    d = sbp.dim
    vx, elements, names = read_gmsh_raw(path)
    if d not in elements:
        raise ValueError(f"gmsh: the file has no {d}-D elements")
    _, el, _ = elements[d]
    tags = {}
    if d - 1 in elements:
        _, bel, btag = elements[d - 1]
        for vv, t in zip(bel, btag):
            tags[tuple(sorted(int(v) for v in vv))] = int(t)
    look = None
    if bc_of_tag is not None:
        by_name = {nm: t for (dd, t), nm in names.items() if dd == d - 1}

        def look(t):
            for key in (t, next((nm for nm, tt in by_name.items() if tt == t), None)):
                if key is not None and key in bc_of_tag:
                    return bc_of_tag[key]
            raise ValueError(f"gmsh: no boundary condition for physical tag {t}")
    # elements of the mesh dimension only; unused vertices are harmless
    return _mesh.from_elements(sbp, vx, el, tags, bc_of_tag=look, bc=bc, default_tag=default_tag,
                               name=name or str(path).rsplit("/", 1)[-1])


def write_gmsh(path, vertices, elements, boundary_tags, names=None):
    """A MSH 2.2 ASCII file of straight-sided triangles or tetrahedra
    (elements [E, d+1], 0-based), with every tagged boundary face
    ({sorted vertex ids: physical tag}) as a line or triangle element, and
    optional physical names {tag: name} of the boundary groups."""
    vx = np.asarray(vertices, dtype=np.float64)
    el = np.asarray(elements, dtype=np.int64)
    d = el.shape[1] - 1
    if d not in (2, 3):
        raise ValueError("write_gmsh: triangles or tetrahedra only")
    btype, etype = (_LINE, _TRI) if d == 2 else (_TRI, _TET)
    out = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat"]
    if names:
        out += ["$PhysicalNames", str(len(names))]
        out += [f'{d - 1} {int(t)} "{nm}"' for t, nm in sorted(names.items())]
        out += ["$EndPhysicalNames"]
    out += ["$Nodes", str(len(vx))]
    for n, x in enumerate(vx):
        xyz = list(x) + [0.0] * (3 - len(x))
        out.append(f"{n + 1} " + " ".join(repr(float(c)) for c in xyz))
    out += ["$EndNodes", "$Elements", str(len(boundary_tags) + len(el))]
    k = 1
    for key, t in sorted(boundary_tags.items()):
        out.append(f"{k} {btype} 2 {int(t)} {int(t)} " + " ".join(str(int(v) + 1) for v in key))
        k += 1
    for vv in el:
        out.append(f"{k} {etype} 2 0 1 " + " ".join(str(int(v) + 1) for v in vv))
        k += 1
    out += ["$EndElements"]
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
