"""Generator for the symmetric cubature rules behind the SBP operators.

Run once (``python pdesolver.jl_gb300/cubature_gen.py``) to regenerate
``cubature_tables.py``; the library only reads the committed tables.

The reference obtains its cubature rules from SummationByParts.jl
(``getTriCubatureOmega``, ``getTriCubatureGamma``, ``getTetCubatureDiagE``;
called from src/solver/common.jl:276-390), a dependency that is not vendored.
These rules are constructed here from the published theory instead:
symmetric orbits in barycentric coordinates whose free parameters and weights
solve the moment equations exactly (Hicken, Del Rey Fernandez & Zingg,
"Multidimensional summation-by-parts operators", SISC 2016, sections 4-5).

Node counts follow src/dofcount.jl:21-88 of the reference (tri Omega p=1..4:
3, 6, 10, 15; tri Gamma p=1..4: 3, 7, 12, 18).  The tet diagonal-E node sets
(p=1..3: 6, 23 and 45 nodes) are this project's own (the reference does not
tabulate them).

Reference elements: triangle (-1,-1), (1,-1), (-1,1); tetrahedron
(-1,-1,-1), (1,-1,-1), (-1,1,-1), (-1,-1,1).
"""
from __future__ import annotations

import itertools
import math
import sys
from fractions import Fraction

import numpy as np
from scipy.optimize import least_squares

# ---------------------------------------------------------------------------
# exact moments of monomials on the reference simplices
# ---------------------------------------------------------------------------


def _binom_expand(i):
    """coefficients of (-1 + 2u)^i in powers of u."""
    return [Fraction(math.comb(i, k)) * (2 ** k) * ((-1) ** (i - k)) for k in range(i + 1)]


def tri_moment(i, j):
    """exact integral of x^i y^j over the reference triangle."""
    ci, cj = _binom_expand(i), _binom_expand(j)
    tot = Fraction(0)
    for a, ca in enumerate(ci):
        for b, cb in enumerate(cj):
            tot += ca * cb * Fraction(math.factorial(a) * math.factorial(b),
                                      math.factorial(a + b + 2))
    return tot * 4


def tet_moment(i, j, k):
    """exact integral of x^i y^j z^k over the reference tetrahedron."""
    ci, cj, ck = _binom_expand(i), _binom_expand(j), _binom_expand(k)
    tot = Fraction(0)
    for a, ca in enumerate(ci):
        for b, cb in enumerate(cj):
            for c, cc in enumerate(ck):
                tot += ca * cb * cc * Fraction(
                    math.factorial(a) * math.factorial(b) * math.factorial(c),
                    math.factorial(a + b + c + 3))
    return tot * 8


TRI_VERTS = np.array([[-1.0, -1.0], [1.0, -1.0], [-1.0, 1.0]])
TET_VERTS = np.array([[-1.0, -1.0, -1.0], [1.0, -1.0, -1.0], [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]])


def _unique_perms(bary):
    out = []
    for p in itertools.permutations(bary):
        if not any(np.allclose(p, q, atol=1e-14) for q in out):
            out.append(p)
    return out


# ---------------------------------------------------------------------------
# orbit descriptions.  Each orbit is (kind, nfree) where the free parameters
# are positions; fixed orbits have nfree = 0.
# ---------------------------------------------------------------------------

def tri_orbit(kind, params):
    if kind == "S3":
        b = [(1 / 3, 1 / 3, 1 / 3)]
    elif kind == "vert":
        b = _unique_perms((0.0, 0.0, 1.0))
    elif kind == "mid":
        b = _unique_perms((0.5, 0.5, 0.0))
    elif kind == "S21":
        a = params[0]
        b = _unique_perms((a, a, 1 - 2 * a))
    elif kind == "edge":       # two points per edge, symmetric about the midpoint
        a = params[0]
        b = _unique_perms((a, 1 - a, 0.0))
    elif kind == "S111":
        a, c = params
        b = _unique_perms((a, c, 1 - a - c))
    else:
        raise ValueError(kind)
    return np.array(b)


def tet_orbit(kind, params):
    if kind == "S4":
        b = [(0.25,) * 4]
    elif kind == "vert":
        b = _unique_perms((0.0, 0.0, 0.0, 1.0))
    elif kind == "mid":
        b = _unique_perms((0.5, 0.5, 0.0, 0.0))
    elif kind == "facecen":
        b = _unique_perms((1 / 3, 1 / 3, 1 / 3, 0.0))
    elif kind == "S31":
        a = params[0]
        b = _unique_perms((a, a, a, 1 - 3 * a))
    elif kind == "face21":    # S21 orbit of the face triangle, on all 4 faces
        a = params[0]
        b = _unique_perms((a, a, 1 - 2 * a, 0.0))
    elif kind == "edge2":     # two points per edge
        a = params[0]
        b = _unique_perms((a, 1 - a, 0.0, 0.0))
    else:
        raise ValueError(kind)
    return np.array(b)


NFREE = {"S3": 0, "S4": 0, "vert": 0, "mid": 0, "facecen": 0, "S21": 1,
         "edge": 1, "S111": 2, "S31": 1, "face21": 1, "edge2": 1}


def _points(dim, orbits, x):
    """expand the free parameters x into cartesian points and orbit sizes."""
    pos, k, sizes = [], 0, []
    verts = TRI_VERTS if dim == 2 else TET_VERTS
    orb = tri_orbit if dim == 2 else tet_orbit
    for kind in orbits:
        nf = NFREE[kind]
        b = orb(kind, x[k:k + nf])
        k += nf
        pos.append(b @ verts)
        sizes.append(len(b))
    return pos, sizes, k


def _monomials(dim, q):
    if dim == 2:
        return [(i, d - i) for d in range(q + 1) for i in range(d + 1)]
    return [(i, j, d - i - j) for d in range(q + 1) for i in range(d + 1) for j in range(d - i + 1)]


def _exact(dim, q):
    mono = _monomials(dim, q)
    f = tri_moment if dim == 2 else tet_moment
    return mono, np.array([float(f(*m)) for m in mono])


def _residual(dim, orbits, q, x):
    pos, sizes, k = _points(dim, orbits, x)
    w = x[k:]
    mono, ex = _exact(dim, q)
    out = np.zeros(len(mono), dtype=np.result_type(x, float))
    for pts, wi in zip(pos, w):
        for mi, m in enumerate(mono):
            out[mi] += wi * np.sum(np.prod(pts ** np.array(m), axis=1))
    return out - ex


def solve_rule(dim, orbits, q, seed=0, tries=400):
    """find positions/weights of the symmetric orbits exact to degree q.

    Returns (points[n, dim], weights[n]) with positive weights and interior
    free positions, or raises.
    """
    rng = np.random.default_rng(seed)
    nfree = sum(NFREE[o] for o in orbits)
    nw = len(orbits)
    best = None
    for _ in range(tries):
        x0 = np.concatenate([rng.uniform(0.02, 0.48, nfree), rng.uniform(0.01, 0.5, nw)])
        lo = np.concatenate([np.full(nfree, 1e-3), np.full(nw, 1e-6)])
        hi = np.concatenate([np.full(nfree, 0.4999), np.full(nw, 10.0)])
        # S111 second parameter and edge positions: keep inside the simplex
        r = least_squares(lambda x: _residual(dim, orbits, q, x), x0, bounds=(lo, hi),
                          xtol=1e-15, ftol=1e-15, gtol=1e-15, max_nfev=2000)
        res = np.max(np.abs(r.fun))
        if best is None or res < best[0]:
            best = (res, r.x)
        if res < 1e-14:
            break
    res, x = best
    if res > 1e-13:
        raise RuntimeError(f"no rule for {orbits} q={q}: residual {res}")
    # polish with Gauss-Newton steps (complex-step Jacobian), keeping a step
    # only while it lowers the residual
    for _ in range(8):
        f = _residual(dim, orbits, q, x)
        J = np.zeros((len(f), len(x)))
        for i in range(len(x)):
            xc = x.astype(complex)
            xc[i] += 1e-30j
            J[:, i] = _residual(dim, orbits, q, xc).imag / 1e-30
        xn = x + np.linalg.lstsq(J, -f, rcond=None)[0]
        if np.max(np.abs(_residual(dim, orbits, q, xn))) < np.max(np.abs(f)):
            x = xn
    pos, sizes, k = _points(dim, orbits, x)
    w = x[k:]
    if np.any(w <= 0):
        raise RuntimeError(f"non-positive weight for {orbits}")
    pts = np.concatenate(pos)
    wts = np.concatenate([np.full(s, wi) for s, wi in zip(sizes, w)])
    return pts, wts, float(np.max(np.abs(_residual(dim, orbits, q, x))))


def solve_linear_weights(dim, orbits_fixed_pts, q):
    """weights only (positions fixed).  Among the exact rules, take the one that
    maximises the smallest weight (a linear program), so the weights are
    positive whenever a positive rule exists for these orbits."""
    from scipy.optimize import linprog
    mono, ex = _exact(dim, q)
    n = len(orbits_fixed_pts)
    A = np.zeros((len(mono), n))
    for j, pts in enumerate(orbits_fixed_pts):
        for mi, m in enumerate(mono):
            A[mi, j] = np.sum(np.prod(pts ** np.array(m), axis=1))
    c = np.zeros(n + 1)
    c[-1] = -1.0
    a_eq = np.hstack([A, np.zeros((A.shape[0], 1))])
    a_ub = np.hstack([-np.eye(n), np.ones((n, 1))])
    r = linprog(c, A_ub=a_ub, b_ub=np.zeros(n), A_eq=a_eq, b_eq=ex,
                bounds=[(None, None)] * (n + 1), method="highs")
    w = r.x[:-1] if r.status == 0 else np.linalg.lstsq(A, ex, rcond=None)[0]
    # restore exactness to round-off: project onto the affine solution set
    w = w + np.linalg.lstsq(A, ex - A @ w, rcond=None)[0]
    res = np.max(np.abs(A @ w - ex))
    return w, res


# ---------------------------------------------------------------------------
# the rule families
# ---------------------------------------------------------------------------

TRI_OMEGA = {  # p: (orbits, degree)
    1: (["S21"], 2),
    2: (["S21", "S21"], 4),
    3: (["S3", "S21", "S111"], 5),
    4: (["S21", "S21", "S21", "S111"], 7),
}
TRI_GAMMA = {
    1: (["vert"], 1),
    2: (["vert", "mid", "S3"], 3),
    3: (["vert", "edge", "S21"], 5),
    4: (["vert", "mid", "edge", "S21", "S21"], 7),
}


def _vand_cond(pts, p):
    mono = [(i, d - i) for d in range(p + 1) for i in range(d + 1)]
    V = np.array([[np.prod(pt ** np.array(e)) for e in mono] for pt in pts])
    return np.linalg.cond(V)


def build_tri(family, p):
    """Where the moment equations leave a family of rules, several seeded
    solves are made and the rule whose nodes are best conditioned for
    degree-p interpolation (smallest Vandermonde condition number) is kept:
    the Omega operators interpolate to faces from all volume nodes."""
    orbits, q = (TRI_OMEGA if family == "omega" else TRI_GAMMA)[p]
    if all(NFREE[o] == 0 for o in orbits):
        pts = [tri_orbit(o, []) @ TRI_VERTS for o in orbits]
        w, res = solve_linear_weights(2, pts, q)
        wts = np.concatenate([np.full(len(pt), wi) for pt, wi in zip(pts, w)])
        return np.concatenate(pts), wts, res
    best = None
    for seed in range(4):
        try:
            pts, wts, res = solve_rule(2, orbits, q, seed=100 * p + seed, tries=25)
        except RuntimeError:
            continue
        c = _vand_cond(pts, p) if family == "omega" else 0.0
        if best is None or c < best[0]:
            best = (c, pts, wts, res)
    if best is None:
        raise RuntimeError(f"no {family} rule for p={p}")
    return best[1], best[2], best[3]


def gauss_legendre(n):
    x, w = np.polynomial.legendre.leggauss(n)
    return x, w


def build_tet_diage(p):
    """tet diagonal-E rule: face nodes (volume nodes on the faces) form a
    degree-2p triangle rule on every face; the volume rule is degree 2p-1."""
    if p == 1:
        # edge midpoints: on each face the 3 midpoints are the degree-2 rule
        face_orbits, face_q = ["mid"], 2
        tet_face_kinds = ["mid"]
        interior = []
    elif p == 2:
        face_orbits, face_q = ["vert", "mid", "S21"], 4
        tet_face_kinds = ["vert", "mid", "face21"]
        interior = ["S4"]
    elif p == 3:
        return _build_tet_diage3()
    else:
        raise ValueError("tet diagonal-E rules are built for p = 1, 2, 3")
    # face rule on the reference triangle
    if all(NFREE[o] == 0 for o in face_orbits):
        fpts = [tri_orbit(o, []) @ TRI_VERTS for o in face_orbits]
        fw, fres = solve_linear_weights(2, fpts, face_q)
        fparams = []
    else:
        fpts_all, fwts, fres = solve_rule(2, face_orbits, face_q, seed=10 + p)
        # recover the free parameter of the S21 orbit from the solved points
        fparams = []
    if fres > 1e-13:
        raise RuntimeError("face rule failed")
    # the face21 parameter: barycentric a of the S21 face orbit
    a_face = None
    if "S21" in face_orbits:
        # find the interior face points: smallest barycentric coordinate > 0
        bary = _tri_bary(fpts_all)
        inner = [b for b in bary if np.min(b) > 1e-8]
        a_face = float(np.min(inner[0]) if np.sum(np.isclose(inner[0], np.min(inner[0]))) == 2
                       else np.max(inner[0]))
        srt = np.sort(inner[0])
        a_face = float(srt[0]) if np.isclose(srt[0], srt[1]) else float(srt[2])
    # volume weights for the tet orbits with fixed positions
    tet_pts = []
    for kind in tet_face_kinds + interior:
        params = [a_face] if kind == "face21" else []
        tet_pts.append(tet_orbit(kind, params) @ TET_VERTS)
    w, vres = solve_linear_weights(3, tet_pts, 2 * p - 1)
    if vres > 1e-13 or np.any(w <= 0):
        raise RuntimeError(f"tet volume weights failed: {w} {vres}")
    pts = np.concatenate(tet_pts)
    wts = np.concatenate([np.full(len(pt), wi) for pt, wi in zip(tet_pts, w)])
    if p == 1:
        fpts_all = np.concatenate(fpts)
        fwts = np.concatenate([np.full(len(pt), wi) for pt, wi in zip(fpts, fw)])
    return pts, wts, fpts_all, fwts, max(fres, vres)


def _s21_param(b):
    """the repeated barycentric coordinate of an S21 point (a, a, 1 - 2a)."""
    srt = np.sort(b)
    return float(srt[0]) if np.isclose(srt[0], srt[1]) else float(srt[2])


def _build_tet_diage3():
    """p = 3: on every face a degree-6 triangle rule with the vertices, two
    points per edge (a, 1 - a) and two S21 orbits (15 face nodes, found by
    solve_rule); in the volume those 40 boundary nodes plus the centroid and
    an S31 orbit (c, c, c, 1 - 3c), with weights exact to degree 5 = 2p - 1.
    The moment equations fix the weights for each c; c is chosen on a grid
    of step 1e-3 in [0.01, 0.24] to maximise the smallest weight (45 nodes)."""
    face_orbits = ["vert", "edge", "S21", "S21"]
    fpts_all, fwts, fres = solve_rule(2, face_orbits, 6, seed=7, tries=60)
    bary = _tri_bary(fpts_all)
    edge = bary[3:9]
    a = float(np.min(edge[edge > 1e-9]))
    b1, b2 = _s21_param(bary[9]), _s21_param(bary[12])
    fixed = [tet_orbit("vert", []) @ TET_VERTS, tet_orbit("edge2", [a]) @ TET_VERTS,
             tet_orbit("face21", [b1]) @ TET_VERTS, tet_orbit("face21", [b2]) @ TET_VERTS,
             tet_orbit("S4", []) @ TET_VERTS]
    best = None
    for c in np.round(np.arange(0.01, 0.2405, 0.001), 6):
        tet_pts = fixed + [tet_orbit("S31", [float(c)]) @ TET_VERTS]
        w, vres = solve_linear_weights(3, tet_pts, 5)
        if vres < 1e-13 and np.all(w > 0) and (best is None or w.min() > best[0]):
            best = (w.min(), tet_pts, w, vres)
    if best is None:
        raise RuntimeError("no positive degree-5 tet rule on the p = 3 face nodes")
    _, tet_pts, w, vres = best
    pts = np.concatenate(tet_pts)
    wts = np.concatenate([np.full(len(pt), wi) for pt, wi in zip(tet_pts, w)])
    return pts, wts, fpts_all, fwts, max(fres, vres)


def _tri_bary(pts):
    # x = -1 + 2 l2, y = -1 + 2 l3 for the reference triangle
    l2 = (pts[:, 0] + 1) / 2
    l3 = (pts[:, 1] + 1) / 2
    return np.stack([1 - l2 - l3, l2, l3], axis=1)


def _fmt(a):
    return "[" + ", ".join(repr(float(v)) for v in np.ravel(a)) + "]"


def main(out_path):
    lines = ['"""Cubature tables for the SBP operators (generated by cubature_gen.py; do not edit).',
             '',
             'Each entry: points (row-major, n x dim, reference element coordinates),',
             'weights (n), and the max moment-equation residual of the solve.',
             '"""', '', 'TRI = {']
    for fam in ("omega", "gamma"):
        for p in (1, 2, 3, 4):
            pts, wts, res = build_tri(fam, p)
            lines.append(f'    ("{fam}", {p}): {{"n": {len(wts)}, "points": {_fmt(pts)},')
            lines.append(f'        "weights": {_fmt(wts)}, "residual": {float(res)!r}}},')
            print(fam, p, len(wts), res, file=sys.stderr)
    lines.append('}')
    lines.append('')
    lines.append('TET_DIAGE = {')
    for p in (1, 2, 3):
        pts, wts, fpts, fwts, res = build_tet_diage(p)
        lines.append(f'    {p}: {{"n": {len(wts)}, "points": {_fmt(pts)},')
        lines.append(f'        "weights": {_fmt(wts)},')
        lines.append(f'        "face_points": {_fmt(fpts)}, "face_weights": {_fmt(fwts)},')
        lines.append(f'        "residual": {float(res)!r}}},')
        print("tet diagE", p, len(wts), res, file=sys.stderr)
    lines.append('}')
    with open(out_path, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    import os
    main(os.path.join(os.path.dirname(os.path.abspath(__file__)), "cubature_tables.py"))
