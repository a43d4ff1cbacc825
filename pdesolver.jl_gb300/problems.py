"""The synthetic workloads the hot path is measured on (seeded).

* ``config1``: FP64 isentropic vortex, quarter annulus r in [1,3],
  16x16 (r, theta) quads split into 512 triangles, SBP-Omega p=2, Roe faces,
  vortex (rho_in = 2, M_in = 0.5) as state and Dirichlet data; state =
  vortex * (1 + N(0, 1e-3)) with seed 1.
* ``config2``: same annulus at 64x64 (8192 triangles), SBP-Gamma p=3, Roe;
  start = free stream (rho 1, Ma = 0.5, aoa 0) * (1 + U(-0.01, 0.01)), seed 2.
* ``config3``: unit cube 24^3 hexes -> 6 tets each (82,944), warped, SBP
  diagonal-E p=2 tets, Ismail-Roe split-form volume and IR faces, Mach 0.5
  free stream with density * (1 + N(0, 0.01)), seed 4.

Initial/boundary states restate the reference's calcIsentropicVortex
(src/solver/euler/common_funcs.jl:25-79, with M_in a parameter) and
calcFreeStream (common_funcs.jl:312-345).
"""
from __future__ import annotations

import numpy as np

from . import mesh as _mesh
from . import sbp as _sbp

R_GAS = 287.058   # read_input.jl:141


def vortex_state(coords, gamma=1.4, M_in=0.5, r_in=1.0, rho_in=2.0):
    x, y = coords[..., 0], coords[..., 1]
    r = np.sqrt(x * x + y * y)
    theta = np.arctan2(y, x)
    tmp1 = ((gamma - 1) / 2) * M_in * M_in
    rho = rho_in * (1 + tmp1 * (1 - (r_in * r_in) / (r * r))) ** (1 / (gamma - 1))
    p = (1 / gamma) * (rho / rho_in) ** gamma
    a = np.sqrt(gamma * p / rho)
    M = np.sqrt((2 / (gamma - 1)) * (rho_in / rho) ** (gamma - 1) * (1 + tmp1) - 2 / (gamma - 1))
    U = M * a
    cv = R_GAS / (gamma - 1)
    e = cv * p / (rho * R_GAS)
    q = np.zeros(coords.shape[:-1] + (4,))
    q[..., 0] = rho
    q[..., 1] = rho * (U * np.sin(theta))
    q[..., 2] = rho * (-U * np.cos(theta))
    q[..., 3] = rho * e + 0.5 * rho * U * U
    return q


def free_stream(dim, shape, gamma=1.4, Ma=0.5, aoa=0.0, rho=1.0, p_free=None):
    p_free = 1.0 / gamma if p_free is None else p_free
    q = np.zeros(shape + (dim + 2,))
    q[..., 0] = rho
    q[..., 1] = rho * Ma * np.cos(aoa)
    if dim == 2:
        q[..., 2] = rho * Ma * np.sin(aoa)
    else:
        q[..., 3] = -rho * Ma * np.sin(aoa)
    q[..., dim + 1] = p_free / (gamma - 1) + 0.5 * rho * Ma * Ma
    return q


def config1(n=16, p=2, family="omega", seed=1):
    op = _sbp.get_operator(2, family, p)
    ms = _mesh.annulus(op, n, n, bc=_mesh.BC_VORTEX)
    opts = {"gamma": 1.4, "Ma": 0.5, "aoa": 0.0, "vortex_M_in": 0.5, "Flux_name": "RoeFlux",
            "volume_integral_type": 1}
    rng = np.random.default_rng(seed)
    q = vortex_state(ms.coords, M_in=0.5)
    q = q * (1.0 + rng.normal(0.0, 1e-3, size=q.shape))
    return ms, opts, np.ascontiguousarray(q)


def config2(n=64, p=3, family="gamma", seed=2, M_in=0.5):
    op = _sbp.get_operator(2, family, p)
    ms = _mesh.annulus(op, n, n, bc=_mesh.BC_VORTEX)
    opts = {"gamma": 1.4, "Ma": M_in, "aoa": 0.0, "vortex_M_in": M_in, "Flux_name": "RoeFlux",
            "volume_integral_type": 1}
    rng = np.random.default_rng(seed)
    q = free_stream(2, ms.coords.shape[:2], Ma=M_in)
    q = q * (1.0 + rng.uniform(-0.01, 0.01, size=q.shape))
    return ms, opts, np.ascontiguousarray(q)


def config3(n=24, p=2, seed=4, warp=0.05, warp_seed=3):
    op = _sbp.get_operator(3, "diage", p)
    ms = _mesh.cube(op, n, warp=warp, seed=warp_seed, bc=_mesh.BC_FREESTREAM)
    opts = {"gamma": 1.4, "Ma": 0.5, "aoa": 0.0, "Flux_name": "IRFlux",
            "volume_integral_type": 2, "Volume_flux_name": "IRFlux"}
    rng = np.random.default_rng(seed)
    q = free_stream(3, ms.coords.shape[:2], Ma=0.5)
    q[..., 0] *= 1.0 + rng.normal(0.0, 0.01, size=q.shape[:2])
    return ms, opts, np.ascontiguousarray(q)


def cube_wall(n=2, p=2, seed=11, warp=0.05, warp_seed=3, Ma=0.5):
    """Entropy-stable steady problem with a wall: the warped cube of n^3
    hexes -> 6 n^3 tets, diagonal-E p, Ismail-Roe split-form volume terms and
    IR interface fluxes, the face z = 0 (tag 4) an entropy-stable
    no-penetration wall (noPenetrationESBC) and the other faces free-stream
    Dirichlet data at Mach Ma along x; start: that free stream times
    (1 + U(-0.01, 0.01)) with `seed`."""
    op = _sbp.get_operator(3, "diage", p)
    ms = _mesh.cube(op, n, warp=warp, seed=warp_seed,
                    bc_of_tag=lambda t: _mesh.BC_NOPENETRATION_ES if t == 4 else _mesh.BC_FREESTREAM)
    opts = {"gamma": 1.4, "Ma": Ma, "aoa": 0.0, "Flux_name": "IRFlux",
            "volume_integral_type": 2, "Volume_flux_name": "IRFlux"}
    rng = np.random.default_rng(seed)
    q = free_stream(3, ms.coords.shape[:2], Ma=Ma)
    return ms, opts, np.ascontiguousarray(q * (1.0 + rng.uniform(-0.01, 0.01, size=q.shape)))


def annulus_wall(n=4, p=2, family="omega", seed=12, M_in=0.5):
    """The quarter annulus with its inner arc r = 1 (tag 0) an entropy-stable
    no-penetration wall (the isentropic vortex is tangential there) and
    vortex Dirichlet data on the other boundaries; Roe faces, weak-form
    volume terms; state: the vortex times (1 + N(0, 1e-3)) with `seed`."""
    op = _sbp.get_operator(2, family, p)
    ms = _mesh.annulus(op, n, n, bc_of_tag=lambda t: _mesh.BC_NOPENETRATION_ES if t == 0 else _mesh.BC_VORTEX)
    opts = {"gamma": 1.4, "Ma": M_in, "aoa": 0.0, "vortex_M_in": M_in, "Flux_name": "RoeFlux",
            "volume_integral_type": 1}
    rng = np.random.default_rng(seed)
    q = vortex_state(ms.coords, M_in=M_in)
    return ms, opts, np.ascontiguousarray(q * (1.0 + rng.normal(0.0, 1e-3, size=q.shape)))


def config4_specs(count=96, seed=5):
    """Batched workload: `count` annulus problems with n ~ logU(8, 96) (E = 2 n^2),
    SBP-Gamma p ~ U{1, 2, 3, 4}, vortex M_in ~ U(0.3, 0.7), each started from
    the free stream times (1 + U(-0.01, 0.01)) with its own seed."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(count):
        n = int(round(np.exp(rng.uniform(np.log(8.0), np.log(96.0)))))
        p = int(rng.integers(1, 5))
        M = float(rng.uniform(0.3, 0.7))
        specs.append({"n": n, "p": p, "M_in": M, "seed": int(rng.integers(0, 2**31 - 1))})
    return specs


def config4_problem(spec):
    """[(mesh, opts)] of the continuation levels (p = 1, then p when p > 1) and
    the initial state of the first level."""
    ps = (1,) if spec["p"] == 1 else (1, spec["p"])
    levels, q0 = [], None
    for p in ps:
        ms, opts, q = config2(n=spec["n"], p=p, seed=spec["seed"], M_in=spec["M_in"])
        levels.append((ms, opts))
        if q0 is None:
            q0 = q
    return levels, q0


def cube_problem(spec, warp=0.05, warp_seed=3):
    """A 3-D steady solve: the warped unit cube of n^3 hexes -> 6 n^3 tets,
    SBP diagonal-E tets of degree p (levels p = 1, then p when p > 1), Roe
    faces, weak-form volume terms, free-stream Dirichlet data at Mach M_in,
    started from that free stream times (1 + U(-0.01, 0.01)) with the spec's
    seed.  Returns ([(mesh, opts)] per level, initial state of level 0)."""
    ps = (1,) if spec["p"] == 1 else (1, spec["p"])
    levels, q0 = [], None
    M = spec["M_in"]
    for p in ps:
        op = _sbp.get_operator(3, "diage", p)
        ms = _mesh.cube(op, spec["n"], warp=warp, seed=warp_seed, bc=_mesh.BC_FREESTREAM)
        opts = {"gamma": 1.4, "Ma": M, "aoa": 0.0, "Flux_name": "RoeFlux",
                "volume_integral_type": 1}
        levels.append((ms, opts))
        if q0 is None:
            rng = np.random.default_rng(spec["seed"])
            q = free_stream(3, ms.coords.shape[:2], Ma=M)
            q0 = np.ascontiguousarray(q * (1.0 + rng.uniform(-0.01, 0.01, size=q.shape)))
    return levels, q0


def config5_specs(count=2000, seed=6, frac_3d=0.2):
    """Serving stream: `count` requests, a fraction `frac_3d` of them 3-D
    warped cubes (n ~ U{8..24}, p ~ U{1, 2}, Mach ~ U(0.3, 0.7)), the rest
    drawn from the batched 2-D distribution (config4_specs).  Each spec has
    "dim" and the unit-rate exponential inter-arrival gap "gap" (the stream's
    arrival times are cumsum(gap) / rate for the chosen rate)."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(count):
        if rng.uniform() < frac_3d:
            sp = {"dim": 3, "n": int(rng.integers(8, 25)), "p": int(rng.integers(1, 3)),
                  "M_in": float(rng.uniform(0.3, 0.7))}
        else:
            n = int(round(np.exp(rng.uniform(np.log(8.0), np.log(96.0)))))
            sp = {"dim": 2, "n": n, "p": int(rng.integers(1, 5)), "M_in": float(rng.uniform(0.3, 0.7))}
        sp["seed"] = int(rng.integers(0, 2**31 - 1))
        sp["gap"] = float(rng.exponential(1.0))
        specs.append(sp)
    return specs


def request_meshes(key):
    """Host meshes of the continuation levels of a geometry key (dim, n, p):
    the annulus n x n with SBP-Gamma (2-D, vortex data) or the warped cube
    n^3 x 6 with diagonal-E tets (3-D, free-stream data), degrees 1 and p."""
    dim, n, p = key
    out = []
    for pl in ((1,) if p == 1 else (1, p)):
        if dim == 2:
            out.append(_mesh.annulus(_sbp.get_operator(2, "gamma", pl), n, n, bc=_mesh.BC_VORTEX))
        else:
            out.append(_mesh.cube(_sbp.get_operator(3, "diage", pl), n, warp=0.05, seed=3,
                                  bc=_mesh.BC_FREESTREAM))
    return out


def request_problem(spec, meshes=None):
    """([(mesh, opts)] per continuation level, initial state) of a 2-D
    (as config4_problem) or 3-D (as cube_problem) serving request; `meshes`
    (from request_meshes) skips building the geometry."""
    dim = spec.get("dim", 2)
    if meshes is None:
        meshes = request_meshes(geometry_key(spec))
    M = spec["M_in"]
    opts = {"gamma": 1.4, "Ma": M, "aoa": 0.0, "Flux_name": "RoeFlux", "volume_integral_type": 1}
    if dim == 2:
        opts["vortex_M_in"] = M
    ms0 = meshes[0]
    rng = np.random.default_rng(spec["seed"])
    q = free_stream(dim, ms0.coords.shape[:2], Ma=M)
    q0 = np.ascontiguousarray(q * (1.0 + rng.uniform(-0.01, 0.01, size=q.shape)))
    return [(ms, dict(opts)) for ms in meshes], q0


def geometry_key(spec):
    """Requests with equal keys share meshes (the same elements, operators
    and boundary tags); they differ only in Mach number and initial state."""
    return (spec.get("dim", 2), spec["n"], spec["p"])
