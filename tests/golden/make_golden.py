"""Regenerates the committed golden residual fixtures from the CPU oracle.

Run from the repository root: ``python tests/golden/make_golden.py [name ...]``
(no names: every fixture).
Each fixture holds every input bit-exactly (SBP operator, mesh arrays,
options, seeded state) and the oracle's residual, for a small case of each
discretisation on the hot path:
  c1:       512-triangle vortex annulus, SBP-Omega p=2, Roe (full config 1)
  gamma3:   8x8 annulus (128 triangles), SBP-Gamma p=3, Roe
  tet2:     warped 2^3 cube (48 tets), diagonal-E p=2, IR split form + IR faces
  tet3:     one warped hex (6 tets), diagonal-E p=3, IR split form + IR faces
  wall3:    warped 2^3 cube (48 tets), diagonal-E p=2, IR split form, the z=0 face an
            entropy-stable no-penetration wall (noPenetrationESBC)
  annwall:  4x4 annulus (32 triangles), SBP-Omega p=2, Roe, the inner arc an
            entropy-stable no-penetration wall
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import __graft_entry__ as graft  # noqa: E402

graft.load_package()
import json  # noqa: E402

from pdesolver_gb300 import abi, build, eulergpu, mesh, problems  # noqa: E402


def load(name):
    """(mesh, opts, q, res) of a committed fixture."""
    ms, extra = mesh.load_npz(os.path.join(HERE, f"residual_{name}.npz"))
    return ms, json.loads(str(extra["opts"])), extra["q"], extra["res"]


def cases():
    yield "c1", problems.config1()
    yield "gamma3", problems.config1(n=8, p=3, family="gamma", seed=11)
    yield "tet2", problems.config3(n=2, seed=12)
    yield "tet3", problems.config3(n=1, p=3, seed=13)
    yield "wall3", problems.cube_wall(n=2, p=2, seed=14)
    yield "annwall", problems.annulus_wall(n=4, p=2, seed=15)


def oracle_residual(lib, ms, opts, q):
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    res = np.zeros_like(q)
    st = lib.oracle_eval_residual(C.byref(desc.desc), C.byref(P), abi.dptr(q), abi.dptr(res))
    assert st == 0
    return res


def main(names=None):
    lib = C.CDLL(build.build_oracle())
    for name, (ms, opts, q) in cases():
        if names and name not in names:
            continue
        res = oracle_residual(lib, ms, opts, q)
        mesh.save_npz(os.path.join(HERE, f"residual_{name}.npz"), ms, q=q, res=res,
                      opts=np.array(json.dumps(opts)))
        print(name, q.shape, float(np.abs(res).max()))


if __name__ == "__main__":
    main(sys.argv[1:])
