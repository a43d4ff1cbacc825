"""Regenerates the committed golden residual fixtures from the CPU oracle.

Run from the repository root: ``python tests/golden/make_golden.py``.
Each fixture holds the seeded input state and the oracle's residual for a
small case of each discretisation on the hot path:
  c1:       512-triangle vortex annulus, SBP-Omega p=2, Roe (full config 1)
  gamma3:   8x8 annulus (128 triangles), SBP-Gamma p=3, Roe
  tet2:     warped 2^3 cube (48 tets), diagonal-E p=2, IR split form + IR faces
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import __graft_entry__ as graft  # noqa: E402

graft.load_package()
from pdesolver_gb300 import abi, build, eulergpu, problems  # noqa: E402


def cases():
    yield "c1", problems.config1()
    yield "gamma3", problems.config1(n=8, p=3, family="gamma", seed=11)
    yield "tet2", problems.config3(n=2, seed=12)


def oracle_residual(lib, ms, opts, q):
    desc = abi.MeshDesc(ms)
    P = eulergpu.params_from_opts(opts)
    res = np.zeros_like(q)
    st = lib.oracle_eval_residual(C.byref(desc.desc), C.byref(P), abi.dptr(q), abi.dptr(res))
    assert st == 0
    return res


def main():
    lib = C.CDLL(build.build_oracle())
    for name, (ms, opts, q) in cases():
        res = oracle_residual(lib, ms, opts, q)
        np.savez_compressed(os.path.join(HERE, f"residual_{name}.npz"), q=q, res=res)
        print(name, q.shape, float(np.abs(res).max()))


if __name__ == "__main__":
    main()
