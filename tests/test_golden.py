"""The oracle reproduces the committed golden residuals (CPU) on the
fixtures' own bit-exact inputs, and the seeded set-up regenerates them."""
import importlib.util
import os

import numpy as np
import pytest

from conftest import oracle_residual
from pdesolver_gb300 import abi, eulergpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["c1", "gamma3", "tet2", "tet3", "wall3", "annwall"]


def _gen():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


GEN = _gen()


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_golden(oracle, name):
    """1e-12 relative to the largest entry, the GPU parity bar: the fixtures
    were written on x86-64, and a compiler that contracts multiply-adds into
    FMAs (gcc on aarch64 does by default) moves the oracle's result by about
    1e-13 of it."""
    ms, opts, q, gold = GEN.load(name)
    res = oracle_residual(oracle, abi.MeshDesc(ms), eulergpu.params_from_opts(opts), q)
    assert np.abs(res - gold).max() <= 1e-12 * np.abs(gold).max()


@pytest.mark.parametrize("name", NAMES)
def test_setup_regenerates_fixture(name):
    """the seeded state and the operator/mesh set-up reproduce the fixture
    (to round-off: numpy's linear algebra and elementary functions may differ
    in the last bits across machines; the vortex state differs by 1.4e-14
    between x86-64 and Arm)."""
    cases = dict(GEN.cases())
    ms, opts, q = cases[name]
    gms, gopts, gq, _ = GEN.load(name)
    assert opts == gopts
    np.testing.assert_allclose(q, gq, rtol=1e-13, atol=0)
    np.testing.assert_allclose(ms.sbp.Q, gms.sbp.Q, atol=1e-12)
    np.testing.assert_allclose(ms.dxidx, gms.dxidx, rtol=1e-12, atol=1e-14)
