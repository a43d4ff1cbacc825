"""The oracle reproduces the committed golden residuals (CPU), and the
seeded inputs regenerate identically."""
import os

import numpy as np
import pytest

from conftest import oracle_residual
from pdesolver_gb300 import abi, eulergpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cases():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return {name: c for name, c in mod.cases()}


CASES = _cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_golden(oracle, name):
    ms, opts, q = CASES[name]
    g = np.load(os.path.join(HERE, f"residual_{name}.npz"))
    np.testing.assert_allclose(q, g["q"], rtol=1e-15, atol=0)
    res = oracle_residual(oracle, abi.MeshDesc(ms), eulergpu.params_from_opts(opts), q)
    scale = np.abs(g["res"]).max()
    assert np.abs(res - g["res"]).max() <= 1e-12 * scale
