"""The C-ABI library loads and exports every symbol include/eulergpu.h
declares (no compute calls: CPU only)."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "eulergpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(eg_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(gpu_lib):
    names = declared_symbols()
    assert "eg_eval_residual" in names and "eg_mesh_create" in names
    for n in names:
        assert hasattr(gpu_lib, n), f"libeulergpu.so does not export {n}"


def test_version_and_error_without_gpu_work(gpu_lib):
    gpu_lib.eg_version.restype = C.c_int
    assert gpu_lib.eg_version() >= 1
    gpu_lib.eg_last_error.restype = C.c_char_p
    assert isinstance(gpu_lib.eg_last_error(), bytes)


def test_mesh_create_rejects_bad_sizes(gpu_lib):
    """invalid descriptors are refused on the host before any device call."""
    from pdesolver_gb300 import abi
    d = abi.EgMeshDesc()
    d.dim = 4
    p = abi.EgParams.make()
    h = C.c_void_p()
    assert gpu_lib.eg_mesh_create(C.byref(d), C.byref(p), C.byref(h)) == abi.EG_ERR_INVALID


def test_host_arrays_are_size_checked():
    """the library takes raw pointers; the Python host layer refuses arrays
    whose size is not the mesh's number of unknowns (before any device call)."""
    import numpy as np
    import pytest
    from pdesolver_gb300 import eulergpu
    with pytest.raises(ValueError):
        eulergpu.GPUMesh._ptr(np.zeros(10), 12)
    with pytest.raises(ValueError):
        eulergpu.GPUMesh._ptr(np.zeros(12, dtype=np.float32), 12)
    ptr, mem = eulergpu.GPUMesh._ptr(np.zeros(12), 12)
    assert mem == 0 and ptr.value
