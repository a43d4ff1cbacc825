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


def test_ctypes_structures_match_the_header(tmp_path):
    """every ctypes structure of the Python binding has the size and field
    offsets of its C struct in include/eulergpu.h (compiled with the host C
    compiler), so no argument block drifts from the ABI."""
    import shutil
    import subprocess
    import pytest
    from pdesolver_gb300 import abi, eulergpu
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {
        "eg_params": abi.EgParams, "eg_mesh_desc": abi.EgMeshDesc, "eg_timings": eulergpu.Timings,
        "eg_ls_stats": eulergpu.LsStats, "eg_newton_opts": eulergpu.NewtonOpts,
        "eg_newton_stats": eulergpu.NewtonStats, "eg_rk4_stats": eulergpu.Rk4Stats,
        "eg_mem_query": abi.EgMemQuery, "eg_mem_estimate": abi.EgMemEstimate,
        "eg_launch_config": abi.EgLaunchConfig, "eg_tune_entry": abi.EgTuneEntry,
    }
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "eulergpu.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "abi_probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "abi_probe"
    r = subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    for cname, cls in structs.items():
        assert int(got[cname]) == C.sizeof(cls), f"sizeof({cname})"
        for fname, _ in cls._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(cls, fname).offset, f"{cname}.{fname}"


def test_binding_argument_counts_match_the_prototypes():
    """every function the Python binding declares argtypes for takes as
    many arguments in include/eulergpu.h (a drifted prototype would pass
    misaligned arguments through ctypes)."""
    from pdesolver_gb300 import eulergpu
    src = open(os.path.join(ROOT, "include", "eulergpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(eg_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", src):
        args = m.group(2).strip()
        protos[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1

    class Recorder:
        def __init__(self):
            self.fns = {}

        def __getattr__(self, name):
            fn = self.fns.setdefault(name, type("Fn", (), {})())
            return fn

    rec = Recorder()
    eulergpu._declare(rec)
    checked = 0
    for name, fn in rec.fns.items():
        if hasattr(fn, "argtypes"):
            assert name in protos, f"{name} is not declared in eulergpu.h"
            assert len(fn.argtypes) == protos[name], f"{name}: {len(fn.argtypes)} vs {protos[name]}"
            checked += 1
    assert checked >= 30
