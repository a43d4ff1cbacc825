"""The Julia binding sketched in INTEGRATION.md (Julia is not installed, so it
cannot run here) is checked against the C header and the tested Python
binding: every ccall names a declared entry point with its number of
arguments, and every Julia struct mirrors its C struct field by field."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _prototypes():
    src = open(os.path.join(ROOT, "include", "eulergpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(eg_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", src):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def _doc():
    return open(os.path.join(ROOT, "INTEGRATION.md")).read()


def test_every_ccall_matches_a_prototype():
    protos = _prototypes()
    calls = re.findall(r"ccall\(\(:(eg_[a-z0-9_]+),\s*lib\),\s*\w+,\s*\((.*?)\)\s*[,)]", _doc(), flags=re.S)
    assert len(calls) >= 15
    for name, types in calls:
        assert name in protos, f"INTEGRATION.md calls {name}, which eulergpu.h does not declare"
        t = types.strip().rstrip(",").strip()
        n = 0 if not t else t.count(",") + 1
        assert n == protos[name], f"{name}: {n} argument types, the prototype takes {protos[name]}"


_JULIA_TO_CTYPES = {"Float64": C.c_double, "Int32": C.c_int32, "UInt64": C.c_uint64,
                    "Int64": C.c_int64}


def test_julia_structs_mirror_the_c_structs():
    from pdesolver_gb300 import abi, eulergpu
    classes = {"EgParams": abi.EgParams, "EgMeshDesc": abi.EgMeshDesc,
               "EgNewtonOpts": eulergpu.NewtonOpts, "EgMemQuery": abi.EgMemQuery,
               "EgMemEstimate": abi.EgMemEstimate}
    seen = 0
    for name, body in re.findall(r"^struct (Eg\w+)[^\n]*\n(.*?)^end", _doc(), flags=re.S | re.M):
        fields = re.findall(r"(\w+)::([\w{}]+)", re.sub(r"#[^\n]*", "", body))
        cls = classes[name]
        assert [f for f, _ in fields] == [f for f, _ in cls._fields_], name
        for (fname, jt), (_, ct) in zip(fields, cls._fields_):
            if jt.startswith("Ptr{"):
                assert C.sizeof(ct) == C.sizeof(C.c_void_p), f"{name}.{fname}"
            else:
                assert _JULIA_TO_CTYPES[jt] == ct, f"{name}.{fname}: {jt} vs {ct}"
        seen += 1
    assert seen == len(classes)
