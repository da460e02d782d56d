"""The C-ABI library: builds for sm_103a, loads, and exports every symbol that
include/tmgpu.h declares (no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

from tensormol_gb300 import _lib, build

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(REPO, "include", "tmgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tm_[a-z_0-9]+)\s*\(", src)))


def test_library_builds_and_exports_header_symbols():
    path = build.build()
    lib = ctypes.CDLL(path)
    declared = header_symbols()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(_lib.EXPORTS) == declared


def test_desc_struct_layout_matches_header():
    # the ctypes mirror must have the same size as the C struct
    import subprocess, tempfile
    code = '#include "tmgpu.h"\n#include <stdio.h>\nint main(){printf("%zu\\n", sizeof(tm_model_desc));return 0;}\n'
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(code)
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-I" + os.path.join(REPO, "include"), c, "-o", exe])
        n = int(subprocess.check_output([exe]).strip())
    assert n == ctypes.sizeof(_lib.tm_model_desc)


def _c_class(decl):
    """Type class of one C parameter or return type."""
    d = decl.strip()
    if "*" in d or "[" in d:    # an array parameter is a pointer
        return "ptr"
    words = d.replace("const", "").split()
    for t, cls in (("double", "f64"), ("size_t", "size"), ("int64_t", "i64"), ("unsigned", "u32"),
                   ("int", "i32"), ("void", "void")):
        if t in words:
            return cls
    raise ValueError(decl)


def _ctypes_class(t):
    if t is None:
        return "void"
    if t in (ctypes.c_void_p, ctypes.c_char_p) or issubclass(t, ctypes._Pointer):
        return "ptr"
    return {ctypes.c_double: "f64", ctypes.c_size_t: "size", ctypes.c_int64: "i64",
            ctypes.c_uint: "u32", ctypes.c_int: "i32"}[t]


def test_ctypes_signatures_match_header():
    """Every prototype of include/tmgpu.h against the ctypes declaration of
    tensormol_gb300/_lib.py: return type and each parameter's class
    (pointer, double, int, unsigned, size_t, int64_t), so that a header
    change cannot silently desynchronise the Python side."""
    build.build()
    lib = _lib.load()
    src = open(os.path.join(REPO, "include", "tmgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = re.findall(r"([A-Za-z_][A-Za-z_0-9 \t]*\**)\s*\b(tm_[a-z_0-9]+)\s*\(([^)]*)\)\s*;", src)
    assert len(protos) == len(header_symbols())
    for ret, name, params in protos:
        f = getattr(lib, name)
        args = [p for p in params.split(",") if p.strip() and p.strip() != "void"]
        assert len(args) == len(f.argtypes), (name, args, f.argtypes)
        assert _c_class(ret) == _ctypes_class(f.restype), (name, ret, f.restype)
        for a, t in zip(args, f.argtypes):
            assert _c_class(a) == _ctypes_class(t), (name, a, t)


def test_product_does_not_use_the_oracle():
    """The package (Python and CUDA sources) never imports, links or names
    the oracle: the oracle checks results, it is never the thing measured or
    shipped, and without the CUDA library every call raises."""
    pkg = os.path.join(REPO, "tensormol_gb300")
    hits = []
    for root, _, files in os.walk(pkg):
        if "__pycache__" in root or "_build" in root:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp", ".c")):
                text = open(os.path.join(root, f), encoding="utf-8").read()
                if re.search(r"\boracle\b|tmoracle", text):
                    hits.append(os.path.relpath(os.path.join(root, f), REPO))
    assert hits == [], hits
