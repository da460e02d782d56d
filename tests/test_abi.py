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
