"""The C-ABI library loads on a machine without a GPU and exports every
entry point that include/*.h declares (no compute calls)."""
import os
import re

import pytest

from conftest import ROOT


def _declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(vdvc_[a-z0-9_]+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    from voxeldvc_gb300 import build, _lib
    build.build()
    return _lib


def test_every_declared_symbol_is_exported(lib):
    L = lib.lib()
    declared = _declared()
    assert len(declared) >= 30
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, missing


def test_every_declared_symbol_has_a_binding(lib):
    declared = _declared()
    assert declared <= set(lib.SIGNATURES), sorted(declared - set(lib.SIGNATURES))


def test_status_strings_without_gpu(lib):
    L = lib.lib()
    assert L.vdvc_abi_version() == 1
    assert L.vdvc_status_string(lib.OK) == b"ok"
    assert L.vdvc_status_string(lib.ERR_ZERO_DIVISION) == b"division by zero"


def test_size_queries_without_gpu(lib):
    L = lib.lib()
    # 64^3 elements of h = 8: two [24][Ne] float element-vector sets dominate
    n = L.vdvc_workspace_bytes(lib.F32, 8, 64, 64, 64)
    assert n >= 2 * 24 * 64 ** 3 * 4
    assert L.vdvc_workspace_bytes(lib.F32, 0, 4, 4, 4) == 0        # invalid h
    assert L.vdvc_workspace_bytes(7, 8, 4, 4, 4) == 0              # invalid dtype
    assert L.vdvc_workspace_bytes(lib.F32, 8, 2000, 2000, 2000) == 0  # int32 guard
    g = L.vdvc_gn_workspace_bytes(lib.F32, 8, 64, 64, 64)
    assert g > 513 ** 3 * 8  # gvals + res per voxel at least


def test_status_mapping(lib):
    with pytest.raises(ValueError):
        lib.check(lib.ERR_ARG)
    with pytest.raises(ValueError):
        lib.check(lib.ERR_INDEX_RANGE)
    with pytest.raises(ZeroDivisionError):
        lib.check(lib.ERR_ZERO_DIVISION)
    with pytest.raises(NotImplementedError):
        lib.check(lib.ERR_UNSUPPORTED)
    with pytest.raises(lib.VdvcError):
        lib.check(lib.ERR_CUDA)
    lib.check(lib.OK)


def test_gn_desc_layout_matches_header(lib, tmp_path):
    """Every field offset of the ctypes mirror equals the C compiler's."""
    import ctypes as C
    import shutil
    import subprocess
    d = lib.GnDesc
    names = [f[0] for f in d._fields_]
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    src = tmp_path / "layout.c"
    body = "".join(f'  printf("{n} %zu\\n", offsetof(vdvc_gn_desc, {n}));\n' for n in names)
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "vdvc.h"\nint main(void) {\n' + body +
                   '  printf("sizeof %zu\\n", sizeof(vdvc_gn_desc));\n  return 0;\n}\n')
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                       text=True).stdout.splitlines())
    for n in names:
        assert getattr(d, n).offset == int(out[n]), n
    assert C.sizeof(d) == int(out["sizeof"])
