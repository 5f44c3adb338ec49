"""The C-ABI library builds, loads and exports every symbol include/kore_gpu.h declares
(no compute calls: these run without a GPU)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "kore_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z0-9_]+\s*\*?\s*(kore_[a-z_]+)\s*\(", src, flags=re.M)))


def test_header_parses():
    names = declared_functions()
    assert "kore_plan_create" in names and "kore_eigs" in names and len(names) >= 10


def test_library_exports_every_declared_symbol():
    from kore_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    for name in declared_functions():
        assert hasattr(lib, name), name
    from kore_gb300 import _lib
    assert set(_lib.EXPORTS) == set(declared_functions())


def test_status_strings_and_counter():
    from kore_gb300 import _lib
    lib = _lib.load()
    for code in range(9):
        assert lib.kore_status_string(code)
    assert lib.kore_kernel_launches() >= 0


def test_plan_create_rejects_bad_desc():
    """Invalid descriptors fail with KORE_EINVAL before touching the device."""
    from kore_gb300 import _lib
    lib = _lib.load()
    d = _lib.PencilDesc()
    d.n = 0
    plan = ctypes.c_void_p()
    assert lib.kore_plan_create(ctypes.byref(d), 0, ctypes.byref(plan)) == 1
    assert lib.kore_plan_create(None, 0, ctypes.byref(plan)) == 1
