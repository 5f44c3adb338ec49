"""The C-ABI library builds, loads and exports every symbol include/kore_gpu.h declares
(no compute calls: these run without a GPU)."""
import ctypes
import os
import re

import pytest

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
    for code in range(11):
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


def test_estimate_bytes_bounds_the_allocations():
    """kore_plan_estimate_bytes (host arithmetic only) is at least the factor and
    workspace sizes of the block structure and grows with precision, shifts and ncv."""
    import numpy as np
    from conftest import load_case
    from kore_gb300.solver import PencilData
    from kore_gb300.structure import layout_from_params
    meta, A, B = load_case("shell_m2_ek1e-4")
    P = PencilData(A, B, layout=layout_from_params(meta))
    K = len(P.layout.block_sizes)
    S = (int(P.layout.block_sizes.max()) + 3) // 4 * 4
    e64, e32 = P.estimate_bytes("fp64"), P.estimate_bytes("mixed")
    assert e64 > e32 >= 4 * K * S * S * 8
    assert P.estimate_bytes("mixed", nshift=4) > 3 * (e32 - (128 << 20))
    assert P.estimate_bytes("mixed", ncv=32) >= e32 + 2 * K * S * 33 * 16


def test_batch_api_rejects_bad_arguments():
    """The serving entry points validate their arguments before starting anything."""
    from kore_gb300 import _lib
    lib = _lib.load()
    b = ctypes.c_void_p()
    assert lib.kore_batch_create(0, 0, 0, ctypes.byref(b)) == 1          # no workers
    t = ctypes.c_uint64()
    assert lib.kore_batch_submit(None, None, ctypes.byref(t)) == 1
    st = ctypes.c_int()
    assert lib.kore_batch_poll(None, 1, 0, ctypes.byref(st)) == 1
    assert lib.kore_batch_destroy(None) == 0


def test_default_basis_size_rule():
    """The eigensolver's basis when none is given (include/kore_gpu.h, kore_eps_opts.ncv
    = 0): SLEPc's max(2 nev, nev + 15), raised to 4 nev up to 64, never above n."""
    from kore_gb300._lib import MAX_NCV, default_ncv
    assert MAX_NCV == 64
    assert default_ncv(240000, 16) == 64      # the headline solve
    assert default_ncv(240000, 8) == 32       # config 3: 4 nev
    assert default_ncv(240000, 4) == 19       # SLEPc's nev + 15 dominates
    assert default_ncv(240000, 40) == 80      # SLEPc's 2 nev above the cap (refused by the engine)
    assert default_ncv(30, 16) == 30          # never above n


def test_ctypes_structs_match_the_header(tmp_path):
    """Sizes and field offsets of the ctypes mirrors in kore_gb300._lib against the C
    structs of include/kore_gpu.h, compiled with the host compiler."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from kore_gb300 import _lib as L
    pairs = [("kore_pencil_desc", L.PencilDesc), ("kore_eps_opts", L.EpsOpts), ("kore_stats", L.Stats),
             ("kore_request", L.Request)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "kore_gpu.h"', "int main(void) {"]
    for cname, cls in pairs:
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = {}
    for row in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        name, field, val = row.split()
        got[(name, field)] = int(val)
    for cname, cls in pairs:
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)
