"""The allocation-free solve entry point (kore_solve_dev_noalloc) against the ordinary
device solve (kore_solve_dev), called through the C-ABI.

kore_solve_dev_noalloc serves callers that cannot allocate device memory when they
solve (a fixed budget or a pool they do not own, a latency-critical loop that must not
take cudaMalloc's device-wide synchronisation).  Its scratch is a fixed file-scope
device array, so it must give the same result as kore_solve_dev on every call, also
when the array still holds the previous call's contents.  This file is collected last
so that a run stopping at the first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KORE_EINVAL = 1


def _pencil(case, name):
    from kore_gb300 import Pencil, layout_from_params
    meta, A, B = case(name)
    return meta, Pencil(A, B, layout=layout_from_params(meta))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_matches_solve_dev(gpu_lib, case, precision):
    import torch
    meta, p = _pencil(case, "shell_m1_ek1e-4")
    with p:
        p.factor(complex(*meta["tau"]), precision)
        n = p.n
        g = torch.Generator(device="cuda").manual_seed(11)
        b = torch.complex(torch.randn(n, dtype=torch.float64, device="cuda", generator=g),
                          torch.randn(n, dtype=torch.float64, device="cuda", generator=g))
        x_ref = torch.zeros_like(b)
        stream = torch.cuda.current_stream().cuda_stream
        p.solve_dev(b.data_ptr(), x_ref.data_ptr(), 1, 1e-15, stream)
        torch.cuda.synchronize()
        for call in range(2):
            x = torch.full_like(b, complex(float("nan"), 0.0))
            rc = p.lib.kore_solve_dev_noalloc(p._plan, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                                              1e-15, ctypes.c_void_p(stream))
            assert rc == 0, (call, rc)
            torch.cuda.synchronize()
            rel = float((x - x_ref).abs().max() / x_ref.abs().max())
            assert np.isfinite(rel) and rel < 1e-12, (call, rel)


def test_noalloc_rejects_oversized_problem(gpu_lib, case):
    """More padded unknowns than the fixed scratch holds: a clear KORE_EINVAL."""
    import torch
    meta, p = _pencil(case, "dormy2004_rac")   # 148 blocks x 148 = 21904 padded unknowns
    with p:
        b = torch.zeros(p.n, dtype=torch.complex128, device="cuda")
        x = torch.zeros_like(b)
        rc = p.lib.kore_solve_dev_noalloc(p._plan, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                                          0.0, ctypes.c_void_p(0))
        assert rc == KORE_EINVAL
