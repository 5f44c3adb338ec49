"""The allocation-free solve entry point (kore_solve_dev_noalloc) against the ordinary
device solve (kore_solve_dev) and the oracle, called through the C-ABI.

kore_solve_dev_noalloc serves callers that cannot allocate device memory when they
solve (a fixed budget or a pool they do not own, a latency-critical loop that must not
take cudaMalloc's device-wide synchronisation).  Its scratch is a fixed file-scope
device array shared by every call, so it must give the same result as kore_solve_dev
on every call, also when the array still holds the contents of a previous call on a
larger problem or of a call that ended on a NaN.  This file is collected last so that
a run stopping at the first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

from oracle.eps_ref import solve_residual

pytestmark = pytest.mark.gpu

KORE_EINVAL, KORE_ENAN = 1, 8


def _pencil(case, name):
    from kore_gb300 import Pencil, layout_from_params
    meta, A, B = case(name)
    return meta, A, B, Pencil(A, B, layout=layout_from_params(meta))


def _noalloc(p, b, x, tol, stream):
    return p.lib.kore_solve_dev_noalloc(p._plan, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                                        float(tol), ctypes.c_void_p(stream))


def _rhs(torch, n, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.complex(torch.randn(n, dtype=torch.float64, device="cuda", generator=g),
                         torch.randn(n, dtype=torch.float64, device="cuda", generator=g))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_matches_solve_dev(gpu_lib, case, precision):
    """Calls alternate between a 4352-unknown plan (64 blocks) and a 1152-unknown one
    (16 blocks), twice each, so the smaller problem runs on scratch that the larger one
    left behind; each result equals kore_solve_dev's and meets the oracle's backward
    error bound."""
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    plans = []
    for name in ("spinover", "mac_dipole_small"):
        meta, A, B, p = _pencil(case, name)
        sigma = complex(*meta["tau"])
        p.factor(sigma, precision)
        b = _rhs(torch, p.n, 11 + len(plans))
        x_ref = torch.zeros_like(b)
        p.solve_dev(b.data_ptr(), x_ref.data_ptr(), 1, 1e-15, stream)
        plans.append((p, (A - sigma * B).tocsr(), b, x_ref))
    torch.cuda.synchronize()
    try:
        for call in range(4):
            p, M, b, x_ref = plans[call % 2]
            x = torch.full_like(b, complex(float("nan"), 0.0))
            rc = _noalloc(p, b, x, 1e-15, stream)
            assert rc == 0, (call, rc)
            torch.cuda.synchronize()
            rel = float((x - x_ref).abs().max() / x_ref.abs().max())
            assert np.isfinite(rel) and rel < 1e-12, (call, rel)
            eta = solve_residual(M, x.cpu().numpy(), b.cpu().numpy())
            assert eta < (1e-15 if precision == "fp64" else 1e-14), (call, eta)
    finally:
        for p, *_ in plans:
            p.close()


def test_noalloc_nan_then_clean_call(gpu_lib, case):
    """Mixed precision: a NaN in the right-hand side ends the call with KORE_ENAN (the
    refinement's residual check keeps it); the next call, on a clean right-hand side,
    starts from cleared flags and succeeds.  (The FP64 path has no refinement loop: like
    kore_solve_dev it leaves a NaN in x for the caller to find.)"""
    precision = "mixed"
    import torch
    meta, A, B, p = _pencil(case, "shell_m1_ek1e-4")
    stream = torch.cuda.current_stream().cuda_stream
    with p:
        p.factor(complex(*meta["tau"]), precision)
        b = _rhs(torch, p.n, 5)
        x_ref = torch.zeros_like(b)
        p.solve_dev(b.data_ptr(), x_ref.data_ptr(), 1, 1e-15, stream)
        bad = b.clone()
        bad[p.n // 2] = complex(float("nan"), 0.0)
        x = torch.zeros_like(b)
        assert _noalloc(p, bad, x, 1e-15, stream) == KORE_ENAN
        x = torch.zeros_like(b)
        assert _noalloc(p, b, x, 1e-15, stream) == 0
        torch.cuda.synchronize()
        assert float((x - x_ref).abs().max() / x_ref.abs().max()) < 1e-12


def test_noalloc_rejects_oversized_problem(gpu_lib, case):
    """More padded unknowns than the fixed scratch holds: a clear KORE_EINVAL."""
    import torch
    meta, A, B, p = _pencil(case, "dormy2004_rac")   # 148 blocks x 148 = 21904 padded unknowns
    with p:
        b = torch.zeros(p.n, dtype=torch.complex128, device="cuda")
        x = torch.zeros_like(b)
        assert _noalloc(p, b, x, 0.0, 0) == KORE_EINVAL


def test_noalloc_rejects_too_many_counters(gpu_lib):
    """8192 unknowns in 2048 blocks of 4: within the unknowns limit, but the sweep needs
    (3 x 11 levels + 2) x 2048 = 71680 completion counters, more than the 32768 the
    scratch holds: KORE_EINVAL before anything runs (the size checks come before the
    plan's factorisation is looked at, so no factorisation is needed)."""
    import scipy.sparse as ss
    import torch
    from kore_gb300 import Pencil
    from kore_gb300.structure import Layout
    K, s = 2048, 4
    n = K * s
    rng = np.random.default_rng(3)
    rows, cols = [], []
    for i in range(K):
        lo, hi = max(0, (i - 1) * s), min(n, (i + 2) * s)
        r, c = np.meshgrid(np.arange(i * s, (i + 1) * s), np.arange(lo, hi), indexing="ij")
        rows.append(r.ravel())
        cols.append(c.ravel())
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    vals = rng.standard_normal(len(rows)) + 1j * rng.standard_normal(len(rows)) + 8.0 * (rows == cols)
    A = ss.csr_matrix((vals, (rows, cols)), shape=(n, n))
    B = ss.identity(n, format="csr")
    lay = Layout(n=n, N1=s, nb=K, perm=np.arange(n, dtype=np.int64), block_sizes=np.full(K, s, dtype=np.int32),
                 block_ell=np.arange(K), sections=("upol",), coupling=1)
    with Pencil(A, B, layout=lay) as p:
        b = torch.zeros(n, dtype=torch.complex128, device="cuda")
        x = torch.zeros_like(b)
        assert _noalloc(p, b, x, 0.0, 0) == KORE_EINVAL


def test_noalloc_rejects_several_shifts(gpu_lib, case):
    """A plan factorised for several shifts (kore_factor_shifts) is rejected."""
    import torch
    meta, A, B, p = _pencil(case, "shell_m1_ek1e-4")
    with p:
        p.factor_shifts([0.5j, 1.0j], "fp64")
        b = _rhs(torch, p.n, 9)
        x = torch.zeros_like(b)
        assert _noalloc(p, b, x, 0.0, 0) == KORE_EINVAL
