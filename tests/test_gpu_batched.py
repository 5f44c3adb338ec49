"""Batched forced solves: many forcing frequencies sigma = i*omega of one pencil
factorised and solved in the same kernel launches (the tidal-forcing frequency sweep at
test size), checked against the oracle and against one-at-a-time solves."""
import numpy as np
import pytest
import scipy.sparse.linalg as ssl

from oracle.eps_ref import forced_solve, solve_residual

pytestmark = pytest.mark.gpu


def pencil(case, name):
    from kore_gb300 import Pencil, layout_from_params
    meta, A, B = case(name)
    return meta, A, B, Pencil(A, B, layout=layout_from_params(meta))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_shifts_match_oracle(gpu_lib, case, precision):
    meta, A, B, p = pencil(case, "shell_m2_ek1e-4")
    omegas = np.linspace(-2.0, 2.0, 12)
    sig = 1j * omegas
    rng = np.random.default_rng(5)
    n = A.shape[0]
    b = rng.standard_normal((n, len(sig))) + 1j * rng.standard_normal((n, len(sig)))
    with p:
        p.factor_shifts(sig, precision)
        x, st = p.solve(b, refine_tol=1e-15 if precision == "mixed" else 0.0, stats=True)
    for s, sg in enumerate(sig):
        M = (A - sg * B).tocsr()
        eta = solve_residual(M, x[:, s], b[:, s])
        assert eta < (1e-15 if precision == "fp64" else 1e-14), (s, eta, st)
        xr = forced_solve(M, b[:, s])
        assert np.linalg.norm(x[:, s] - xr) / np.linalg.norm(xr) < 1e-9


def test_batched_equals_alone(gpu_lib, case):
    """Each shift's result is the same solved alone and in the batch."""
    meta, A, B, p = pencil(case, "shell_m2_ek1e-4")
    sig = 1j * np.array([-1.3, 0.2, 0.7, 1.9])
    rng = np.random.default_rng(9)
    n = A.shape[0]
    b = rng.standard_normal((n, 4)) + 1j * rng.standard_normal((n, 4))
    with p:
        p.factor_shifts(sig, "fp64")
        xb = p.solve(b)
        for s, sg in enumerate(sig):
            p.factor(sg, "fp64")
            xa = p.solve(b[:, s])
            assert np.linalg.norm(xa - xb[:, s]) / np.linalg.norm(xa) < 1e-13


def test_forced_problem_from_eigen_pencil(gpu_lib, case):
    """forcing=10 at omega=0.7: the forced matrix is ||u||_F (A_eig - i omega B_eig), so
    the batched shifted solve on the eigen pencil reproduces the forced solution."""
    meta_f, Af, bf = case("forced_m2_f10")
    meta, A, B, p = pencil(case, "shell_m2_ek1e-4")
    w = meta_f["forcing_frequency"]
    M = A - (1j * w) * B
    unorm = np.abs(Af).sum() / np.abs(M).sum()
    b = bf.toarray().ravel() / unorm
    xr = forced_solve(Af, bf.toarray().ravel())
    with p:
        p.factor_shifts([0.1j, 1j * w, -0.4j], "mixed")
        x = p.solve(np.column_stack([b, b, b]), refine_tol=1e-15)
    assert np.linalg.norm(x[:, 1] - xr) / np.linalg.norm(xr) < 1e-9
