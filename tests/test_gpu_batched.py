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


def test_forced_sweep_escalates_to_fp64(gpu_lib, case):
    """The escalation path of forced_sweep, forced by a bound no refinement meets: every
    group is factorised again in FP64 and the results are the FP64 path's."""
    from kore_gb300 import forced_sweep
    meta, A, B, p = pencil(case, "shell_m2_ek1e-4")
    omegas = np.linspace(-1.5, 1.5, 6)
    rng = np.random.default_rng(9)
    b = rng.standard_normal(A.shape[0]) + 1j * rng.standard_normal(A.shape[0])
    info = {}
    with p:
        x, _ = forced_sweep(p, omegas, b, "mixed", 4, refine_tol=1e-14, escalate_tol=1e-300, info=info)
        x64, _ = forced_sweep(p, omegas, b, "fp64", 4)
    assert info["escalated"] == len(omegas) and info["mixed_resid_max"] < 1e-12
    assert np.abs(x - x64).max() <= 1e-13 * np.abs(x64).max()


def test_forced_sweep_badly_conditioned_instance(gpu_lib):
    """An uneven instance of the forcing sweep (m=1, N=80, lmax=248, Ek=1.67e-7: a thin
    Ekman layer on 80 radial coefficients) whose complex64 factors leave the refinement
    near 1e-9: the returned solve meets 1e-12 all the same, escalated to FP64 factors."""
    from kore_gb300 import Pencil, forced_sweep, layout_from_params
    from kore_gb300.assembly import forcing_vector, hydro_params, hydro_pencil
    m, N, lmax, Ek, w = 1, 80, 248, 1.67e-7, 0.3729
    A, B, nrm = hydro_pencil(m, 1, Ek, N, lmax, 0.35, with_norm=True)
    b = forcing_vector(m, 1, N, lmax, 0.35, 10).toarray().ravel()
    info = {}
    with Pencil(A, B, layout=layout_from_params(hydro_params(m, 1, Ek, N, lmax, 0.35))) as p:
        x, _ = forced_sweep(p, [w], b, "mixed", 1, refine_tol=1e-14, scale=nrm, info=info)
    M = (A - 1j * w * B).tocsr()
    assert solve_residual(M, x[:, 0], b / nrm) < 1e-12
    assert info["escalated"] == 1 or info["mixed_resid_max"] <= 1e-10, info
