"""The CPU oracle (scipy restatement of bin/solve.py) against the reference's own
golden values, on pencils produced by the reference's own assembly."""
import numpy as np
import pytest

from oracle.eps_ref import (eig_residuals, forced_solve, shift_invert_eigs, solve_residual,
                            sort_which)

# tests/spinover/reference.eig:1 in the reference
SPINOVER_GOLDEN = np.array([-1.019947097016500742e-01, 1.005733690103750355e+00])
# tests/jones2000/reference.jones:1 and tests/dormy2004/reference.dormy04:1 (omega_c column)
JONES_OMEGA_C = -1.93444e-02
DORMY_OMEGA_C = -1.10162e-02


def test_spinover_golden(case):
    """Same check as tests/test_spinover.py: max-Re eigenvalue vs reference.eig, rtol 1e-8."""
    meta, A, B = case("spinover")
    lam, X = shift_invert_eigs(A, B, complex(*meta["tau"]), meta["nev"], meta["which_eigenpairs"])
    i = np.argmax(lam.real)
    np.testing.assert_allclose([lam[i].real, lam[i].imag], SPINOVER_GOLDEN, rtol=1e-8, atol=1e-20)
    # the restatement reproduces it far below the test's tolerance
    assert abs(lam[i].real - SPINOVER_GOLDEN[0]) / abs(SPINOVER_GOLDEN[0]) < 1e-12
    assert eig_residuals(A, B, lam, X).max() < 1e-12


@pytest.mark.parametrize("name,omega_c", [("jones2000_rac", JONES_OMEGA_C), ("dormy2004_rac", DORMY_OMEGA_C)])
def test_convective_onset_golden(case, name, omega_c):
    """At the golden critical Rayleigh number the max-Re eigenvalue (find_Rac.py's
    argmax) is marginal and its frequency is the golden omega_c (5 digits)."""
    meta, A, B = case(name)
    lam, X = shift_invert_eigs(A, B, complex(*meta["tau"]), meta["nev"], "TR")
    i = np.argmax(lam.real)
    assert abs(lam[i].real) < 1e-5
    assert abs(lam[i].imag - omega_c) < 1e-6


def test_which_ordering():
    lam = np.array([1 + 1j, -0.5 + 0.2j, 0.1 - 3j, 2 + 0j])
    tau = 0.5j
    assert list(sort_which(lam, "TM", tau)) == list(np.argsort(np.abs(lam - tau), kind="stable"))
    assert list(sort_which(lam, "TR", tau)) == [2, 1, 0, 3]
    assert list(sort_which(lam, "LR", tau)) == [3, 0, 2, 1]
    assert list(sort_which(lam, "SI", tau)) == [2, 3, 1, 0]


def test_forced_is_shifted_eigen_pencil(case):
    """Forced A(w) = |u|_F (A_eig - i w B_eig): the forced solve is the shifted system
    with sigma = i w on the eigen pencil (B_eig = -u/|u|_F, A_eig = (cori - visc)/|u|_F,
    bin/assemble.py:446,582-584,1164-1165; the forced A adds i w u, :685-689)."""
    import scipy.sparse.linalg as ssl
    meta_f, Af, bf = case("forced_m2_f10")
    meta_e, Ae, Be = case("shell_m2_ek1e-4")
    w = meta_f["forcing_frequency"]
    assert ssl.norm(Be) == pytest.approx(1.0, rel=1e-14)
    M = Ae - (1j * w) * Be
    scale = np.abs(Af).sum() / np.abs(M).sum()
    assert abs(ssl.norm(Af - scale * M) / ssl.norm(Af)) < 1e-13
    b = bf.toarray().ravel()
    x = forced_solve(Af, b)
    assert solve_residual(Af, x, b) < 1e-15
