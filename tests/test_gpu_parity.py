"""GPU parity: the sm_103a path through the C-ABI against the CPU oracle and the
reference's golden values."""
import numpy as np
import pytest

from oracle.eps_ref import eig_residuals, forced_solve, shift_invert_eigs, solve_residual

pytestmark = pytest.mark.gpu

SPINOVER_GOLDEN = np.array([-1.019947097016500742e-01, 1.005733690103750355e+00])

SOLVE_CASES = ["shell_m1_ek1e-4", "spinover", "jones2000_rac", "dormy2004_rac", "mac_dipole_small", "mac_dipole_medium",
               "mac_quadrupole_small", "shell_m2_small"]


def make_pencil(meta, A, B):
    from kore_gb300 import Pencil, layout_from_params
    return Pencil(A, B if B.shape[0] == B.shape[1] else None, layout=layout_from_params(meta))


def match_eigs(lam, ref):
    """Relative error of each reference eigenvalue against its nearest computed one."""
    return np.array([np.min(np.abs(lam - r)) / abs(r) for r in ref])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", SOLVE_CASES)
def test_shifted_solve_matches_oracle(gpu_lib, case, name, precision):
    meta, A, B = case(name)
    sigma = complex(*meta["tau"])
    M = (A - sigma * B).tocsr()
    rng = np.random.default_rng(7)
    b = rng.standard_normal(A.shape[0]) + 1j * rng.standard_normal(A.shape[0])
    with make_pencil(meta, A, B) as p:
        p.factor(sigma, precision)
        x, st = p.solve(b, refine_tol=1e-15 if precision == "mixed" else 0.0, stats=True)
    xr = forced_solve(M, b)
    eta = solve_residual(M, x, b)
    assert eta < (1e-15 if precision == "fp64" else 1e-14), (eta, st)
    # forward agreement with the oracle is limited by conditioning; the pencils at the
    # critical Rayleigh number with target 0 have ||x|| / ||b|| ~ 1e13
    growth = np.linalg.norm(xr) / np.linalg.norm(b)
    tol = 1e-8 if growth < 1e8 else 1e-5
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_forced_problem(gpu_lib, case, precision):
    """Forced solve (KSP preonly + LU, bin/solve.py:207-268) on a forced pencil."""
    from kore_gb300 import KSP
    meta, A, bf = case("forced_m2_f10")
    b = bf.toarray().ravel()
    with make_pencil(meta, A, bf) as p:
        k = KSP()
        k.setOperators(p)
        k.setFromOptions({"kore_precision": precision, "kore_refine_tol": 1e-15})
        x = k.solve(b)
    xr = forced_solve(A, b)
    assert solve_residual(A, x, b) < (1e-15 if precision == "fp64" else 1e-14)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-9
    assert np.isfinite(x).all()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_forced_nan_rhs_reports_enan(gpu_lib, case, precision):
    """A NaN in the right-hand side ends the solve with KORE_ENAN, as bin/solve.py:263-268
    stops on a NaN solution.  In mixed precision the refinement's residual maxima are
    taken on the bits of |r|, which keep a NaN (fmax would drop it), so the loop stops
    at its first check."""
    from kore_gb300 import KSP
    from kore_gb300._lib import KoreError
    meta, A, bf = case("forced_m2_f10")
    b = bf.toarray().ravel().astype(complex)
    b[len(b) // 2] = np.nan
    with make_pencil(meta, A, bf) as p:
        k = KSP()
        k.setOperators(p)
        k.setFromOptions({"kore_precision": precision})
        with pytest.raises(KoreError) as e:
            k.solve(b)
    assert e.value.status == 8   # KORE_ENAN


def run_eps(p, meta, precision, which=None, nev=None, seed=1):
    from kore_gb300 import EPS
    E = EPS()
    E.setOperators(p)
    E.setProblemType(EPS.ProblemType.GNHEP)
    E.setDimensions(nev or meta["nev"])
    E.setTolerances(meta["tol"], meta["maxit"])
    E.setWhichEigenpairs(which or meta["which_eigenpairs"])
    E.setTarget(complex(*meta["tau"]))
    E.setFromOptions({"st_type": "sinvert", "kore_precision": precision, "kore_seed": seed})
    E.solve()
    return E


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-10)])
def test_eigs_shell_m1(gpu_lib, case, precision, tol):
    """Hydrodynamic shell, m=1, Ek=1e-4, N=48, lmax=40, target 1i, nev=10."""
    meta, A, B = case("shell_m1_ek1e-4")
    tau = complex(*meta["tau"])
    ref, Xr = shift_invert_eigs(A, B, tau, meta["nev"], "TM")
    with make_pencil(meta, A, B) as p:
        E = run_eps(p, meta, precision)
    lam, X = E.eigenvalues(), E.eigenvectors()
    assert len(lam) >= meta["nev"], E.stats
    err = match_eigs(lam[:meta["nev"]], ref)
    assert err.max() < tol, (err, E.stats)
    # SLEPc order: sorted by distance to the target
    d = np.abs(lam - tau)
    assert np.all(np.diff(d) >= -1e-12 * d.max())
    # eigenvectors: unit norm, residual small (checked up to phase by the residual)
    assert np.allclose(np.linalg.norm(X, axis=0), 1.0, atol=1e-12)
    assert eig_residuals(A, B, lam, X).max() < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_eigs_spinover_golden(gpu_lib, case, precision):
    """tests/test_spinover.py of the reference: max-Re eigenvalue vs reference.eig."""
    meta, A, B = case("spinover")
    with make_pencil(meta, A, B) as p:
        E = run_eps(p, meta, precision)
    lam = E.eigenvalues()
    i = np.argmax(lam.real)
    np.testing.assert_allclose([lam[i].real, lam[i].imag], SPINOVER_GOLDEN, rtol=1e-8, atol=1e-20)
    assert abs(lam[i] - complex(*SPINOVER_GOLDEN)) / abs(complex(*SPINOVER_GOLDEN)) < 1e-11


@pytest.mark.parametrize("name,omega_c", [("jones2000_rac", -1.93444e-02), ("dormy2004_rac", -1.10162e-02)])
def test_eigs_convective_onset(gpu_lib, case, name, omega_c):
    """Critical mode at the golden Ra: which='TR', target 0 (find_Rac.py's criterion)."""
    meta, A, B = case(name)
    with make_pencil(meta, A, B) as p:
        E = run_eps(p, meta, "fp64", which="TR", nev=meta["nev"])
    lam = E.eigenvalues()
    i = np.argmax(lam.real)
    assert abs(lam[i].real) < 1e-5 and abs(lam[i].imag - omega_c) < 1e-6


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-10)])
@pytest.mark.parametrize("name", ["mac_dipole_small", "mac_dipole_medium", "mac_dipole_internal",
                                  "mac_quadrupole_small", "shell_m2_small"])
def test_eigs_other_pencils(gpu_lib, case, name, precision, tol):
    """Magneto-Archimedes-Coriolis pencils (dipole: superblocks {upol, btor, theta} /
    {utor, bpol}; quadrupole: degree pairs merged for the l +- 2 coupling) and an m=2
    shell, at the bars of the eigenvalue comparison: FP64 1e-12, mixed 1e-10."""
    meta, A, B = case(name)
    tau = complex(*meta["tau"])
    ref, _ = shift_invert_eigs(A, B, tau, meta["nev"], "TM")
    with make_pencil(meta, A, B) as p:
        E = run_eps(p, meta, precision, which="TM")
    lam, X = E.eigenvalues(), E.eigenvectors()
    err = match_eigs(lam[:meta["nev"]], ref)
    assert err.max() < tol, err
    assert eig_residuals(A, B, lam[:meta["nev"]], X[:, :meta["nev"]]).max() < 1e-12
