"""Batched eigensolves (kore_eigs_shifts): several targets on one pencil stepping
together in shared launches.  Each target's eigenpairs must be those of the same solve
run alone (kore_eigs with the same seed) and match the oracle at that target."""
import numpy as np
import pytest

from oracle.eps_ref import eig_residuals, shift_invert_eigs

pytestmark = pytest.mark.gpu


def alone(p, tau, nev, precision, seed, which="TM"):
    from kore_gb300 import EPS
    E = EPS()
    E.setOperators(p)
    E.setProblemType(EPS.ProblemType.GNHEP)
    E.setDimensions(nev)
    E.setTolerances(1e-15, 100)
    E.setWhichEigenpairs(which)
    E.setTarget(tau)
    E.setFromOptions({"st_type": "sinvert", "kore_precision": precision, "kore_seed": seed})
    p.sigma = None
    E.solve()
    return E.eigenvalues(), E.eigenvectors()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-10)])
def test_targets_batched_equal_alone_and_oracle(gpu_lib, case, precision, tol):
    """Three targets with different nev on the m=1 shell (1,920 unknowns)."""
    from kore_gb300 import Pencil, eigs_targets, layout_from_params
    meta, A, B = case("shell_m1_ek1e-4")
    targets = [1.0j, 0.6j, 0.05 + 1.4j]
    nevs = [10, 6, 8]
    seeds = [3, 4, 5]
    with Pencil(A, B, layout=layout_from_params(meta)) as p:
        res = eigs_targets(p, targets, nevs, "TM", precision, tol=1e-15, maxit=100, seeds=seeds)
        single = [alone(p, t, k, precision, s) for t, k, s in zip(targets, nevs, seeds)]
    for (lam, X, st), (lam1, X1), tau, nev in zip(res, single, targets, nevs):
        assert len(lam) >= nev, st
        # the same solve alone: identical arithmetic per target
        assert len(lam) == len(lam1)
        assert np.max(np.abs(lam - lam1) / np.abs(lam1)) < 1e-13
        for j in range(nev):
            ph = np.vdot(X1[:, j], X[:, j])
            assert np.linalg.norm(X[:, j] - X1[:, j] * ph / abs(ph)) < 1e-10
        # the oracle at this target
        ref, _ = shift_invert_eigs(A, B, tau, nev, "TM")
        err = np.array([np.min(np.abs(lam[:nev] - r)) / abs(r) for r in ref])
        assert err.max() < tol, (tau, err)
        assert eig_residuals(A, B, lam[:nev], X[:, :nev]).max() < 1e-12
        d = np.abs(lam - tau)
        assert np.all(np.diff(d) >= -1e-12 * d.max())


def test_targets_batched_quadrupole_mixed(gpu_lib, case):
    """Block-pentadiagonal-in-degree (merged superblock) MAC pencil, two targets, mixed."""
    from kore_gb300 import Pencil, eigs_targets, layout_from_params
    meta, A, B = case("mac_quadrupole_small")
    nev = meta["nev"]
    targets = [complex(*meta["tau"]), complex(*meta["tau"]) + 0.3j]
    with Pencil(A, B, layout=layout_from_params(meta)) as p:
        res = eigs_targets(p, targets, nev, "TM", "mixed", seeds=[1, 2])
    for (lam, X, st), tau in zip(res, targets):
        ref, _ = shift_invert_eigs(A, B, tau, nev, "TM")
        err = np.array([np.min(np.abs(lam[:nev] - r)) / abs(r) for r in ref])
        assert err.max() < 1e-10, (tau, err)
        assert eig_residuals(A, B, lam[:nev], X[:, :nev]).max() < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_targets_through_fewer_slots(gpu_lib, case, precision):
    """Five targets through two slots: a finished target's slot is re-factorised for the
    next target while the other slot carries on; every target's pairs equal its lone
    solve and the oracle's."""
    from kore_gb300 import Pencil, eigs_targets, layout_from_params
    meta, A, B = case("shell_m1_ek1e-4")
    targets = [1.0j, 0.6j, 0.05 + 1.4j, 0.8j, 1.2j]
    nevs = [8, 4, 6, 5, 7]
    seeds = [11, 12, 13, 14, 15]
    with Pencil(A, B, layout=layout_from_params(meta)) as p:
        res = eigs_targets(p, targets, nevs, "TM", precision, tol=1e-15, maxit=100, seeds=seeds, slots=2)
        single = [alone(p, t, k, precision, s) for t, k, s in zip(targets, nevs, seeds)]
    tol = 1e-12 if precision == "fp64" else 1e-10
    for (lam, X, st), (lam1, X1), tau, nev in zip(res, single, targets, nevs):
        assert len(lam) >= nev, st
        assert len(lam) == len(lam1)
        assert np.max(np.abs(lam - lam1) / np.abs(lam1)) < 1e-13
        ref, _ = shift_invert_eigs(A, B, tau, nev, "TM")
        err = np.array([np.min(np.abs(lam[:nev] - r)) / abs(r) for r in ref])
        assert err.max() < tol, (tau, err)
        assert eig_residuals(A, B, lam[:nev], X[:, :nev]).max() < 1e-12
