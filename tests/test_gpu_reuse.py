"""Factors and Krylov vectors reused across nearby targets.

* A spectral-transformation shift apart from the target (SLEPc's -st_shift): OP is
  (A - sigma B)^-1 B, the eigenvalues are lambda = sigma + 1/theta and `which` still
  measures from the target; the result is the target's nearest eigenvalues, as the
  oracle computes them at the target itself.
* Batched and served eigensolves with a reuse radius: a target near an idle slot's
  shift runs on that slot's factors without re-factorising (optionally started from the
  seeded vector plus the eigenvectors the slot returned last) and gets the same
  eigenpairs as a fresh solve within the solver's tolerance."""
import numpy as np
import pytest

from oracle.eps_ref import eig_residuals, shift_invert_eigs

pytestmark = pytest.mark.gpu


def make_pencil(meta, A, B):
    from kore_gb300 import Pencil, layout_from_params
    return Pencil(A, B, layout=layout_from_params(meta))


def match_eigs(lam, ref):
    return np.array([np.min(np.abs(lam - r)) / abs(r) for r in ref])


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-10)])
def test_shift_apart_from_target(gpu_lib, case, precision, tol):
    from kore_gb300 import EPS
    meta, A, B = case("shell_m1_ek1e-4")
    tau = complex(*meta["tau"])
    nev = meta["nev"]
    ref, _ = shift_invert_eigs(A, B, tau, nev, "TM")
    with make_pencil(meta, A, B) as p:
        E = EPS()
        E.setOperators(p)
        E.setProblemType(EPS.ProblemType.GNHEP)
        E.setDimensions(nev)
        E.setTolerances(1e-15, 100)
        E.setWhichEigenpairs("TM")
        E.setTarget(tau)
        E.setFromOptions({"st_type": "sinvert", "st_shift": tau + 0.01 - 0.01j, "kore_precision": precision,
                          "kore_seed": 4})
        E.solve()
        assert p.sigma == tau + 0.01 - 0.01j
        lam, X = E.eigenvalues(), E.eigenvectors()
        st = E.stats
    assert len(lam) >= nev, st
    assert complex(st["shift_re"], st["shift_im"]) == tau + 0.01 - 0.01j
    assert match_eigs(lam[:nev], ref).max() < tol
    d = np.abs(lam - tau)
    assert np.all(np.diff(d) >= -1e-12 * d.max())           # ordered from the target, not the shift
    assert eig_residuals(A, B, lam[:nev], X[:, :nev]).max() < 1e-12


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-10)])
def test_batched_targets_reuse_nearby_slot(gpu_lib, case, precision, tol):
    """Three targets 0.01 apart through one slot: with a radius of 0.05 the second and third
    run on the first one's factors (warm started); without, each is factorised afresh.
    Both give the oracle's eigenvalues at every target."""
    from kore_gb300 import eigs_targets
    meta, A, B = case("shell_m1_ek1e-4")
    tau = complex(*meta["tau"])
    nev = meta["nev"]
    targets = [tau, tau + 0.01j, tau + 0.02j]
    with make_pencil(meta, A, B) as p:
        reused = eigs_targets(p, targets, nev, "TM", precision, seeds=[7, 8, 9], slots=1, reuse_radius=0.05,
                              warm=True)
        fresh = eigs_targets(p, targets, nev, "TM", precision, seeds=[7, 8, 9], slots=1)
    for k, (t, (lr, Xr, sr), (lf, Xf, sf)) in enumerate(zip(targets, reused, fresh)):
        ref, _ = shift_invert_eigs(A, B, t, nev, "TM")
        assert match_eigs(lr[:nev], ref).max() < tol, (t, sr)
        assert match_eigs(lf[:nev], ref).max() < tol, (t, sf)
        assert eig_residuals(A, B, lr[:nev], Xr[:, :nev]).max() < 1e-12
        if k > 0:
            assert sr["factor_reused"] == 1 and sr["warm_started"] == 1, sr
            assert complex(sr["shift_re"], sr["shift_im"]) == tau, sr
            assert sf["factor_reused"] == 0 and complex(sf["shift_re"], sf["shift_im"]) == t, sf


def test_served_request_reuses_cached_factor(gpu_lib, case):
    """A served eigen request near a target its pencil's plan has already factorised runs on
    those factors (no re-factorisation; here not warm) and matches a fresh solve at its
    target."""
    from kore_gb300.serve import PencilData, Server
    from kore_gb300.structure import layout_from_params
    meta, A, B = case("shell_m2_ek1e-4")
    P = PencilData(A, B, layout=layout_from_params(meta))
    tau = complex(*meta["tau"])
    nev = meta["nev"]
    with Server(workers=1) as srv:
        r0 = srv.result(srv.submit_eigen(P, tau, nev, seed=3))
        r1 = srv.result(srv.submit_eigen(P, tau + 0.01j, nev, seed=4, reuse_radius=0.05, vectors=True))
        hits = srv.stats()["factor_cache_hits"]
    with Server(workers=1) as srv:
        f1 = srv.result(srv.submit_eigen(P, tau + 0.01j, nev, seed=4))
    s1 = r1["stats"]
    assert s1["factor_reused"] == 1 and s1["warm_started"] == 0, s1
    assert complex(s1["shift_re"], s1["shift_im"]) == tau
    assert hits >= 1
    assert r0["stats"]["factor_reused"] == 0
    ref, _ = shift_invert_eigs(A, B, tau + 0.01j, nev, "TM")
    assert match_eigs(r1["evals"][:nev], ref).max() < 1e-10
    assert match_eigs(f1["evals"][:nev], ref).max() < 1e-10
    assert eig_residuals(A, B, r1["evals"][:nev], r1["evecs"][:, :nev]).max() < 1e-12
