"""How well the computed eigenvalues of a pencil are determined, measured with the FP64
GPU path.

At kore's small Ekman numbers the eigenvalues near a target are extremely
ill-conditioned: on the 240,000-unknown shell (Ek = 1e-7, target 0.5i) the condition
numbers ||x|| ||y|| / |y^H B x| of the 16 nearest eigenvalues are 1e15-1e17, so a
backward-stable solver determines them only to about kappa * u, far above 1e-10.  Two
FP64 runs that share one factorisation agree much more closely than that (they see the
same rounding of A - tau B), which says nothing about the accuracy of either.  This
module measures what a comparison can rest on:

* ``reference``: the FP64 path at twice nev, the eigenvalue set the others are compared
  with;
* ``perturbation_band``: the FP64 path again on A with every entry multiplied by
  (1 + eps u), u uniform in [-1, 1] and eps at rounding level, and how far that moves
  the eigenvalues (relative distance to the nearest reference eigenvalue): the spread
  that rounding alone produces;
* ``condition_numbers``: kappa_i = ||x_i|| ||y_i|| / |y_i^H B x_i| from the left
  eigenvectors y (an eigensolve of the adjoint pencil (A^H, B^T) at conj(tau)).

``compare`` then places a computed set of eigenpairs against them: distances to the
FP64 eigenvalues (reference and perturbed runs), membership of the window of the nev
nearest, residuals, and the first-order bound kappa * eta.
"""
import numpy as np
import scipy.sparse as ss
import scipy.sparse.linalg as ssl

from .solver import EPS, Pencil


def rel_residuals(A, B, lam, X):
    """||A x - lambda B x|| / ((||A||_1 + |lambda| ||B||_1) ||x||) per pair."""
    na, nb = ssl.norm(A, 1), ssl.norm(B, 1)
    return np.array([np.linalg.norm(A @ X[:, j] - l * (B @ X[:, j])) / ((na + abs(l) * nb) * np.linalg.norm(X[:, j]))
                     for j, l in enumerate(lam)])


def solve(p, tau, nev, precision="fp64", seed=1, which="TM", tol=1e-15, maxit=100):
    """One eigensolve through the public EPS API; returns (eigenvalues, eigenvectors)."""
    E = EPS()
    E.setOperators(p)
    E.setProblemType(EPS.ProblemType.GNHEP)
    E.setDimensions(nev)
    E.setTolerances(tol, maxit)
    E.setWhichEigenpairs(which)
    E.setTarget(tau)
    E.setFromOptions({"st_type": "sinvert", "kore_precision": precision, "kore_seed": seed})
    p.sigma = None
    E.solve()
    return E.eigenvalues(), E.eigenvectors()


def perturbed(A, eps, seed):
    """A with every stored entry multiplied by (1 + eps u), u uniform in [-1, 1]."""
    Ap = ss.csr_matrix(A, copy=True)
    Ap.data = Ap.data * (1.0 + eps * np.random.default_rng(seed).uniform(-1.0, 1.0, Ap.data.shape))
    return Ap


def reference(A, B, layout, tau, nev, seed=1):
    """FP64 eigenpairs nearest tau (2 nev of them) and their residuals."""
    with Pencil(A, B, layout=layout) as p:
        lam, X = solve(p, tau, 2 * nev, "fp64", seed)
    return lam, X, rel_residuals(A, B, lam, X)


def perturbation_band(A, B, layout, tau, nev, ref, eps=1e-16, seeds=(5, 6)):
    """FP64 eigenvalues of A perturbed at level eps (one run per seed) and the largest
    relative distance of any of them to the reference set: (band, list of sets)."""
    sets = []
    band = 0.0
    for s in seeds:
        with Pencil(perturbed(A, eps, s), B, layout=layout) as p:
            lam, _ = solve(p, tau, nev, "fp64", 2)
        sets.append(lam[:nev])
        band = max(band, max(np.min(np.abs(ref - l)) / abs(l) for l in lam[:nev]))
    return band, sets


def condition_numbers(A, B, layout, tau, lam, X, nev_left=None, seed=1):
    """kappa_i = ||x_i|| ||y_i|| / |y_i^H B x_i| for the eigenpairs (lam, X), with y_i the
    left eigenvector whose eigenvalue is nearest lam_i (NaN when none is within 1e-3)."""
    with Pencil(A.conj().T.tocsr(), B.T.tocsr(), layout=layout) as q:
        ll, Y = solve(q, np.conj(tau), nev_left or 2 * len(lam), "fp64", seed)
    ll = np.conj(ll)
    kap = np.full(len(lam), np.nan)
    for i, l in enumerate(lam):
        j = int(np.argmin(np.abs(ll - l)))
        if abs(ll[j] - l) <= 1e-3 * abs(l):
            x, y = X[:, i], Y[:, j]
            kap[i] = np.linalg.norm(x) * np.linalg.norm(y) / abs(np.vdot(y, B @ x))
    return kap


def compare(A, B, tau, nev, lam, X, ref, ref_res, band, sets, kappa=None):
    """Where the eigenpairs (lam, X) stand against the FP64 measurements.

    Returns a dict: ``d`` relative distance of each eigenvalue to the nearest FP64
    eigenvalue (reference or perturbed runs), ``band``, ``within_band`` (count with d <=
    4 band or d <= 1e-10), ``in_window`` (count no farther from tau than the reference's
    (nev+1)-th nearest eigenvalue), ``resid`` and ``fp64_resid`` maxima, and with kappa
    the count with d <= kappa (||A|| + |lambda| ||B||) / |lambda| * eta.
    """
    lam = np.asarray(lam)[:nev]
    pool = np.concatenate([np.asarray(ref)] + [np.asarray(s) for s in sets])
    d = np.array([np.min(np.abs(pool - l)) / abs(l) for l in lam])
    dist = np.sort(np.abs(np.asarray(ref) - tau))
    r_out = dist[nev] if len(dist) > nev else np.inf
    res = rel_residuals(A, B, lam, X[:, :nev])
    out = {"d": d, "d_max": float(d.max()), "band": float(band),
           "within_band": int(np.sum((d <= 4.0 * band) | (d <= 1e-10))),
           "in_window": int(np.sum(np.abs(lam - tau) <= r_out * (1 + 1e-12))),
           "match_1e-10": int(np.sum(d <= 1e-10)),
           "resid": float(res.max()), "fp64_resid": float(np.max(ref_res[:nev])), "n": int(len(lam))}
    if kappa is not None:
        na, nb = ssl.norm(A, 1), ssl.norm(B, 1)
        bound = kappa * (na + np.abs(lam) * nb) / np.abs(lam) * res
        ok = np.isfinite(bound)
        out["kappa_min"] = float(np.nanmin(kappa)) if ok.any() else None
        out["kappa_max"] = float(np.nanmax(kappa)) if ok.any() else None
        out["kappa_known"] = int(ok.sum())
        out["within_kappa_eta"] = int(np.sum(d[ok] <= bound[ok]))
    return out
