"""scipy FP64 restatement of ``bin/solve.py``'s arithmetic — TEST INFRASTRUCTURE ONLY.

Used by the tests and the CPU-baseline leg of ``bench.py`` as the checker; never by
the product path.

Reference behaviour restated here:

* ``bin/utils.py:1253-1256`` ``load_csr``: CSR from an ``np.savez`` archive.
* ``bin/solve.py:91-123``: SLEPc EPS, problem type GNHEP, ``nev`` from the
  parameters, tolerances ``(tol, maxit)``, ``which`` from ``which_eigenpairs``,
  target ``tau``, spectral transformation shift-and-invert from argv.  SLEPc sorts
  the back-transformed eigenvalues lambda with the comparison function of ``which``
  (a target criterion measures the distance to ``tau``), so the oracle computes more
  Ritz pairs than requested and applies the same ordering.
* ``bin/solve.py:145-158``: eigenvectors normalised to unit 2-norm.
* ``bin/solve.py:207-233``: forced solve by one direct LU solve.
"""
import numpy as np
import scipy.sparse as ss
import scipy.sparse.linalg as ssl

WHICH = ("LM", "SM", "LR", "SR", "LI", "SI", "TM", "TR", "TI")


def load_csr_npz(path, prefix=""):
    """CSR matrix from a ``np.savez`` archive (``bin/utils.py:1253-1256``)."""
    z = np.load(path)
    return ss.csr_matrix((z[prefix + "data"], z[prefix + "indices"], z[prefix + "indptr"]),
                         shape=tuple(z[prefix + "shape"]))


def which_key(lam, which, tau):
    """Sort key for SLEPc's comparison functions; ascending key = wanted first.

    LM/SM: |lambda| descending/ascending; LR/SR: Re lambda; LI/SI: Im lambda;
    TM/TR/TI: |lambda - tau|, |Re(lambda - tau)|, |Im(lambda - tau)| ascending.
    """
    lam = np.asarray(lam)
    d = lam - tau
    return {
        "LM": -np.abs(lam), "SM": np.abs(lam),
        "LR": -lam.real, "SR": lam.real,
        "LI": -lam.imag, "SI": lam.imag,
        "TM": np.abs(d), "TR": np.abs(d.real), "TI": np.abs(d.imag),
    }[which]


def sort_which(lam, which, tau):
    return np.argsort(which_key(lam, which, tau), kind="stable")


def shift_invert_eigs(A, B, tau, nev, which="TM", over=None, tol=0.0, seed=0, ncv=None):
    """Eigenpairs of A x = lambda B x nearest ``tau`` in the sense of ``which``.

    Factor A - tau*B once (SuperLU), run ARPACK on OP = (A - tau B)^-1 B, map
    theta -> lambda = tau + 1/theta, order by ``which`` and keep ``nev``.
    ``over`` Ritz pairs are computed (default ``nev`` for TM, else 3*nev+10) so that
    a non-magnitude criterion sees enough candidates.
    Returns (lam[nev], X[n, nev]) with unit-2-norm columns.
    """
    n = A.shape[0]
    M = (A - tau * B).tocsc().astype(np.complex128)
    lu = ssl.splu(M, permc_spec="COLAMD")
    Bc = B.tocsr().astype(np.complex128)
    op = ssl.LinearOperator((n, n), matvec=lambda x: lu.solve(Bc @ x), dtype=np.complex128)
    if over is None:
        over = nev if which == "TM" else 3 * nev + 10
    k = min(over, n - 2)
    rng = np.random.default_rng(seed)
    v0 = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    if ncv is None:
        ncv = min(n, max(2 * k + 1, k + 16))
    theta, V = ssl.eigs(op, k=k, which="LM", v0=v0, tol=tol, ncv=ncv)
    lam = tau + 1.0 / theta
    order = sort_which(lam, which, tau)[:nev]
    lam = lam[order]
    X = V[:, order]
    X = X / np.linalg.norm(X, axis=0, keepdims=True)
    return lam, X


def forced_solve(A, b):
    """x = A^-1 b by one sparse direct solve (``-ksp_type preonly -pc_type lu``)."""
    lu = ssl.splu(A.tocsc().astype(np.complex128), permc_spec="COLAMD")
    return lu.solve(np.asarray(b, dtype=np.complex128))


def eig_residuals(A, B, lam, X):
    """Relative eigen-residuals ||A x - lambda B x|| / ((||A||_1 + |lambda| ||B||_1) ||x||)."""
    na = ssl.norm(A, 1)
    nb = ssl.norm(B, 1)
    out = []
    for j, l in enumerate(np.atleast_1d(lam)):
        x = X[:, j]
        r = A @ x - l * (B @ x)
        out.append(np.linalg.norm(r) / ((na + abs(l) * nb) * np.linalg.norm(x)))
    return np.array(out)


def solve_residual(M, x, b):
    """||b - M x|| / (||M||_1 ||x|| + ||b||)."""
    r = b - M @ x
    return np.linalg.norm(r) / (ssl.norm(M, 1) * np.linalg.norm(x) + np.linalg.norm(b))
