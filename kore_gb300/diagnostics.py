"""Diagnostics of computed eigenmodes: what ``bin/spin_doctor.py`` prints for the
hydrodynamic problem, computed on the GPU (``kore_flow_diagnostics``).

For each eigenvector (velocity part, ``bin/assemble.py``'s order: poloidal degrees
then toroidal degrees, N Chebyshev coefficients each) and its eigenvalue
lambda = sigma + i omega:

* KE, KP, KT: kinetic energy, total, poloidal and toroidal (``spin_doctor.py:148-150``);
* Dkin = OmgTau Ek integral(u . lap u) and Dint = OmgTau Ek (internal dissipation)
  (``:151-153``);
* resid0 = |Dint + Dkin| / max(|Dint|, |Dkin|) and resid1 = |2 sigma KE - Dkin| /
  max(|2 sigma KE|, |Dkin|): the power balance of an unforced hydrodynamic mode
  (``:225-236``).  Both are small for a resolved, accurate eigenpair whatever the size
  of the problem, so they check eigenvectors where no oracle can run.

The radial integrals per degree come from the GPU; the sums over degrees and the
residuals are formed here.
"""
import numpy as np

from . import _lib as L
from .structure import ell


def flow_integrals(X, m, symm, lmax, N, ricb, device=0):
    """Per vector (columns of X, original order, velocity part first) and degree block:
    (kinetic energy, diffusion, internal dissipation) integrals, shape (k, blocks, 3),
    with the degrees of the blocks (poloidal first, then toroidal)."""
    lp, lt = ell(m, lmax, symm)
    nb = len(lp) + len(lt)
    X = np.asarray(X)
    if X.ndim == 1:
        X = X[:, None]
    k = X.shape[1]
    xs = np.ascontiguousarray(X[:nb * N, :].T, dtype=np.complex128)   # (k, nb N)
    out = np.zeros((k, nb, 3))
    lpi = L.as_i32(lp)
    lti = L.as_i32(lt)
    L.check(L.load().kore_flow_diagnostics(int(device), int(N), float(ricb), len(lp), L.ptr(lpi), len(lt),
                                           L.ptr(lti), L.ptr(xs), k, L.ptr(out)), "kore_flow_diagnostics")
    return out, np.concatenate([lp, lt])


def flow_diagnostics(X, lam, m, symm, lmax, N, ricb, Ek, OmgTau=1.0, device=0):
    """spin_doctor's hydrodynamic power balance of eigenpairs (lam, X): a list of dicts."""
    per, _ = flow_integrals(X, m, symm, lmax, N, ricb, device)
    npol = len(ell(m, lmax, symm)[0])
    out = []
    for j, l in enumerate(np.atleast_1d(lam)):
        kp = per[j, :npol].sum(axis=0)
        kt = per[j, npol:].sum(axis=0)
        tot = kp + kt
        d = {"KE": tot[0], "KP": kp[0], "KT": kt[0], "Dkin0": tot[1], "Dint0": tot[2],
             "Dkin": OmgTau * Ek * tot[1], "Dint": OmgTau * Ek * tot[2]}
        d["resid0"] = abs(tot[2] + tot[1]) / max(abs(tot[2]), abs(tot[1]))
        a, b = 2 * complex(l).real * d["KE"], d["Dkin"]
        d["resid1"] = abs(a - b) / max(abs(a), abs(b))
        out.append(d)
    return out
