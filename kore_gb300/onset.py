"""Critical Rayleigh number of convective onset, with the GPU eigensolver.

Restates the search of ``tests/jones2000/find_Rac.py:36-78`` (the same script drives
``tests/dormy2004``): the growth rate sigma(Ra) is the largest real part among the
converged eigenvalues of one solve (``get_sigma``, ``find_Rac.py:36-56``), and the
critical Rayleigh number is its root in log10(Ra).  A bracket is searched from a
starting point in steps of ``dx`` (downwards while the mode grows, upwards while it
decays; ``bracket_brentq``, ``find_Rac.py:59-78``), then refined with Brent's method
(scipy ``brentq`` with ``xtol = rtol = tol``, as the reference calls it).

The reference re-assembles A and B for every Ra and runs ``bin/solve.py`` on them.
Only the buoyancy coupling of A depends on Ra, so here A(Ra) is the affine
interpolation of two assemblies (``tests/golden/make_fixtures.py`` writes them from the
reference) and every step is one plan upload, one factorisation and one eigensolve on
the device.
"""
import numpy as np
import scipy.sparse as ss
from scipy.optimize import brentq

from .solver import EPS, Pencil

__all__ = ["OnsetSearch"]


class OnsetSearch:
    """A(Ra) = A_a + (Ra - Ra_a) / (Ra_b - Ra_a) dA with B fixed; eigensolves around
    `tau` with SLEPc's `which` (``'TR'`` in the reference's onset tests)."""

    def __init__(self, A_a, dA, Ra_a, Ra_b, B, layout, nev=12, which="TR", tau=0.0, tol=1e-15, maxit=50,
                 precision="fp64", seed=1, device=0):
        self.A_a = ss.csr_matrix(A_a)
        self.dA = ss.csr_matrix(dA)
        self.Ra_a, self.Ra_b = float(Ra_a), float(Ra_b)
        self.B = B
        self.layout = layout
        self.nev, self.which, self.tau, self.tol, self.maxit = nev, which, complex(tau), tol, maxit
        self.precision, self.seed, self.device = precision, seed, device
        self.cache = {}          # Ra -> (sigma, eigenvalue with the largest real part)
        self.evaluations = 0

    def A(self, Ra):
        return (self.A_a + ((Ra - self.Ra_a) / (self.Ra_b - self.Ra_a)) * self.dA).tocsr()

    def leading(self, Ra):
        """(growth rate, eigenvalue) of the leading mode at Ra (find_Rac.py: get_sigma)."""
        if Ra in self.cache:
            return self.cache[Ra]
        with Pencil(self.A(Ra), self.B, layout=self.layout, device=self.device) as p:
            E = EPS()
            E.setOperators(p)
            E.setProblemType(EPS.ProblemType.GNHEP)
            E.setDimensions(self.nev)
            E.setTolerances(self.tol, self.maxit)
            E.setWhichEigenpairs(self.which)
            E.setTarget(self.tau)
            E.setFromOptions({"st_type": "sinvert", "kore_precision": self.precision, "kore_seed": self.seed})
            E.solve()
            lam = E.eigenvalues()
        self.evaluations += 1
        if len(lam) == 0:
            raise RuntimeError(f"no eigenpair converged at Ra = {Ra:g}")
        i = int(np.argmax(lam.real))
        self.cache[Ra] = (float(lam[i].real), complex(lam[i]))
        return self.cache[Ra]

    def sigma(self, log10_ra):
        return self.leading(10.0 ** log10_ra)[0]

    def bracket(self, x1, x2=None, dx=0.01, maxsteps=100):
        """A bracket [x1, x2] of the growth-rate root in log10(Ra) (find_Rac.py: bracket_brentq).
        The search gives up (RuntimeError) after ``maxsteps`` steps of dx without a sign change."""
        y1 = self.sigma(x1)
        dx = abs(dx)
        if x2 is not None:
            y2 = self.sigma(x2)
            if y1 * y2 > 0:
                if abs(y2) < abs(y1):
                    x1, y1 = x2, y2
                x2 = None
        if x2 is None:
            step = -dx if y1 > 0 else dx
            x2 = x1
            for _ in range(maxsteps):
                x2 += step
                y2 = self.sigma(x2)
                if y1 * y2 < 0:
                    break
                x1, y1 = x2, y2
            else:
                raise RuntimeError(f"no sign change of the growth rate within {maxsteps} steps of {dx} from {x1 - maxsteps * step:g}")
        return x1, x2

    def critical(self, log10_ra0, dx=0.01, tol=1e-6, maxiter=200, maxsteps=100):
        """(Ra_c, omega_c): the Rayleigh number where the leading growth rate vanishes and the
        frequency of that mode (the imaginary part of its eigenvalue)."""
        x1, x2 = self.bracket(log10_ra0, dx=dx, maxsteps=maxsteps)
        lo, hi = min(x1, x2), max(x1, x2)
        xc = brentq(self.sigma, lo, hi, xtol=tol, rtol=tol, maxiter=maxiter)
        Ra_c = 10.0 ** xc
        return Ra_c, self.leading(Ra_c)[1].imag
