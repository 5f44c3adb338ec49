"""numpy restatement of kore's flow diagnostics — TEST INFRASTRUCTURE ONLY.

Used by the tests (and nothing in the product) as the checker of the GPU diagnostics
(``kore_flow_diagnostics``).  It restates, for the hydrodynamic problem in a spherical
shell (ricb > 0, so no parity expansion of the radial coefficients):

* ``bin/utils4pp.py:794-829`` (``diagnose``): Chebyshev-Gauss points x_k = cos((k+1/2)
  pi/N) mapped to r in [ricb, rcmb], with sqrt(1 - x_k^2) quadrature weights;
* ``bin/utils.py:273-314`` (``Dcheb``, ``Dn_cheb``) and ``bin/utils4pp.py:28-51``
  (``funcheb``): a radial function and its r-derivatives from its Chebyshev
  coefficients;
* ``bin/utils4pp.py:163-218`` (``cheb2space_pol``, ``cheb2space_tor``): the radial
  (q), consoidal (s) and toroidal (t) components of degree l and their derivatives;
* ``bin/utils4pp.py:221-296`` (``energy_*``, ``diffus_*``, ``internl_dissip_*``): the
  integrands of the kinetic energy, of the diffusion term integral(u . lap u) and of the
  internal dissipation;
* ``bin/utils4pp.py:54-64`` (``cg_quad``) for the radial integrals;
* ``bin/spin_doctor.py:148-160,225-236`` for the sums over l, the scaling by
  OmgTau * Ek, and the power-balance residuals resid0 = |Dint + Dkin| / max and
  resid1 = |2 sigma KE - Dkin| / max (no forcing, no magnetic field, no buoyancy).
"""
import numpy as np
import numpy.polynomial.chebyshev as ch


def quad_grid(N, ricb, rcmb=1.0):
    """Chebyshev-Gauss points in r, their position in the basis domain, and sqrt(1-x^2)."""
    i = np.arange(N)
    xk = np.cos((i + 0.5) * np.pi / N)
    rk = 0.5 * (rcmb - ricb) * (xk + 1) + ricb
    x0 = 2 * (rk - ricb) / (rcmb - ricb) - 1
    return rk, x0, np.sqrt(1 - xk ** 2)


def dcheb(ck, ricb, rcmb=1.0):
    """Chebyshev coefficients of d/dr of the expansion ck on [ricb, rcmb]."""
    s = ck.size
    out = np.zeros_like(ck)
    if s > 1:
        out[-2] = 2.0 * (s - 1) * ck[-1]
    for k in range(s - 3, -1, -1):
        out[k] = out[k + 2] + 2.0 * (k + 1) * ck[k + 1]
    out[0] = out[0] / 2.0
    return 2 * out / (rcmb - ricb)


def fun_and_derivs(ck, x0, ricb, n, rcmb=1.0):
    """The expansion ck and its first n r-derivatives at the points x0 (columns)."""
    out = np.zeros((x0.size, n + 1), dtype=ck.dtype)
    c = ck
    for j in range(n + 1):
        out[:, j] = ch.chebval(x0, c)
        c = dcheb(c, ricb, rcmb)
    return out


def flow_l(l, coeffs, toroidal, N, ricb, rcmb=1.0):
    """(kinetic energy, diffusion, internal dissipation) radial integrals of degree l."""
    rk, x0, sqx = quad_grid(N, ricb, rcmb)
    r2 = rk ** 2
    L = l * (l + 1)
    f0 = 4 * np.pi / (2 * l + 1)
    if not toroidal:
        p = fun_and_derivs(coeffs, x0, ricb, 3, rcmb)
        q0 = L * p[:, 0] / rk
        s0 = p[:, 1] + p[:, 0] / rk
        q1 = (L * p[:, 1] - q0) / rk
        s1 = p[:, 2] + q1 / L
        q2 = (L * p[:, 2] - 2 * q1) / rk
        s2 = p[:, 3] + q2 / L
        ke = f0 * (r2 * np.abs(q0) ** 2 + r2 * L * np.abs(s0) ** 2)
        dk = 2 * np.real(f0 * (L * r2 * np.conj(s0) * s2 + 2 * rk * L * np.conj(s0) * s1
                               - L ** 2 * np.conj(s0) * s0 - (l ** 2 + l + 2) * np.conj(q0) * q0
                               + 2 * rk * np.conj(q0) * q1 + r2 * np.conj(q0) * q2
                               + 2 * L * (np.conj(q0) * s0 + q0 * np.conj(s0))))
        di = 2 * f0 * (L * np.abs(q0 + rk * s1 - s0) ** 2 + 3 * np.abs(rk * q1) ** 2
                       + L * (l - 1) * (l + 2) * np.abs(s0) ** 2)
    else:
        t = fun_and_derivs(coeffs, x0, ricb, 2, rcmb)
        t0, t1, t2 = t[:, 0], t[:, 1], t[:, 2]
        ke = f0 * r2 * L * np.abs(t0) ** 2
        dk = 2 * np.real(f0 * (L * r2 * np.conj(t0) * t2 + 2 * rk * L * np.conj(t0) * t1 - L ** 2 * np.conj(t0) * t0))
        di = 2 * f0 * (L * np.abs(rk * t1 - t0) ** 2 + L * (l - 1) * (l + 2) * np.abs(t0) ** 2)
    quad = lambda f: (np.pi / N) * np.sum(sqx * f) * (rcmb - ricb) / 2
    return quad(ke), quad(dk), quad(di)


def flow_diagnostics(x, lp, lt, N, ricb, lam=None, Ek=1.0, OmgTau=1.0):
    """Per eigenvector x (original order: poloidal blocks of degrees lp, then toroidal
    blocks of degrees lt, N coefficients each): KE, KP, KT, Dkin, Dint and, with the
    eigenvalue lam, the power-balance residuals resid0 and resid1."""
    nb = len(lp)
    P = np.asarray(x[:nb * N]).reshape(nb, N)
    T = np.asarray(x[nb * N:2 * nb * N]).reshape(len(lt), N)
    kp = np.zeros(3)
    kt = np.zeros(3)
    for b, l in enumerate(lp):
        kp += np.array(flow_l(int(l), P[b], False, N, ricb))
    for b, l in enumerate(lt):
        kt += np.array(flow_l(int(l), T[b], True, N, ricb))
    tot = kp + kt
    out = {"KE": tot[0], "KP": kp[0], "KT": kt[0], "Dkin0": tot[1], "Dint0": tot[2],
           "Dkin": OmgTau * Ek * tot[1], "Dint": OmgTau * Ek * tot[2]}
    out["resid0"] = abs(tot[2] + tot[1]) / max(abs(tot[2]), abs(tot[1]))
    if lam is not None:
        sigma = complex(lam).real
        a, b = 2 * sigma * out["KE"], out["Dkin"]
        out["resid1"] = abs(a - b) / max(abs(a), abs(b))
    return out
