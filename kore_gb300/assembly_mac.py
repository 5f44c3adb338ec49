"""Magnetohydrodynamic pencil of kore with a dipole background field and buoyancy,
built on the host from the parameters.

Restates, for a spherical shell (``ricb > 0``) with an imposed dipole field
(``B0 = 'dipole'``), insulating inner core and mantle, uniform magnetic diffusivity,
Boussinesq thermal convection with 'differential' or 'internal' heating and
isothermal or fixed-flux thermal boundaries, what the reference's
``bin/submatrices.py``, ``bin/operators.py`` and ``bin/assemble.py`` compute:

* unknowns in five sections of l-blocks: poloidal and toroidal velocity (degrees lp,
  lt), poloidal and toroidal magnetic field (degrees lt, lp: the dipole is
  equatorially antisymmetric, so b has the opposite symmetry of u,
  ``bin/assemble.py:50-74``), temperature (degrees lp);
* momentum (``bin/operators.py:22-124,136-195``): with the dipole the double-curl
  equation is multiplied by r^2 more and the single-curl one by r^3 more
  (``bin/submatrices.py:204-300``, ``labelit`` rplus), plus the Lorentz force
  (``lorentz``, ``:198-383``, dipole branches: l +- 1 from the poloidal field in
  section u, l from the toroidal field; l from the poloidal and l +- 1 from the
  toroidal field in section v) and the buoyancy ``BV2 L r^6`` (``:386-406``);
* induction (``induction``, ``:471-643``, dipole branches) and magnetic diffusion
  (``:646-696``), the equations multiplied by r^2 (poloidal) and r^3 (toroidal) more;
* heat (``:699-775``): theta, advection of the background temperature, diffusion;
* boundary rows: velocity as in the hydrodynamic problem, insulating magnetic
  boundaries (``bc_b_icb``, ``bc_b_cmb``, ``bin/assemble.py:1472-1560``, inner
  boundary on the first row), thermal (``bc_theta_spherical``, ``:1300-1341``, outer
  boundary on the first row);
* B = diag(-u, -u, -b, -b, theta), A and B divided by ||B||_F (``:582-584,1164-1165``).

The field enters through the Chebyshev coefficients of r^X h^(J)(r), h = r^-2 / 2 the
dipole's poloidal scalar, scaled to unit magnetic energy (``dipole_norm``).  Only the
eigenproblem (no forcing) is assembled.
"""
import contextlib

import numpy as np
import scipy.sparse as ss

from .assembly import (RCMB, RadialOperators, assemble_grid, bc_block, boundary_values, dipole_norm, kron_sum,
                       lazy_blocks, momentum_blocks, velocity_bc_blocks)
from .structure import ell

__all__ = ["mac_pencil", "mac_pencil_parts", "mac_params"]


def _lorentz_u(op, m, lmag_p, lmag_t, lp):
    """Lorentz force in section u (rows of degrees lp), dipole field, before the factor Le^2."""
    h = lambda rx, hx, dx: op(rx, dx, "u", h=hx)
    L = lambda l: l * (l + 1)
    c_lo = lambda l: np.sqrt(l ** 2 - m ** 2) * (l ** 2 - 1) / (2 * l - 1)
    c_hi = lambda l: np.sqrt((1 + l + m) * (1 + l - m)) * l * (l + 2) / (2 * l + 3)
    lo = [(lambda l: -2 * (l ** 2 + 2), h(3, 0, 1)), (lambda l: -2 * (l - 2), h(4, 1, 1)),
          (lambda l: -(l - 4), h(4, 0, 2)), (lambda l: -(l - 2), h(5, 1, 2)),
          (lambda l: L(l) * (l + 2), h(2, 0, 0)), (lambda l: L(l) * (l - 4), h(3, 1, 0)),
          (lambda l: l, h(4, 2, 0)), (lambda l: l, h(5, 3, 0)), (lambda l: 2 + 0 * l, h(5, 0, 3))]
    hi = [(lambda l: -2 * (l ** 2 + 2 * l + 3), h(3, 0, 1)), (lambda l: 2 * (l + 3), h(4, 1, 1)),
          (lambda l: l + 5, h(4, 0, 2)), (lambda l: l + 3, h(5, 1, 2)),
          (lambda l: -L(l) * (l - 1), h(2, 0, 0)), (lambda l: -L(l) * (l + 5), h(3, 1, 0)),
          (lambda l: -(l + 1), h(4, 2, 0)), (lambda l: -(l + 1), h(5, 3, 0)), (lambda l: 2 + 0 * l, h(5, 0, 3))]
    bpol = kron_sum(lp, lmag_p, [(-1, (lambda f: lambda l: c_lo(l) * f(l))(f), M) for f, M in lo] +
                    [(1, (lambda f: lambda l: c_hi(l) * f(l))(f), M) for f, M in hi])
    tor = [(lambda l: -1 + 0 * l, h(3, 0, 0)), (lambda l: -(l ** 2 + l - 1), h(4, 1, 0)),
           (lambda l: 1 + 0 * l, h(4, 0, 1)), (lambda l: 1 + 0 * l, h(5, 1, 1)), (lambda l: 1 + 0 * l, h(5, 0, 2))]
    btor = kron_sum(lp, lmag_t, [(0, (lambda f: lambda l: 2j * m * f(l))(f), M) for f, M in tor])
    return bpol, btor


def _lorentz_v(op, m, lmag_p, lmag_t, lt):
    """Lorentz force in section v (rows of degrees lt), dipole field, before the factor Le^2."""
    h = lambda rx, hx, dx: op(rx, dx, "v", h=hx)
    L = lambda l: l * (l + 1)
    pol = [(lambda l: 4 + 0 * l, h(3, 0, 1)), (lambda l: -2 * L(l), h(3, 1, 0)),
           (lambda l: -L(l), h(4, 2, 0)), (lambda l: 2 + 0 * l, h(4, 0, 2))]
    bpol = kron_sum(lt, lmag_p, [(0, (lambda f: lambda l: 1j * m * f(l))(f), M) for f, M in pol])
    c_lo = lambda l: np.sqrt((l - m) * (l + m)) * (l ** 2 - 1) / (2 * l - 1)
    c_hi = lambda l: -np.sqrt((l + m + 1) * (l + 1 - m)) * l * (l + 2) / (2 * l + 3)
    lo = [(lambda l: l - 2, h(3, 0, 0)), (lambda l: l, h(4, 1, 0)), (lambda l: -2 + 0 * l, h(4, 0, 1))]
    hi = [(lambda l: l + 3, h(3, 0, 0)), (lambda l: l + 1, h(4, 1, 0)), (lambda l: 2 + 0 * l, h(4, 0, 1))]
    btor = kron_sum(lt, lmag_t, [(-1, (lambda f: lambda l: c_lo(l) * f(l))(f), M) for f, M in lo] +
                    [(1, (lambda f: lambda l: c_hi(l) * f(l))(f), M) for f, M in hi])
    return bpol, btor


def _induction(op, m, lp, lt, lmag_p, lmag_t):
    """Induction curl(B0 x u), dipole field: rows of the poloidal field (section f,
    degrees lmag_p) and of the toroidal field (section g, degrees lmag_t), columns of
    the poloidal (lp) and toroidal (lt) velocity."""
    f = lambda rx, hx, dx: op(rx, dx, "f", h=hx)
    g = lambda rx, hx, dx: op(rx, dx, "g", h=hx)
    L = lambda l: l * (l + 1)
    c_lo = lambda l: np.sqrt(l ** 2 - m ** 2) * (l ** 2 - 1) / (2 * l - 1)
    c_hi = lambda l: np.sqrt((l + 1) ** 2 - m ** 2) * l * (l + 2) / (2 * l + 3)
    f_lo = [(lambda l: l - 2, f(2, 0, 0)), (lambda l: l, f(3, 1, 0)), (lambda l: -2 + 0 * l, f(3, 0, 1))]
    f_hi = [(lambda l: -(l + 3), f(2, 0, 0)), (lambda l: -(l + 1), f(3, 1, 0)), (lambda l: -2 + 0 * l, f(3, 0, 1))]
    f_up = kron_sum(lmag_p, lp, [(-1, (lambda q: lambda l: c_lo(l) * q(l))(q), M) for q, M in f_lo] +
                    [(1, (lambda q: lambda l: c_hi(l) * q(l))(q), M) for q, M in f_hi])
    f_ut = kron_sum(lmag_p, lt, [(0, lambda l: -2j * m + 0 * l, f(3, 0, 0))])
    g_pol = [(lambda l: 1 + 0 * l, g(3, 0, 1)), (lambda l: 1 + 0 * l, g(4, 1, 1)),
             (lambda l: -(l ** 2 + l + 1), g(2, 0, 0)), (lambda l: 1 + 0 * l, g(3, 1, 0)),
             (lambda l: L(l) / 2, g(4, 2, 0)), (lambda l: 1 + 0 * l, g(4, 0, 2))]
    g_up = kron_sum(lmag_t, lp, [(0, (lambda q: lambda l: 2j * m * q(l))(q), M) for q, M in g_pol])
    g_lo = [(lambda l: l, g(3, 0, 0)), (lambda l: -2 + 0 * l, g(4, 0, 1)), (lambda l: l - 2, g(4, 1, 0))]
    g_hi = [(lambda l: -2 + 0 * l, g(4, 0, 1)), (lambda l: -(l + 1), g(3, 0, 0)), (lambda l: -(l + 3), g(4, 1, 0))]
    g_ut = kron_sum(lmag_t, lt, [(-1, (lambda q: lambda l: c_lo(l) * q(l))(q), M) for q, M in g_lo] +
                    [(1, (lambda q: lambda l: c_hi(l) * q(l))(q), M) for q, M in g_hi])
    return f_up, f_ut, g_up, g_ut


def mac_pencil_parts(m, symm, Ek, N, lmax, ricb=0.35, Em=None, Le2=None, Prandtl=1.0, cnorm="mag_energy",
                     heating="differential", bci=1, bco=1, bci_thermal=0, bco_thermal=0, Gaspard=1.0,
                     device=None, assemble_on_device=False):
    """(A0, Ab, B, bnorm): the unnormalised eigen pencil with A = A0 + BV2 Ab, where
    BV2 = -Ra Ek^2 / Prandtl is the buoyancy factor (``bin/parameters.py:175-186``), so
    that A is affine in the Rayleigh number; B does not depend on it.
    ``assemble_on_device``: A0 and B assembled on the GPU (``device``, else GPU 0) from the
    radial operators (``assemble_grid``); Ab, one operator per block, stays on the host."""
    if ricb <= 0:
        raise ValueError("the dipole field needs an inner core (ricb > 0)")
    if (lmax - m + 1) % 2:
        raise ValueError("lmax - m + 1 must be even")
    if heating not in ("differential", "internal"):
        raise ValueError(f"heating {heating!r} is not assembled here")
    if Em is None or Le2 is None:
        raise ValueError("Em and Le2 are required")
    N1 = N
    lp, lt = ell(m, lmax, symm)
    lmag_p, lmag_t = ell(m, lmax, -symm)   # b has the opposite symmetry of u
    R = RadialOperators(N, ricb, device=device, field=dipole_norm(ricb, cnorm))
    op = R.op
    mf = float(m)
    L = lambda l: l * (l + 1)
    nb = lp.size

    with lazy_blocks() if assemble_on_device else contextlib.nullcontext():
        A0g, Bg = _mac_blocks(op, mf, L, N, N1, ricb, Ek, Em, Le2, Prandtl, heating, bci, bco, bci_thermal,
                              bco_thermal, Gaspard, lp, lt, lmag_p, lmag_t)
    if assemble_on_device:
        gpu = 0 if device is None else device
        A0 = assemble_grid(A0g, N1, gpu)
        B = assemble_grid(Bg, N1, gpu).real.astype(np.float64)
    else:
        A0 = ss.bmat(A0g, format="csr").astype(np.complex128)
        A0.eliminate_zeros()
        B = ss.block_diag([Bg[k][k] for k in range(5)], format="csr").real.astype(np.float64)
    B.eliminate_zeros()
    Ubuoy = kron_sum(lp, lp, [(0, L, op(6, 0, "u"))])   # L r^6 theta in section u
    n = nb * N1
    Ub = Ubuoy.tocoo()
    Ab = ss.csr_matrix((Ub.data, (Ub.row, Ub.col + 4 * n)), shape=A0.shape, dtype=np.complex128)
    Ab.eliminate_zeros()
    return A0, Ab, B, float(ss.linalg.norm(B))


def _mac_blocks(op, mf, L, N, N1, ricb, Ek, Em, Le2, Prandtl, heating, bci, bco, bci_thermal, bco_thermal,
                Gaspard, lp, lt, lmag_p, lmag_t):
    """The 5 x 5 section grid of A0 and the block diagonal of B (sparse blocks, or
    LazyBlock term lists inside ``lazy_blocks()``)."""
    App, Apt, Atp, Att, Up, Ut = momentum_blocks(op, mf, lp, lt, Ek, 0.0, Gaspard, pu=2, pv=3)
    BCp, BCt = velocity_bc_blocks(lp, lt, N, ricb, bci, bco)
    u_bpol, u_btor = _lorentz_u(op, mf, lmag_p, lmag_t, lp)
    v_bpol, v_btor = _lorentz_v(op, mf, lmag_p, lmag_t, lt)
    f_up, f_ut, g_up, g_ut = _induction(op, mf, lp, lt, lmag_p, lmag_t)

    # b (r^4 and r^5 with the dipole) and magnetic diffusion (uniform diffusivity: the
    # derivative of the profile vanishes and its terms with it)
    Bf = kron_sum(lmag_p, lmag_p, [(0, L, op(4, 0, "f"))])
    Bg = kron_sum(lmag_t, lmag_t, [(0, L, op(5, 0, "g"))])
    Df = kron_sum(lmag_p, lmag_p, [(0, lambda l: -L(l) * L(l), op(2, 0, "f")), (0, lambda l: 2 * L(l), op(3, 1, "f")),
                                   (0, L, op(4, 2, "f"))])
    Dg = kron_sum(lmag_t, lmag_t, [(0, lambda l: 2 * L(l), op(4, 1, "g")), (0, lambda l: -L(l) * L(l), op(3, 0, "g")),
                                   (0, L, op(5, 2, "g"))])

    # heat: theta, advection of the background temperature, diffusion
    if heating == "differential":   # dT/dr = -beta r^-2, equation times r^3
        Th = kron_sum(lp, lp, [(0, lambda l: 1 + 0 * l, op(3, 0, "h"))])
        Hu = kron_sum(lp, lp, [(0, lambda l: L(l) * (ricb / (RCMB - ricb)), op(0, 0, "h"))])
        Dh = kron_sum(lp, lp, [(0, lambda l: -L(l), op(1, 0, "h")), (0, lambda l: 2 + 0 * l, op(2, 1, "h")),
                               (0, lambda l: 1 + 0 * l, op(3, 2, "h"))])
    else:                           # dT/dr = -beta r, equation times r^2
        Th = kron_sum(lp, lp, [(0, lambda l: 1 + 0 * l, op(2, 0, "h"))])
        Hu = kron_sum(lp, lp, [(0, L, op(2, 0, "h"))])
        Dh = kron_sum(lp, lp, [(0, lambda l: -L(l), op(0, 0, "h")), (0, lambda l: 2 + 0 * l, op(1, 1, "h")),
                               (0, lambda l: 1 + 0 * l, op(2, 2, "h"))])

    # boundary rows: insulating magnetic boundaries (inner on the first row), thermal
    Ta = boundary_values(-1, N, 4, ricb)
    Tb = boundary_values(1, N, 5, ricb)

    def rows_f(l):
        r = np.zeros((2, N1), dtype=complex)
        r[0] = l * Ta[:, 0] - ricb * Ta[:, 1]
        r[1] = (l + 1) * Tb[:, 0] + RCMB * Tb[:, 1]
        return r

    rg = np.zeros((2, N1), dtype=complex)
    rg[0] = Ta[:, 0]
    rg[1] = Tb[:, 0]
    rh = np.zeros((2, N1), dtype=complex)
    rh[0] = Tb[:, bco_thermal]
    rh[1] = Ta[:, bci_thermal]
    BCf = bc_block([rows_f(float(l)) for l in lmag_p], 2, N1)
    BCg = bc_block([rg for _ in lmag_t], 2, N1)
    BCh = bc_block([rh for _ in lp], 2, N1)

    thermaD = Ek / Prandtl
    A0 = [[App + BCp, Apt, Le2 * u_bpol, Le2 * u_btor, None],
          [Atp, Att + BCt, Le2 * v_bpol, Le2 * v_btor, None],
          [f_up, f_ut, -Em * Df + BCf, None, None],
          [g_up, g_ut, None, -Em * Dg + BCg, None],
          [Hu, None, None, None, thermaD * Dh + BCh]]
    diag = [-Up, -Ut, -Bf, -Bg, Th]
    B = [[diag[a] if a == b else None for b in range(5)] for a in range(5)]
    return A0, B


def mac_pencil(m, symm, Ek, N, lmax, ricb=0.35, Em=None, Le2=None, Prandtl=1.0, Ra=0.0, with_norm=False, **kw):
    """(A, B) of the eigenproblem as ``bin/assemble.py`` writes them for the dipole MAC
    problem at Rayleigh number Ra (``Ra = Ra_gap / (1 - ricb)^3`` in the reference's
    parameters), both divided by ||B||_F."""
    A0, Ab, B, bnorm = mac_pencil_parts(m, symm, Ek, N, lmax, ricb, Em, Le2, Prandtl, **kw)
    bv2 = -Ra * Ek ** 2 / Prandtl
    A = (A0 + bv2 * Ab) / bnorm
    if with_norm:
        return A.tocsr(), (B / bnorm).tocsr(), bnorm
    return A.tocsr(), (B / bnorm).tocsr()


def mac_params(m, symm, Ek, N, lmax, ricb=0.35, **kw):
    """The parameter mapping structure.layout_from_params expects for mac_pencil."""
    d = dict(m=m, symm=symm, Ek=Ek, N=N, lmax=lmax, ricb=ricb, hydro=1, magnetic=1, thermal=1,
             compositional=0, B0="dipole")
    d.update(kw)
    return d
