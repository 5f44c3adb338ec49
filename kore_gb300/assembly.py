"""Hydrodynamic pencil of kore, built on the host from the parameters.

Restates, for the hydrodynamic problem in a spherical shell (``ricb > 0``, no
magnetic field, no buoyancy, Boussinesq), what the reference computes in three
stages:

* ``bin/submatrices.py``: radial operators ``r^X D^Y`` in the Gegenbauer (ultraspherical)
  basis.  Chebyshev coefficients of powers of r (``bin/utils.py:251-269``), basis
  conversion C^(l) -> C^(l+1) (``Slam``, ``bin/utils.py:911-926``), derivatives
  (``Dlam``, ``bin/utils.py:895-908``) and the multiplication operator by a series in
  C^(l) (``Mlam``, ``bin/utils.py:962-1051``), assembled as
  ``G[g][g-Y] * M(S_Y r^X, Y) * D_Y`` with the top ``g`` rows left empty for the tau
  boundary rows (``bin/submatrices.py:540-590``).  ``g`` = 4 for the poloidal (2curl)
  equation, 2 for the toroidal (1curl) one.
* ``bin/operators.py:22-124,141-215``: time-derivative, Coriolis and viscous terms
  with their degree-dependent coefficients (non-dipole, non-anelastic branches).
* ``bin/assemble.py``: A = i w u + Coriolis - viscous per degree l, Coriolis coupling
  l -> l+-1 between the poloidal and toroidal sections, tau rows from
  ``bc_u_spherical`` (``bin/assemble.py:1188-1296``), B = -u, both divided by ||B||_F
  for the eigenproblem (``:582-584,1164-1165``); forcing vectors 7, 9 and 10
  (``:279-427``).

The multiplication operator uses the ultraspherical linearisation coefficients of
Olver & Townsend (SIAM Review 55, 2013): a closed-form first coefficient followed by
a three-term ratio recurrence, evaluated here for all (row, column) pairs of the
band at once.
"""
import contextlib
import math
import threading

import numpy as np
import scipy.fft as sfft
import scipy.sparse as ss

from .structure import ell, radial_size

RCMB = 1.0


def ncheb(Ek):
    """Radial truncation for an Ekman number (``bin/parameters.py:6-16``)."""
    out = int(17 * Ek ** -0.2) if Ek != 0 else 48
    return max(48, out + out % 2)


def gauss_radii(N, ricb, rcmb=RCMB):
    """The radii of the N Chebyshev-Gauss points x_i = cos(pi (i + 1/2) / N)."""
    i = np.arange(N)
    xi = np.cos(np.pi * (i + 0.5) / N)
    if ricb == 0:
        return rcmb * xi
    return ricb + (rcmb - ricb) * (xi + 1) / 2.0


def chebco_values(fi, tol):
    """Chebyshev coefficients of the function whose values at the Chebyshev-Gauss points
    are fi (DCT-II), entries of magnitude <= tol set to zero (``bin/utils.py:200-222``)."""
    N = fi.size
    out = sfft.dct(fi, type=2) / N
    out[0] = out[0] / 2.0
    out[np.abs(out) <= tol] = 0.0
    return out


def chebco(powr, N, tol, ricb, rcmb=RCMB):
    """First N Chebyshev coefficients of r^powr on [ricb, rcmb] (``bin/utils.py:251-269``)."""
    return chebco_values(gauss_radii(N, ricb, rcmb) ** powr, tol)


# Poloidal scalar of the dipole background field outside a point dipole, h(r) = r^-2 / 2,
# and its r-derivatives: h^(j)(r) = c_j r^e_j (``bin/utils.py:555-760``, kind 'dipole').
_DIPOLE_H = ((0.5, -2), (-1.0, -3), (3.0, -4), (-12.0, -5))


def dipole_h(r, j, rpow=0):
    """r^rpow times the j-th r-derivative of the dipole's poloidal scalar."""
    c, e = _DIPOLE_H[j]
    return c * r ** (e + rpow)


def dipole_norm(ricb, cnorm="mag_energy"):
    """Amplitude of the dipole background field (``bin/utils.py:837-890``): unit total
    magnetic energy in the shell ('mag_energy', twice that for 'Schmitt2012', by a
    240-point Chebyshev-Gauss quadrature), unit rms radial field at the outer boundary
    ('rms_cmb'), or a number given as is."""
    l, L = 1, 2
    if cnorm == "rms_cmb":
        return float(np.sqrt(2 * l + 1) / (L * dipole_h(np.array([1.0]), 0)[0]))
    if cnorm in ("mag_energy", "Schmitt2012"):
        N = 240
        xk = np.cos((np.arange(N) + 0.5) * np.pi / N)
        sqx = np.sqrt(1 - xk ** 2)
        rk = 0.5 * (1 - ricb) * (xk + 1) + ricb
        y0, y1 = dipole_h(rk, 0), dipole_h(rk, 1)
        f0 = 4 * np.pi * L / (2 * l + 1)
        integ = (np.pi / N) * ((1 - ricb) / 2) * np.sum(sqx * f0 * ((L + 1) * y0 ** 2 + 2 * rk * y0 * y1 + rk ** 2 * y1 ** 2))
        return float((1.0 if cnorm == "mag_energy" else 2.0) / np.sqrt(integ))
    return float(cnorm)


def conv_mat(lam, N):
    """C^(lam) -> C^(lam+1) coefficient conversion (bidiagonal, offsets 0 and 2)."""
    if lam == 0:
        d0 = 0.5 * np.ones(N)
        d0[0] = 1.0
        d2 = -0.5 * np.ones(N - 2)
    else:
        t = np.arange(0.0, N)
        d0 = lam / (lam + t)
        d2 = -lam / (lam + t[2:])
    return ss.diags([d0, d2], [0, 2], shape=(N, N), format="csr")


def diff_mat(lam, N, ricb, rcmb=RCMB):
    """d^lam/dr^lam from C^(0) to C^(lam) coefficients."""
    c1 = (1.0 / rcmb) ** lam if ricb == 0 else (2.0 / (rcmb - ricb)) ** lam
    c2 = math.factorial(lam - 1) * 2.0 ** (lam - 1)
    t = lam + np.arange(0, N - lam, dtype=float)
    return c1 * c2 * ss.diags(t, lam, shape=(N, N), format="csr")


def _lin_coeff_first(s, lam, j, k):
    """Closed form of the first linearisation coefficient c_s^lam(j, k) (vectorised)."""
    s = np.asarray(s, dtype=np.int64)
    j = np.asarray(j, dtype=np.int64)
    k = np.asarray(k, dtype=np.int64)
    p1 = np.ones(s.shape)
    p3 = np.ones(s.shape)
    smax = int(s.max()) if s.size else 0
    for t in range(smax):
        on = t < s
        p1 = np.where(on, p1 * (lam + t) / float(1 + t), p1)
        p3 = np.where(on, p3 * (2 * lam + j + k - 2 * s + t) / (lam + j + k - 2 * s + t), p3)
    p2 = np.ones(s.shape)
    p4 = np.ones(s.shape)
    js = j - s
    jmax = int(js.max()) if js.size else 0
    for t in range(jmax):
        on = t < js
        p2 = np.where(on, p2 * (lam + t) / float(1 + t), p2)
        p4 = np.where(on, p4 * (k - s + 1 + t) / (k - s + lam + t), p4)
    return p1 * p2 * p3 * p4 * (j + k + lam - 2.0 * s) / (j + k + lam - s)


def mult_mat(a0, lam):
    """Multiplication by the C^(lam) series a0, as an operator on C^(lam) coefficients
    (no parity reduction: the shell case)."""
    a0 = np.asarray(a0, dtype=float)
    N = a0.size
    if not np.any(a0):
        return ss.csr_matrix((N, N))
    if lam == 0:
        a2 = a0.copy()
        a2[0] *= 2.0
        i = np.arange(N)
        T = a2[np.abs(i[:, None] - i[None, :])]
        Hk = i[:, None] + i[None, :]
        H = np.where(Hk < N, a2[np.minimum(Hk, N - 1)], 0.0)
        H[0, :] = 0.0
        return ss.csr_matrix(0.5 * (T + H))
    bw = int(np.nonzero(a0)[0].max())
    a1 = np.zeros(2 * N)
    a1[:N] = a0
    rows, cols = [], []
    for j in range(N):
        k1, k2 = max(0, j - bw - 1), min(N, j + bw + 2)
        for k in range(k1, k2):
            rows.append(j)
            cols.append(k)
    rows = np.array(rows)
    cols = np.array(cols)
    # pair (j, k): sum over s = s0..k of a1[2s + j - k] * c_s, with c the recurrence
    # started at s0 = max(0, k - j) for the index pair (k, |j - k|)
    s0 = np.maximum(0, cols - rows)
    jj = cols.copy()
    kk = np.abs(rows - cols)
    c = _lin_coeff_first(s0, lam, jj, kk)
    nsteps = cols - s0 + 1
    acc = a1[2 * s0 + rows - cols] * c
    s = s0.astype(float)
    kcur = kk.astype(float)
    jf = jj.astype(float)
    for step in range(1, int(nsteps.max()) if nsteps.size else 0):
        on = step < nsteps
        t1 = (jf + kcur + lam - s) * (lam + s) * (jf - s) * (2 * lam + jf + kcur - s) * (kcur - s + lam)
        t2 = (jf + kcur + lam - s + 1) * (s + 1) * (lam + jf - s - 1) * (lam + jf + kcur - s) * (kcur - s + 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            cn = c * t1 / t2
        c = np.where(on, cn, c)
        s = np.where(on, s + 1, s)
        kcur = np.where(on, kcur + 2, kcur)
        idx = np.where(on, (2 * s + rows - cols).astype(np.int64), 0)
        acc = acc + np.where(on, a1[idx] * c, 0.0)
    M = ss.csr_matrix((acc, (rows, cols)), shape=(N, N))
    M.eliminate_zeros()
    return M


def mult_mat_gpu(a0, lam, device=0):
    """``mult_mat`` computed on the GPU (``kore_gegenbauer_mult``): the same operator,
    one thread per band entry."""
    from . import _lib as L
    a0 = np.ascontiguousarray(a0, dtype=np.float64)
    N = a0.size
    nz = np.nonzero(a0)[0]
    if nz.size == 0:
        return ss.csr_matrix((N, N))
    h = min(int(nz.max()) + 1, N - 1)
    band = np.zeros((2 * h + 1, N))
    L.check(L.load().kore_gegenbauer_mult(int(device), N, L.ptr(a0), float(lam), h, L.ptr(band)),
            "kore_gegenbauer_mult")
    offs = np.arange(-h, h + 1)
    # dia storage indexes column k of diagonal d; band is indexed by row j = k - d
    data = np.zeros_like(band)
    for i, d in enumerate(offs):
        if d >= 0:
            data[i, d:] = band[i, :N - d]
        else:
            data[i, :N + d] = band[i, -d:]
    M = ss.dia_matrix((data, offs), shape=(N, N)).tocsr()
    M.eliminate_zeros()
    return M


class RadialOperators:
    """The radial operators ``r^X D^Y`` (and, with a background field of amplitude
    ``field``, ``r^X h^(J) D^Y``) of the equations' sections for one (N, ricb).
    Section 'u' (the double-curl momentum equation) leaves 4 rows for boundary
    conditions, every other section 2.  ``device``: compute the multiplication operators
    on that GPU (``mult_mat_gpu``)."""

    def __init__(self, N, ricb, tol=1e-9, device=None, field=None):
        self.N = N
        self.ricb = ricb
        self.tol = tol
        self.device = device
        self.field = field
        rp = [chebco(x, N, tol, ricb) for x in range(7)]
        S = [conv_mat(l, N) for l in range(4)]
        D = [None] + [diff_mat(l, N, ricb) for l in range(1, 5)]
        ident = ss.identity(N, format="csr")
        Sto = [ident, S[0], S[1] @ S[0], S[2] @ S[1] @ S[0], S[3] @ S[2] @ S[1] @ S[0]]
        G4 = [ident, S[3], S[3] @ S[2], S[3] @ S[2] @ S[1], S[3] @ S[2] @ S[1] @ S[0]]
        G2 = [ident, S[1], S[1] @ S[0]]
        self._rp, self._Sto, self._D, self._G = rp, Sto, D, {4: G4, 2: G2}
        self._cache = {}

    def field_coeffs(self, rx, j):
        """Chebyshev coefficients of field * r^rx h^(j)(r); as the reference, small
        coefficients are dropped before the amplitude is applied (``bin/utils.py:800-834``,
        ``bin/submatrices.py:121-128``)."""
        key = ("h", rx, j)
        if key not in self._cache:
            fi = dipole_h(gauss_radii(self.N, self.ricb), j, rx)
            self._cache[key] = self.field * chebco_values(fi, self.tol)
        return self._cache[key]

    def op(self, rx, dx, section, h=None):
        """Operator ``r<rx>_D<dx>_<section>`` (``r<rx>_h<h>_D<dx>_<section>`` with h) with
        the boundary rows emptied."""
        key = (rx, dx, section, h)
        if key in self._cache:
            return self._cache[key]
        g = 4 if section == "u" else 2
        c0 = self._rp[rx] if h is None else self.field_coeffs(rx, h)
        a = self._Sto[dx] @ c0
        Mm = mult_mat(a, dx) if self.device is None else mult_mat_gpu(a, dx, self.device)
        M = self._G[g][g - dx] @ Mm
        if dx > 0:
            M = M @ self._D[dx]
        M = ss.csr_matrix(M)
        M = ss.vstack([ss.csr_matrix((g, self.N)), M[:-g, :]], format="csr")
        self._cache[key] = M
        return M


def boundary_values(x, N, nder, ricb, rcmb=RCMB):
    """T_k and its first nder r-derivatives at x = +-1 (``bin/bc_variables.py:8-28``)."""
    ric = -rcmb if ricb == 0 else ricb
    out = np.zeros((N, nder + 1))
    for k in range(N):
        out[k, 0] = x ** k
        t = 1.0
        for i in range(nder):
            t = t * (k ** 2 - i ** 2) / (2 * i + 1)
            out[k, i + 1] = x ** (k + i + 1) * t * (2 / (rcmb - ric)) ** (i + 1)
    return out


# Inside ``lazy_blocks()`` kron_sum and bc_block return LazyBlock term lists instead of
# sparse matrices, for assemble_grid to assemble on the GPU (per thread).
_LAZY_STATE = threading.local()


def _lazy():
    return getattr(_LAZY_STATE, "on", False)


@contextlib.contextmanager
def lazy_blocks():
    """Build the blocks of the pencil as term lists (LazyBlock) for ``assemble_grid``."""
    prev = _lazy()
    _LAZY_STATE.on = True
    try:
        yield
    finally:
        _LAZY_STATE.on = prev


class LazyBlock:
    """A block of the section grid (nrow x ncol l-blocks of n1 unknowns) kept as its terms:
    (ks, js, vals, M) puts vals[t] * M at block (ks[t], js[t]); ``bc`` = (g, rows) puts
    rows[k] (g x n1) in the first g rows of diagonal block k.  Supports the scalar
    products, sums and differences the assembly uses."""

    def __init__(self, nrow, ncol, terms=(), bc=None):
        self.nrow, self.ncol = nrow, ncol
        self.terms = list(terms)
        self.bc = bc

    def __mul__(self, a):
        a = complex(a)
        return LazyBlock(self.nrow, self.ncol, [(ks, js, a * v, M) for ks, js, v, M in self.terms],
                         None if self.bc is None else (self.bc[0], a * self.bc[1]))

    __rmul__ = __mul__

    def __neg__(self):
        return self * -1.0

    def __add__(self, o):
        if o is None:
            return self
        if (o.nrow, o.ncol) != (self.nrow, self.ncol) or (self.bc is not None and o.bc is not None):
            raise ValueError("incompatible lazy blocks")
        return LazyBlock(self.nrow, self.ncol, self.terms + o.terms, self.bc if o.bc is None else o.bc)

    __radd__ = __add__

    def __sub__(self, o):
        return self + (-o)


def kron_sum(lrow, lcol, terms):
    """Sum over terms (d, coef, M) of kron(P, M), where P[k, j] = coef(l_k) for the blocks
    k of degree l_k = lrow[k] and j of degree lcol[j] = l_k + d: the coupling of degree l
    to degree l + d in the l-block layout of two sections.  ``coef`` takes an array of
    degrees.  None if no block couples (a LazyBlock inside ``lazy_blocks()``)."""
    lrow = np.asarray(lrow)
    lcol = np.asarray(lcol)
    pos = {int(l): j for j, l in enumerate(lcol)}
    out = LazyBlock(lrow.size, lcol.size) if _lazy() else None
    for d, coef, M in terms:
        ks = np.array([k for k, l in enumerate(lrow) if int(l) + d in pos], dtype=np.int64)
        if ks.size == 0:
            continue
        js = np.array([pos[int(lrow[k]) + d] for k in ks], dtype=np.int64)
        vals = np.asarray(coef(lrow[ks].astype(float)), dtype=complex) * np.ones(ks.size)
        if _lazy():
            out.terms.append((ks, js, vals, M))
            continue
        P = ss.csr_matrix((vals, (ks, js)), shape=(lrow.size, lcol.size))
        t = ss.kron(P, M, format="csr")
        out = t if out is None else out + t
    return out


def grid_arrays(grid, n1):
    """The arrays ``kore_assemble_blocks`` takes for a grid of LazyBlock (or None) cells,
    sections of l-blocks of n1 unknowns: the dense operators, the entries (row block,
    column block, operator, coefficient) sorted by row block, the boundary rows, the row
    patterns of the distinct block signatures (the (block offset, operator) pairs and
    boundary rows of a row block) and the CSR row pointer."""
    nsec_r, nsec_c = len(grid), len(grid[0])
    nrow_sec = [next((c.nrow for c in row if c is not None), None) for row in grid]
    ncol_sec = [next((grid[a][b].ncol for a in range(nsec_r) if grid[a][b] is not None), None) for b in range(nsec_c)]
    if None in nrow_sec or None in ncol_sec:
        raise ValueError("every section row and column of the grid needs at least one block")
    ro = np.concatenate([[0], np.cumsum(nrow_sec)])
    co = np.concatenate([[0], np.cumsum(ncol_sec)])
    nblk = int(ro[-1])
    if int(co[-1]) != nblk:
        raise ValueError("assemble_grid builds square matrices")
    ops, op_id = [], {}
    R_l, C_l, O_l, V_l = [], [], [], []
    bc_g = np.zeros(nblk, dtype=np.int32)
    bc_rows = [None] * nblk
    for a in range(nsec_r):
        for b in range(nsec_c):
            cell = grid[a][b]
            if cell is None:
                continue
            for ks, js, vals, M in cell.terms:
                if id(M) not in op_id:
                    op_id[id(M)] = len(ops)
                    ops.append(M)
                R_l.append(ro[a] + ks)
                C_l.append(co[b] + js)
                O_l.append(np.full(ks.size, op_id[id(M)], dtype=np.int32))
                V_l.append(vals)
            if cell.bc is not None:
                if ro[a] != co[b]:
                    raise ValueError("boundary rows belong to diagonal blocks")
                g, rows = cell.bc
                for k in range(cell.nrow):
                    bc_g[ro[a] + k] = g
                    bc_rows[ro[a] + k] = rows[k]
    R = np.concatenate(R_l).astype(np.int64)
    order = np.argsort(R, kind="stable")
    R = R[order]
    ent_col = np.concatenate(C_l).astype(np.int32)[order]
    ent_op = np.concatenate(O_l)[order]
    ent_coef = np.ascontiguousarray(np.concatenate(V_l).astype(np.complex128)[order])
    ent_ptr = np.concatenate([[0], np.cumsum(np.bincount(R, minlength=nblk))]).astype(np.int64)
    # the operators' row patterns and dense copies
    dense = np.zeros((len(ops), n1, n1), dtype=np.complex128)
    pat = []
    for q, M in enumerate(ops):
        Mc = ss.csr_matrix(M)
        dense[q] = Mc.toarray()
        rr = np.repeat(np.arange(n1), np.diff(Mc.indptr))
        pat.append((rr, Mc.indices.astype(np.int64)))
    # signatures: the (block offset, operator) pairs and boundary rows of a row block
    sig_of = np.zeros(nblk, dtype=np.int32)
    sigs, keys = [], {}
    for Rb in range(nblk):
        e0, e1 = ent_ptr[Rb], ent_ptr[Rb + 1]
        key = (tuple(sorted(set(zip((ent_col[e0:e1] - Rb).tolist(), ent_op[e0:e1].tolist())))), int(bc_g[Rb]))
        if key not in keys:
            keys[key] = len(sigs)
            sigs.append(key)
        sig_of[Rb] = keys[key]
    sig_rowptr = np.zeros((len(sigs), n1 + 1), dtype=np.int32)
    pats, rowlen, base = [], np.zeros((len(sigs), n1), dtype=np.int64), 0
    for s, (pairs, g) in enumerate(sigs):
        ii, dd, jj = [], [], []
        for dC, q in pairs:
            rr, cc = pat[q]
            keep = rr >= g
            ii.append(rr[keep]); dd.append(np.full(int(keep.sum()), dC)); jj.append(cc[keep])
        if g > 0:
            ii.append(np.repeat(np.arange(g), n1)); dd.append(np.zeros(g * n1, dtype=np.int64))
            jj.append(np.tile(np.arange(n1), g))
        ii, dd, jj = (np.concatenate(x).astype(np.int64) for x in (ii, dd, jj))
        # one integer key per (row, block offset, column), ordered as those triples
        span = 2 * nblk + 1
        key = np.unique((ii * span + (dd + nblk)) * n1 + jj)   # sorted by row, then (dC, j)
        u_j = key % n1
        u_d = (key // n1) % span - nblk
        u_i = key // (n1 * span)
        rowlen[s] = np.bincount(u_i, minlength=n1)
        sig_rowptr[s] = base + np.concatenate([[0], np.cumsum(rowlen[s])])
        pats.append(np.stack([u_d, u_j], axis=1).astype(np.int32))
        base += len(key)
    sig_pat = np.ascontiguousarray(np.concatenate(pats)) if pats else np.zeros((0, 2), np.int32)
    indptr = np.concatenate([[0], np.cumsum(rowlen[sig_of].ravel())]).astype(np.int64)
    nnz = int(indptr[-1])
    bc_ptr = np.full(nblk, -1, dtype=np.int64)
    chunks, off = [], 0
    for Rb in range(nblk):
        if bc_g[Rb] > 0:
            bc_ptr[Rb] = off
            chunks.append(np.asarray(bc_rows[Rb], dtype=np.complex128).reshape(-1))
            off += chunks[-1].size
    bc_vals = np.ascontiguousarray(np.concatenate(chunks)) if chunks else np.zeros(1, np.complex128)
    return dict(n1=int(n1), nblk=nblk, ops=np.ascontiguousarray(dense), sig_of=sig_of,
                sig_rowptr=np.ascontiguousarray(sig_rowptr), sig_pat=sig_pat, ent_ptr=ent_ptr,
                ent_col=np.ascontiguousarray(ent_col), ent_op=np.ascontiguousarray(ent_op), ent_coef=ent_coef,
                bc_g=bc_g, bc_ptr=bc_ptr, bc_len=int(off), bc_vals=bc_vals, indptr=indptr, nnz=nnz)


def assemble_grid(grid, n1, device=0):
    """CSR matrix of a grid of LazyBlock (or None) cells, sections of l-blocks of n1
    unknowns, assembled on the GPU (``kore_assemble_blocks``): the row patterns are formed
    here once per distinct block signature (``grid_arrays``), the values and column indices
    of every row on the device.  Explicit zeros are removed, as in the host assembly."""
    from . import _lib as L
    g = grid_arrays(grid, n1)
    indices = np.zeros(g["nnz"], dtype=np.int32)
    values = np.zeros(g["nnz"], dtype=np.complex128)
    L.check(L.load().kore_assemble_blocks(
        int(device), g["n1"], len(g["ops"]), L.ptr(g["ops"]), g["nblk"], L.ptr(g["sig_of"]), len(g["sig_rowptr"]),
        L.ptr(g["sig_rowptr"]), len(g["sig_pat"]), L.ptr(g["sig_pat"]), L.ptr(g["ent_ptr"]), L.ptr(g["ent_col"]),
        L.ptr(g["ent_op"]), L.ptr(g["ent_coef"]), L.ptr(g["bc_g"]), L.ptr(g["bc_ptr"]), g["bc_len"],
        L.ptr(g["bc_vals"]), L.ptr(g["indptr"]), g["nnz"], L.ptr(indices), L.ptr(values)), "kore_assemble_blocks")
    n = g["nblk"] * g["n1"]
    out = ss.csr_matrix((values, indices, g["indptr"]), shape=(n, n))
    out.eliminate_zeros()
    return out


def momentum_blocks(op, m, lp, lt, visc, wf, Gaspard=1.0, pu=0, pv=0):
    """Blocks of the momentum equation (``bin/operators.py:22-124,136-195``, non-anelastic):
    section u (r.curl curl, poloidal degrees lp) and section v (r.curl, toroidal degrees
    lt).  Returns (App, Apt, Atp, Att, Up, Ut): the time derivative i w u plus Coriolis
    minus viscous terms on the diagonal, the Coriolis coupling l -> l +- 1 between the
    sections, and the time-derivative operators Up, Ut of B.  The reference multiplies
    the equations by r^2 (section u) and r^3 (section v) more for the dipole field: pu,
    pv raise the powers of r accordingly."""
    m = float(m)
    u = lambda rx, dx: op(rx + pu, dx, "u")
    v = lambda rx, dx: op(rx + pv, dx, "v")
    L = lambda l: l * (l + 1)
    # section u, degree l: u = L (L r2 - 2 r3 D - r4 D2), Coriolis 2im (-L r2 + 2 r3 D + r4 D2),
    # viscous L (-L (l+2)(l-1) r0 + 2L r2 D2 - 4 r3 D3 - r4 D4)
    Up = kron_sum(lp, lp, [(0, lambda l: L(l) * L(l), u(2, 0)), (0, lambda l: -2 * L(l), u(3, 1)),
                           (0, lambda l: -L(l), u(4, 2))])
    Cp = kron_sum(lp, lp, [(0, lambda l: -L(l) * 2 * m, u(2, 0)), (0, lambda l: 4 * m + 0 * l, u(3, 1)),
                           (0, lambda l: 2 * m + 0 * l, u(4, 2))])
    Vp = kron_sum(lp, lp, [(0, lambda l: -L(l) * L(l) * (l + 2) * (l - 1), u(0, 0)),
                           (0, lambda l: 2 * L(l) * L(l), u(2, 2)), (0, lambda l: -4 * L(l), u(3, 3)),
                           (0, lambda l: -L(l), u(4, 4))])
    Ut = kron_sum(lt, lt, [(0, L, v(2, 0))])
    Ct = kron_sum(lt, lt, [(0, lambda l: -2 * m + 0 * l, v(2, 0))])
    Vt = kron_sum(lt, lt, [(0, lambda l: -L(l) * L(l), v(0, 0)), (0, lambda l: 2 * L(l), v(1, 1)),
                           (0, L, v(2, 2))])
    App = (1j * wf) * Up + (1j * Gaspard) * Cp - visc * Vp
    Att = (1j * wf) * Ut + (1j * Gaspard) * Ct - visc * Vt
    # Coriolis coupling: to degree l-1 with C- = (l^2-1) sqrt(l^2-m^2) / (2l-1),
    # 2C- ((l-1) r^a - r^b D); to l+1 with C+ = l (l+2) sqrt((l+m+1)(l-m+1)) / (2l+3),
    # 2C+ (-(l+2) r^a - r^b D); (a, b) = (3, 4) in section u and (1, 2) in section v
    cm = lambda l: (l ** 2 - 1) * np.sqrt(l ** 2 - m ** 2) / (2 * l - 1.0)
    cp = lambda l: l * (l + 2.0) * np.sqrt((l + m + 1.0) * (l - m + 1)) / (2.0 * l + 3.0)

    def coriolis(lrow, lcol, w, a, b):
        return Gaspard * kron_sum(lrow, lcol, [
            (-1, lambda l: 2 * cm(l) * (l - 1), w(a, 0)), (-1, lambda l: -2 * cm(l), w(b, 1)),
            (1, lambda l: 2 * cp(l) * -(l + 2), w(a, 0)), (1, lambda l: -2 * cp(l), w(b, 1))])

    Apt = coriolis(lp, lt, u, 3, 4)
    Atp = coriolis(lt, lp, v, 1, 2)
    return App, Apt, Atp, Att, Up, Ut


def bc_block(rows_list, nrow, N1):
    """Block-diagonal matrix holding, for each l-block k, the boundary rows rows_list[k]
    (nrow rows of N1 Chebyshev coefficients) in its first nrow rows (a LazyBlock inside
    ``lazy_blocks()``)."""
    if _lazy():
        return LazyBlock(len(rows_list), len(rows_list), bc=(nrow, np.stack([np.asarray(r)[:nrow] for r in rows_list])))
    data, ri, ci = [], [], []
    for k, rows in enumerate(rows_list):
        for q in range(nrow):
            nz = np.nonzero(rows[q])[0]
            data.append(rows[q][nz])
            ri.append(np.full(nz.size, k * N1 + q))
            ci.append(k * N1 + nz)
    n = len(rows_list) * N1
    return ss.csr_matrix((np.concatenate(data).astype(complex), (np.concatenate(ri), np.concatenate(ci))),
                         shape=(n, n))


def velocity_bc_blocks(lp, lt, N, ricb, bci=1, bco=1, forcing=0):
    """Boundary rows of the velocity (``bc_u_spherical``, ``bin/assemble.py:1188-1296``,
    ricb > 0): in section u, u_r = 0 and no-slip (bc = 1) or stress-free (0) at the outer
    then the inner boundary; in section v, no-slip or stress-free at both."""
    N1 = N
    Tb = boundary_values(1, N, 5, ricb)
    Ta = boundary_values(-1, N, 4, ricb)

    def rows_u(l):
        L = l * (l + 1)
        rows = np.zeros((4, N1), dtype=complex)
        rows[0] = Tb[:, 0]
        if bco == 0:
            rows[1] = (Tb[:, 2] - (2 - L) * Tb[:, 0] / RCMB ** 2) if forcing == 9 else RCMB * Tb[:, 2]
        else:
            rows[1] = (Tb[:, 1] + Tb[:, 0]) if forcing == 9 else Tb[:, 1]
        rows[2] = Ta[:, 0]
        rows[3] = ricb * Ta[:, 2] if bci == 0 else Ta[:, 1]
        return rows

    rv = np.zeros((2, N1), dtype=complex)
    rv[0] = (-RCMB * Tb[:, 1] + Tb[:, 0]) if bco == 0 else Tb[:, 0]
    rv[1] = (-ricb * Ta[:, 1] + Ta[:, 0]) if bci == 0 else Ta[:, 0]
    return bc_block([rows_u(float(l)) for l in lp], 4, N1), bc_block([rv for _ in lt], 2, N1)


def hydro_pencil(m, symm, Ek, N, lmax, ricb=0.35, bci=1, bco=1, forcing=0, forcing_frequency=0.0,
                 forcing_amplitude_cmb=1.0, forcing_amplitude_icb=0.0, Gaspard=1.0, ViscosD=None,
                 with_norm=False, device=None, assemble_on_device=False):
    """(A, B) as bin/assemble.py writes them for the hydrodynamic shell problem.

    forcing == 0: eigenproblem, B is the (sizmat x sizmat) float64 matrix, A and B
    divided by ||B||_F (with_norm=True also returns that norm).  forcing in (7, 9, 10):
    forced problem, A = i w u + Coriolis - viscous (unnormalised) and B is the
    (sizmat x 1) forcing column.  The forced matrix at frequency w is therefore
    ||B||_F (A_eig - i w B_eig) of the eigen pencil.  ``device``: build the Gegenbauer
    multiplication operators on that GPU instead of the host.  ``assemble_on_device``:
    assemble A and B from the radial operators on the GPU (``device``, else GPU 0) with
    ``assemble_grid``; the host then forms only the row patterns of the distinct block
    signatures.
    """
    if ricb <= 0:
        raise ValueError("only the spherical shell (ricb > 0) is assembled here")
    if (lmax - m + 1) % 2:
        raise ValueError("lmax - m + 1 must be even")
    visc = Ek if ViscosD is None else ViscosD
    lp, lt = ell(m, lmax, symm)
    wf = forcing_frequency if forcing else 0.0
    R = RadialOperators(N, ricb, device=device)
    with lazy_blocks() if assemble_on_device else contextlib.nullcontext():
        App, Apt, Atp, Att, u_p, u_t = momentum_blocks(R.op, m, lp, lt, visc, wf, Gaspard)
        BCp, BCt = velocity_bc_blocks(lp, lt, N, ricb, bci, bco, forcing)
    gpu = 0 if device is None else device
    if assemble_on_device:
        A = assemble_grid([[App + BCp, Apt], [Atp, Att + BCt]], N, gpu)
    else:
        A = ss.bmat([[App + BCp, Apt], [Atp, Att + BCt]], format="csr").astype(np.complex128)
        A.eliminate_zeros()
    if forcing == 0:
        if assemble_on_device:
            B = assemble_grid([[-u_p, None], [None, -u_t]], N, gpu).real.astype(np.float64)
        else:
            B = ss.bmat([[-u_p, None], [None, -u_t]], format="csr").real.astype(np.float64)
        B.eliminate_zeros()
        bnorm = ss.linalg.norm(B)
        if with_norm:
            return (A / bnorm).tocsr(), (B / bnorm).tocsr(), float(bnorm)
        return (A / bnorm).tocsr(), (B / bnorm).tocsr()
    return A, forcing_vector(m, symm, N, lmax, ricb, forcing, forcing_frequency, forcing_amplitude_cmb,
                             forcing_amplitude_icb, bci, bco)


def forcing_vector(m, symm, N, lmax, ricb, forcing, forcing_frequency=0.0, forcing_amplitude_cmb=1.0,
                   forcing_amplitude_icb=0.0, bci=1, bco=1):
    """The (sizmat x 1) forcing column of the forced problem (bin/assemble.py:279-427):
    forcing 10 and 9 are boundary forcings independent of the frequency, forcing 7
    (libration) is proportional to it."""
    N1 = radial_size(N, ricb)
    nb = (lmax - m + 1) // 2
    lp, lt = ell(m, lmax, symm)
    n = 2 * nb * N1
    if forcing == 10:
        if symm != 1:
            raise ValueError("forcing 10 needs symm = 1")
        l = m
        L = l * (l + 1)
        pos = N1 * int(np.nonzero(lp == l)[0][0])
        vals = np.array([1.0 / L, 0.0])
    elif forcing == 9:
        if not (symm == 1 and m == 2 and bci == 1):
            raise ValueError("forcing 9 needs symm = 1, m = 2, bci = 1")
        L = 6
        pos = N1 * int(np.nonzero(lp == 2)[0][0])
        vals = np.array([forcing_amplitude_cmb * RCMB / L, forcing_amplitude_icb * ricb / L])
    elif forcing == 7:
        if not (m == 2 and symm == 1 and bci == 1 and bco == 1):
            raise ValueError("forcing 7 is coded here for m = 2, symm = 1, no-slip")
        L = 6
        pos = N1 * int(np.nonzero(lp == 2)[0][0])
        vals = np.array([-forcing_frequency / L * forcing_amplitude_cmb,
                         -forcing_frequency / L * forcing_amplitude_icb * ricb ** 2])
    else:
        raise ValueError(f"forcing {forcing} is not assembled here")
    rows = np.arange(pos, pos + 2)
    keep = vals != 0
    return ss.csr_matrix((vals[keep].astype(complex), (rows[keep], np.zeros(keep.sum(), int))), shape=(n, 1))


def hydro_params(m, symm, Ek, N, lmax, ricb=0.35, **kw):
    """The parameter mapping structure.layout_from_params expects for hydro_pencil."""
    d = dict(m=m, symm=symm, Ek=Ek, N=N, lmax=lmax, ricb=ricb, hydro=1, magnetic=0, thermal=0,
             compositional=0, B0="axial")
    d.update(kw)
    return d
