"""l-major block structure of kore's pencil.

bin/assemble.py orders the unknowns section-major: for each field section
(upol, utor, bpol, btor, theta, xi; ``bin/assemble.py:442-534``) the N1-long radial
blocks of all its harmonic degrees l, in the order of ``ut.ell``
(``bin/utils.py:174-183``).  The operators couple degree l only with l+-1 (Coriolis,
``bin/operators.py:48-124``; antisymmetric B0) or l+-2 (symmetric B0, e.g. the
quadrupole ``Luo_S2``), so ordering the blocks by degree turns A - sigma B into a
block-tridiagonal matrix (block-pentadiagonal in degree for l+-2 coupling, which is
tridiagonal again after grouping pairs of degrees).  This module computes that
permutation and the diagonal block sizes from the parameters alone, mirroring the
reference's own size formulas (``bin/utils.py:24-44``).
"""
from dataclasses import dataclass

import numpy as np

SECTIONS = ("upol", "utor", "bpol", "btor", "theta", "xi")


def ell(m, lmax, vsymm):
    """Degrees of the poloidal and toroidal sections (``bin/utils.py:174-183``)."""
    lm1 = lmax - m + 1
    s = int(vsymm * 0.5 + 0.5)
    sg = int(np.sign(m))
    idp = np.arange((sg + s) % 2, lm1, 2, dtype=int)
    idt = np.arange((sg + s + 1) % 2, lm1, 2, dtype=int)
    ll = np.arange(m + 1 - sg, lmax + 2 - sg, dtype=int)
    return ll[idp], ll[idt]


def symm_b0(B0, B0_l=1):
    """Equatorial symmetry of the imposed field (``bin/utils.py:46-55``)."""
    if B0 in ("axial", "dipole", "G21 dipole", "Luo_S1"):
        return -1
    if B0 == "Luo_S2":
        return 1
    if B0 == "FDM":
        return int((-1) ** B0_l)
    raise ValueError(f"unknown B0 {B0!r}")


@dataclass
class Layout:
    n: int                 # sizmat
    N1: int                # radial block size
    nb: int                # blocks per section
    perm: np.ndarray       # perm[i] = original index of l-major unknown i (int64)
    block_sizes: np.ndarray  # int32, diagonal blocks of the block-tridiagonal form
    block_ell: np.ndarray  # degree of each N1 block in l-major order
    sections: tuple        # active section names, in original (section-major) order
    coupling: int          # max |l_row - l_col| of the operator (1 or 2)

    @property
    def nblocks(self):
        return int(len(self.block_sizes))


def radial_size(N, ricb):
    """N1: N/2 without an inner core, N with one (``bin/utils.py:24``)."""
    sg = int(np.sign(ricb))
    return int(N / 2) * int(1 + sg) + int((N % 2) * sg)


def layout(m, lmax, symm, N, ricb, hydro=1, magnetic=0, thermal=0, compositional=0, B0="axial", B0_l=1,
           coupling=None):
    """Permutation and block sizes for the given kore parameters."""
    if (lmax - m + 1) % 2:
        raise ValueError("lmax - m + 1 must be even (the reference requires it, bin/parameters.py:301-304)")
    N1 = radial_size(N, ricb)
    nb = (lmax - m + 1) // 2
    sb = symm_b0(B0, B0_l) if magnetic else -1
    flo = ell(m, lmax, symm)
    mag = ell(m, lmax, symm * sb)
    secs, lists = [], []
    if hydro:
        secs += ["upol", "utor"]; lists += [flo[0], flo[1]]
    if magnetic:
        secs += ["bpol", "btor"]; lists += [mag[0], mag[1]]
    if thermal:
        secs += ["theta"]; lists += [flo[0]]
    if compositional:
        secs += ["xi"]; lists += [flo[0]]
    blocks = []
    for si, ls in enumerate(lists):
        for k, l in enumerate(ls):
            blocks.append((int(l), si, (si * nb + k) * N1))
    blocks.sort(key=lambda t: (t[0], t[1]))
    perm = np.concatenate([np.arange(st, st + N1, dtype=np.int64) for _, _, st in blocks])
    ells = np.array([b[0] for b in blocks], dtype=np.int64)
    if coupling is None:
        coupling = 2 if (magnetic and sb == 1) else 1
    uniq, counts = np.unique(ells, return_counts=True)
    sizes = counts * N1
    if coupling == 2:
        sizes = np.array([sizes[i:i + 2].sum() for i in range(0, len(sizes), 2)])
    elif coupling != 1:
        raise ValueError("coupling must be 1 or 2")
    n = len(perm)
    return Layout(n=n, N1=N1, nb=nb, perm=perm, block_sizes=sizes.astype(np.int32), block_ell=ells,
                  sections=tuple(secs), coupling=coupling)


def layout_from_params(par, coupling=None):
    """Layout from a kore ``parameters`` module or a mapping with the same names."""
    g = (lambda k, d=None: par.get(k, d)) if isinstance(par, dict) else (lambda k, d=None: getattr(par, k, d))
    return layout(int(g("m")), int(g("lmax")), int(g("symm")), int(g("N")), float(g("ricb")),
                  hydro=int(g("hydro", 1)), magnetic=int(g("magnetic", 0)), thermal=int(g("thermal", 0)),
                  compositional=int(g("compositional", 0)), B0=g("B0", "axial"), B0_l=int(g("B0_l", 1)),
                  coupling=coupling)


def band_of(A, lay):
    """Largest |l_row - l_col| over the nonzeros of A (structural check of ``coupling``)."""
    Ac = A.tocoo()
    inv = np.empty(lay.n, dtype=np.int64)
    inv[lay.perm] = np.arange(lay.n)
    lrow = np.repeat(lay.block_ell, lay.N1)
    return int(np.abs(lrow[inv[Ac.row]] - lrow[inv[Ac.col]]).max()) if Ac.nnz else 0


def field_offsets(n_per_section, hydro, magnetic, thermal, compositional, forced=False):
    """Section slices of the solution vector exactly as bin/solve.py takes them.

    The eigen branch (``bin/solve.py:169-190``) places temperature at 2n + 2n*magnetic
    and composition after it whatever ``hydro`` is; the forced branch
    (``bin/solve.py:241-261``) multiplies the flow part by ``hydro``.
    """
    n = n_per_section
    h = hydro if forced else 1
    off = {}
    if hydro:
        off["flow"] = (0, 2 * n)
    if magnetic:
        o = 2 * n * hydro
        off["magnetic"] = (o, o + 2 * n)
    if thermal:
        o = 2 * n * h + magnetic * 2 * n
        off["temperature"] = (o, o + n)
    if compositional:
        o = 2 * n * h + magnetic * 2 * n + thermal * n
        off["composition"] = (o, o + n)
    return off
