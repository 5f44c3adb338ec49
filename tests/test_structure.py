"""l-major permutation and block sizes against the reference's pencils."""
import numpy as np
import pytest

from kore_gb300.structure import band_of, ell, field_offsets, layout_from_params

CASES = ["spinover", "shell_m1_ek1e-4", "shell_m2_small", "forced_m2_f10", "jones2000_rac",
         "dormy2004_rac", "mac_dipole_small", "mac_quadrupole_small"]


@pytest.mark.parametrize("name", CASES)
def test_layout_is_block_tridiagonal(case, name):
    meta, A, B = case(name)
    lay = layout_from_params(meta)
    assert lay.n == meta["sizmat"] == A.shape[0]
    assert lay.N1 == meta["N1"]
    assert sorted(lay.perm.tolist()) == list(range(lay.n))      # a permutation
    assert band_of(A, lay) == lay.coupling
    # every entry within the block-tridiagonal band of the (merged) blocks
    off = np.concatenate([[0], np.cumsum(lay.block_sizes)])
    inv = np.empty(lay.n, dtype=np.int64)
    inv[lay.perm] = np.arange(lay.n)
    blk = np.searchsorted(off, np.arange(lay.n), side="right") - 1
    Ac = A.tocoo()
    d = blk[inv[Ac.row]] - blk[inv[Ac.col]]
    assert np.abs(d).max() <= 1
    if B.shape[1] == B.shape[0]:
        Bc = B.tocoo()
        assert np.all(blk[inv[Bc.row]] == blk[inv[Bc.col]])   # B is block diagonal


def test_permutation_roundtrip(case):
    meta, A, B = case("spinover")
    lay = layout_from_params(meta)
    x = np.random.default_rng(1).standard_normal(lay.n)
    xp = x[lay.perm]
    back = np.empty_like(xp)
    back[lay.perm] = xp
    assert np.array_equal(back, x)
    Ap = A[lay.perm][:, lay.perm]
    assert abs(Ap @ xp - (A @ x)[lay.perm]).max() == 0.0


def test_ell_lists():
    # bin/utils.py:174-183 for m=1 symmetric: poloidal l = 1,3,..., toroidal 2,4,...
    p, t = ell(1, 40, 1)
    assert p[0] == 1 and t[0] == 2 and len(p) == len(t) == 20
    p, t = ell(0, 9, 1)
    assert p[0] == 2 and t[0] == 1
    p, t = ell(2, 31, -1)
    assert p[0] == 3 and t[0] == 2


def test_field_offsets():
    off = field_offsets(100, 1, 1, 1, 0)
    assert off == {"flow": (0, 200), "magnetic": (200, 400), "temperature": (400, 500)}
    assert field_offsets(100, 1, 0, 0, 1)["composition"] == (200, 300)


def test_invalid_lmax():
    with pytest.raises(ValueError):
        layout_from_params(dict(m=1, lmax=41, symm=1, N=48, ricb=0.35))
