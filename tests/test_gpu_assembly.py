"""A and B assembled on the GPU (kore_assemble_blocks) against the reference's own
assembly: the fixtures its submatrices.py/assemble.py wrote, and the fingerprint of the
240,000-unknown benchmark pencil."""
import json
import os
import sys

import numpy as np
import pytest
import scipy.sparse.linalg as ssl

from kore_gb300.assembly import hydro_pencil

pytestmark = pytest.mark.gpu

HYDRO = ["spinover", "shell_m1_ek1e-4", "shell_m2_small", "shell_m2_ek1e-4", "forced_m2_f10", "forced_m2_f7"]


def assert_same_structure(ref, got):
    """Same column indices row by row, except entries that are zero to rounding in one
    and stored in the other (a sum of operator terms that cancels): B matches exactly, A
    in all but 3-52 entries of the fixtures, each below 1e-13 of its row's largest."""
    X, Y = ref.tocsr().copy(), got.tocsr().copy()
    for M in (X, Y):
        M.eliminate_zeros()
        M.sort_indices()
    PX, PY = (abs(X) > 0).astype(np.int8), (abs(Y) > 0).astype(np.int8)
    diff = (PX != PY).tocoo()
    rowmax = np.asarray(abs(X).max(axis=1).todense()).ravel()
    for r, c in zip(diff.row, diff.col):
        assert max(abs(X[r, c]), abs(Y[r, c])) <= 1e-13 * rowmax[r], (r, c)
    return diff.nnz


@pytest.mark.parametrize("name", HYDRO)
def test_device_assembly_matches_reference(gpu_lib, case, name):
    meta, A, B = case(name)
    A2, B2 = hydro_pencil(meta["m"], meta["symm"], meta["Ek"], meta["N"], meta["lmax"], meta["ricb"],
                          forcing=meta["forcing"], forcing_frequency=meta["forcing_frequency"],
                          assemble_on_device=True)
    assert A2.shape == A.shape and B2.shape == B.shape
    assert ssl.norm(A2 - A) <= 1e-14 * ssl.norm(A)
    assert ssl.norm(B2 - B) <= 1e-14 * ssl.norm(B)
    D = abs(A2 - A).tocsr()
    rowmax = np.asarray(abs(A).max(axis=1).todense()).ravel()
    assert (D.multiply(1.0 / np.maximum(rowmax, 1e-300)[:, None])).max() < 1e-13
    assert np.all(np.diff(A2.indptr) >= 0) and A2.has_sorted_indices
    assert assert_same_structure(B, B2) == 0
    assert assert_same_structure(A, A2) <= 1e-3 * A.nnz


def test_device_assembly_fullsize_fingerprint(gpu_lib):
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, "shell2_fingerprint.npz"))
    meta = json.loads(str(z["meta"]))
    sys.path.insert(0, GOLDEN)
    from make_fullsize_fingerprint import fingerprint
    args = (meta["m"], meta["symm"], meta["Ek"], meta["N"], meta["lmax"], meta["ricb"])
    A, B = hydro_pencil(*args, assemble_on_device=True, device=0)
    Ah, Bh = hydro_pencil(*args)
    # against the host assembly on this machine: the same sums in another order
    assert ssl.norm(A - Ah) <= 1e-15 * ssl.norm(Ah)
    assert ssl.norm(B - Bh) <= 1e-15 * ssl.norm(Bh)
    f = fingerprint(A, B)
    assert tuple(f["shape"]) == tuple(z["shape"])
    assert np.array_equal(f["rows"], z["rows"])
    # scipy's sparse Frobenius norm sums 8.5 million squares with an error of ~2e-13 that
    # depends on the host's numpy build (x86 and Arm differ by that much for the same
    # matrix); the rows of A v and B v below are the tight check
    assert abs(f["A_fro"] - float(z["A_fro"])) <= 1e-12 * float(z["A_fro"])
    assert abs(f["B_fro"] - float(z["B_fro"])) <= 1e-12 * float(z["B_fro"])
    scale_a = z["A_row1"] * 6.0
    scale_b = np.maximum(z["B_row1"], 1e-300) * 6.0
    assert np.all(np.abs(f["Av"] - z["Av"]) <= 1e-13 * scale_a)
    assert np.all(np.abs(f["Bv"] - z["Bv"]) <= 1e-13 * scale_b)
    assert np.allclose(f["A_row1"], z["A_row1"], rtol=1e-13, atol=0)
    assert abs(int(f["A_nnz"]) - int(z["A_nnz"])) <= 0.001 * int(z["A_nnz"])


@pytest.mark.parametrize("name", ["mac_dipole_small", "mac_dipole_medium", "mac_dipole_internal"])
def test_mac_device_assembly_matches_reference(gpu_lib, case, name):
    from kore_gb300.assembly_mac import mac_pencil
    meta, A, B = case(name)
    A2, B2 = mac_pencil(meta["m"], meta["symm"], meta["Ek"], meta["N"], meta["lmax"], meta["ricb"],
                        Em=meta["Em"], Le2=meta["Le2"], Prandtl=meta["Prandtl"], Ra=meta["Ra"],
                        heating=meta["heating"], bci_thermal=meta["bci_thermal"],
                        bco_thermal=meta["bco_thermal"], cnorm=meta["cnorm"], assemble_on_device=True, device=0)
    assert A2.shape == A.shape and B2.shape == B.shape
    assert ssl.norm(A2 - A) <= 1e-14 * ssl.norm(A)
    assert ssl.norm(B2 - B) <= 1e-14 * ssl.norm(B)
    D = abs(A2 - A).tocsr()
    rowmax = np.asarray(abs(A).max(axis=1).todense()).ravel()
    assert (D.multiply(1.0 / np.maximum(rowmax, 1e-300)[:, None])).max() < 1e-13
    assert assert_same_structure(B, B2) == 0
    assert assert_same_structure(A, A2) <= 1e-3 * A.nnz


def test_mac_device_assembly_fullsize_matches_host(gpu_lib):
    """The 100,000-unknown MAC pencil (m=1, Ek=1e-6, N=200, lmax=200) assembled on the GPU
    against the host assembly, whose restatement is pinned to the reference by the
    fixtures above and by the full-size solve's parity."""
    from kore_gb300.assembly_mac import mac_pencil_parts
    kw = dict(Em=1e-3, Le2=1e-8, Prandtl=1.0)
    A0, Ab, B, nrm = mac_pencil_parts(1, 1, 1e-6, 200, 200, 0.35, assemble_on_device=True, device=0, **kw)
    A0h, Abh, Bh, nrmh = mac_pencil_parts(1, 1, 1e-6, 200, 200, 0.35, **kw)
    assert A0.shape == (100000, 100000)
    # the radial operators come from the GPU too (kore_gegenbauer_mult): rounding apart
    assert ssl.norm(A0 - A0h) <= 1e-14 * ssl.norm(A0h)
    assert ssl.norm(B - Bh) <= 1e-14 * ssl.norm(Bh)
    assert abs(nrm - nrmh) <= 1e-14 * nrmh
    assert ssl.norm(Ab - Abh) <= 1e-14 * ssl.norm(Abh)
