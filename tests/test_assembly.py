"""The host restatement of the hydrodynamic assembly (kore_gb300.assembly) against
the pencils the reference's own submatrices.py/assemble.py produced."""
import numpy as np
import pytest
import scipy.sparse.linalg as ssl

from kore_gb300.assembly import chebco, hydro_pencil, mult_mat, ncheb

HYDRO = ["spinover", "shell_m1_ek1e-4", "shell_m2_small", "shell_m2_ek1e-4", "forced_m2_f10", "forced_m2_f7"]


@pytest.mark.parametrize("name", HYDRO)
def test_matches_reference_assembly(case, name):
    meta, A, B = case(name)
    A2, B2 = hydro_pencil(meta["m"], meta["symm"], meta["Ek"], meta["N"], meta["lmax"], meta["ricb"],
                          forcing=meta["forcing"], forcing_frequency=meta["forcing_frequency"])
    assert A2.shape == A.shape and B2.shape == B.shape
    assert ssl.norm(A2 - A) <= 1e-14 * ssl.norm(A)
    assert ssl.norm(B2 - B) <= 1e-14 * ssl.norm(B)
    # entrywise, relative to the largest entry of the row
    D = abs(A2 - A).tocsr()
    rowmax = np.asarray(abs(A).max(axis=1).todense()).ravel()
    assert (D.multiply(1.0 / np.maximum(rowmax, 1e-300)[:, None])).max() < 1e-13


def test_chebyshev_coefficients_of_powers():
    # r^2 on [0.35, 1] has exactly three nonzero Chebyshev coefficients
    c = chebco(2, 16, 1e-9, 0.35)
    assert np.count_nonzero(c) == 3
    x = 0.3
    r = 0.35 + 0.65 * (x + 1) / 2
    assert abs(np.polynomial.chebyshev.chebval(x, c) - r * r) < 1e-14


def test_multiplication_operator_lambda0_is_chebyshev_product():
    a = chebco(1, 12, 1e-12, 0.35)
    b = np.zeros(12)
    b[:5] = [0.3, -0.2, 0.1, 0.05, 0.01]
    prod = mult_mat(a, 0) @ b
    full = np.polynomial.chebyshev.chebmul(a, b)
    ref = np.zeros(12)
    ref[:min(12, full.size)] = full[:12]
    assert np.abs(prod - ref).max() < 1e-14


def test_ncheb_rule():
    # bin/parameters.py:6-16
    assert ncheb(1e-3) == 68 and ncheb(1e-7) == 428 and ncheb(0) == 48


def test_forced_matrix_is_scaled_shift_of_eigen_pencil():
    """kore's forced matrix at frequency w equals ||B||_F (A_eig - i w B_eig), and the
    forcing column built alone equals the one assembled with the forced matrix; the
    batched frequency sweep relies on both."""
    from kore_gb300.assembly import forcing_vector, hydro_pencil
    m, symm, Ek, N, lmax, ricb = 2, 1, 1e-4, 24, 13, 0.35
    Ae, Be, nrm = hydro_pencil(m, symm, Ek, N, lmax, ricb, with_norm=True)
    for w in (-1.3, 0.0, 0.7):
        Af, bf = hydro_pencil(m, symm, Ek, N, lmax, ricb, forcing=10, forcing_frequency=w)
        M = nrm * (Ae - (1j * w) * Be)
        assert abs(Af - M).max() <= 1e-12 * abs(Af).max()
        assert abs(bf - forcing_vector(m, symm, N, lmax, ricb, 10, w)).max() == 0


MAC = ["mac_dipole_small", "mac_dipole_medium", "mac_dipole_internal"]


@pytest.mark.parametrize("name", MAC)
def test_mac_dipole_matches_reference_assembly(case, name):
    """The dipole MAC restatement (kore_gb300.assembly_mac) against the pencils the
    reference's own compute_profiles.py/submatrices.py/assemble.py produced: both
    symmetries, differential and internal heating, isothermal and fixed-flux thermal
    boundaries."""
    from kore_gb300.assembly_mac import mac_pencil
    meta, A, B = case(name)
    A2, B2 = mac_pencil(meta["m"], meta["symm"], meta["Ek"], meta["N"], meta["lmax"], meta["ricb"],
                        Em=meta["Em"], Le2=meta["Le2"], Prandtl=meta["Prandtl"], Ra=meta["Ra"],
                        heating=meta["heating"], bci_thermal=meta["bci_thermal"],
                        bco_thermal=meta["bco_thermal"], cnorm=meta["cnorm"])
    assert A2.shape == A.shape and B2.shape == B.shape
    assert ssl.norm(A2 - A) <= 1e-14 * ssl.norm(A)
    assert ssl.norm(B2 - B) <= 1e-14 * ssl.norm(B)
    D = abs(A2 - A).tocsr()
    rowmax = np.asarray(abs(A).max(axis=1).todense()).ravel()
    assert (D.multiply(1.0 / np.maximum(rowmax, 1e-300)[:, None])).max() < 1e-13


def test_mac_pencil_is_affine_in_rayleigh_number():
    from kore_gb300.assembly_mac import mac_pencil, mac_pencil_parts
    kw = dict(Em=0.1, Le2=1e-3, Prandtl=1.0)
    A0, Ab, B, nrm = mac_pencil_parts(1, -1, 1e-3, 20, 12, 0.35, **kw)
    for Ra in (0.0, 3.7e5):
        A, B2 = mac_pencil(1, -1, 1e-3, 20, 12, 0.35, Ra=Ra, **kw)
        assert ssl.norm(A - (A0 - Ra * 1e-6 * Ab) / nrm) <= 1e-15 * ssl.norm(A)
        assert ssl.norm(B2 - B / nrm) == 0.0


def test_fullsize_bench_pencil_matches_reference_fingerprint():
    """The 240,000-unknown benchmark pencil (m=2, Ek=1e-7, N=400, lmax=601) built by the
    restatement against the reference's own assembly of it, through the fingerprint
    tests/golden/make_fullsize_fingerprint.py stored: norms, nonzero counts, and 4096
    seeded rows of A v and B v for a seeded v."""
    import json
    import os
    import sys
    from conftest import GOLDEN
    path = os.path.join(GOLDEN, "shell2_fingerprint.npz")
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    sys.path.insert(0, GOLDEN)
    from make_fullsize_fingerprint import fingerprint
    A, B = hydro_pencil(meta["m"], meta["symm"], meta["Ek"], meta["N"], meta["lmax"], meta["ricb"])
    f = fingerprint(A, B)
    assert tuple(f["shape"]) == tuple(z["shape"])
    assert np.array_equal(f["rows"], z["rows"])
    assert abs(f["A_fro"] - float(z["A_fro"])) <= 1e-14 * float(z["A_fro"])
    assert abs(f["B_fro"] - float(z["B_fro"])) <= 1e-14 * float(z["B_fro"])
    # rows of A v and B v, relative to the row's 1-norm times max |v| (~5 for this v)
    scale_a = z["A_row1"] * 6.0
    scale_b = np.maximum(z["B_row1"], 1e-300) * 6.0
    assert np.all(np.abs(f["Av"] - z["Av"]) <= 1e-13 * scale_a)
    assert np.all(np.abs(f["Bv"] - z["Bv"]) <= 1e-13 * scale_b)
    assert np.allclose(f["A_row1"], z["A_row1"], rtol=1e-13, atol=0)
    # explicit zeros aside, the sparsity matches
    assert abs(int(f["A_nnz"]) - int(z["A_nnz"])) <= 0.001 * int(z["A_nnz"])


def _emulate_assemble_kernel(g):
    """What kore_assemble_blocks computes, row by row in numpy: the column indices and
    values of each row from its signature's pattern, the boundary rows and the entries."""
    import scipy.sparse as ss
    n1, nblk = g["n1"], g["nblk"]
    indices = np.zeros(g["nnz"], dtype=np.int64)
    values = np.zeros(g["nnz"], dtype=np.complex128)
    for R in range(nblk):
        rp = g["sig_rowptr"][g["sig_of"][R]]
        e0, e1 = g["ent_ptr"][R], g["ent_ptr"][R + 1]
        for i in range(n1):
            pat = g["sig_pat"][rp[i]:rp[i + 1]]
            C = R + pat[:, 0].astype(np.int64)
            j = pat[:, 1].astype(np.int64)
            if i < g["bc_g"][R]:
                v = np.where(pat[:, 0] == 0, g["bc_vals"][g["bc_ptr"][R] + i * n1 + j], 0)
            else:
                v = np.zeros(len(pat), dtype=np.complex128)
                for e in range(e0, e1):
                    v = v + np.where(C == g["ent_col"][e], g["ent_coef"][e] * g["ops"][g["ent_op"][e], i, j], 0)
            out = g["indptr"][R * n1 + i]
            indices[out:out + len(pat)] = C * n1 + j
            values[out:out + len(pat)] = v
    n = nblk * n1
    M = ss.csr_matrix((values, indices, g["indptr"]), shape=(n, n))
    assert np.all(np.diff(indices[:g["indptr"][1]]) > 0)
    M.eliminate_zeros()
    return M


@pytest.mark.parametrize("forcing", [0, 7])
def test_device_assembly_inputs_rebuild_host_pencil(forcing):
    """The lazy blocks and grid arrays that the GPU assembly takes rebuild the host
    assembly's A and B: signatures, row patterns (sorted columns), boundary rows and
    entry coefficients, checked through a numpy restatement of the kernel."""
    import scipy.sparse as ss
    from kore_gb300 import assembly as asm
    m, symm, Ek, N, lmax, ricb = 2, 1, 1e-3, 24, 13, 0.35
    lp, lt = asm.ell(m, lmax, symm)
    R = asm.RadialOperators(N, ricb)
    wf = 0.7 if forcing else 0.0
    with asm.lazy_blocks():
        App, Apt, Atp, Att, Up, Ut = asm.momentum_blocks(R.op, m, lp, lt, Ek, wf)
        BCp, BCt = asm.velocity_bc_blocks(lp, lt, N, ricb, forcing=forcing)
    gA = asm.grid_arrays([[App + BCp, Apt], [Atp, Att + BCt]], N)
    assert len(gA["sig_rowptr"]) <= 8          # row blocks share a few signatures
    A = _emulate_assemble_kernel(gA)
    if forcing:
        Ah, _ = asm.hydro_pencil(m, symm, Ek, N, lmax, ricb, forcing=forcing, forcing_frequency=wf)
        assert ssl.norm(A - Ah) <= 1e-14 * ssl.norm(Ah)
        return
    B = _emulate_assemble_kernel(asm.grid_arrays([[-Up, None], [None, -Ut]], N)).real
    Ah, Bh, nrm = asm.hydro_pencil(m, symm, Ek, N, lmax, ricb, with_norm=True)
    assert ssl.norm(A / nrm - Ah) <= 1e-14 * ssl.norm(Ah)
    assert ssl.norm(ss.csr_matrix(B) / nrm - Bh) <= 1e-14 * ssl.norm(Bh)
    assert abs(ssl.norm(B) - nrm) <= 1e-14 * nrm


def test_mac_device_assembly_inputs_rebuild_host_pencil():
    """The same for the dipole MAC pencil's 5 x 5 section grid (Lorentz, induction and
    heat blocks, insulating and thermal boundary rows)."""
    import scipy.sparse as ss
    from kore_gb300 import assembly as asm
    from kore_gb300 import assembly_mac as mac
    from kore_gb300.structure import ell
    m, symm, Ek, N, lmax, ricb = 1, 1, 1e-3, 16, 8, 0.35
    kw = dict(Em=0.1, Le2=1e-3, Prandtl=1.0)
    A0h, _, Bh, nrm = mac.mac_pencil_parts(m, symm, Ek, N, lmax, ricb, **kw)
    lp, lt = ell(m, lmax, symm)
    lmag_p, lmag_t = ell(m, lmax, -symm)
    R = asm.RadialOperators(N, ricb, field=asm.dipole_norm(ricb, "mag_energy"))
    with asm.lazy_blocks():
        A0g, Bg = mac._mac_blocks(R.op, float(m), lambda l: l * (l + 1), N, N, ricb, Ek, kw["Em"], kw["Le2"],
                                  kw["Prandtl"], "differential", 1, 1, 0, 0, 1.0, lp, lt, lmag_p, lmag_t)
    A0 = _emulate_assemble_kernel(asm.grid_arrays(A0g, N))
    B = ss.csr_matrix(_emulate_assemble_kernel(asm.grid_arrays(Bg, N)).real)
    assert ssl.norm(A0 - A0h) <= 1e-14 * ssl.norm(A0h)
    assert ssl.norm(B - Bh) <= 1e-14 * ssl.norm(Bh)


def test_lazy_blocks_are_per_thread_and_grid_checks():
    import threading
    from kore_gb300 import assembly as asm
    seen = {}

    def other():
        seen["other"] = asm.kron_sum([2, 3], [2, 3], [(0, lambda l: l, np.eye(4))])

    with asm.lazy_blocks():
        mine = asm.kron_sum([2, 3], [2, 3], [(0, lambda l: l, np.eye(4))])
        t = threading.Thread(target=other)
        t.start()
        t.join()
    assert isinstance(mine, asm.LazyBlock) and not isinstance(seen["other"], asm.LazyBlock)
    assert not isinstance(asm.kron_sum([2], [2], [(0, lambda l: l, np.eye(2))]), asm.LazyBlock)
    with pytest.raises(ValueError):
        asm.grid_arrays([[mine, None], [None, None]], 4)


def test_device_assembly_pattern_covers_fullsize_pencil():
    """At the 240,000-unknown bench size (too large for the kernel's numpy restatement):
    the row patterns that grid_arrays gives the GPU kernel hold every stored entry of the
    host assembly, A and B, so the kernel writes every value somewhere."""
    import scipy.sparse as ss
    from kore_gb300 import assembly as asm
    m, symm, Ek, N, lmax, ricb = 2, 1, 1e-7, 400, 601, 0.35
    lp, lt = asm.ell(m, lmax, symm)
    R = asm.RadialOperators(N, ricb)
    with asm.lazy_blocks():
        App, Apt, Atp, Att, Up, Ut = asm.momentum_blocks(R.op, m, lp, lt, Ek, 0.0)
        BCp, BCt = asm.velocity_bc_blocks(lp, lt, N, ricb)
    Ah, Bh = asm.hydro_pencil(m, symm, Ek, N, lmax, ricb)
    for grid, H in (([[App + BCp, Apt], [Atp, Att + BCt]], Ah), ([[-Up, None], [None, -Ut]], Bh)):
        g = asm.grid_arrays(grid, N)
        n = g["nblk"] * N
        rows = np.repeat(np.arange(n), np.diff(g["indptr"]))
        R_of = rows // N
        i_of = rows % N
        # the kernel's column of each output slot: (R + dC) N + j from the signature pattern
        sig = g["sig_of"][R_of]
        start = g["sig_rowptr"][sig, i_of]
        k = np.arange(g["nnz"]) - g["indptr"][rows]
        pat = g["sig_pat"][start + k]
        cols = (R_of + pat[:, 0]) * N + pat[:, 1]
        P = ss.csr_matrix((np.ones(g["nnz"]), (rows, cols)), shape=(n, n))
        assert P.max() == 1                                  # no column twice in a row
        Hp = H.copy()
        Hp.data[:] = 1.0
        assert (Hp - Hp.multiply(P)).nnz == 0                # host entries all in the pattern
        same_row = rows[1:] == rows[:-1]
        assert np.all(np.diff(cols)[same_row] > 0)          # columns increase along each row
