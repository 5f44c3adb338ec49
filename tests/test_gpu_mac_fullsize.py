"""The dipole MAC shell at full size (m=1, Ek=1e-6, N=200, lmax=200: 100,000 unknowns in
ℓ-superblocks of 600 and 400, the pencil restated by kore_gb300.assembly_mac and pinned
to the reference's assembly by tests/test_assembly.py): the critical Rayleigh number
found by the onset search of tests/jones2000/find_Rac.py in both precisions, and the
eigenpairs at twice it placed against FP64 measurements of how well they are determined
(kore_gb300.conditioning), as for the hydrodynamic headline problem."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mac3():
    import bench
    from kore_gb300 import layout_from_params
    from kore_gb300.assembly_mac import mac_params, mac_pencil_parts
    c = bench.MAC["mac3"]
    A0, Ab, B, nrm = mac_pencil_parts(c["m"], c["symm"], c["Ek"], c["N"], c["lmax"], c["ricb"], Em=c["Em"],
                                      Le2=c["Le2"], Prandtl=c["Prandtl"])
    lay = layout_from_params(mac_params(c["m"], c["symm"], c["Ek"], c["N"], c["lmax"], c["ricb"]))
    bv = -(c["Ek"] ** 2) / c["Prandtl"]
    return c, (A0 / nrm).tocsr(), (bv * Ab / nrm).tocsr(), (B / nrm).tocsr(), lay


def search(mac3, precision):
    from kore_gb300.onset import OnsetSearch
    c, A0, dA, B, lay = mac3
    S = OnsetSearch(A0, dA, 0.0, 1.0, B, lay, nev=16, which="TR", tau=0.0, precision=precision)
    Rac, wc = S.critical(c["log10_ra0"], dx=0.02, tol=1e-6, maxsteps=40)
    return S, Rac, wc


def test_critical_rayleigh_number_both_precisions(gpu_lib, mac3):
    """The growth rate of the leading mode changes sign at Ra_c, and the mixed path's
    search lands on the FP64 one's Ra_c and drift frequency."""
    S, Rac, wc = search(mac3, "fp64")
    assert S.sigma(np.log10(Rac) - 1e-3) < 0 < S.sigma(np.log10(Rac) + 1e-3)
    assert 1e8 < Rac < 1e10 and abs(wc) < 1e-2, (Rac, wc)
    Sm, Racm, wcm = search(mac3, "mixed")
    assert abs(Racm - Rac) <= 1e-4 * Rac, (Racm, Rac)
    assert abs(wcm - wc) <= 1e-3 * abs(wc), (wcm, wc)


def test_eigenpairs_at_twice_critical(gpu_lib, mac3):
    """At Ra = 2 Ra_c, target 0.1i, 8 pairs: mixed residuals at the FP64 level, every
    mixed eigenvalue within the band that a 1e-16 relative perturbation of A opens in the
    FP64 eigenvalues, and inside the window of the 8 nearest."""
    import bench
    from kore_gb300 import Pencil
    from kore_gb300 import conditioning as cd
    c, A0, dA, B, lay = mac3
    _, Rac, _ = search(mac3, "fp64")
    A = (A0 + (2 * Rac) * dA).tocsr()
    tau, nev = c["tau"], c["nev"]
    ref, Xref, ref_res = cd.reference(A, B, lay, tau, nev)
    band, sets = cd.perturbation_band(A, B, lay, tau, nev, ref)
    with Pencil(A, B, layout=lay) as p:
        E = bench.run_eps(p, tau, nev, c["which"], "mixed", 5)
        lam, X = E.eigenvalues(), E.eigenvectors()
    assert len(lam) >= nev
    r = cd.compare(A, B, tau, nev, lam, X, ref, ref_res, band, sets)
    assert r["in_window"] == nev, r
    assert r["within_band"] == nev, r
    assert r["resid"] <= max(4.0 * r["fp64_resid"], 1e-15), r
    assert max(ref_res[:nev]) < 1e-14
