"""The critical Rayleigh number search on the GPU eigensolver (kore_gb300.onset,
restating tests/jones2000/find_Rac.py) finds the reference's golden onset
(tests/jones2000/reference.jones: Ra_c = 4.66986e6, omega_c = -1.93444e-2)."""
import numpy as np
import pytest

from test_onset import JONES_OMEGA, JONES_RAC, load_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_critical_rayleigh(gpu_lib, precision):
    from kore_gb300.onset import OnsetSearch
    from kore_gb300.structure import layout_from_params
    meta, Aa, dA, B = load_pair("jones2000_onset")
    s = OnsetSearch(Aa, dA, meta["Ra_a"], meta["Ra_b"], B, layout_from_params(meta), nev=meta["nev"], which="TR",
                    tau=complex(*meta["tau"]), precision=precision)
    Ra_c, omega = s.critical(np.log10(4.6e6), dx=0.01, tol=1e-6)
    assert abs(Ra_c / JONES_RAC - 1) < 2e-6, (Ra_c, s.evaluations)
    assert abs(omega - JONES_OMEGA) < 1e-6, omega
