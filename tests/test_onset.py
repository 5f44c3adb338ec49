"""Critical Rayleigh number search (tests/jones2000/find_Rac.py restated in
kore_gb300.onset): the affine model of A(Ra) is pinned against the reference's own
assembly at a third Rayleigh number, and the search run with the oracle's eigensolver
finds the reference's golden critical Rayleigh number and frequency
(tests/jones2000/reference.jones)."""
import json
import os

import numpy as np
import scipy.sparse as ss

from conftest import GOLDEN, load_case

# tests/jones2000/reference.jones: Ek, -, Ra_c, m, omega_c
JONES_RAC, JONES_OMEGA = 4.66986e6, -1.93444e-2


def load_pair(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    M = {k: ss.csr_matrix((z[k + "_data"], z[k + "_indices"], z[k + "_indptr"]), shape=tuple(z[k + "_shape"]))
         for k in ("A", "dA", "B")}
    return meta, M["A"], M["dA"], M["B"]


def test_affine_model_matches_reference_assembly():
    """A(Ra_c) interpolated from the assemblies at 4.6e6 and 4.8e6 equals the reference's
    assembly at Ra_c = 4.66986e6 (tests/golden/jones2000_rac.npz)."""
    meta, Aa, dA, B = load_pair("jones2000_onset")
    m2, Ac, Bc = load_case("jones2000_rac")
    A = Aa + ((JONES_RAC - meta["Ra_a"]) / (meta["Ra_b"] - meta["Ra_a"])) * dA
    assert abs(A - Ac).max() <= 1e-12 * abs(Ac).max()
    assert abs(B - Bc).max() == 0
    assert dA.nnz < Aa.nnz // 4      # only the buoyancy coupling depends on Ra


class OracleSearch:
    """The search of kore_gb300.onset with the oracle's CPU eigensolver in place of the GPU."""

    def __new__(cls, *a, **k):
        from kore_gb300.onset import OnsetSearch
        from oracle.eps_ref import shift_invert_eigs

        class _S(OnsetSearch):
            def leading(self, Ra):
                if Ra in self.cache:
                    return self.cache[Ra]
                lam, _ = shift_invert_eigs(self.A(Ra), self.B, self.tau, self.nev, self.which, seed=1)
                i = int(np.argmax(lam.real))
                self.cache[Ra] = (float(lam[i].real), complex(lam[i]))
                self.evaluations += 1
                return self.cache[Ra]
        return _S(*a, **k)


def test_oracle_search_finds_the_golden_onset():
    from kore_gb300.structure import layout_from_params
    meta, Aa, dA, B = load_pair("jones2000_onset")
    s = OracleSearch(Aa, dA, meta["Ra_a"], meta["Ra_b"], B, layout_from_params(meta), nev=meta["nev"],
                     which="TR", tau=complex(*meta["tau"]))
    Ra_c, omega = s.critical(np.log10(4.6e6), dx=0.01, tol=1e-6)
    assert abs(Ra_c / JONES_RAC - 1) < 2e-6, Ra_c
    assert abs(omega - JONES_OMEGA) < 1e-6, omega
