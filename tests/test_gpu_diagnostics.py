"""GPU flow diagnostics (kore_flow_diagnostics, kore_gb300.diagnostics) against the
reference's own bin/utils4pp.py diagnose() (golden per-degree integrals written by
tests/golden/make_diag_golden.py), against the oracle's restatement on GPU eigenpairs,
and, at the full 240k-unknown size where no oracle runs, through the power balance of
the modes (bin/spin_doctor.py's resid0 and resid1) for both precisions."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle.diag_ref import flow_diagnostics as flow_ref

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["shell_m1_ek1e-4", "shell_m2_ek1e-4"])
def test_per_degree_integrals_match_reference(gpu_lib, name):
    from kore_gb300.diagnostics import flow_integrals
    z = np.load(os.path.join(GOLDEN, f"diag_{name}.npz"))
    meta = json.loads(str(z["meta"]))
    per, degrees = flow_integrals(z["X"], meta["m"], meta["symm"], meta["lmax"], meta["N"], meta["ricb"])
    order = np.argsort(degrees, kind="stable")   # the reference lists degrees in increasing order
    ref = z["per_l"]
    for j in range(ref.shape[0]):
        scale = np.abs(ref[j]).max(axis=0)
        assert np.all(np.abs(per[j, order] - ref[j]) <= 1e-11 * scale), j


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_diagnostics_of_gpu_eigenpairs(gpu_lib, case, precision):
    from kore_gb300 import Pencil, layout_from_params
    from kore_gb300 import conditioning as cd
    from kore_gb300.diagnostics import flow_diagnostics
    from kore_gb300.structure import ell
    meta, A, B = case("shell_m1_ek1e-4")
    tau = complex(*meta["tau"])
    with Pencil(A, B, layout=layout_from_params(meta)) as p:
        lam, X = cd.solve(p, tau, 6, precision, 1)
    got = flow_diagnostics(X[:, :6], lam[:6], meta["m"], meta["symm"], meta["lmax"], meta["N"], meta["ricb"],
                           meta["Ek"])
    lp, lt = ell(meta["m"], meta["lmax"], meta["symm"])
    for j in range(6):
        ref = flow_ref(X[:, j], lp, lt, meta["N"], meta["ricb"], lam[j], Ek=meta["Ek"])
        for k in ("KE", "KP", "KT", "Dkin", "Dint"):
            assert abs(got[j][k] - ref[k]) <= 1e-11 * abs(ref[k]), (j, k)
        # the power balance of a mode of this (coarse, N = 48) discretisation
        assert got[j]["resid1"] < 1e-4 and got[j]["resid0"] < 1e-2, got[j]


def test_power_balance_at_full_size(gpu_lib):
    """240k-unknown shell at 0.5i: the mixed eigenpairs satisfy the modes' power balance
    as well as the FP64 path's do."""
    import bench
    from kore_gb300 import Pencil
    from kore_gb300 import conditioning as cd
    from kore_gb300.diagnostics import flow_diagnostics
    A, B, lay = bench.build_pencil("shell2")
    m, symm, Ek, N, lmax, ricb, tau, nev, which = bench.WORKLOADS["shell2"]
    with Pencil(A, B, layout=lay) as p:
        res = {prec: cd.solve(p, tau, nev, prec, 5, maxit=50) for prec in ("fp64", "mixed")}
    r1 = {}
    for prec, (lam, X) in res.items():
        d = flow_diagnostics(X[:, :nev], lam[:nev], m, symm, lmax, N, ricb, Ek)
        r1[prec] = np.array([x["resid1"] for x in d])
        assert all(x["KE"] > 0 for x in d)
    assert r1["mixed"].max() <= 4 * max(r1["fp64"].max(), 1e-12), r1
