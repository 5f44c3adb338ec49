"""The flow-diagnostics restatement of the oracle (oracle/diag_ref.py) against the
reference's own bin/utils4pp.py diagnose(), whose per-degree kinetic energy, diffusion
and internal-dissipation integrals tests/golden/make_diag_golden.py stored for
eigenvectors of two fixture pencils."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle.diag_ref import flow_l


@pytest.mark.parametrize("name", ["shell_m1_ek1e-4", "shell_m2_ek1e-4"])
def test_flow_integrals_match_reference(name):
    from kore_gb300.structure import ell
    z = np.load(os.path.join(GOLDEN, f"diag_{name}.npz"))
    meta = json.loads(str(z["meta"]))
    X, per_l = z["X"], z["per_l"]
    lp, lt = ell(meta["m"], meta["lmax"], meta["symm"])
    ll = np.sort(np.concatenate([lp, lt]))
    N, nb = meta["N"], len(lp)
    for j in range(X.shape[1]):
        P = X[:nb * N, j].reshape(nb, N)
        T = X[nb * N:, j].reshape(len(lt), N)
        for i, l in enumerate(ll):
            if l in lp:
                got = flow_l(int(l), P[list(lp).index(l)], False, N, meta["ricb"])
            else:
                got = flow_l(int(l), T[list(lt).index(l)], True, N, meta["ricb"])
            ref = per_l[j, i]
            scale = np.abs(per_l[j]).max(axis=0)
            assert np.all(np.abs(np.array(got) - ref) <= 1e-12 * scale), (j, l, got, ref)
