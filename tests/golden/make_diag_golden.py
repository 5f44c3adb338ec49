#!/usr/bin/env python3
"""Golden values of kore's flow diagnostics, computed by the reference's own code.

For each case this script takes the fixture pencil of ``tests/golden/<case>.npz``,
computes a few eigenpairs with the oracle (unit eigenvectors, original unknown order),
and runs the reference's unmodified ``bin/utils4pp.py`` ``diagnose`` on them (in a copy
of the reference's ``bin/`` with the case's ``parameters.py``, as ``bin/spin_doctor.py``
calls it).  It stores the eigenvectors, the eigenvalues and the per-degree kinetic
energy, diffusion and internal-dissipation integrals in
``tests/golden/diag_<case>.npz``, so the tests never read the reference at run time.

    KORE_REF=<kore checkout> python tests/golden/make_diag_golden.py
"""
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, HERE)

from make_fixtures import CASES, REF, edit_params  # noqa: E402

DIAG_CASES = {"shell_m1_ek1e-4": 4, "shell_m2_ek1e-4": 3}

# run inside the reference's bin/ copy: diagnose() of every vector in vecs.npy
PROBE = r"""
import json, sys
import numpy as np
sys.path.insert(0, 'bin')
import parameters as par, utils as ut, utils4pp as upp
X = np.load('vecs.npy')
out = []
for j in range(X.shape[1]):
    u2 = upp.expand_reshape_sol(X[:, j], par.symm)
    udgn = upp.diagnose(u2, 0, 0, 0, par.ricb, ut.rcmb, 1)[0]
    out.append(np.asarray(udgn)[:, :3].tolist())
print(json.dumps(out))
"""


def make(name, nvec):
    from conftest import load_case
    from oracle.eps_ref import shift_invert_eigs
    meta, A, B = load_case(name)
    lam, X = shift_invert_eigs(A, B, complex(*meta["tau"]), nvec, "TM")
    base, overrides, _ = CASES[name]
    with tempfile.TemporaryDirectory(prefix=f"korediag_{name}_") as tmp:
        shutil.copytree(os.path.join(REF, "bin"), os.path.join(tmp, "bin"))
        with open(os.path.join(REF, base)) as f:
            text = edit_params(f.read(), overrides)
        with open(os.path.join(tmp, "bin", "parameters.py"), "w") as f:
            f.write(text)
        np.save(os.path.join(tmp, "vecs.npy"), X)
        r = subprocess.run([sys.executable, "-c", PROBE], cwd=tmp, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stderr[-4000:])
        per_l = np.array(json.loads(r.stdout.strip().splitlines()[-1]))   # (nvec, degrees, 3)
    dst = os.path.join(HERE, f"diag_{name}.npz")
    np.savez_compressed(dst, lam=lam, X=X, per_l=per_l, meta=np.array(json.dumps(meta)))
    return dst


if __name__ == "__main__":
    if not REF or not os.path.isdir(os.path.join(REF, "bin")):
        sys.exit("set KORE_REF to a checkout of the reference (the directory holding bin/assemble.py)")
    for name, nvec in DIAG_CASES.items():
        print(make(name, nvec))
