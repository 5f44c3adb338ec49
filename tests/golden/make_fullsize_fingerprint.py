#!/usr/bin/env python3
"""Fingerprint of the reference's own assembly of the full benchmark pencil.

The 240,000-unknown hydrodynamic shell (m=2, symm=1, Ek=1e-7, N=400, lmax=601,
ricb=0.35) is assembled by the reference's unmodified ``submatrices.py`` and
``assemble.py`` (through ``make_fixtures.make_case``, in a scratch directory); its A.npz is
172 MB, too large to commit.  This script stores instead, in
``tests/golden/shell2_fingerprint.npz``:

* the shapes, nonzero counts and Frobenius norms of A and B;
* for 4096 rows drawn with a fixed seed: those rows of A v and B v for a seeded complex
  standard-normal vector v, and the rows' 1-norms in A and B.

``tests/test_assembly.py`` builds the same pencil with ``kore_gb300.assembly`` and
compares these numbers.

    KORE_REF=<kore checkout> python tests/golden/make_fullsize_fingerprint.py
"""
import json
import os
import sys
import tempfile

import numpy as np
import scipy.sparse as ss
import scipy.sparse.linalg as ssl

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import make_fixtures as mf  # noqa: E402

CASE = ("bin/parameters.py", {
    "m": "2", "symm": "1", "Ek": "1e-7", "N": "400", "lmax": "601", "itau": "0.5",
    "nev": "16", "which_eigenpairs": "'TM'"}, False)
ROW_SEED, VEC_SEED, NROWS = 2024, 77, 4096


def fingerprint(A, B):
    """The stored quantities of a pencil (see the module docstring)."""
    n = A.shape[0]
    rows = np.sort(np.random.default_rng(ROW_SEED).choice(n, NROWS, replace=False))
    rng = np.random.default_rng(VEC_SEED)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    A, B = A.tocsr(), B.tocsr()
    return {"rows": rows, "Av": (A @ v)[rows], "Bv": (B @ v)[rows],
            "A_row1": np.asarray(abs(A[rows]).sum(axis=1)).ravel(),
            "B_row1": np.asarray(abs(B[rows]).sum(axis=1)).ravel(),
            "A_fro": ssl.norm(A), "B_fro": ssl.norm(B), "A_nnz": A.nnz, "B_nnz": B.nnz,
            "shape": np.array(A.shape)}


def main():
    if not mf.REF or not os.path.isdir(os.path.join(mf.REF, "bin")):
        sys.exit("set KORE_REF to a checkout of the reference (the directory holding bin/assemble.py)")
    mf.CASES["shell2_full"] = CASE
    with tempfile.TemporaryDirectory(prefix="korefp_") as tmp:
        dst = os.path.join(tmp, "full.npz")
        mf.make_case("shell2_full", dst=dst)
        z = np.load(dst)
        A = ss.csr_matrix((z["A_data"], z["A_indices"], z["A_indptr"]), shape=tuple(z["A_shape"]))
        B = ss.csr_matrix((z["B_data"], z["B_indices"], z["B_indptr"]), shape=tuple(z["B_shape"]))
        meta = json.loads(str(z["meta"]))
    out = fingerprint(A, B)
    out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, "shell2_fingerprint.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
