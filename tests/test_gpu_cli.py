"""The drop-in solve.py run like the reference's own end-to-end tests
(tests/test_spinover.py: solve in a case directory, read eigenvalues0.dat, compare the
max-Re eigenvalue with reference.eig at rtol 1e-8)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT
from oracle.eps_ref import forced_solve

pytestmark = pytest.mark.gpu

SPINOVER_GOLDEN = np.array([-1.019947097016500742e-01, 1.005733690103750355e+00])


def write_case(tmp, meta, A, B):
    os.makedirs(os.path.join(tmp, "bin"), exist_ok=True)
    tau = complex(*meta["tau"])
    lines = [f"{k} = {meta[k]!r}" for k in ("hydro", "magnetic", "thermal", "compositional", "m", "symm", "ricb",
                                            "N", "lmax", "forcing", "nev", "tol", "maxit", "which_eigenpairs", "B0",
                                            "Ek")]
    lines.append(f"tau = complex({tau.real!r}, {tau.imag!r})")
    lines.append("B0_l = 1")
    with open(os.path.join(tmp, "bin", "parameters.py"), "w") as f:
        f.write("\n".join(lines) + "\n")
    np.savez(os.path.join(tmp, "A.npz"), data=A.data, indices=A.indices, indptr=A.indptr, shape=A.shape)
    name = "B.npz" if meta["forcing"] == 0 else "B_forced.npz"
    np.savez(os.path.join(tmp, name), data=B.data, indices=B.indices, indptr=B.indptr, shape=B.shape)


def run_cli(tmp, *args):
    cmd = [sys.executable, os.path.join(ROOT, "kore_gb300", "cli", "solve.py")] + list(args)
    r = subprocess.run(cmd, cwd=tmp, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return r.stdout


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cli_spinover(gpu_lib, case, tmp_path, precision):
    meta, A, B = case("spinover")
    write_case(str(tmp_path), meta, A, B)
    out = run_cli(str(tmp_path), "-st_type", "sinvert", "-eps_error_relative", "::ascii_info_detail",
                  "-kore_precision", precision)
    assert "Solve done in" in out
    dat = np.loadtxt(tmp_path / "eigenvalues0.dat")
    i = np.argmax(dat[:, 0])
    np.testing.assert_allclose(dat[i, :], SPINOVER_GOLDEN, rtol=1e-8, atol=1e-20)
    n = meta["sizmat"] // 2
    rf = np.loadtxt(tmp_path / "real_flow.field")
    imf = np.loadtxt(tmp_path / "imag_flow.field")
    assert rf.shape == (2 * n, dat.shape[0]) and imf.shape == rf.shape
    # unit-norm eigenvectors satisfy A x = lambda B x
    lam = dat[:, 0] + 1j * dat[:, 1]
    X = rf + 1j * imf
    for k in range(len(lam)):
        x = X[:, k]
        assert abs(np.linalg.norm(x) - 1.0) < 1e-10
        assert np.linalg.norm(A @ x - lam[k] * (B @ x)) < 1e-9 * (abs(lam[k]) + 1)
    assert os.path.exists(tmp_path / "timing.dat")


def test_cli_forced(gpu_lib, case, tmp_path):
    meta, A, bf = case("forced_m2_f10")
    write_case(str(tmp_path), meta, A, bf)
    out = run_cli(str(tmp_path), "-ksp_type", "preonly", "-pc_type", "lu", "-kore_precision", "fp64")
    assert "Solution(s) computed" in out
    x = np.loadtxt(tmp_path / "real_flow.field") + 1j * np.loadtxt(tmp_path / "imag_flow.field")
    ref = forced_solve(A, bf.toarray().ravel())
    assert x.shape == ref.shape
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-9




def test_cli_binary_output_matches_text(gpu_lib, case, tmp_path):
    """-kore_binary writes the eigenvalues and fields also as .npy, equal to the text files
    up to the text format's 18 significant digits."""
    meta, A, B = case("spinover")
    write_case(str(tmp_path), meta, A, B)
    run_cli(str(tmp_path), "-st_type", "sinvert", "-kore_precision", "fp64", "-kore_binary")
    dat = np.loadtxt(tmp_path / "eigenvalues0.dat")
    np.testing.assert_allclose(np.load(tmp_path / "eigenvalues0.npy"), dat, rtol=1e-17, atol=0)
    for part in ("real", "imag"):
        txt = np.loadtxt(tmp_path / f"{part}_flow.field")
        np.testing.assert_allclose(np.load(tmp_path / f"{part}_flow.field.npy"), txt, rtol=1e-17, atol=0)


def test_cli_spin_doctor(gpu_lib, case, tmp_path):
    """solve.py then spin_doctor.py in a case directory (the reference's post-processing
    order): the printed table and flow.dat hold the power balance of every solution,
    equal to the oracle's diagnostics of the written fields."""
    from kore_gb300.structure import ell
    from oracle.diag_ref import flow_diagnostics
    meta, A, B = case("shell_m1_ek1e-4")
    write_case(str(tmp_path), meta, A, B)
    run_cli(str(tmp_path), "-st_type", "sinvert", "-kore_precision", "mixed")
    cmd = [sys.executable, os.path.join(ROOT, "kore_gb300", "cli", "spin_doctor.py")]
    r = subprocess.run(cmd, cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    dat = np.loadtxt(tmp_path / "eigenvalues0.dat").reshape(-1, 2)
    flow = np.loadtxt(tmp_path / "flow.dat").reshape(-1, 14)
    assert flow.shape[0] == dat.shape[0]
    n = meta["sizmat"] // 2
    X = np.loadtxt(tmp_path / "real_flow.field") + 1j * np.loadtxt(tmp_path / "imag_flow.field")
    lp, lt = ell(meta["m"], meta["lmax"], meta["symm"])
    for k in range(dat.shape[0]):
        ref = flow_diagnostics(X[:, k], lp, lt, meta["N"], meta["ricb"], dat[k, 0] + 1j * dat[k, 1], Ek=meta["Ek"])
        got = dict(zip(("KE", "KP", "KT", "Dkin", "Dint"), flow[k, :5]))
        for key, v in got.items():
            assert abs(v - ref[key]) <= 1e-9 * abs(ref[key]), (k, key)
        assert abs(flow[k, 9] - ref["resid1"]) <= 1e-5 * max(ref["resid1"], 1e-12)
        assert flow[k, 9] < 1e-4
