#!/usr/bin/env python3
"""Generate the golden pencil fixtures in ``tests/golden/`` from the reference itself.

For each case this script
  1. copies the reference's ``bin/`` into a scratch directory,
  2. writes ``bin/parameters.py`` from a base parameter file plus overrides
     (the same ``sed`` style edit the reference's own tests and tools use,
     ``tests/jones2000/find_Rac.py:31``),
  3. runs the reference's unmodified ``compute_profiles.py`` (magnetic cases),
     ``submatrices.py`` and ``assemble.py``, the latter under the single-rank
     ``mpi4py`` stand-in in ``_standin/``,
  4. stores A, B (or the forcing column) and the derived sizes in
     ``tests/golden/<case>.npz``.

It needs a checkout of the reference, named by ``$KORE_REF``, and is run by hand;
the fixtures it writes are committed so that the tests never read the reference at
run time.

    KORE_REF=<kore checkout> python tests/golden/make_fixtures.py [case ...]
"""
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("KORE_REF", "")
STANDIN = os.path.join(HERE, "_standin")

# case name -> (base parameter file relative to the reference root, overrides, needs profiles)
CASES = {
    # the reference's spin-over test, byte-identical parameters (tests/spinover/params.spinover)
    "spinover": ("tests/spinover/params.spinover", {}, False),
    # hydrodynamic shell, m=1 symmetric, Ek=1e-4, N=48, lmax=40 (2k unknowns)
    "shell_m1_ek1e-4": ("bin/parameters.py", {
        "symm": "1", "Ek": "1e-4", "N": "48", "lmax": "40", "itau": "1.0",
        "nev": "10", "which_eigenpairs": "'TM'"}, False),
    # smaller hydrodynamic shell with an m=2 target on the imaginary axis
    "shell_m2_small": ("bin/parameters.py", {
        "m": "2", "symm": "1", "Ek": "1e-5", "N": "40", "lmax": "31", "itau": "0.5",
        "nev": "16", "which_eigenpairs": "'TM'"}, False),
    # forced problem: m=2 radial boundary forcing (forcing 10), omega = 0.7
    "forced_m2_f10": ("bin/parameters.py", {
        "m": "2", "symm": "1", "Ek": "1e-4", "N": "40", "lmax": "31",
        "forcing": "10", "forcing_frequency": "0.7"}, False),
    # forced problem: m=2 libration (forcing 7), omega = -1.3
    "forced_m2_f7": ("bin/parameters.py", {
        "m": "2", "symm": "1", "Ek": "1e-4", "N": "32", "lmax": "21",
        "forcing": "7", "forcing_frequency": "-1.3"}, False),
    # the same m=2 shell as an eigenproblem (forced A = |B|_F (A_eig - i w B_eig))
    "shell_m2_ek1e-4": ("bin/parameters.py", {
        "m": "2", "symm": "1", "Ek": "1e-4", "N": "40", "lmax": "31", "itau": "0.5",
        "nev": "8"}, False),
    # Jones et al. 2000 onset at the golden critical Rayleigh number (tests/jones2000)
    "jones2000_rac": ("tests/jones2000/params.jones", {
        "Ra_gap": "4.66986e6", "nev": "12", "which_eigenpairs": "'TR'"}, False),
    # Dormy et al. 2004 onset at the golden critical Rayleigh number (tests/dormy2004)
    "dormy2004_rac": ("tests/dormy2004/params.dormy04", {
        "Ra_gap": "1.65404e6", "nev": "12", "which_eigenpairs": "'TR'"}, False),
    # small magneto-Archimedes-Coriolis case: dipole B0, insulating mantle, thermal
    "mac_dipole_small": ("bin/parameters.py", {
        "symm": "1", "Ek": "1e-3", "N": "24", "lmax": "16", "itau": "0.1",
        "magnetic": "1", "thermal": "1", "B0": "'dipole'", "Pm": "1e-3",
        "Lambda": "0.1", "Ra_gap": "1e5", "nev": "8"}, True),
    # dipole MAC case of 3,200 unknowns, antisymmetric flow, fixed heat flux at the outer boundary
    "mac_dipole_medium": ("bin/parameters.py", {
        "symm": "-1", "Ek": "1e-4", "N": "40", "lmax": "32", "itau": "0.1",
        "magnetic": "1", "thermal": "1", "B0": "'dipole'", "Pm": "1e-3",
        "Lambda": "1e-4", "Ra_gap": "5e5", "bco_thermal": "1", "nev": "8"}, True),
    # dipole MAC case with internal heating, m=2, fixed heat flux at the inner boundary
    "mac_dipole_internal": ("bin/parameters.py", {
        "m": "2", "symm": "1", "Ek": "1e-3", "N": "24", "lmax": "17", "itau": "0.1",
        "magnetic": "1", "thermal": "1", "B0": "'dipole'", "heating": "'internal'",
        "Pm": "1e-3", "Lambda": "0.1", "Ra_gap": "1e5", "bci_thermal": "1", "nev": "8"}, True),
    # small quadrupole-field case (l +- 2 coupling through B0)
    "mac_quadrupole_small": ("bin/parameters.py", {
        "symm": "1", "Ek": "1e-3", "N": "24", "lmax": "16", "itau": "0.1",
        "magnetic": "1", "B0": "'Luo_S2'", "Pm": "1e-3", "Lambda": "0.1",
        "nev": "8"}, True),
}

DERIVED = ("m symm ricb N lmax hydro magnetic thermal compositional B0 forcing "
           "forcing_frequency nev tol maxit which_eigenpairs Ek Em Le2 Prandtl Ra heating "
           "bci_thermal bco_thermal cnorm").split()


def edit_params(text, overrides):
    for name, value in overrides.items():
        pat = re.compile(r"^(\s*)" + re.escape(name) + r"\s*=.*$", re.M)
        if not pat.search(text):
            raise KeyError(f"parameter {name} not found")
        text = pat.sub(lambda mo: f"{mo.group(1)}{name} = {value}", text, count=1)
    return text


def run(cmd, cwd, env=None):
    r = subprocess.run(cmd, cwd=cwd, env=env, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)} failed:\n{r.stdout[-2000:]}\n{r.stderr[-4000:]}")
    return r.stdout


# Pencils whose A is affine in the Rayleigh number (only the buoyancy coupling depends
# on Ra_gap): the reference assembles A at two Rayleigh numbers; the fixture stores
# A_a = A(Ra_a), dA = A(Ra_b) - A(Ra_a) and B (which does not depend on Ra), so that
# A(Ra) = A_a + (Ra - Ra_a) / (Ra_b - Ra_a) dA.  Used by the critical-Rayleigh search
# (tests/jones2000/find_Rac.py).
RA_PAIRS = {
    "jones2000_onset": ("jones2000_rac", 4.6e6, 4.8e6),
}


def make_case(name, extra=None, dst=None):
    base, overrides, profiles = CASES[name]
    if extra:
        overrides = dict(overrides, **extra)
    with tempfile.TemporaryDirectory(prefix=f"korefx_{name}_") as tmp:
        shutil.copytree(os.path.join(REF, "bin"), os.path.join(tmp, "bin"))
        with open(os.path.join(REF, base)) as f:
            text = edit_params(f.read(), overrides)
        with open(os.path.join(tmp, "bin", "parameters.py"), "w") as f:
            f.write(text)
        env = dict(os.environ)
        env["PYTHONPATH"] = STANDIN + os.pathsep + env.get("PYTHONPATH", "")
        py = sys.executable
        if profiles:
            run([py, "bin/compute_profiles.py"], tmp, env)
        run([py, "bin/submatrices.py", "4"], tmp, env)
        run([py, "bin/assemble.py"], tmp, env)
        probe = ("import sys, json; sys.path.insert(0, 'bin'); import parameters as par, utils as ut;"
                 "d = {k: getattr(par, k) for k in %r};"
                 "d['tau'] = [float(par.tau.real), float(par.tau.imag)];"
                 "d.update(N1=int(ut.N1), n=int(ut.n), sizmat=int(ut.sizmat), symmB0=int(ut.symmB0));"
                 "print(json.dumps(d, default=lambda v: v.item() if hasattr(v, 'item') else str(v)))"
                 % (DERIVED,))
        meta = json.loads(run([py, "-c", probe], tmp, env).strip().splitlines()[-1])
        out = {"meta": np.array(json.dumps(meta))}
        a = np.load(os.path.join(tmp, "A.npz"))
        for k in ("data", "indices", "indptr", "shape"):
            out["A_" + k] = a[k]
        bname = "B.npz" if meta["forcing"] == 0 else "B_forced.npz"
        b = np.load(os.path.join(tmp, bname))
        for k in ("data", "indices", "indptr", "shape"):
            out["B_" + k] = b[k]
        dst = dst or os.path.join(HERE, name + ".npz")
        np.savez_compressed(dst, **out)
        return name, meta["sizmat"], os.path.getsize(dst)


def make_ra_pair(name):
    import scipy.sparse as ss
    case, ra_a, ra_b = RA_PAIRS[name]
    with tempfile.TemporaryDirectory(prefix=f"korefx_{name}_") as tmp:
        za, zb = os.path.join(tmp, "a.npz"), os.path.join(tmp, "b.npz")
        make_case(case, {"Ra_gap": repr(ra_a)}, za)
        make_case(case, {"Ra_gap": repr(ra_b)}, zb)
        a, b = np.load(za), np.load(zb)
        A = [ss.csr_matrix((z["A_data"], z["A_indices"], z["A_indptr"]), shape=tuple(z["A_shape"])) for z in (a, b)]
        Bd = [ss.csr_matrix((z["B_data"], z["B_indices"], z["B_indptr"]), shape=tuple(z["B_shape"])) for z in (a, b)]
        if abs(Bd[0] - Bd[1]).max() != 0:
            raise RuntimeError("B depends on Ra")
        dA = (A[1] - A[0]).tocsr()
        dA.eliminate_zeros()
        meta = json.loads(str(a["meta"]))
        meta.update(Ra_a=ra_a, Ra_b=ra_b)
        out = {"meta": np.array(json.dumps(meta))}
        for k, M in (("A", A[0]), ("dA", dA)):
            M = M.tocsr()
            out[k + "_data"], out[k + "_indices"], out[k + "_indptr"] = M.data, M.indices, M.indptr
            out[k + "_shape"] = np.array(M.shape)
        for k in ("data", "indices", "indptr", "shape"):
            out["B_" + k] = a["B_" + k]
        dst = os.path.join(HERE, name + ".npz")
        np.savez_compressed(dst, **out)
        return name, meta["sizmat"], os.path.getsize(dst)


def make_any(name):
    return make_ra_pair(name) if name in RA_PAIRS else make_case(name)


if __name__ == "__main__":
    if not REF or not os.path.isdir(os.path.join(REF, "bin")):
        sys.exit("set KORE_REF to a checkout of the reference (the directory holding bin/assemble.py)")
    names = sys.argv[1:] or list(CASES) + list(RA_PAIRS)
    from concurrent.futures import ProcessPoolExecutor
    with ProcessPoolExecutor(max_workers=min(4, len(names))) as ex:
        for name, sizmat, size in ex.map(make_any, names):
            print(f"{name}: sizmat={sizmat} file={size/1e6:.2f} MB")
