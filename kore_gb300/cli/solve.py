#!/usr/bin/env python3
"""Drop-in replacement for kore's ``bin/solve.py`` running on the GB300 solve path.

Run it from a kore case directory, with the same options the reference takes::

    python kore_gb300/cli/solve.py -st_type sinvert -eps_error_relative ::ascii_info_detail

It reads what ``bin/solve.py`` reads and writes what it writes:
  * ``parameters`` imported from ``./bin`` (``bin/solve.py:24``), ``A.npz`` and ``B.npz``
    (eigenproblem) or ``B_forced.npz`` (forced problem, ``par.forcing != 0``) in the CSR
    form ``np.savez`` wrote (``bin/utils.py:1253-1256``);
  * ``eigenvalues0.dat`` (one row per converged pair: Re, Im),
    ``{real,imag}_{flow,magnetic,temperature,composition}.field`` (one column per
    solution, original unknown order), ``timing.dat`` (appended) and
    ``no_conv_solution`` when nothing converged (``bin/solve.py:163-311``).
Options with no effect on this path (MUMPS/PC choices, balancing, viewers) are
accepted and ignored with a warning; ``-kore_precision fp64|mixed`` (default mixed),
``-kore_seed``, ``-kore_device`` and ``-kore_refine_tol`` select this path's settings.
``-kore_binary`` also writes the same arrays in binary form next to the text files
(``eigenvalues0.npy``, ``{real,imag}_<field>.field.npy``): the text files of a 240k
unknown case hold millions of numbers and take longer to write than the solve.
"""
import os
import sys
from timeit import default_timer as timer

import numpy as np
import scipy.sparse as ss

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

KNOWN = {"st_type", "eps_nev", "eps_ncv", "eps_tol", "eps_max_it", "eps_purify", "ksp_type", "pc_type", "nbl",
         "kore_precision", "kore_seed", "kore_device", "kore_refine_tol", "kore_binary"}
IGNORED_PREFIX = ("mat_mumps", "st_pc_factor", "pc_factor", "eps_balance", "eps_true_residual", "eps_view",
                  "eps_error", "log_view", "ksp_view", "ksp_monitor", "eps_monitor", "st_ksp", "st_pc")


def parse_options(argv):
    """PETSc-style argv -> dict (option name without the dash -> value or True)."""
    opts = {}
    i = 0
    while i < len(argv):
        a = argv[i]
        if a.startswith("-") and len(a) > 1 and not _is_number(a):
            name = a[1:]
            if i + 1 < len(argv) and (not argv[i + 1].startswith("-") or _is_number(argv[i + 1])):
                opts[name] = argv[i + 1]
                i += 2
            else:
                opts[name] = True
                i += 1
        else:
            i += 1
    return opts


def _is_number(s):
    try:
        float(s)
        return True
    except ValueError:
        return False


def load_csr(path):
    """CSR from an np.savez archive (bin/utils.py:1253-1256)."""
    z = np.load(path)
    return ss.csr_matrix((z["data"], z["indices"], z["indptr"]), shape=tuple(z["shape"]))


def write_fields(vec, n, par, forced, binary=False):
    from kore_gb300.structure import field_offsets
    off = field_offsets(n, int(par.hydro), int(par.magnetic), int(par.thermal),
                        int(getattr(par, "compositional", 0)), forced=forced)
    names = {"flow": "flow", "magnetic": "magnetic", "temperature": "temperature", "composition": "composition"}
    for key, (a, b) in off.items():
        part = vec[a:b]
        if part.ndim == 1:
            part = part.reshape(-1, 1)
        with open(f"real_{names[key]}.field", "wb") as f:
            np.savetxt(f, np.real(part))
        with open(f"imag_{names[key]}.field", "wb") as f:
            np.savetxt(f, np.imag(part))
        if binary:
            np.save(f"real_{names[key]}.field.npy", np.ascontiguousarray(np.real(part)))
            np.save(f"imag_{names[key]}.field.npy", np.ascontiguousarray(np.imag(part)))


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    opts = parse_options(argv)
    for k in opts:
        if k not in KNOWN:
            if not k.startswith(IGNORED_PREFIX):
                sys.stderr.write(f"kore_gb300 solve: option -{k} ignored\n")
    sys.path.insert(0, os.path.join(os.getcwd(), "bin"))
    import parameters as par
    from kore_gb300 import EPS, KSP, Pencil, layout_from_params
    from kore_gb300.structure import radial_size

    tic = timer()
    n = int(radial_size(par.N, par.ricb) * (par.lmax - par.m + 1) / 2)   # bin/utils.py:24-25
    precision = str(opts.get("kore_precision", "mixed"))
    device = int(opts.get("kore_device", 0))
    A = load_csr("A.npz")
    lay = layout_from_params(par)
    forced = int(getattr(par, "forcing", 0)) != 0
    binary = bool(opts.get("kore_binary", False)) and str(opts.get("kore_binary")) != "0"
    success = 0
    if not forced:
        B = load_csr("B.npz")
        if "nbl" in opts and int(opts["nbl"]) != B.shape[0]:
            sys.stderr.write("kore_gb300 solve: -nbl differs from the size of B; the size of B is used\n")
        with Pencil(A, B, layout=lay, device=device) as p:
            E = EPS()
            E.setOperators(p)
            E.setProblemType(EPS.ProblemType.GNHEP)
            E.setDimensions(par.nev)
            E.setTolerances(par.tol, par.maxit)
            E.setWhichEigenpairs(par.which_eigenpairs)
            E.setTarget(par.tau)
            E.setFromOptions({k: v for k, v in opts.items() if k in KNOWN})
            E.solve()
            nconv = E.getConverged()
            if nconv > 0:
                lam = E.eigenvalues()
                X = E.eigenvectors()
                if "eps_error_relative" in opts:
                    print(" ---------------------- --------------------")
                    print("            k             ||Ax-kBx||/||kx||")
                    print(" ---------------------- --------------------")
                    for i in range(nconv):
                        r = p.residual(lam[i], X[:, i])
                        err = np.linalg.norm(r) / (abs(lam[i]) * np.linalg.norm(X[:, i]))
                        print(f" {lam[i].real:+.6f}{lam[i].imag:+.6f}i {err:12g}")
                    print(" ---------------------- --------------------")
                eigval = np.column_stack([lam.real, lam.imag])
                with open("eigenvalues0.dat", "wb") as f:
                    np.savetxt(f, eigval)
                if binary:
                    np.save("eigenvalues0.npy", eigval)
                write_fields(X, n, par, forced=False, binary=binary)
                success = nconv
            else:
                print("No converged solution found")
                np.savetxt("no_conv_solution", [0])
    else:
        b = load_csr("B_forced.npz").toarray().ravel().astype(np.complex128)
        with Pencil(A, None, layout=lay, device=device) as p:
            K = KSP()
            K.setOperators(p)
            K.setTolerances(rtol=par.tol, max_it=par.maxit)
            K.setFromOptions({k: v for k, v in opts.items() if k in KNOWN})
            try:
                x = K.solve(b)
            except RuntimeError as e:
                if "KORE_ENAN" not in str(e):
                    raise
                x = np.full_like(b, np.nan)
        if np.isnan(x).any() or np.isinf(x).any():
            print("Solver crashed, got nan's!")
        else:
            success = 1
            print("Solution(s) computed")
            write_fields(x, n, par, forced=True, binary=binary)
    toc = timer()
    print("Solve done in", toc - tic, "seconds")
    with open("timing.dat", "ab") as f:
        np.savetxt(f, np.array([toc - tic]))
    return 0


if __name__ == "__main__":
    sys.exit(main())
