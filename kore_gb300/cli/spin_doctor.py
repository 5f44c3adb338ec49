#!/usr/bin/env python3
"""Drop-in for kore's ``bin/spin_doctor.py`` (hydrodynamic problem in a shell), with the
diagnostics computed on the GPU.

Run it from a kore case directory after a solve::

    python kore_gb300/cli/spin_doctor.py [-kore_device 0]

It reads what ``bin/spin_doctor.py`` reads (``parameters`` from ``./bin``,
``eigenvalues0.dat``, ``{real,imag}_flow.field``, ``bin/spin_doctor.py:22-70``), prints
the same table (damping, frequency, resid0, resid1, poloidal/toroidal energy ratio,
``:117-119, 239-242``) and appends one row per solution to ``flow.dat`` in the
reference's 14 columns (``:357-364``): KE, KP, KT, Dkin, Dint, Wlor, Wthm, Wcmp,
resid0, resid1 and the viscous torques on the mantle and the inner core (real and
imaginary parts).  The power terms Wlor, Wthm and Wcmp are zero for the hydrodynamic
problem; the torque columns are NaN, because the reference's torque operators
(``bin/utils.py:1288-1402``) are tables for a spheroidal container that this path does
not carry.  Magnetic, thermal and compositional diagnostics are not computed: the
script stops with a message for such cases.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from kore_gb300.cli.solve import parse_options  # noqa: E402


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    opts = parse_options(argv)
    device = int(opts.get("kore_device", 0))
    sys.path.insert(0, os.path.join(os.getcwd(), "bin"))
    import parameters as par
    from kore_gb300.diagnostics import flow_diagnostics
    from kore_gb300.structure import radial_size

    if getattr(par, "magnetic", 0) or getattr(par, "thermal", 0) or getattr(par, "compositional", 0):
        sys.exit("kore_gb300 spin_doctor: only the hydrodynamic problem is diagnosed on this path")
    if not par.ricb > 0:
        sys.exit("kore_gb300 spin_doctor: only the spherical shell (ricb > 0) is diagnosed on this path")
    if getattr(par, "forcing", 0) != 0:
        sys.exit("kore_gb300 spin_doctor: forced solutions are not diagnosed on this path")
    n = int(radial_size(par.N, par.ricb) * (par.lmax - par.m + 1) / 2)
    eig = np.loadtxt("eigenvalues0.dat").reshape((-1, 2))
    ru = np.loadtxt("real_flow.field").reshape((2 * n, -1))
    iu = np.loadtxt("imag_flow.field").reshape((2 * n, -1))
    lam = eig[:, 0] + 1j * eig[:, 1]
    X = ru + 1j * iu
    OmgTau = getattr(par, "OmgTau", 1.0)
    d = flow_diagnostics(X, lam[:X.shape[1]], par.m, par.symm, par.lmax, par.N, par.ricb, par.Ek, OmgTau, device)
    print("\n  *     Damping sigma   Frequency w     resid0     resid1     Tor/Pol")
    rows = []
    for i, (l, x) in enumerate(zip(lam, d)):
        print(" {:2d}   {: 12.9f}   {: 12.9f}   {:8.2e}   {:8.2e}   {:8.2e}".format(
            i, l.real, l.imag, x["resid0"], x["resid1"], x["KT"] / x["KP"]))
        rows.append([x["KE"], x["KP"], x["KT"], x["Dkin"], x["Dint"], 0.0, 0.0, 0.0, x["resid0"], x["resid1"],
                     np.nan, np.nan, np.nan, np.nan])
    with open("flow.dat", "ab") as f:
        np.savetxt(f, np.array(rows))
    return 0


if __name__ == "__main__":
    sys.exit(main())
