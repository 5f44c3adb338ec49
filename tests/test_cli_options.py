"""Option parsing of the drop-in solve.py (PETSc-style argv)."""
import os
import sys

from conftest import ROOT


def test_cli_option_parsing():
    from kore_gb300.cli.solve import parse_options
    o = parse_options(["-st_type", "sinvert", "-eps_error_relative", "::ascii_info_detail", "-eps_true_residual",
                       "-mat_mumps_icntl_14", "1000", "-kore_refine_tol", "-1e-3"])
    assert o["st_type"] == "sinvert" and o["eps_true_residual"] is True and o["mat_mumps_icntl_14"] == "1000"
    assert float(o["kore_refine_tol"]) == -1e-3
