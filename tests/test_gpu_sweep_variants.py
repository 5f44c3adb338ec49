"""Every compiled variant of the sweep kernel (2, 3, 4 CTAs per SM x 8 and 16 KB ring
slots, complex64 and complex128 factors), pinned with kore_sweep_variant, solves
(A - sigma B) x = b to the oracle's accuracy.  The autotuner runs every variant on the
first sweep of a plan shape but keeps the output of the one it chooses only, so without
this test a variant that computed a wrong result would go unseen."""
import numpy as np
import pytest

from oracle.eps_ref import solve_residual

pytestmark = pytest.mark.gpu

VARIANTS = [(2, 16384), (3, 16384), (4, 16384), (2, 8192), (3, 8192), (4, 8192)]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("cps,chunk", VARIANTS)
def test_sweep_variant_solves(gpu_lib, case, precision, cps, chunk):
    from kore_gb300 import Pencil, layout_from_params, sweep_variant
    meta, A, B = case("spinover")
    rng = np.random.default_rng(cps * 7 + chunk)
    b = rng.standard_normal(A.shape[0]) + 1j * rng.standard_normal(A.shape[0])
    sigma = 0.37j
    sweep_variant(cps, chunk)
    try:
        with Pencil(A, B, layout=layout_from_params(meta)) as p:
            p.factor(sigma, precision)
            x = p.solve(b, refine_tol=1e-14)
            prof = p.profile(False)
    finally:
        sweep_variant()
    assert (prof["sweep_ctas_per_sm"], prof["sweep_chunk_bytes"]) == (cps, chunk)
    assert solve_residual((A - sigma * B).tocsr(), x, b) < 1e-14


def test_sweep_variant_rejects_unknown(gpu_lib):
    assert gpu_lib.kore_sweep_variant(5, 8192) == 1   # KORE_EINVAL
    assert gpu_lib.kore_sweep_variant(4, 4096) == 1
    assert gpu_lib.kore_sweep_variant(0, 0) == 0
