"""The tensor-core (tcgen05, 3xTF32) complex64 GEMM of the mixed-precision
factorisation against an FP64 product (kore_tc_selftest), and its effect on the
factorisation: with accurate complex64 factors the FP64 refinement converges in few
corrections."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("S", [48, 100, 240, 400])
def test_tc_gemm_matches_fp64(gpu_lib, S):
    err = ctypes.c_double(-1.0)
    assert gpu_lib.kore_tc_selftest(0, S, 6, ctypes.byref(err)) == 0
    # 3xTF32 with FP32 accumulation: a few units of 2^-24 times sqrt(S) relative to sum |a||b|
    assert 0.0 <= err.value < 4e-6, err.value


def test_mixed_factor_needs_few_corrections(gpu_lib, case):
    """Mixed-precision solves on a pencil with several reduction levels (the levels >= 1
    use the tensor-core update): backward error 1e-14 within three corrections."""
    from kore_gb300 import Pencil, layout_from_params
    from oracle.eps_ref import solve_residual
    meta, A, B = case("spinover")
    rng = np.random.default_rng(4)
    b = rng.standard_normal(A.shape[0]) + 1j * rng.standard_normal(A.shape[0])
    with Pencil(A, B, layout=layout_from_params(meta)) as p:
        assert len(p.layout.block_sizes) >= 8
        p.factor(0.37j, "mixed")
        x, st = p.solve(b, refine_tol=1e-14, stats=True)
    assert solve_residual((A - 0.37j * B).tocsr(), x, b) < 1e-14
    assert st["refine_iters_max"] <= 3, st


def test_gegenbauer_mult_matches_host(gpu_lib):
    """The GPU multiplication operators (kore_gegenbauer_mult) against the host ones,
    which tests/test_assembly.py pins to the reference's Mlam through its matrices: the
    r^X coefficients converted to C^(Y) for every operator the hydro assembly uses, at
    N = 48 and N = 400."""
    import numpy as np
    from kore_gb300.assembly import RadialOperators, mult_mat, mult_mat_gpu
    for N in (48, 400):
        R = RadialOperators(N, 0.35)
        for rx in range(7):
            for dx in range(5):
                a = R._Sto[dx] @ R._rp[rx]
                Mh, Mg = mult_mat(a, dx), mult_mat_gpu(a, dx)
                ref = abs(Mh).max()
                assert abs(Mh - Mg).max() <= 1e-13 * max(ref, 1e-300), (N, rx, dx)


def test_hydro_pencil_with_gpu_operators(gpu_lib):
    """The whole hydro pencil assembled with the GPU multiplication operators equals the
    host-assembled one."""
    import numpy as np
    from kore_gb300.assembly import hydro_pencil
    A, B = hydro_pencil(1, 1, 1e-4, 48, 40, 0.35)
    Ag, Bg = hydro_pencil(1, 1, 1e-4, 48, 40, 0.35, device=0)
    assert abs(A - Ag).max() <= 1e-13 * abs(A).max()
    assert abs(B - Bg).max() <= 1e-13 * abs(B).max()
