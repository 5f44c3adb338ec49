"""Serving queue (kore_batch_*): eigen and forced requests of several pencils run
concurrently, admitted by device memory, with plans and factors shared per pencil.

The key property: a request's result is the same whether it runs alone or in a mix of
concurrent requests of other sizes (each request has its own plan and stream, and every
kernel reduces in a fixed order)."""
import numpy as np
import pytest

from oracle.eps_ref import forced_solve, shift_invert_eigs, solve_residual

pytestmark = pytest.mark.gpu


def data_of(case, name):
    from kore_gb300.serve import PencilData
    from kore_gb300.structure import layout_from_params
    meta, A, B = case(name)
    return meta, A, B, PencilData(A, B, layout=layout_from_params(meta))


def match_eigs(lam, ref):
    return np.array([np.min(np.abs(lam - r)) / abs(r) for r in ref])


def test_request_alone_equals_in_mix(gpu_lib, case):
    from kore_gb300.serve import Server
    meta, A, B, P = data_of(case, "shell_m2_ek1e-4")
    tau = complex(*meta["tau"])
    with Server(workers=1) as srv:
        alone = srv.result(srv.submit_eigen(P, tau, meta["nev"], seed=3, vectors=True))
    others = [data_of(case, n) for n in ("shell_m1_ek1e-4", "spinover", "mac_dipole_small")]
    rng = np.random.default_rng(0)
    with Server(workers=4) as srv:
        tickets = []
        for k, (m2, A2, B2, P2) in enumerate(others):
            tickets.append(srv.submit_eigen(P2, complex(*m2["tau"]), m2["nev"], seed=k + 1))
            b = rng.standard_normal(P2.n) + 1j * rng.standard_normal(P2.n)
            tickets.append(srv.submit_forced(P2, 0.3j + 0.1 * k, b))
        mine = srv.submit_eigen(P, tau, meta["nev"], seed=3, vectors=True)
        for k, (m2, A2, B2, P2) in enumerate(others):
            tickets.append(srv.submit_eigen(P2, complex(*m2["tau"]), m2["nev"], seed=k + 7, precision="fp64"))
        mixed = srv.result(mine)
        for t in tickets:
            assert srv.result(t)["status"] == 0
        st = srv.stats()
    assert st["finished"] == st["submitted"] and st["running"] == 0 and st["queued"] == 0
    assert alone["nconv"] == mixed["nconv"] >= meta["nev"]
    assert np.array_equal(alone["evals"], mixed["evals"])
    assert np.array_equal(alone["evecs"], mixed["evecs"])
    ref, _ = shift_invert_eigs(A, B, tau, meta["nev"], "TM")
    assert match_eigs(mixed["evals"][:meta["nev"]], ref).max() < 1e-10


def test_factor_cache_and_forced_parity(gpu_lib, case):
    """Forced requests at the same shift on the same pencil reuse the factorised plan,
    and each solution matches the oracle."""
    from kore_gb300.serve import Server
    meta, A, B, P = data_of(case, "shell_m2_ek1e-4")
    rng = np.random.default_rng(1)
    sig = 0.7j
    bs = [rng.standard_normal(P.n) + 1j * rng.standard_normal(P.n) for _ in range(4)]
    with Server(workers=1) as srv:
        res = [srv.result(srv.submit_forced(P, sig, b, scale=2.0, refine_tol=1e-15)) for b in bs]
        st = srv.stats()
    assert st["factor_cache_hits"] >= 3 and st["plans_created"] == 1
    M = (A - sig * B).tocsr()
    for b, r in zip(bs, res):
        assert solve_residual(M, r["x"], b / 2.0) < 1e-14
        xr = forced_solve(M, b / 2.0)
        assert np.linalg.norm(r["x"] - xr) / np.linalg.norm(xr) < 1e-9


def test_admission_under_a_small_budget(gpu_lib, case):
    """With room for about one plan at a time every request still finishes: requests wait
    for memory and idle cached plans are freed to make room."""
    from kore_gb300.serve import Server
    datas = [data_of(case, n) for n in ("shell_m1_ek1e-4", "shell_m2_ek1e-4", "spinover")]
    need = max(P.estimate_bytes("mixed", ncv=32) for _, _, _, P in datas)
    rng = np.random.default_rng(2)
    with Server(workers=3, hbm_budget=int(need * 1.2)) as srv:
        ts = []
        for rep in range(2):
            for m, A, B, P in datas:
                b = rng.standard_normal(P.n) + 1j * rng.standard_normal(P.n)
                ts.append((srv.submit_forced(P, 0.2j * (rep + 1), b, refine_tol=1e-15), A, B, b, 0.2j * (rep + 1)))
        for t, A, B, b, s in ts:
            r = srv.result(t)
            assert solve_residual((A - s * B).tocsr(), r["x"], b) < 1e-14
        st = srv.stats()
    assert st["finished"] == len(ts)
    assert st["plans_evicted"] >= 1
    assert st["device_bytes"] <= int(need * 1.2)


def test_eigen_requests_join_a_running_engine(gpu_lib, case):
    """Six eigen requests of one pencil: the first starts the batched engine on the
    pencil's plan, the others are admitted into its slots (four) as they free up and
    share its launches; each result equals the same request served alone."""
    from kore_gb300.serve import Server
    meta, A, B, P = data_of(case, "shell_m2_ek1e-4")
    targets = [0.4j, 0.7j, 1.0j, 1.3j, 0.55j, 0.85j]
    with Server(workers=1) as srv:
        ts = [srv.submit_eigen(P, t, 6, seed=k + 1, vectors=True) for k, t in enumerate(targets)]
        together = [srv.result(t) for t in ts]
        st = srv.stats()
    assert st["joined_running_engine"] >= len(targets) - 1, st
    assert st["plans_created"] == 1
    for k, (t, r) in enumerate(zip(targets, together)):
        with Server(workers=1) as srv:
            alone = srv.result(srv.submit_eigen(P, t, 6, seed=k + 1, vectors=True))
        assert r["status"] == 0 and alone["nconv"] == r["nconv"] >= 6
        assert np.array_equal(alone["evals"], r["evals"])
        assert np.array_equal(alone["evecs"], r["evecs"])
        ref, _ = shift_invert_eigs(A, B, t, 6, "TM")
        assert match_eigs(r["evals"][:6], ref).max() < 1e-10


def test_served_forced_request_escalates_when_refinement_stalls(gpu_lib):
    """A served mixed-precision forced request on the badly conditioned uneven instance
    of the forcing sweep (m=1, N=80, lmax=248, Ek=1.67e-7): the result meets 1e-12, with
    FP64 factors when the complex64 refinement stopped above 1e-10; a well-conditioned
    request is not escalated."""
    from kore_gb300.assembly import forcing_vector, hydro_params, hydro_pencil
    from kore_gb300.serve import PencilData, Server
    from kore_gb300.structure import layout_from_params
    m, N, lmax, Ek, w = 1, 80, 248, 1.67e-7, 0.3729
    A, B, nrm = hydro_pencil(m, 1, Ek, N, lmax, 0.35, with_norm=True)
    b = forcing_vector(m, 1, N, lmax, 0.35, 10).toarray().ravel()
    P = PencilData(A, B, layout=layout_from_params(hydro_params(m, 1, Ek, N, lmax, 0.35)))
    with Server(workers=1) as srv:
        r = srv.result(srv.submit_forced(P, 1j * w, b, scale=nrm, refine_tol=1e-14))
    st = r["stats"]
    assert solve_residual((A - 1j * w * B).tocsr(), r["x"], b / nrm) < 1e-12, st
    assert st["escalated"] == 1 or st["solve_resid_max"] <= 1e-10, st


def test_served_forced_request_not_escalated(gpu_lib, case):
    from kore_gb300.serve import Server
    meta, A, B, P = data_of(case, "shell_m2_ek1e-4")
    rng = np.random.default_rng(2)
    b = rng.standard_normal(P.n) + 1j * rng.standard_normal(P.n)
    with Server(workers=1) as srv:
        r = srv.result(srv.submit_forced(P, 0.4j, b, refine_tol=1e-14))
    assert r["stats"]["escalated"] == 0 and r["stats"]["solve_resid_max"] <= 1e-10, r["stats"]
    assert solve_residual((A - 0.4j * B).tocsr(), r["x"], b) < 1e-13
