#!/usr/bin/env python3
"""Benchmark of the GB300 solve path: converged eigenpairs/s of the shift-and-invert
Krylov-Schur solve, mixed precision (complex64 block factorisation + FP64 refinement)
against the plain FP64 GPU path, with p50/p99 per-solve latency.

Workload (default ``--workload shell2``): hydrodynamic inertial modes in a spherical
shell, ricb=0.35, no-slip, m=2, equatorially symmetric, Ek=1e-7, N=400, lmax=601
(240,000 complex unknowns, 600 l-blocks of 400), target 0.5i, nev=16, which='TM'.
The pencil is assembled on the host by kore_gb300.assembly (a restatement of
bin/assemble.py that reproduces the reference's matrices to ~1e-16).

A step is one complete eigen solve (factorise A - tau B, Krylov-Schur to nev converged
pairs) with the pencil resident on the device.  ``e2e`` times the same solve through
the C-ABI with host buffers: plan creation from the host CSR (host->device copy),
factorisation, eigensolve and the eigenvalues+eigenvectors back to host memory.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (m, symm, Ek, N, lmax, ricb, tau, nev, which)
    "shell2": (2, 1, 1e-7, 400, 601, 0.35, 0.5j, 16, "TM"),
    "shell1": (1, 1, 1e-4, 48, 40, 0.35, 1.0j, 10, "TM"),
    # the same shell with 120 l-blocks: small case for profiler captures
    "shell2s": (2, 1, 1e-7, 400, 121, 0.35, 0.5j, 16, "TM"),
}


# Batched forced solves (the tidal-forcing sweep): forcing 10 (a boundary forcing whose
# right-hand side does not depend on the frequency) on the eigen pencil, nfreq
# frequencies uniform in [-2, 2] solved `group` at a time, then `instances` uneven
# problems (m, N, lmax, Ek drawn from the sweep's ranges) solved concurrently.
FORCED = {
    "forced4": dict(m=2, symm=1, Ek=1e-6, N=240, lmax=301, ricb=0.35, nfreq=512, group=16, instances=256),
    # small version of the same for quick checks
    "forced4s": dict(m=2, symm=1, Ek=1e-5, N=96, lmax=61, ricb=0.35, nfreq=64, group=16, instances=4),
}


# DRAM traffic of one sweep launch over its algorithmic bytes, from one ncu capture of
# the 120-block shell (dram__bytes_read.sum + dram__bytes_write.sum = 542.4 MB against
# 551.7 MB algorithmic).  Both grow with the block count, so the ratio carries over to
# the 600-block workload.
SWEEP_TRAFFIC_RATIO = 542.4 / 551.7


def describe_forced(c):
    return (f"batched forced solves: hydro shell ricb={c['ricb']} no-slip m={c['m']} symm={c['symm']} "
            f"Ek={c['Ek']:g} N={c['N']} lmax={c['lmax']}, forcing 10, {c['nfreq']} frequencies in [-2, 2] "
            f"({c['group']} per batch), plus {c['instances']} uneven instances")


def describe(w):
    if w in FORCED:
        return describe_forced(FORCED[w])
    m, symm, Ek, N, lmax, ricb, tau, nev, which = WORKLOADS[w]
    return (f"hydro shell ricb={ricb} no-slip m={m} symm={symm} Ek={Ek:g} N={N} lmax={lmax}, "
            f"target {tau.imag:g}i, nev={nev}, which={which}")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], d.get("bf16_tflops"), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 3 + i and r[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def build_pencil(w):
    from kore_gb300.assembly import hydro_params, hydro_pencil
    from kore_gb300.structure import layout_from_params
    m, symm, Ek, N, lmax, ricb, tau, nev, which = WORKLOADS[w]
    t0 = time.perf_counter()
    A, B = hydro_pencil(m, symm, Ek, N, lmax, ricb)
    ASSEMBLY["host_s"] = time.perf_counter() - t0
    lay = layout_from_params(hydro_params(m, symm, Ek, N, lmax, ricb))
    return A, B, lay


ASSEMBLY = {}


def assembly_bench(w, A, B, device, reps=2):
    """The pencil assembled on the GPU (kore_assemble_blocks) against the host assembly:
    wall time of each (radial operators, patterns, values, the copy back) and the
    relative Frobenius difference of the two results."""
    import scipy.sparse.linalg as ssl
    from kore_gb300.assembly import hydro_pencil
    m, symm, Ek, N, lmax, ricb, tau, nev, which = WORKLOADS[w]
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        Ad, Bd = hydro_pencil(m, symm, Ek, N, lmax, ricb, assemble_on_device=True, device=device)
        ts.append(time.perf_counter() - t0)
    out = {"host_s": ASSEMBLY.get("host_s"), "device_s": min(ts), "device_gpu": device,
           "rel_diff_A": float(ssl.norm(Ad - A) / ssl.norm(A)), "rel_diff_B": float(ssl.norm(Bd - B) / ssl.norm(B)),
           "nnz": int(Ad.nnz + Bd.nnz)}
    out["speedup"] = out["host_s"] / out["device_s"] if out["host_s"] else None
    return out


def run_eps(p, tau, nev, which, precision, seed, want_vectors=True, tol=1e-15, maxit=50):
    from kore_gb300 import EPS
    E = EPS()
    E.setOperators(p)
    E.setProblemType(EPS.ProblemType.GNHEP)
    E.setDimensions(nev)
    E.setTolerances(tol, maxit)
    E.setWhichEigenpairs(which)
    E.setTarget(tau)
    E.setFromOptions({"st_type": "sinvert", "kore_precision": precision, "kore_seed": seed})
    p.sigma = None  # every step factorises afresh
    E.solve()
    return E


def rel_residuals(A, B, lam, X):
    import scipy.sparse.linalg as ssl
    na, nb = ssl.norm(A, 1), ssl.norm(B, 1)
    out = []
    for j, l in enumerate(lam):
        x = X[:, j]
        out.append(np.linalg.norm(A @ x - l * (B @ x)) / ((na + abs(l) * nb) * np.linalg.norm(x)))
    return np.array(out)


def time_arm(p, torch, stream, spec, precision, steps, warmup, seed0=1):
    """Timed eigensolves of (tau, nev, which) = spec: CUDA events on the plan's stream."""
    tau, nev, which = spec
    for s in range(warmup):
        run_eps(p, tau, nev, which, precision, seed0 + s)
    lat, pairs = [], 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(steps):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        E = run_eps(p, tau, nev, which, precision, seed0 + warmup + s)
        ev1.record(stream)
        ev1.synchronize()
        lat.append(ev0.elapsed_time(ev1))
        pairs += min(E.getConverged(), nev)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    return E, lat, pairs, wall


# The headline metric, the same string in both arms' lines (the mixed / FP64 detail is in
# other keys of the GPU arm's line).
METRIC = "eigenpairs/s (shift-invert Krylov-Schur, nev converged, resid<=1e-10)"

# wall-clock budget of the reference arm's timed full-size solves: at least one solve is
# timed, further ones only while the total stays under this
REFERENCE_BUDGET_S = 600.0


def replica_aggregate(dist, total_ms, units, device):
    """Whole-job figures of N independent replicas (one per GPU, no data-path
    collective): the slowest replica's time (max over ranks) and the units every rank
    processed (sum).  With dist None (one process) the rank's own figures."""
    if dist is None:
        return total_ms, units
    import torch
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), int(round(u.item()))


def reference_arm(args, rank, world):
    """The reference's CPU solve path restated by the oracle (SuperLU factorisation of
    A - tau B + ARPACK shift-invert, SLEPc's `which` ordering), timed on the host cores on
    the full workload.  One full solve takes minutes, so the run times as many of the
    requested steps as fit in REFERENCE_BUDGET_S (at least one) and reports how many it
    timed; its warm-up steps are solves of the small m=1 shell (1,920 unknowns), which
    load the libraries and threads without minutes of extra work."""
    if rank != 0:
        return
    from kore_gb300.assembly import hydro_pencil
    from oracle.eps_ref import shift_invert_eigs
    m, symm, Ek, N, lmax, ricb, tau, nev, which = WORKLOADS[args.workload]
    ws = WORKLOADS["shell1"]
    Aw, Bw = hydro_pencil(ws[0], ws[1], ws[2], ws[3], ws[4], ws[5])
    for s in range(args.warmup):
        shift_invert_eigs(Aw, Bw, ws[6], ws[7], ws[8], seed=s)
    A, B = hydro_pencil(m, symm, Ek, N, lmax, ricb)
    ts, pairs = [], 0
    t_all = time.perf_counter()
    for s in range(max(1, args.steps)):
        t = time.perf_counter()
        lam, X = shift_invert_eigs(A, B, tau, nev, which, seed=s)
        ts.append(time.perf_counter() - t)
        pairs += len(lam)
        if time.perf_counter() - t_all + ts[-1] > REFERENCE_BUDGET_S:
            break
    per = float(np.mean(ts))
    value = pairs / float(np.sum(ts))
    cores = os.cpu_count()
    sample = (f"scipy SuperLU + ARPACK (restatement of SLEPc/MUMPS solve.py) on the full {A.shape[0]}-unknown "
              f"pencil, {len(ts)} timed solve(s) of {args.steps} requested (budget {REFERENCE_BUDGET_S:.0f} s), "
              f"{per:.1f} s each; SuperLU is single-threaded, ARPACK's BLAS uses the host's threads")
    line = {"metric": METRIC, "value": value,
            "unit": "eigenpairs/s", "n_gpus": args.gpus, "steps": len(ts), "steps_requested": args.steps,
            "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic: pencil assembled from the kore parameters",
            "config": {"workload": describe(args.workload)}, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "eigenpairs/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "eigenpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline(args):
    """The oracle on a bounded sample (about 10-30 s of CPU work): the same shell with 40
    of its 600 l-blocks, reported unscaled.  The full-size CPU time is the reference arm's
    (`--impl reference`)."""
    from kore_gb300.assembly import hydro_pencil
    from oracle.eps_ref import shift_invert_eigs
    m, symm, Ek, N, lmax, ricb, tau, nev, which = WORKLOADS[args.workload]
    lsample = min(lmax, 41)
    if (lsample - m + 1) % 2:
        lsample += 1
    A, B = hydro_pencil(m, symm, Ek, N, lsample, ricb)
    t = time.perf_counter()
    lam, _ = shift_invert_eigs(A, B, tau, nev, which, seed=0)
    dt = time.perf_counter() - t
    return {"value": len(lam) / dt, "unit": "eigenpairs/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"scipy SuperLU + ARPACK on the same shell with lmax={lsample} ({A.shape[0]} unknowns, "
                      f"{lsample - m + 1} of {lmax - m + 1} l-blocks): {dt:.1f} s for {len(lam)} pairs, not scaled; "
                      f"the full-size CPU time is the reference arm's line"}


def batched_arm(p, torch, stream, args, tau, nev, which):
    """The batched form: `args.batch` targets spaced 0.04 apart on the imaginary axis,
    tau among them, nev pairs each, in one kore_eigs_shifts per step (factorisation of all
    shifts included).  Warm-up and timed steps as the main arm, with other seeds."""
    from kore_gb300 import eigs_targets
    T = args.batch
    targets = tau + 0.04j * (np.arange(T) - T // 2)   # target T // 2 is tau itself
    torch.cuda.nvtx.range_push("batched")   # lets a profiler select this arm's launches
    for s in range(max(1, args.warmup // 2)):
        eigs_targets(p, targets, nev, which, "mixed", seeds=400 + T * s + np.arange(T))
    lat, pairs = [], 0
    torch.cuda.synchronize()
    p.profile(True)
    for s in range(max(1, args.steps // 2)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        res = eigs_targets(p, targets, nev, which, "mixed", seeds=500 + T * s + np.arange(T))
        e1.record(stream)
        e1.synchronize()
        lat.append(e0.elapsed_time(e1))
        pairs += sum(min(len(r[0]), nev) for r in res)
    prof = p.profile(False)
    total = sum(lat) / 1e3
    torch.cuda.nvtx.range_pop()
    return {"targets": [[float(t.real), float(t.imag)] for t in targets], "nev": nev, "steps": len(lat),
            "value": pairs / total, "unit": "eigenpairs/s", "ms_per_step": float(np.mean(lat)),
            "latency_ms_per_batch": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
            "step_breakdown_ms": {k: prof[k] / len(lat) for k in ("sweep_ms", "factor_ms", "spmv_ms", "ortho_ms",
                                                                  "schur_ms")},
            "sweeps_per_step": prof["sweeps"] / len(lat),
            "restarts": [r[2]["restarts"] for r in res], "op_applies": [r[2]["op_applies"] for r in res],
            "results": res}


def parity_block(A, B, lay, tau, nev, lam, X, batched):
    """Mixed eigenpairs against FP64 GPU measurements (kore_gb300.conditioning): the FP64
    set of 2 nev pairs, the spread a 1e-16 relative perturbation of A causes in it, the
    adjoint-pencil condition numbers, and where the mixed pairs fall."""
    from kore_gb300 import conditioning as cd
    t = time.perf_counter()
    ref, _, ref_res = cd.reference(A, B, lay, tau, nev)
    band, sets = cd.perturbation_band(A, B, lay, tau, nev, ref)
    kap = cd.condition_numbers(A, B, lay, tau, lam[:nev], X[:, :nev])
    r = cd.compare(A, B, tau, nev, lam, X, ref, ref_res, band, sets, kap)
    out = {k: v for k, v in r.items() if k != "d"}
    out["d_median"] = float(np.median(r["d"]))
    out["note"] = ("d = relative distance of each mixed eigenvalue to the nearest FP64 eigenvalue (reference set or "
                   "a run on A perturbed by 1e-16 relative); band = largest such distance of the perturbed FP64 "
                   "runs, i.e. what rounding of A alone moves; within_band counts d <= 4 band")
    if batched:
        lb, Xb, _ = batched["results"][len(batched["results"]) // 2]
        tb = complex(*batched["targets"][len(batched["targets"]) // 2])
        if abs(tb - tau) < 1e-12:
            rb = cd.compare(A, B, tau, nev, lb, Xb, ref, ref_res, band, sets)
            out["batched_at_target"] = {k: v for k, v in rb.items() if k != "d"}
    out["seconds"] = time.perf_counter() - t
    return out


def tracking_bench(A, B, lay, local, tau, nev, which, steps=8, spacing=0.004j, radius=0.01):
    """A target followed along the imaginary axis (parameter tracking: tau, tau + spacing,
    ...), one served eigen request at a time on one pencil, in both precisions.  Without
    reuse every request factorises its target; with `radius` a request runs on the cached
    factors of a shift within that distance.  Latency is the serving queue's run time of
    each request."""
    from kore_gb300.serve import PencilData, Server
    P = PencilData(A, B, layout=lay)
    out = {"targets": [[float(tau.real), float(tau.imag)], [float(spacing.real), float(spacing.imag)], steps],
           "nev": nev, "radius": radius}
    for name, prec, r in (("mixed_fresh", "mixed", 0.0), ("mixed_reuse", "mixed", radius),
                          ("fp64_fresh", "fp64", 0.0), ("fp64_reuse", "fp64", radius)):
        lat, reused, warm, applies, resid = [], 0, 0, [], []
        with Server(workers=1, device=local) as srv:
            for k in range(steps):
                res = srv.result(srv.submit_eigen(P, tau + k * spacing, nev, which, seed=900 + k, precision=prec,
                                                  reuse_radius=r, vectors=True))
                lat.append(res["run_ms"])
                st = res["stats"]
                reused += st["factor_reused"]
                warm += st["warm_started"]
                applies.append(st["op_applies"])
                resid.append(float(rel_residuals(A, B, res["evals"][:nev], res["evecs"][:, :nev]).max()))
        out[name] = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                     "mean_ms": float(np.mean(lat)), "factor_reused": reused, "warm_started": warm,
                     "op_applies_mean": float(np.mean(applies)), "max_eig_resid": max(resid)}
    out["reuse_speedup_mean_latency"] = {p: out[p + "_fresh"]["mean_ms"] / out[p + "_reuse"]["mean_ms"]
                                         for p in ("mixed", "fp64")}
    return out


def uneven_instances(count, seed=7):
    """Uneven forced problems drawn from the sweep's ranges: m in 1..8 (forcing 10 acts on
    l = m, so m = 0 has no forcing), N even in [64, 320], lmax in [60, 400] with
    lmax - m + 1 even, Ek log-uniform in [1e-7, 1e-4], one frequency in [-2, 2] each."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        m = int(rng.integers(1, 9))
        N = 2 * int(rng.integers(32, 161))
        lmax = int(rng.integers(60, 401))
        if (lmax - m + 1) % 2:
            lmax += 1 if lmax < 400 else -1
        out.append(dict(m=m, symm=1, Ek=float(10 ** rng.uniform(-7, -4)), N=N, lmax=lmax, ricb=0.35,
                        w=float(rng.uniform(-2, 2))))
    return out


def forced_bench(args, local, c=None, emit=True):
    """Batched forced solves: forced solves/s, mixed (complex64 batched factorisation +
    FP64 refinement) against the FP64 GPU path, through the public Python API
    (kore_gb300.forced_sweep: host right-hand sides in, host solutions out).  Prints the
    JSON line (emit) and returns it."""
    import torch
    import scipy.sparse as ss
    from concurrent.futures import ThreadPoolExecutor
    from kore_gb300 import Pencil, forced_sweep, kernel_launches
    from kore_gb300 import build as kb
    from kore_gb300.assembly import forcing_vector, hydro_params, hydro_pencil
    from kore_gb300.structure import layout_from_params
    kb.build()
    torch.cuda.set_device(local)
    c = c or FORCED[args.workload]
    geo = dict(m=c["m"], symm=c["symm"], Ek=c["Ek"], N=c["N"], lmax=c["lmax"], ricb=c["ricb"])
    Ae, Be, nrm = hydro_pencil(geo["m"], geo["symm"], geo["Ek"], geo["N"], geo["lmax"], geo["ricb"], with_norm=True)
    b = forcing_vector(geo["m"], geo["symm"], geo["N"], geo["lmax"], geo["ricb"], 10).toarray().ravel()
    lay = layout_from_params(hydro_params(**geo))
    p = Pencil(Ae, Be, layout=lay, device=local)
    om = np.linspace(-2.0, 2.0, c["nfreq"])
    G = c["group"]

    def resid(x, w):
        M = (Ae - (1j * w) * Be).tocsr()
        r = M @ x - b / nrm
        return np.abs(r).max() / (abs(M).sum(axis=1).max() * np.abs(x).max() + np.abs(b / nrm).max())

    # warm-up: `warmup` batches of the first frequencies
    for _ in range(max(args.warmup, 1)):
        forced_sweep(p, om[:G], b, "mixed", G, refine_tol=1e-14, scale=nrm)
    launches0 = kernel_launches()
    clocks = ClockSampler(local)
    with clocks:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        X, gt = forced_sweep(p, om, b, "mixed", G, refine_tol=1e-14, scale=nrm)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = kernel_launches() - launches0
    sample = np.linspace(0, len(om) - 1, 9).astype(int)
    res = np.array([resid(X[:, j], om[j]) for j in sample])
    # FP64 plain path on the first `fp64` batches
    nb64 = max(1, min(len(gt), args.fp64_steps if args.fp64_steps is not None else 2))
    t0 = time.perf_counter()
    X64, gt64 = forced_sweep(p, om[:nb64 * G], b, "fp64", G, scale=nrm)
    wall64 = time.perf_counter() - t0
    diff = max(np.linalg.norm(X[:, j] - X64[:, j]) / np.linalg.norm(X64[:, j]) for j in range(0, nb64 * G, 7))
    n = int(Ae.shape[0])
    p.close()

    # uneven instances, four plans in flight at once (each plan has its own stream); the
    # pencils are assembled on the GPU 16 at a time, outside the timed region
    inst = uneven_instances(c["instances"])

    def assemble(d):
        A_i, B_i, nrm_i = hydro_pencil(d["m"], 1, d["Ek"], d["N"], d["lmax"], d["ricb"], with_norm=True,
                                       assemble_on_device=True, device=local)
        b_i = forcing_vector(d["m"], 1, d["N"], d["lmax"], d["ricb"], 10).toarray().ravel()
        return d, A_i, B_i, nrm_i, b_i

    def one(item):
        d, A_i, B_i, nrm_i, b_i = item
        q = Pencil(A_i, B_i, layout=layout_from_params(hydro_params(d["m"], 1, d["Ek"], d["N"], d["lmax"], d["ricb"])),
                   device=local)
        info = {}
        with q:
            x, _ = forced_sweep(q, [d["w"]], b_i, "mixed", 1, refine_tol=1e-14, scale=nrm_i, info=info)
        M = (A_i - (1j * d["w"]) * B_i).tocsr()
        r = M @ x[:, 0] - b_i / nrm_i
        return (np.abs(r).max() / (abs(M).sum(axis=1).max() * np.abs(x).max() + np.abs(b_i / nrm_i).max()),
                info["escalated"], info["mixed_resid_max"], d)

    res_i, wall_i = [], 0.0
    for k0 in range(0, len(inst), 16):
        built = [assemble(d) for d in inst[k0:k0 + 16]]
        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=4) as ex:
            res_i += list(ex.map(one, built))
        wall_i += time.perf_counter() - t0
        del built
    ns_i = [(d["lmax"] - d["m"] + 1) * d["N"] for d in inst]
    worst = sorted(res_i, key=lambda r: -r[2])[:3]
    esc = sum(r[1] for r in res_i)
    res_i = [r[0] for r in res_i]
    value = len(om) / wall
    hbytes = (len(om) * n * 16, len(om) * n * 16)
    line = {
        "metric": "forced solves/s (batched frequency sweep, resid<=1e-10), mixed vs FP64 GPU",
        "value": value, "unit": "solves/s", "n_gpus": 1, "steps": len(gt), "warmup": max(args.warmup, 1),
        "ms_per_step": 1e3 * wall / len(gt), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 factor + f64 refinement", "data": "synthetic: pencil assembled from the kore parameters",
        "config": {"workload": describe_forced(c), "n": n, "blocks": int(lay.nblocks),
                   "block": int(lay.block_sizes.max()), "batch": G, "l2": "inputs larger than L2",
                   "parallelism": "replicas x1"},
        "latency_ms": {"batch_p50": 1e3 * float(np.percentile(gt, 50)), "batch_p99": 1e3 * float(np.percentile(gt, 99))},
        "max_resid": float(res.max()),
        "fp64": {"value": nb64 * G / wall64, "unit": "solves/s", "frequencies": nb64 * G,
                 "max_rel_diff_mixed_vs_fp64": float(diff)},
        "speedup_vs_fp64": value / (nb64 * G / wall64),
        "uneven": {"instances": len(inst), "value": len(inst) / wall_i, "unit": "solves/s (plan + factor + solve, "
                   "4 plans in flight, 16 instances per round)", "max_resid": float(max(res_i)),
                   "unknowns": {"min": min(ns_i), "max": max(ns_i), "mean": float(np.mean(ns_i))},
                   "escalated_to_fp64": int(esc),
                   "worst_mixed_refinement": [{"m": d["m"], "N": d["N"], "lmax": d["lmax"], "Ek": float(f"{d['Ek']:.3g}"),
                                               "w": float(f"{d['w']:.4g}"), "mixed_eta": float(e)}
                                              for _, _, e, d in worst],
                   "first_sizes_m_N_lmax_Ek": [[d["m"], d["N"], d["lmax"], float(f"{d['Ek']:.3g}")] for d in inst[:8]]},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": hbytes[0] // len(gt),
                "d2h_bytes_per_step": hbytes[1] // len(gt)},
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


# Serving: a seeded Poisson stream of requests over a pool of pencils drawn from the
# serving ranges (lmax in [60, 600], N in [48, 400], Ek log-uniform in [1e-7, 1e-4],
# m in 0..8); 70% eigen (nev 4..16, target i*U[-2, 2]) and 30% forced (forcing 10,
# shift i*U[-2, 2]), at each arrival rate in `rates` (requests/s).
# Config 3: the dipole MAC shell (Lorentz force, induction, buoyancy; insulating inner
# core and mantle; differential heating) at twice the critical Rayleigh number of its
# m mode.  The critical Rayleigh number comes from the onset search of
# tests/jones2000/find_Rac.py (FP64, target 0, 'TR', 16 pairs) started at log10_ra0;
# the timed solves are at the target tau.  symm = 1: equatorially symmetric flow, as in
# the reference's onset tests.
MAC = {
    "mac3": dict(m=1, symm=1, Ek=1e-6, N=200, lmax=200, ricb=0.35, Em=1e-3, Le2=1e-8, Prandtl=1.0,
                 tau=0.1j, nev=8, which="TM", log10_ra0=8.9),
    # the same physics with 60 of the 100 l-superblocks and N=120: small case for profiler
    # captures (factors of ~0.3 GB, above the L2 size)
    "mac3s": dict(m=1, symm=1, Ek=1e-6, N=120, lmax=120, ricb=0.35, Em=1e-3, Le2=1e-8, Prandtl=1.0,
                  tau=0.1j, nev=8, which="TM", log10_ra0=8.9),
}


def describe_mac(c):
    return (f"dipole MAC shell ricb={c['ricb']} no-slip, insulating, m={c['m']} symm={c['symm']} Ek={c['Ek']:g} "
            f"Em={c['Em']:g} Le2={c['Le2']:g} Pr={c['Prandtl']:g} N={c['N']} lmax={c['lmax']}, differential heating, "
            f"Ra = 2 Ra_c, target {c['tau'].imag:g}i, nev={c['nev']}, which={c['which']}")


def mac_bench(args, local, c=None, emit=True):
    """Config 3: eigenpairs/s of the dipole MAC shell at Ra = 2 Ra_c, mixed against the FP64
    GPU path, pencil resident on the device (as the headline's `value`).  Set-up, not
    timed: the host assembly (kore_gb300.assembly_mac) and the onset search for Ra_c
    (kore_gb300.onset, FP64 eigensolves on the device).  Parity as for the headline:
    FP64 measurements, the rounding band and condition numbers (kore_gb300.conditioning)."""
    import torch
    from kore_gb300 import Pencil, kernel_launches, layout_from_params
    from kore_gb300.assembly_mac import mac_params, mac_pencil_parts
    from kore_gb300.onset import OnsetSearch
    c = c or MAC[args.workload]
    tau, nev, which = c["tau"], c["nev"], c["which"]
    t0 = time.perf_counter()
    A0, Ab, B, nrm = mac_pencil_parts(c["m"], c["symm"], c["Ek"], c["N"], c["lmax"], c["ricb"], Em=c["Em"],
                                      Le2=c["Le2"], Prandtl=c["Prandtl"])
    lay = layout_from_params(mac_params(c["m"], c["symm"], c["Ek"], c["N"], c["lmax"], c["ricb"]))
    Bn = (B / nrm).tocsr()
    t_asm = time.perf_counter() - t0
    bv = -(c["Ek"] ** 2) / c["Prandtl"]      # buoyancy factor per unit Ra
    t0 = time.perf_counter()
    S = OnsetSearch(A0 / nrm, bv * Ab / nrm, 0.0, 1.0, Bn, lay, nev=16, which="TR", tau=0.0,
                    precision="fp64", device=local)
    Rac, wc = S.critical(c["log10_ra0"], dx=0.02, tol=1e-5, maxsteps=40)
    t_onset = time.perf_counter() - t0
    Ra = 2.0 * Rac
    A = ((A0 + (Ra * bv) * Ab) / nrm).tocsr()
    p = Pencil(A, Bn, layout=lay, device=local)
    stream = torch.cuda.ExternalStream(p.stream(), device=torch.device("cuda", local))
    steps = max(2, args.steps // 2)
    spec = (tau, nev, which)
    E64, lat64, pairs64, _ = time_arm(p, torch, stream, spec, "fp64", steps, 1, seed0=600)
    l0 = kernel_launches()
    p.profile(True)
    E, lat, pairs, _ = time_arm(p, torch, stream, spec, "mixed", steps, 1, seed0=600)
    prof = p.profile(False)
    launches = kernel_launches() - l0
    hbm, _, src = peaks()
    sweep_ms = prof["sweep_ms"] / max(prof["sweeps"], 1)
    achieved = prof["sweep_bytes"] / (sweep_ms * 1e-3) / 1e9
    lam, X = E.eigenvalues(), E.eigenvectors()
    lam64, X64 = E64.eigenvalues(), E64.eigenvectors()
    res = rel_residuals(A, Bn, lam[:nev], X[:, :nev])
    res64 = rel_residuals(A, Bn, lam64[:nev], X64[:, :nev])
    dists = np.array([np.min(np.abs(lam64 - l)) / abs(l) for l in lam[:nev]])
    value = pairs / (sum(lat) / 1e3)
    v64 = pairs64 / (sum(lat64) / 1e3)
    out = {"metric": METRIC, "value": value, "unit": "eigenpairs/s", "ms_per_step": float(np.mean(lat)),
           "config": {"workload": describe_mac(c), "n": int(lay.n), "blocks": int(lay.nblocks),
                      "block": int(lay.block_sizes.max()), "l2": "inputs larger than L2",
                      "parallelism": "replicas x1"},
           "Ra_c": Rac, "omega_c": wc, "Ra": Ra, "onset_evaluations": S.evaluations,
           "setup_s": {"assembly": t_asm, "onset_search": t_onset},
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
           "fp64": {"value": v64, "p50_ms": float(np.percentile(lat64, 50)), "p99_ms": float(np.percentile(lat64, 99)),
                    "max_eig_resid": float(res64.max()), "factor_s": E64.stats.get("factor_s"),
                    "solver_stats": {k: E64.stats.get(k) for k in ("restarts", "op_applies", "sweeps")}},
           "speedup_vs_fp64": value / v64, "max_eig_resid": float(res.max()),
           "factor_s": E.stats.get("factor_s"),
           "solver_stats": {k: E.stats.get(k) for k in ("restarts", "op_applies", "sweeps", "refine_iters_max")},
           "max_rel_eig_diff_vs_fp64": float(dists.max()), "eigs_matching_fp64_1e-10": int((dists < 1e-10).sum()),
           "gpu_launches": int(launches),
           "roofline": {"bound": "hbm", "kernel": "k_sweep_tma", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                        "frac": achieved / hbm, "peak_source": src, "bytes_per_launch": prof["sweep_bytes"],
                        "avg_launch_ms": sweep_ms, "ctas_per_sm": prof["sweep_ctas_per_sm"],
                        "chunk_bytes": prof["sweep_chunk_bytes"],
                        "step_breakdown_ms": {k: prof[k] / len(lat) for k in ("sweep_ms", "factor_ms", "spmv_ms",
                                                                             "ortho_ms", "schur_ms")}}}
    if not args.no_parity:
        out["parity"] = parity_block(A, Bn, lay, tau, nev, lam, X, None)
    p.close()
    if emit:
        line = dict(out, n_gpus=1, steps=steps, warmup=1, higher_is_better=True, scaling="weak",
                    vs_baseline=None, dtype="c64 factor + f64 refinement/Krylov",
                    data="synthetic: pencil assembled from the kore parameters (restatement of the reference's "
                         "dipole MAC assembly, matches it to 6e-16)")
        print(json.dumps(line), flush=True)
    return out


SERVE = {
    "serve5": dict(pool=8, requests=120, rates=(2.0, 6.0), workers=4),
    # the summary carried on the headline line: one arrival rate
    "serve5h": dict(pool=8, requests=120, rates=(3.0,), workers=4),
    "serve5s": dict(pool=3, requests=24, rates=(4.0,), workers=3, small=True),
}


def serve_pool(count, seed=11, small=False):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        m = int(rng.integers(0, 9))
        N = 2 * int(rng.integers(24, 201)) if not small else 2 * int(rng.integers(12, 33))
        lmax = int(rng.integers(60, 601)) if not small else int(rng.integers(20, 61))
        if (lmax - m + 1) % 2:
            lmax += 1
        out.append(dict(m=m, N=N, lmax=lmax, Ek=float(10 ** rng.uniform(-7, -4)), ricb=0.35))
    return out


def serve_bench(args, local, c=None, emit=True):
    """Serving queue (kore_gb300.serve.Server): p50/p99 request latency and throughput of
    a Poisson request stream at several arrival rates.  Prints the JSON line (emit) and
    returns it."""
    import torch
    from kore_gb300 import build as kb
    from kore_gb300.assembly import forcing_vector, hydro_params, hydro_pencil
    from kore_gb300.serve import PencilData, Server
    from kore_gb300.structure import layout_from_params
    kb.build()
    torch.cuda.set_device(local)
    c = c or SERVE[args.workload]
    pool = []
    for d in serve_pool(c["pool"], small=c.get("small", False)):
        A, B, nrm = hydro_pencil(d["m"], 1, d["Ek"], d["N"], d["lmax"], d["ricb"], with_norm=True)
        b = (forcing_vector(d["m"], 1, d["N"], d["lmax"], d["ricb"], 10).toarray().ravel() / nrm
             if d["m"] >= 1 else None)
        P = PencilData(A, B, layout=layout_from_params(hydro_params(d["m"], 1, d["Ek"], d["N"], d["lmax"],
                                                                    d["ricb"])))
        pool.append((d, P, b))
    rng = np.random.default_rng(21)
    per_rate = []
    for rate in c["rates"]:
        reqs = []
        t = 0.0
        for _ in range(c["requests"]):
            t += rng.exponential(1.0 / rate)
            i = int(rng.integers(len(pool)))
            d, P, b = pool[i]
            eigen = rng.uniform() < 0.7 or b is None
            reqs.append((t, i, eigen, int(rng.integers(4, 17)), 1j * float(rng.uniform(-2, 2))))
        with Server(device=local, workers=c["workers"]) as srv:
            # warm-up: one request per pencil
            for d, P, b in pool:
                srv.result(srv.submit_eigen(P, 0.5j, 4, seed=1))
            tickets = []
            t0 = time.perf_counter()
            for (ta, i, eigen, nev, tgt) in reqs:
                now = time.perf_counter() - t0
                if ta > now:
                    time.sleep(ta - now)
                d, P, b = pool[i]
                if eigen:
                    tickets.append((srv.submit_eigen(P, tgt, nev, seed=len(tickets) + 1), nev, True))
                else:
                    tickets.append((srv.submit_forced(P, tgt, b), 0, False))
            lat, ok, short = [], 0, 0
            for tk, nev, eigen in tickets:
                r = srv.poll(tk, wait_ms=-1)
                lat.append(r["total_ms"])
                if r["status"] == 0:
                    ok += 1
                    if eigen and r["nconv"] < nev:
                        short += 1
            wall = time.perf_counter() - t0
            st = srv.stats()
        per_rate.append({"arrival_rate": rate, "requests": len(reqs), "ok": ok, "eigen_short_of_nev": short,
                         "throughput": len(reqs) / wall, "p50_ms": float(np.percentile(lat, 50)),
                         "p99_ms": float(np.percentile(lat, 99)), "factor_cache_hits": st["factor_cache_hits"],
                         "joined_running_engine": st["joined_running_engine"],
                         "plans_created": st["plans_created"], "plans_evicted": st["plans_evicted"]})
    best = max(per_rate, key=lambda r: r["throughput"])
    line = {
        "metric": "served solves/s and p50/p99 latency (Poisson stream, 70% eigen / 30% forced, mixed precision)",
        "value": best["throughput"], "unit": "requests/s", "n_gpus": 1, "steps": sum(r["requests"] for r in per_rate),
        "warmup": len(pool), "ms_per_step": best["p50_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 factor + f64 refinement/Krylov",
        "data": "synthetic: pencils assembled from the kore parameters",
        "config": {"workload": f"serving: {c['pool']} pencils "
                               + ", ".join(f"(m={d['m']}, N={d['N']}, lmax={d['lmax']}, Ek={d['Ek']:.2g})"
                                           for d, _, _ in pool)
                               + f"; {c['requests']} requests per arrival rate; {c['workers']} workers",
                   "parallelism": "replicas x1"},
        "rates": per_rate,
    }
    if emit:
        print(json.dumps(line), flush=True)
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="shell2",
                    choices=sorted(WORKLOADS) + sorted(FORCED) + sorted(SERVE) + sorted(MAC))
    ap.add_argument("--fp64-steps", type=int, default=None)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--no-forced", action="store_true", help="leave the batched forced-solve summary out")
    ap.add_argument("--no-serve", action="store_true", help="leave the serving summary out")
    ap.add_argument("--no-mac", action="store_true", help="leave the dipole MAC summary out")
    ap.add_argument("--no-track", action="store_true", help="leave the target-tracking serving summary out")
    ap.add_argument("--no-asm", action="store_true", help="leave the GPU assembly timing out")
    ap.add_argument("--batch", type=int, default=8, help="targets of the batched form (1: skip it)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if args.workload in FORCED:
        if rank == 0:
            forced_bench(args, local)
        return
    if args.workload in SERVE:
        if rank == 0:
            serve_bench(args, local)
        return
    if args.workload in MAC:
        if rank == 0:
            mac_bench(args, local)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)

    from kore_gb300 import Pencil, kernel_launches
    from kore_gb300 import build as kb
    kb.build()
    m, symm, Ek, N, lmax, ricb, tau, nev, which = WORKLOADS[args.workload]
    A, B, lay = build_pencil(args.workload)
    asm = None if args.no_asm or local != 0 else assembly_bench(args.workload, A, B, local)

    # ---- device-resident arms (pencil uploaded once, outside the timed region)
    p = Pencil(A, B, layout=lay, device=local)
    stream = torch.cuda.ExternalStream(p.stream(), device=torch.device("cuda", local))

    # FP64 plain GPU path
    fsteps = args.fp64_steps if args.fp64_steps is not None else args.steps
    lat64, pairs64, stats64 = [], 0, {}
    if fsteps > 0:
        # the timed FP64 solves use the mixed arm's seeds (200, 201, ...), so that the last
        # of each starts from the same vector and their eigenvalues can be compared
        w64 = min(args.warmup, 1)
        E64, lat64, pairs64, wall64 = time_arm(p, torch, stream, (tau, nev, which), "fp64", fsteps, w64,
                                               seed0=200 + args.steps - fsteps - w64)
        lam64, X64 = E64.eigenvalues(), E64.eigenvectors()
        stats64 = dict(E64.stats)

    # mixed (chosen form): timed region
    for s in range(args.warmup):
        run_eps(p, tau, nev, which, "mixed", 100 + s)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = kernel_launches()
    p.profile(True)
    lat, pairs = [], 0
    torch.cuda.nvtx.range_push("mixed_timed")   # lets a profiler select the timed solves
    with ClockSampler(local) as clocks:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for s in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            E = run_eps(p, tau, nev, which, "mixed", 200 + s)
            e1.record(stream)
            e1.synchronize()
            lat.append(e0.elapsed_time(e1))
            pairs += min(E.getConverged(), nev)
        t1.record(stream)
        t1.synchronize()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    prof = p.profile(False)
    launches = kernel_launches() - launches0
    total_ms = t0.elapsed_time(t1)
    total_ms, pairs = replica_aggregate(dist, total_ms, pairs, "cuda")
    value = pairs / (total_ms / 1e3)
    lam, X = E.eigenvalues(), E.eigenvectors()
    res = rel_residuals(A, B, lam[:nev], X[:, :nev])
    if lat64:
        res64 = rel_residuals(A, B, lam64[:nev], X64[:, :nev])
        # The shell's spectrum near the target is a dense cluster, so the two arms (same
        # start vector, operators equal to ~1e-14) can converge to different subsets of
        # the nearest eigenvalues; each is checked by its own residual above.  An
        # eigenvalue that both found agrees to the refinement's accuracy.
        dists = np.array([np.min(np.abs(lam64 - l)) / abs(l) for l in lam[:nev]])
        diff, nmatch = float(dists.max()), int((dists < 1e-10).sum())
        both = dists[dists < 1e-8]
        diff_both = float(both.max()) if both.size else None
        far64 = float(np.max(np.abs(lam64[:nev] - tau)))
        far = float(np.max(np.abs(lam[:nev] - tau)))
    else:
        res64, diff, nmatch, diff_both, far64, far = np.zeros(1), None, None, None, None, None
    stats = dict(E.stats)

    # ---- batched form: `batch` targets around the workload's target in one kore_eigs_shifts
    batched = None
    if args.batch > 1:
        batched = batched_arm(p, torch, stream, args, tau, nev, which)
    p.close()

    # ---- parity against FP64 measurements of how well the eigenvalues are determined
    parity = None
    if not args.no_parity:
        parity = parity_block(A, B, lay, tau, nev, lam, X, batched)

    # ---- e2e through the C-ABI with host buffers
    e2e = None
    if not args.no_e2e:
        ev_ms = []
        h2d = A.nnz * (16 + 4) + (A.shape[0] + 1) * 4 + B.nnz * (8 + 4) + (B.shape[0] + 1) * 4 + lay.n * 8
        d2h = 0
        for s in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t = time.perf_counter()
            with Pencil(A, B, layout=lay, device=local) as q:
                Eq = run_eps(q, tau, nev, which, "mixed", 300 + s)
                lam_q, X_q = Eq.eigenvalues(), Eq.eigenvectors()
            torch.cuda.synchronize()
            ev_ms.append((time.perf_counter() - t) * 1e3)
            d2h = lam_q.nbytes + X_q.nbytes
        e2e = {"value": nev / (np.mean(ev_ms) / 1e3), "unit": "eigenpairs/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": float(np.mean(ev_ms))}

    # ---- configs 3, 4 and 5 on the same line (their own sizes are in their config keys)
    forced = serve = mac = track = None
    if rank == 0 and not args.no_track:
        track = tracking_bench(A, B, lay, local, tau, nev, which)
    if rank == 0 and not args.no_mac:
        mac = mac_bench(args, local, MAC["mac3"], emit=False)
    if rank == 0 and not args.no_forced:
        forced = forced_bench(args, local, FORCED["forced4"], emit=False)
    if rank == 0 and not args.no_serve:
        serve = serve_bench(args, local, SERVE["serve5h"], emit=False)

    if rank != 0:
        return
    hbm, _, src = peaks()
    sweep_ms = prof["sweep_ms"] / max(prof["sweeps"], 1)
    achieved = prof["sweep_bytes"] / (sweep_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "detail": "mixed precision (complex64 factors + FP64 refinement) against the plain FP64 "
        "GPU path; `batched`: several targets in one batched solve",
        "value": value, "unit": "eigenpairs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 factor + f64 refinement/Krylov", "data": "synthetic: pencil assembled from the kore parameters "
        "(restatement of bin/assemble.py, matches the reference to 1e-16)",
        "config": {"workload": describe(args.workload), "n": int(lay.n), "blocks": int(lay.nblocks),
                   "block": int(lay.block_sizes.max()), "l2": "inputs larger than L2 (factors >= 2.3 GB)",
                   "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "fp64": ({"value": pairs64 / (sum(lat64) / 1e3), "unit": "eigenpairs/s",
                  "p50_ms": float(np.percentile(lat64, 50)), "p99_ms": float(np.percentile(lat64, 99)),
                  "max_eig_resid": float(res64.max()),
                  "solver_stats": {k: stats64.get(k) for k in ("restarts", "op_applies", "sweeps")}}
                 if lat64 else None),
        "speedup_vs_fp64": (value / (pairs64 / (sum(lat64) / 1e3))) if lat64 else None,
        "batched": batched and dict({k: v for k, v in batched.items() if k != "results"},
                                    speedup_vs_fp64_single=(batched["value"] / (pairs64 / (sum(lat64) / 1e3))
                                                            if lat64 else None)),
        "parity": parity,
        "max_eig_resid": float(res.max()), "max_rel_eig_diff_vs_fp64": diff,
        "eigs_matching_fp64_1e-10": nmatch, "max_rel_eig_diff_found_by_both": diff_both,
        "max_dist_to_target": {"mixed": far, "fp64": far64},
        "solver_stats": {k: stats.get(k) for k in ("restarts", "op_applies", "sweeps", "refine_iters_max",
                                                   "solve_resid_max")},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_sweep_tma (block-tridiagonal forward+back sweep, TMA-fed dataflow)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": src, "traffic": SWEEP_TRAFFIC_RATIO * prof["sweep_bytes"],
                     "traffic_source": "dram bytes read + written / algorithmic bytes = 542.4 MB / 551.7 MB in one "
                                       "ncu capture of the 120-block case, scaled by the block count",
                     "bytes_per_launch": prof["sweep_bytes"],
                     "avg_launch_ms": sweep_ms, "launches": prof["sweeps"],
                     "ctas_per_sm": prof["sweep_ctas_per_sm"], "chunk_bytes": prof["sweep_chunk_bytes"],
                     "sweep_share_of_step": prof["sweep_ms"] / total_ms,
                     "factor_ms_avg": prof["factor_ms"] / max(prof["factors"], 1),
                     "step_breakdown_ms": {k: prof[k] / args.steps for k in ("sweep_ms", "factor_ms", "spmv_ms",
                                                                            "ortho_ms", "schur_ms")}},
        "clocks": clocks.summary(),
        "e2e": e2e,
        "forced_sweep": forced and {k: forced[k] for k in ("metric", "value", "unit", "config", "latency_ms",
                                                           "max_resid", "fp64", "speedup_vs_fp64", "uneven",
                                                           "gpu_launches", "e2e")},
        "serving": serve and {k: serve[k] for k in ("metric", "value", "unit", "config", "rates")},
        "mac_dipole": mac,
        "serving_tracking": track,
        "assembly": asm,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
