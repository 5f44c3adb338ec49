"""Serving: eigen and forced solves of many pencils through one request queue
(``kore_batch_*`` in include/kore_gpu.h).

kore runs one ``bin/solve.py`` process per problem.  Here a :class:`Server` keeps a
queue of requests, each doing what one such run does (an eigensolve at a target,
``bin/solve.py:91-158``, or a forced solve at a shift, ``bin/solve.py:207-268``), runs
several at once, admits them by the device memory their plans need and keeps uploaded,
factorised plans for later requests on the same pencil.  Eigen requests of one pencil
are batched continuously: they run in the factor slots of one plan (the batched engine
of ``kore_eigs_shifts``), sharing every launch, and a request that arrives while others
of its pencil are on the GPU takes the next free slot.

    srv = Server(workers=4)
    P = PencilData(A, B, layout)                    # host arrays, no device memory yet
    t1 = srv.submit_eigen(P, target=0.5j, nev=8, key=1)
    t2 = srv.submit_forced(P, sigma=0.3j, rhs=b, key=1)
    lam = srv.result(t1)["evals"]; x = srv.result(t2)["x"]
"""
import ctypes as C
import itertools
import threading

import numpy as np

from . import _lib as L
from .solver import PencilData

__all__ = ["Server", "PencilData"]


class Server:
    """A request queue over plans on one GPU.

    hbm_budget: device bytes the plans may hold (0: 90% of the free memory).
    workers: requests running at once (each on its own CUDA stream).
    """

    def __init__(self, device=0, hbm_budget=0, workers=4):
        self.lib = L.load()
        self._b = C.c_void_p()
        L.check(self.lib.kore_batch_create(int(device), int(hbm_budget), int(workers), C.byref(self._b)),
                "kore_batch_create")
        self._live = {}          # ticket -> (request struct, kept arrays, result template)
        self._keys = {}          # id(PencilData) -> pencil key
        self._next_key = itertools.count(1)
        self._mu = threading.Lock()

    def key_of(self, data):
        """The pencil key of a PencilData (requests on the same object share plans)."""
        with self._mu:
            k = self._keys.get(id(data))
            if k is None:
                k = self._keys[id(data)] = next(self._next_key)
            return k

    def _submit(self, req, keep, result):
        t = C.c_uint64()
        L.check(self.lib.kore_batch_submit(self._b, C.byref(req), C.byref(t)), "kore_batch_submit")
        with self._mu:
            self._live[t.value] = (req, keep, result)
        return t.value

    def submit_eigen(self, data, target, nev, which="TM", tol=1e-15, maxit=50, ncv=0, precision="mixed", seed=1,
                     vectors=False, key=None, refine_tol=0.0, reuse_radius=0.0, warm=False):
        """Eigensolve of data's pencil around `target` (kore_eigs); returns a ticket.

        reuse_radius > 0: when an idle slot of the pencil's cached plan holds factors at a
        shift within this distance of the target, the request runs there with that shift
        (no re-factorisation; eigenvalues still sorted from the target).  warm: start from
        the seeded vector plus the eigenvectors that slot returned last.  Either makes the
        result depend on earlier requests, within the solver's tolerance."""
        target = complex(target)
        ncv_eff = ncv if ncv > 0 else L.default_ncv(data.n, nev)
        evals = np.zeros(ncv_eff, dtype=np.complex128)
        evecs = np.zeros((ncv_eff, data.n), dtype=np.complex128) if vectors else None
        nconv = C.c_int32(0)
        timing = np.zeros(3)
        r = L.Request()
        r.kind = L.REQ_EIGEN
        r.pencil = C.pointer(data.desc)
        r.pencil_key = self.key_of(data) if key is None else int(key)
        r.precision = L.PREC[precision]
        r.sigma_re, r.sigma_im = target.real, target.imag
        r.opts = L.EpsOpts(nev=nev, ncv=ncv, tol=tol, maxit=maxit, which=L.WHICH[which], target_re=target.real,
                           target_im=target.imag, seed=seed, purify=1, refine_tol=refine_tol,
                           reuse_radius=float(reuse_radius), warm=int(bool(warm)))
        r.evals = evals.ctypes.data
        r.evecs = evecs.ctypes.data if vectors else None
        r.max_pairs = ncv_eff
        r.nconv = C.pointer(nconv)
        r.timing_ms = timing.ctypes.data
        st = L.Stats()
        r.stats = C.addressof(st)
        keep = (data, evals, evecs, nconv, timing, st)
        return self._submit(r, keep, {"kind": "eigen", "evals": evals, "evecs": evecs, "nconv": nconv,
                                      "timing": timing, "target": target, "stats_struct": st})

    def submit_forced(self, data, sigma, rhs, scale=1.0, precision="mixed", refine_tol=0.0, key=None):
        """x = (A - sigma B)^-1 rhs / scale (kore_solve); returns a ticket.  In mixed
        precision a solve whose refinement stops above a backward error of 1e-10 is redone
        with FP64 factors (result["stats"]["escalated"])."""
        sigma = complex(sigma)
        b = np.ascontiguousarray(np.asarray(rhs, dtype=np.complex128).ravel())
        if b.size != data.n:
            raise ValueError("right-hand side size does not match the pencil")
        x = np.zeros(data.n, dtype=np.complex128)
        timing = np.zeros(3)
        r = L.Request()
        r.kind = L.REQ_FORCED
        r.pencil = C.pointer(data.desc)
        r.pencil_key = self.key_of(data) if key is None else int(key)
        r.precision = L.PREC[precision]
        r.sigma_re, r.sigma_im = sigma.real, sigma.imag
        r.rhs = b.ctypes.data
        r.rhs_scale = float(scale)
        r.refine_tol = float(refine_tol)
        r.x = x.ctypes.data
        r.timing_ms = timing.ctypes.data
        st = L.Stats()
        r.stats = C.addressof(st)
        keep = (data, b, x, timing, st)
        return self._submit(r, keep, {"kind": "forced", "x": x, "timing": timing, "sigma": sigma,
                                      "stats_struct": st})

    def poll(self, ticket, wait_ms=0):
        """None while the request runs, else its result (see :meth:`result`)."""
        st = C.c_int(0)
        rc = self.lib.kore_batch_poll(self._b, C.c_uint64(ticket), int(wait_ms), C.byref(st))
        if rc == L.KORE_EPENDING:
            return None
        L.check(rc, "kore_batch_poll")
        with self._mu:
            _, _, res = self._live.pop(ticket)
        out = dict(res)
        out["status"] = st.value
        t = res["timing"]
        out["queued_ms"], out["run_ms"], out["total_ms"] = float(t[0]), float(t[1]), float(t[2])
        out["stats"] = out.pop("stats_struct").as_dict()
        if res["kind"] == "eigen":
            k = res["nconv"].value
            out["nconv"] = k
            out["evals"] = res["evals"][:k]
            if res["evecs"] is not None:
                out["evecs"] = res["evecs"][:k].T
        return out

    def result(self, ticket):
        """Wait for the request and return a dict: status, timing (queued_ms, run_ms,
        total_ms) and evals/evecs/nconv (eigen) or x (forced).  Raises on a failed request."""
        out = self.poll(ticket, wait_ms=-1)
        if out["status"] != L.KORE_OK:
            raise L.KoreError(out["status"], "request")
        return out

    def stats(self):
        a = np.zeros(9, dtype=np.int64)
        L.check(self.lib.kore_batch_stats(self._b, a.ctypes.data), "kore_batch_stats")
        names = ("submitted", "finished", "running", "queued", "device_bytes", "factor_cache_hits",
                 "plans_created", "plans_evicted", "joined_running_engine")
        return dict(zip(names, (int(v) for v in a)))

    def close(self):
        if self._b:
            self.lib.kore_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
