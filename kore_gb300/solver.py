"""Python host of the GB300 solve path: the objects bin/solve.py builds, backed by
libkoregpu.so.

``bin/solve.py`` drives petsc4py/slepc4py:
  * ``Mat`` assembled from the CSR in ``A.npz`` / ``B.npz`` (``bin/solve.py:40-86``),
  * ``SLEPc.EPS`` configured with ``setProblemType(GNHEP)``, ``setDimensions(nev)``,
    ``setTolerances(tol, maxit)``, ``setWhichEigenpairs``, ``setTarget`` and
    ``setFromOptions`` (``bin/solve.py:91-120``), then ``solve()`` and ``getEigenpair``
    (``bin/solve.py:123-158``),
  * ``PETSc.KSP`` with ``setOperators(A)``, ``setTolerances``, ``setFromOptions``,
    ``solve(b, x)`` (``bin/solve.py:219-227``).
``Pencil``, ``EPS`` and ``KSP`` below keep those names and argument meanings; all
arithmetic runs in the CUDA library (there is no CPU fallback: a missing library
raises).
"""
import ctypes as C
import time

import numpy as np
import scipy.sparse as ss

from . import _lib as L
from .structure import Layout, band_of, layout_from_params


def _csr(M, dtype):
    M = ss.csr_matrix(M)
    M.sum_duplicates()
    M.sort_indices()
    return (L.as_i32(M.indptr), L.as_i32(M.indices), np.ascontiguousarray(M.data, dtype=dtype))


class PencilData:
    """The host CSR arrays of A (complex128) and B (float64, optional) with the l-major
    layout, held in the form ``kore_pencil_desc`` points to (``desc``)."""

    def __init__(self, A, B=None, layout=None, params=None):
        if layout is None:
            if params is None:
                raise ValueError("need a layout or the kore parameters")
            layout = layout_from_params(params)
        self.layout = layout
        n = A.shape[0]
        if n != layout.n:
            raise ValueError(f"matrix size {n} does not match the layout ({layout.n})")
        self.n = n
        self._a = _csr(A, np.complex128)
        self._b = _csr(B, np.float64) if B is not None else None
        self._perm = np.ascontiguousarray(layout.perm, dtype=np.int64)
        self._bs = L.as_i32(layout.block_sizes)
        d = L.PencilDesc()
        d.n = n
        d.a_nnz = len(self._a[1])
        d.a_indptr = self._a[0].ctypes.data_as(C.POINTER(C.c_int32))
        d.a_indices = self._a[1].ctypes.data_as(C.POINTER(C.c_int32))
        d.a_data = self._a[2].view(np.float64).ctypes.data_as(C.POINTER(C.c_double))
        if self._b is not None:
            d.b_nnz = len(self._b[1])
            d.b_indptr = self._b[0].ctypes.data_as(C.POINTER(C.c_int32))
            d.b_indices = self._b[1].ctypes.data_as(C.POINTER(C.c_int32))
            d.b_data = self._b[2].ctypes.data_as(C.POINTER(C.c_double))
        d.perm = self._perm.ctypes.data_as(C.POINTER(C.c_int64))
        d.nblocks = len(self._bs)
        d.block_sizes = self._bs.ctypes.data_as(C.POINTER(C.c_int32))
        self.desc = d

    def estimate_bytes(self, precision="mixed", nshift=1, ncv=0):
        """Upper bound of the device bytes of a plan of this pencil (kore_plan_estimate_bytes)."""
        out = C.c_int64()
        L.check(L.load().kore_plan_estimate_bytes(C.byref(self.desc), L.PREC[precision], int(nshift), int(ncv),
                                                   C.byref(out)), "kore_plan_estimate_bytes")
        return int(out.value)


class Pencil:
    """A (complex128) and optionally B (float64) on the device in l-major block form.

    ``layout`` is a :class:`~kore_gb300.structure.Layout` (or the kore parameters to
    derive one from).  The device copies are owned by the plan; ``close()`` frees them.
    """

    def __init__(self, A, B=None, layout=None, params=None, device=0):
        self.lib = L.load()
        self.data = PencilData(A, B, layout, params)
        self.layout = self.data.layout
        self.n = self.data.n
        self._plan = C.c_void_p()
        t = time.perf_counter()
        L.check(self.lib.kore_plan_create(C.byref(self.data.desc), int(device), C.byref(self._plan)),
                "kore_plan_create")
        self.create_s = time.perf_counter() - t
        self.sigma = None
        self.precision = None
        self.factor_s = None

    # -- factor / solve ---------------------------------------------------------------
    def factor(self, sigma, precision="fp64"):
        """Factorise A - sigma*B (block cyclic reduction, csrc/factor.cu)."""
        sigma = complex(sigma)
        t = time.perf_counter()
        L.check(self.lib.kore_factor(self._plan, sigma.real, sigma.imag, L.PREC[precision]), "kore_factor")
        self.factor_s = time.perf_counter() - t
        self.sigma, self.precision = sigma, precision
        return self

    def factor_shifts(self, sigmas, precision="fp64"):
        """Factorise A - sigma_s B for every shift at once (batched kernels); then
        ``solve`` takes an (n, k * nshift) array whose column j uses shift j % nshift."""
        sig = np.ascontiguousarray(np.asarray(sigmas, dtype=np.complex128).ravel())
        t = time.perf_counter()
        L.check(self.lib.kore_factor_shifts(self._plan, len(sig), L.ptr(sig.view(np.float64)), L.PREC[precision]),
                "kore_factor_shifts")
        self.factor_s = time.perf_counter() - t
        self.sigma = complex(sig[0]) if len(sig) == 1 else tuple(sig)
        self.precision = precision
        return self

    def solve(self, b, refine_tol=0.0, stats=False):
        """x = (A - sigma B)^-1 b for a vector or the columns of an (n, k) array."""
        b = np.asarray(b)
        one = b.ndim == 1
        bc = L.as_c128(b.reshape(self.n, -1).T)  # (k, n) rows contiguous
        x = np.empty_like(bc)
        st = L.Stats()
        L.check(self.lib.kore_solve(self._plan, L.ptr(bc), L.ptr(x), bc.shape[0], float(refine_tol), C.byref(st)),
                "kore_solve")
        out = x[0] if one else np.ascontiguousarray(x.T)
        return (out, st.as_dict()) if stats else out

    def solve_dev(self, b_ptr, x_ptr, nrhs=1, refine_tol=0.0, stream=None):
        """Device-pointer form (complex128, original order); ``stream`` is a cudaStream_t value."""
        st = L.Stats()
        L.check(self.lib.kore_solve_dev(self._plan, C.c_void_p(b_ptr), C.c_void_p(x_ptr), int(nrhs),
                                        float(refine_tol), C.c_void_p(stream or 0), C.byref(st)), "kore_solve_dev")
        return st.as_dict()

    def residual(self, lam, x):
        """A x - lam B x (FP64 on the device)."""
        lam = complex(lam)
        x = L.as_c128(x)
        y = np.empty_like(x)
        L.check(self.lib.kore_residual(self._plan, lam.real, lam.imag, L.ptr(x), L.ptr(y)), "kore_residual")
        return y

    def stream(self):
        """cudaStream_t (as an int) the plan launches its kernels on."""
        s = C.c_void_p()
        L.check(self.lib.kore_plan_stream(self._plan, C.byref(s)), "kore_plan_stream")
        return int(s.value or 0)

    def profile(self, enable):
        """Start (True) / stop (False) CUDA-event timing of the sweep and factorisation
        kernels; returns the totals recorded so far."""
        out = np.zeros(14)
        L.check(self.lib.kore_profile(self._plan, 1 if enable else 0, L.ptr(out)), "kore_profile")
        return {"sweep_ms": out[0], "sweeps": int(out[1]), "factor_ms": out[2], "factors": int(out[3]),
                "sweep_bytes": out[4], "factor_flops": out[5], "spmv_ms": out[6], "spmv_n": int(out[7]),
                "ortho_ms": out[8], "ortho_n": int(out[9]), "schur_ms": out[10], "schur_n": int(out[11]),
                "sweep_ctas_per_sm": int(out[12]), "sweep_chunk_bytes": int(out[13])}

    def device_bytes(self):
        v = C.c_int64()
        L.check(self.lib.kore_plan_bytes(self._plan, C.byref(v)), "kore_plan_bytes")
        return int(v.value)

    def close(self):
        if getattr(self, "_plan", None) and self._plan.value:
            self.lib.kore_plan_destroy(self._plan)
            self._plan = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def kernel_launches():
    return int(L.load().kore_kernel_launches())


def sweep_variant(ctas_per_sm=0, chunk_bytes=0):
    """Pin the sweep variant for every later sweep of the process (2, 3 or 4 CTAs per SM;
    8192 or 16384-byte ring slots); sweep_variant() returns to the autotuner's choice."""
    L.check(L.load().kore_sweep_variant(int(ctas_per_sm), int(chunk_bytes)), "kore_sweep_variant")


def forced_sweep(pencil, omegas, b, precision="mixed", group=16, refine_tol=0.0, scale=1.0, escalate_tol=1e-10,
                 info=None):
    """Forced solves over a frequency sweep on one eigen pencil.

    kore's forced matrix at forcing frequency w is ||B||_F (A_eig - i w B_eig)
    (``bin/assemble.py:582-584``), so each forced solve of ``bin/solve.py:207-268`` is the
    shifted solve x_w = (A_eig - i w B_eig)^-1 b_w / scale with scale = ||B||_F.  The
    frequencies are factorised and solved ``group`` at a time in batched kernels.

    Mixed precision: when the FP64 refinement of a group stops above ``escalate_tol``
    (normwise backward error; the complex64 factors of a badly conditioned shift do not
    contract the error), that group is factorised again in FP64 and solved with those
    factors, so every returned solve meets the bound the direct FP64 solve meets.

    b: (n,) right-hand side shared by every frequency, or (n, F) one per frequency.
    Returns (X (n, F), per-group wall seconds); ``info`` (a dict) receives the number of
    escalated frequencies and the largest backward error the mixed refinement reached.
    """
    om = np.asarray(omegas, dtype=np.float64).ravel()
    F = len(om)
    b = np.asarray(b)
    X = np.empty((pencil.n, F), dtype=np.complex128)
    times = []
    escalated, resid = 0, 0.0
    for g0 in range(0, F, group):
        sl = slice(g0, min(F, g0 + group))
        t = time.perf_counter()
        pencil.factor_shifts(1j * om[sl], precision)
        rhs = (b[:, sl] if b.ndim == 2 else np.repeat(b.reshape(-1, 1), sl.stop - sl.start, axis=1)) / scale
        X[:, sl], st = pencil.solve(rhs, refine_tol=refine_tol, stats=True)
        if precision == "mixed":
            resid = max(resid, st["solve_resid_max"])
            if escalate_tol and not st["solve_resid_max"] <= escalate_tol:
                pencil.factor_shifts(1j * om[sl], "fp64")
                X[:, sl] = pencil.solve(rhs)
                escalated += sl.stop - sl.start
        times.append(time.perf_counter() - t)
    if info is not None:
        info.update(escalated=escalated, mixed_resid_max=resid)
    return X, times


def eigs_targets(pencil, targets, nev, which="TM", precision="mixed", tol=1e-15, maxit=50, seeds=None, ncv=0,
                 purify=True, refine_tol=0.0, vectors=True, slots=None, reuse_radius=0.0, warm=False):
    """Shift-and-invert Krylov-Schur at several targets of one pencil, the targets
    stepping together in shared launches (``kore_eigs_shifts``).  ``slots`` targets run
    at a time (default: all); when one finishes, the next takes its slot (its shift is
    factorised then), so a long list of targets keeps every slot busy.

    The reference computes one target per ``bin/solve.py`` run (``bin/solve.py:91-158``,
    with ``tau`` from ``parameters.py``), fanned out over parameter sweeps by its tools;
    target t here gives what that run gives: the converged eigenvalues nearest ``tau_t``
    in SLEPc's order for ``which`` and their unit eigenvectors.  ``nev`` and ``seeds``
    may be one value or one per target.  Factorises ``A - tau_t B`` for every target
    first (one batched factorisation).

    ``reuse_radius`` > 0: a later target runs on an idle slot whose shift lies within this
    distance of it (that shift is the spectral transformation's, the eigenvalues are still
    sorted from the target), without re-factorising.  ``warm``: a target starts from its
    seeded vector plus the eigenvectors its slot returned last.

    Returns a list of (eigenvalues, eigenvectors or None, stats dict), one per target.
    """
    tg = np.asarray(targets, dtype=np.complex128).ravel()
    T = len(tg)
    nevs = np.broadcast_to(np.asarray(nev, dtype=int), (T,))
    sds = np.broadcast_to(np.asarray(seeds if seeds is not None else np.arange(T), dtype=np.uint64), (T,))
    ns = T if slots is None else max(1, min(int(slots), T))
    pencil.factor_shifts(tg[:ns], precision)
    opts = (L.EpsOpts * T)()
    mx = 0
    for t in range(T):
        k = int(nevs[t])
        m = int(ncv) or L.default_ncv(pencil.n, k)
        mx = max(mx, m)
        opts[t] = L.EpsOpts(nev=k, ncv=int(ncv), tol=tol, maxit=maxit, which=L.WHICH[which], target_re=tg[t].real,
                            target_im=tg[t].imag, seed=int(sds[t]), purify=int(purify),
                            refine_tol=refine_tol, reuse_radius=float(reuse_radius), warm=int(bool(warm)))
    ev = np.zeros((T, mx), dtype=np.complex128)
    X = np.zeros((T, mx, pencil.n), dtype=np.complex128) if vectors else None
    nconv = (C.c_int * T)()
    st = (L.Stats * T)()
    s = pencil.lib.kore_eigs_shifts(pencil._plan, T, opts, L.ptr(ev), L.ptr(X) if vectors else None, mx, nconv, st)
    if s not in (L.KORE_OK, 5):   # KORE_ENOCONV: a target with nconv = 0
        L.check(s, "kore_eigs_shifts")
    out = []
    for t in range(T):
        k = nconv[t]
        out.append((ev[t, :k].copy(), np.ascontiguousarray(X[t, :k].T) if vectors else None, st[t].as_dict()))
    return out


class EPS:
    """Shift-and-invert Krylov-Schur eigensolver with the slepc4py EPS call sequence
    that ``bin/solve.py:91-123`` uses."""

    class ProblemType:
        GNHEP = "GNHEP"

    class Which:
        LARGEST_MAGNITUDE = "LM"
        SMALLEST_MAGNITUDE = "SM"
        LARGEST_REAL = "LR"
        SMALLEST_REAL = "SR"
        LARGEST_IMAGINARY = "LI"
        SMALLEST_IMAGINARY = "SI"
        TARGET_MAGNITUDE = "TM"
        TARGET_REAL = "TR"
        TARGET_IMAGINARY = "TI"

    def __init__(self):
        self.pencil = None
        self.nev, self.ncv = 1, 0
        self.tol, self.maxit = 1e-8, 100
        self.which = "LM"
        self.target = 0j
        self.shift = None          # spectral-transformation shift (SLEPc -st_shift); None: the target
        self.st_type = "sinvert"
        self.precision = "fp64"
        self.seed = 0
        self.purify = True
        self.purify_steps = 1
        self.refine_tol = 0.0
        self._lam = np.zeros(0, complex)
        self._X = None
        self.stats = {}
        self.its = 0

    def create(self, comm=None):
        return self

    def setOperators(self, pencil, B=None):
        if not isinstance(pencil, Pencil):
            raise TypeError("EPS.setOperators takes a kore_gb300 Pencil holding A and B")
        self.pencil = pencil

    def setProblemType(self, ptype):
        if ptype != "GNHEP":
            raise ValueError("only the generalized non-Hermitian problem (GNHEP) is on the kore path")

    def setDimensions(self, nev=None, ncv=None, mpd=None):
        if nev is not None:
            self.nev = int(nev)
        if ncv is not None:
            self.ncv = int(ncv)

    def setTolerances(self, tol=None, max_it=None):
        if tol is not None:
            self.tol = float(tol)
        if max_it is not None:
            self.maxit = int(max_it)

    def setWhichEigenpairs(self, which):
        if which not in L.WHICH:
            raise ValueError(f"unknown which {which!r}")
        self.which = which

    def setTarget(self, tau):
        self.target = complex(tau)

    def setFromOptions(self, options=None):
        """Apply PETSc-style options (dict of option -> value, without the dash)."""
        o = options or {}
        if "st_type" in o:
            if o["st_type"] != "sinvert":
                raise ValueError("only -st_type sinvert is on the kore path")
        if "eps_nev" in o:
            self.nev = int(o["eps_nev"])
        if "eps_ncv" in o:
            self.ncv = int(o["eps_ncv"])
        if "eps_tol" in o:
            self.tol = float(o["eps_tol"])
        if "eps_max_it" in o:
            self.maxit = int(o["eps_max_it"])
        if "eps_purify" in o:
            self.purify = str(o["eps_purify"]).lower() not in ("0", "false", "no")
        if "kore_purify_steps" in o:
            self.purify_steps = int(o["kore_purify_steps"])
        if "kore_precision" in o:
            self.precision = o["kore_precision"]
        if "kore_seed" in o:
            self.seed = int(o["kore_seed"])
        if "kore_refine_tol" in o:
            self.refine_tol = float(o["kore_refine_tol"])
        if "st_shift" in o:
            self.shift = complex(o["st_shift"])

    def setShift(self, sigma):
        """Shift of the spectral transformation, apart from the target (SLEPc's
        ST.setShift / -st_shift): OP = (A - sigma B)^-1 B, eigenvalues sorted by `which`
        from the target."""
        self.shift = None if sigma is None else complex(sigma)

    def getDimensions(self):
        n = self.pencil.n
        ncv = self.ncv or L.default_ncv(n, self.nev)
        return self.nev, ncv, ncv

    def getTolerances(self):
        return self.tol, self.maxit

    def getTarget(self):
        return self.target

    def getType(self):
        return "krylovschur"

    def solve(self):
        p = self.pencil
        if self.which not in ("TM", "TR", "TI"):
            # SLEPc's EPSSetUp stops here under -st_type sinvert, the kore path's transformation
            raise ValueError(f"shift-and-invert requires a target 'which' (TM, TR or TI), not {self.which!r}")
        sigma = self.target if self.shift is None else self.shift
        if p.sigma != sigma or p.precision != self.precision:
            p.factor(sigma, self.precision)
        nev, ncv, _ = self.getDimensions()
        o = L.EpsOpts(nev=nev, ncv=ncv, tol=self.tol, maxit=self.maxit, which=L.WHICH[self.which],
                      target_re=self.target.real, target_im=self.target.imag, seed=self.seed,
                      purify=self.purify_steps if self.purify else 0, refine_tol=self.refine_tol,
                      shift_re=sigma.real, shift_im=sigma.imag, has_shift=int(self.shift is not None))
        ev = np.zeros(ncv, dtype=np.complex128)
        X = np.zeros((ncv, p.n), dtype=np.complex128)
        nconv = C.c_int(0)
        st = L.Stats()
        t = time.perf_counter()
        s = p.lib.kore_eigs(p._plan, C.byref(o), L.ptr(ev), L.ptr(X), ncv, C.byref(nconv), C.byref(st))
        self.solve_s = time.perf_counter() - t
        self.stats = st.as_dict()
        self.stats["factor_s"] = p.factor_s
        if s not in (L.KORE_OK, 5):  # KORE_ENOCONV leaves nconv = 0 (bin/solve.py:192-199)
            L.check(s, "kore_eigs")
        k = nconv.value
        self.its = st.restarts
        self._lam = ev[:k].copy()
        self._X = np.ascontiguousarray(X[:k].T)
        return self

    def getConverged(self):
        return len(self._lam)

    def getIterationNumber(self):
        return self.its

    def getEigenpair(self, i, Vr=None, Vi=None):
        """Eigenvalue i; if ``Vr`` is a numpy array it receives the eigenvector."""
        if Vr is not None:
            Vr[...] = self._X[:, i]
        return complex(self._lam[i])

    def eigenvalues(self):
        return self._lam.copy()

    def eigenvectors(self):
        return self._X


class KSP:
    """Direct solve ``-ksp_type preonly -pc_type lu`` (``bin/solve.py:219-227``)."""

    def __init__(self):
        self.pencil = None
        self.rtol, self.max_it = 1e-8, 10000
        self.precision = "fp64"
        self.refine_tol = 0.0
        self.escalate_tol = 1e-10   # mixed: refactorise in FP64 when the refinement stops above it
        self.stats = {}

    def create(self, comm=None):
        return self

    def setOperators(self, pencil):
        if not isinstance(pencil, Pencil):
            raise TypeError("KSP.setOperators takes a kore_gb300 Pencil holding A")
        self.pencil = pencil

    def setTolerances(self, rtol=None, max_it=None):
        if rtol is not None:
            self.rtol = float(rtol)
        if max_it is not None:
            self.max_it = int(max_it)

    def setFromOptions(self, options=None):
        o = options or {}
        if o.get("ksp_type", "preonly") != "preonly" or o.get("pc_type", "lu") != "lu":
            raise ValueError("only -ksp_type preonly -pc_type lu is on the kore path")
        if "kore_precision" in o:
            self.precision = o["kore_precision"]
        if "kore_refine_tol" in o:
            self.refine_tol = float(o["kore_refine_tol"])

    def solve(self, b, x=None):
        p = self.pencil
        if p.sigma != 0j or p.precision != self.precision:
            p.factor(0.0, self.precision)
        sol, st = p.solve(b, refine_tol=self.refine_tol, stats=True)
        st["escalated"] = 0
        if self.precision == "mixed" and self.escalate_tol and not st["solve_resid_max"] <= self.escalate_tol:
            p.factor(0.0, "fp64")
            sol = p.solve(b)
            st["escalated"] = 1
        self.stats = st
        if x is not None:
            x[...] = sol
            return x
        return sol
