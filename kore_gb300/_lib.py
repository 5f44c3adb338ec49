"""ctypes binding of libkoregpu.so (declarations in include/kore_gpu.h).

The library is the only compute path: there is no CPU fallback.  If it is missing
or cannot be loaded, every entry point raises ``KoreError`` naming the cause.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libkoregpu.so")

KORE_OK = 0
STATUS = {
    0: "KORE_OK", 1: "KORE_EINVAL", 2: "KORE_ENOMEM", 3: "KORE_ECUDA", 4: "KORE_ESINGULAR",
    5: "KORE_ENOCONV", 6: "KORE_ETIMEOUT", 7: "KORE_ENOTFACTORED", 8: "KORE_ENAN", 9: "KORE_EPENDING",
    10: "KORE_ECANCELLED",
}
KORE_EPENDING = 9
REQ_EIGEN, REQ_FORCED = 0, 1
PREC = {"fp64": 0, "mixed": 1}
WHICH = {"LM": 0, "SM": 1, "LR": 2, "SR": 3, "LI": 4, "SI": 5, "TM": 6, "TR": 7, "TI": 8}
MAX_NCV = 64   # largest Krylov basis of the eigensolver


def default_ncv(n, nev):
    """The eigensolver's basis size when none is given (kore_eps_opts.ncv = 0): SLEPc's
    max(2 nev, nev + 15), raised to 4 nev up to MAX_NCV."""
    return min(int(n), max(2 * nev, nev + 15, min(MAX_NCV, 4 * nev)))

# every function include/kore_gpu.h declares
EXPORTS = ("kore_plan_create", "kore_factor", "kore_factor_shifts", "kore_solve", "kore_solve_dev",
           "kore_solve_dev_noalloc", "kore_eigs", "kore_eigs_shifts", "kore_residual", "kore_plan_stream", "kore_profile",
           "kore_plan_bytes", "kore_plan_estimate_bytes", "kore_batch_create", "kore_batch_submit",
           "kore_batch_poll", "kore_batch_stats", "kore_batch_destroy", "kore_tc_selftest", "kore_gegenbauer_mult", "kore_flow_diagnostics", "kore_assemble_blocks", "kore_sweep_variant", "kore_kernel_launches",
           "kore_status_string", "kore_plan_destroy")


class KoreError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        name = STATUS.get(status, str(status))
        msg = f"{what}: {name}"
        if _lib is not None and status in STATUS:
            msg += " (" + _lib.kore_status_string(status).decode() + ")"
        super().__init__(msg)


class PencilDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("a_nnz", C.c_int64),
        ("a_indptr", C.POINTER(C.c_int32)),
        ("a_indices", C.POINTER(C.c_int32)),
        ("a_data", C.POINTER(C.c_double)),
        ("b_nnz", C.c_int64),
        ("b_indptr", C.POINTER(C.c_int32)),
        ("b_indices", C.POINTER(C.c_int32)),
        ("b_data", C.POINTER(C.c_double)),
        ("perm", C.POINTER(C.c_int64)),
        ("nblocks", C.c_int32),
        ("block_sizes", C.POINTER(C.c_int32)),
    ]


class EpsOpts(C.Structure):
    _fields_ = [
        ("nev", C.c_int32),
        ("ncv", C.c_int32),
        ("tol", C.c_double),
        ("maxit", C.c_int32),
        ("which", C.c_int32),
        ("target_re", C.c_double),
        ("target_im", C.c_double),
        ("seed", C.c_uint64),
        ("purify", C.c_int32),
        ("refine_tol", C.c_double),
        ("shift_re", C.c_double),
        ("shift_im", C.c_double),
        ("has_shift", C.c_int32),
        ("warm", C.c_int32),
        ("reuse_radius", C.c_double),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("nconv", C.c_int32),
        ("restarts", C.c_int32),
        ("op_applies", C.c_int32),
        ("sweeps", C.c_int32),
        ("refine_iters_max", C.c_int32),
        ("solve_resid_max", C.c_double),
        ("factor_ms", C.c_double),
        ("iterate_ms", C.c_double),
        ("factor_reused", C.c_int32),
        ("warm_started", C.c_int32),
        ("shift_re", C.c_double),
        ("shift_im", C.c_double),
        ("escalated", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Request(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("pencil", C.POINTER(PencilDesc)),
        ("pencil_key", C.c_uint64),
        ("precision", C.c_int32),
        ("sigma_re", C.c_double),
        ("sigma_im", C.c_double),
        ("opts", EpsOpts),
        ("rhs", C.c_void_p),
        ("rhs_scale", C.c_double),
        ("refine_tol", C.c_double),
        ("x", C.c_void_p),
        ("evals", C.c_void_p),
        ("evecs", C.c_void_p),
        ("max_pairs", C.c_int32),
        ("nconv", C.POINTER(C.c_int32)),
        ("timing_ms", C.c_void_p),
        ("stats", C.c_void_p),
    ]


_lib = None
_load_error = None


def _bind(lib):
    P = C.c_void_p
    lib.kore_plan_create.argtypes = [C.POINTER(PencilDesc), C.c_int, C.POINTER(P)]
    lib.kore_factor.argtypes = [P, C.c_double, C.c_double, C.c_int]
    lib.kore_factor_shifts.argtypes = [P, C.c_int, P, C.c_int]
    lib.kore_solve.argtypes = [P, P, P, C.c_int, C.c_double, C.POINTER(Stats)]
    lib.kore_solve_dev.argtypes = [P, P, P, C.c_int, C.c_double, P, C.POINTER(Stats)]
    lib.kore_solve_dev_noalloc.argtypes = [P, P, P, C.c_double, P]
    lib.kore_eigs.argtypes = [P, C.POINTER(EpsOpts), P, P, C.c_int, C.POINTER(C.c_int), C.POINTER(Stats)]
    lib.kore_eigs_shifts.argtypes = [P, C.c_int, C.POINTER(EpsOpts), P, P, C.c_int, C.POINTER(C.c_int),
                                     C.POINTER(Stats)]
    lib.kore_residual.argtypes = [P, C.c_double, C.c_double, P, P]
    lib.kore_plan_stream.argtypes = [P, C.POINTER(P)]
    lib.kore_profile.argtypes = [P, C.c_int, P]
    lib.kore_plan_bytes.argtypes = [P, C.POINTER(C.c_int64)]
    lib.kore_kernel_launches.argtypes = []
    lib.kore_kernel_launches.restype = C.c_int64
    lib.kore_status_string.argtypes = [C.c_int]
    lib.kore_status_string.restype = C.c_char_p
    lib.kore_plan_destroy.argtypes = [P]
    lib.kore_plan_estimate_bytes.argtypes = [C.POINTER(PencilDesc), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64)]
    lib.kore_batch_create.argtypes = [C.c_int, C.c_int64, C.c_int, C.POINTER(P)]
    lib.kore_batch_submit.argtypes = [P, C.POINTER(Request), C.POINTER(C.c_uint64)]
    lib.kore_batch_poll.argtypes = [P, C.c_uint64, C.c_int, C.POINTER(C.c_int)]
    lib.kore_batch_stats.argtypes = [P, P]
    lib.kore_batch_destroy.argtypes = [P]
    lib.kore_tc_selftest.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.kore_gegenbauer_mult.argtypes = [C.c_int, C.c_int, P, C.c_double, C.c_int, P]
    lib.kore_flow_diagnostics.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, P, C.c_int, P, P, C.c_int, P]
    lib.kore_sweep_variant.argtypes = [C.c_int, C.c_int]
    lib.kore_assemble_blocks.argtypes = [C.c_int, C.c_int, C.c_int, P, C.c_int64, P, C.c_int, P, C.c_int64, P, P, P,
                                         P, P, P, P, C.c_int64, P, P, C.c_int64, P, P]
    for name in EXPORTS:
        if name not in ("kore_kernel_launches", "kore_status_string"):
            getattr(lib, name).restype = C.c_int
    return lib


def load(path=None):
    """Load (once) and return the library; raise RuntimeError if it is absent."""
    global _lib, _load_error
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"libkoregpu.so not built ({path}); run kore_gb300.build.build()")
    try:
        _lib = _bind(C.CDLL(path))
    except OSError as e:  # pragma: no cover - depends on the machine
        _load_error = e
        raise RuntimeError(f"cannot load {path}: {e}") from e
    return _lib


def check(status, what):
    if status != KORE_OK:
        raise KoreError(status, what)


def ptr(a):
    """Data pointer of a C-contiguous numpy array."""
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return C.c_void_p(a.ctypes.data)


def as_i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def as_c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)
