"""kore_gb300 — GB300-native (sm_103a) solve path of kore.

The shift-and-invert Krylov-Schur eigensolve and the forced solve (A - sigma B) x = b
on the pencil that kore's ``bin/assemble.py`` writes, behind the entry points of
``include/kore_gpu.h`` (``libkoregpu.so``).
"""
from .structure import Layout, layout, layout_from_params, ell, field_offsets  # noqa: F401
from .solver import Pencil, EPS, KSP, kernel_launches, forced_sweep, eigs_targets, sweep_variant  # noqa: F401
from .onset import OnsetSearch  # noqa: F401
from . import _lib  # noqa: F401

__all__ = ["Layout", "layout", "layout_from_params", "ell", "field_offsets", "Pencil", "EPS", "KSP",
           "kernel_launches", "forced_sweep", "eigs_targets", "sweep_variant", "OnsetSearch"]
