"""CPU oracle for the kore solve path — TEST INFRASTRUCTURE ONLY.

Nothing in the product (``kore_gb300``) imports this package. Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it, and only as
the checker or the timed CPU baseline.

The reference path (``bin/solve.py``) hands all arithmetic to PETSc/SLEPc and a
sparse direct solver (MUMPS / SuperLU_dist); none of those are installed here, so
``eps_ref`` restates that arithmetic with scipy:

* ``E.solve()`` with ``-st_type sinvert`` (``bin/solve.py:91-123``): sparse LU of
  A - tau*B (scipy SuperLU), Krylov iteration on (A - tau*B)^-1 B (ARPACK), back
  transformation lambda = tau + 1/theta, SLEPc's ``which`` ordering
  (``bin/solve.py:99-117``) and unit-2-norm eigenvectors.
* ``K.solve`` with ``-ksp_type preonly -pc_type lu`` (``bin/solve.py:207-227``):
  one sparse LU solve of A x = b.

Parity is pinned by the reference's own golden values (``tests/spinover/reference.eig``,
``tests/jones2000/reference.jones``, ``tests/dormy2004/reference.dormy04``) on pencils
produced by the reference's own assembly (``tests/golden/make_fixtures.py``).
"""
