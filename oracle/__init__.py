"""CPU oracle for the implicit nodal pressure projection -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain NumPy/SciPy FP64, the reference algorithm of
pyBELLA's implicit nodal pressure projection (``second_projection.py`` and
``laplacian.py`` of the reference).  Each function cites the reference
file:line that it follows.

It is the checker, never the product: only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it.  The product path
(``pybella_gb300``) never imports or calls anything in here and fails loudly
when its CUDA library is missing.

Parity pins
-----------
* 2D nodal operator, Jacobi diagonal, coefficients, divergence, correction and
  the whole projection step: pinned against the reference itself, imported in
  a container that has it (``tests/golden/make_golden.py``), through the
  committed fixtures under ``tests/golden/``.
* 3D 27-point operator: the reference's 3D glue cannot run as shipped
  (``second_projection.py:183-203`` uses ``diag_inv``/``p2`` before
  assignment), so the 3D operator here follows ``lap3D``'s arithmetic with the
  2D path's boundary conventions and is pinned only by self-consistency tests
  (z-invariant fields reproduce the 2D operator, adjoint/symmetry checks).
"""
