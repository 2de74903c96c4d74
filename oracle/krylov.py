"""SciPy BiCGStab with the reference's call semantics (oracle; tests only).

The reference calls ``scipy.sparse.linalg.bicgstab(lap, rhs_inner, tol=ud.tol,
maxiter=ud.max_iterations, callback=counter)`` (second_projection.py:230)
against SciPy 1.7.3 (requirements.txt:11).  SciPy 1.7's ``tol`` keyword used
"legacy" semantics: ``atol = tol * ||b||`` and an immediate exit with ``x = 0``
when ``||b - A x0|| <= tol``.  Newer SciPy spells this ``rtol=tol, atol=0``;
this module adds the legacy early exit on top of the installed SciPy.
"""
import numpy as np
import scipy.sparse.linalg as spla


def bicgstab_legacy(op_or_matvec, b, tol, maxiter, x0=None):
    """Solve with SciPy BiCGStab; returns ``(x, info, iterations)``.

    ``op_or_matvec`` is either a callable ``matvec`` or a packed operator dict
    from :mod:`oracle.nodal2d` / :mod:`oracle.nodal3d`.
    """
    b = np.asarray(b, dtype=np.float64)
    if callable(op_or_matvec):
        mv = op_or_matvec
    elif "nz" in op_or_matvec:
        from oracle.nodal3d import lap3d
        mv = lambda v: lap3d(v, op_or_matvec)
    else:
        from oracle.nodal2d import lap2d_gather
        mv = lambda v: lap2d_gather(v, op_or_matvec)
    n = b.shape[0]
    if x0 is None:
        if np.linalg.norm(b) <= tol:
            return np.zeros_like(b), 0, 0
    A = spla.LinearOperator((n, n), matvec=mv, dtype=np.float64)
    count = [0]

    def cb(xk):
        count[0] += 1

    x, info = spla.bicgstab(A, b, x0=x0, rtol=tol, atol=0.0, maxiter=maxiter, callback=cb)
    return x, info, count[0]


def true_relres(op_or_matvec, x, b):
    """``||b - A x|| / ||b||`` evaluated with the FP64 oracle operator."""
    if callable(op_or_matvec):
        mv = op_or_matvec
    elif "nz" in op_or_matvec:
        from oracle.nodal3d import lap3d
        mv = lambda v: lap3d(v, op_or_matvec)
    else:
        from oracle.nodal2d import lap2d_gather
        mv = lambda v: lap2d_gather(v, op_or_matvec)
    r = b - mv(x)
    nb = np.linalg.norm(b)
    return np.linalg.norm(r) / (nb if nb > 0 else 1.0)
