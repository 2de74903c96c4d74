"""Import shim for the pyBELLA reference (fixture generation only).

Used by ``make_golden.py`` in a container that has the reference checked out.
It makes the reference's hot path importable with the packages present here:

* ``numba`` is absent: ``jit``/``njit`` become identity decorators (the
  decorated functions then run as plain Python, which is slower but
  numerically the same FP64 arithmetic).  ``numba.stencil`` becomes a loop
  that applies the kernel at every point whose neighbourhood lies inside the
  first array, with the kernel's relative indices resolved against each array
  argument, and leaves the border at 0 (numba's default ``cval``); the
  neighbourhood is one point each way, that of the one stencil on the
  projection path (``kernel_9pt``, laplacian.py:749-856, used when
  ``ud.LAMB_BDRY`` is set).
* ``h5py``, ``dill``, ``yaml``, ``termcolor``, ``dask`` and ``matplotlib``
  are absent: they are replaced by empty modules (only imported, never
  used on the projection path).
* SciPy >= 1.14 removed ``bicgstab(..., tol=...)``: a wrapper maps the
  legacy keyword onto ``rtol`` with ``atol=0`` and keeps the SciPy 1.7
  "legacy" early exit ``||b|| <= tol  ->  x = 0`` (the reference pins
  scipy 1.7.3, requirements.txt:11).
* ``np.float`` was removed in numpy 1.24; the reference's test cases use it.
"""
import os
import sys
import types

import numpy as np
import scipy as sp
import scipy.sparse.linalg as spla


def _identity_decorator(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f


class _Relative:
    """An array seen from one point of a stencil: a[di, dj] reads a[i + di, j + dj]."""

    def __init__(self, a, i, j):
        self.a, self.i, self.j = a, i, j

    def __getitem__(self, idx):
        di, dj = idx
        return self.a[self.i + di, self.j + dj]


def _stencil(func=None, **kwargs):
    def wrap(kernel):
        def run(*args):
            a0 = args[0]
            out = np.zeros(a0.shape, dtype=np.float64)
            for i in range(1, a0.shape[0] - 1):
                for j in range(1, a0.shape[1] - 1):
                    out[i, j] = kernel(*[_Relative(a, i, j) if isinstance(a, np.ndarray) else a for a in args])
            return out
        return run
    return wrap(func) if callable(func) else wrap


def _stub_getattr(attr):
    if attr.startswith("__"):
        raise AttributeError(attr)
    return lambda *a, **k: None


def _install_stub_modules():
    nb = types.ModuleType("numba")
    nb.jit = _identity_decorator
    nb.njit = _identity_decorator
    nb.stencil = _stencil
    nb.prange = range
    sys.modules.setdefault("numba", nb)
    for name in ["h5py", "dill", "yaml", "termcolor", "dask", "dask.distributed",
                 "dask.array", "dask.delayed", "matplotlib", "matplotlib.pyplot",
                 "matplotlib.colors", "matplotlib.gridspec", "mpl_toolkits",
                 "mpl_toolkits.axes_grid1", "pyemd"]:
        if name in sys.modules:
            continue
        try:
            __import__(name)
        except ImportError:
            m = types.ModuleType(name)
            m.__path__ = []
            m.__getattr__ = _stub_getattr
            sys.modules[name] = m
    if not hasattr(np, "float"):
        np.float = float


_orig_bicgstab = spla.bicgstab


def legacy_bicgstab(A, b, x0=None, tol=None, maxiter=None, M=None, callback=None,
                    atol=None, rtol=None):
    """SciPy-1.7 ``bicgstab`` keyword semantics on top of the installed SciPy."""
    if tol is None:
        tol = 1e-5 if rtol is None else rtol
    b = np.asarray(b)
    if x0 is None and np.linalg.norm(b) <= tol:
        return np.zeros_like(b), 0
    return _orig_bicgstab(A, b, x0=x0, rtol=tol, atol=0.0 if atol is None else atol,
                          maxiter=maxiter, M=M, callback=callback)


def install(reference_root):
    """Put the reference's ``src`` and repo root on ``sys.path`` and shim it."""
    _install_stub_modules()
    spla.bicgstab = legacy_bicgstab
    sp.sparse.linalg.bicgstab = legacy_bicgstab
    src = os.path.join(reference_root, "src")
    for p in (src, reference_root):
        if p not in sys.path:
            sys.path.insert(0, p)
