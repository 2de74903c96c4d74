"""Background solve of the nodal operators (libbella_gb300 ``bella_spectral3d_*`` /
``bella_spectral2d_create``).

The exact inverse of the 27-point (3D) or 9-point (2D) operator with every
cell coefficient replaced by its mean over the horizontal axes per y-cell (the
stratified background) and ``hcenter`` by its mean per y-node: Hartley
(periodic axis) or DCT-I (wall axis) transforms along x and z, a tridiagonal
solve along y for every horizontal mode, pseudo-inverse on the modes of the
operator's null space.  The transforms are two-pass register FFTs for
power-of-two lengths (dense FP32 GEMMs otherwise); the line solves sweep in FP32
with Thomas factors computed once per operator in FP64.  As a right
preconditioner it bounds the condition number by the spread of the cell
coefficients about their horizontal means.  The reference solves without a
preconditioner (second_projection.py:230 passes no ``M`` to scipy's bicgstab);
this is the slot it fills.
"""
import ctypes

import torch

from . import _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class BackgroundSolve:
    """Background inverse of a :class:`pybella_gb300.linalg.NodalHelmholtz3D` or
    :class:`~pybella_gb300.linalg.NodalHelmholtz2D` (y must be a wall axis; in 2D the
    transform runs along x and the Coriolis cross terms are left out).

    ``apply(r)`` maps a residual of the Jacobi-scaled system (FP32 CUDA tensor)
    to ``A_bg^+ (r / diag_inv)``; pass the object as ``preconditioner=`` to
    :meth:`~pybella_gb300.linalg.NodalHelmholtz3D.solve`, alone or inside a
    :class:`pybella_gb300.learned.LearnedPreconditioner`.
    """

    kind = "background"

    def __init__(self, op):
        self.op = op
        self.dev = op.dev
        self.n = op.n
        self._lib = op.ws._lib
        h = ctypes.c_void_p()
        create = (self._lib.bella_spectral2d_create if isinstance(op._op, _lib.Op2D)
                  else self._lib.bella_spectral3d_create)
        with torch.cuda.device(self.dev):
            _lib.check(create(ctypes.byref(h), ctypes.byref(op._op), self.dev.index,
                              ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)),
                       "bella_spectral_create")
        self.handle = h

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def apply(self, r, out=None):
        x = r.detach().to(device=self.dev, dtype=torch.float32).contiguous().reshape(-1)
        if x.numel() != self.n:
            raise ValueError("vector has %d entries, operator has %d unknowns" % (x.numel(), self.n))
        y = torch.empty_like(x) if out is None else out
        with torch.cuda.device(self.dev):
            _lib.check(self._lib.bella_spectral3d_apply(self.handle, _ptr(x), _ptr(y), self._stream()),
                       "bella_spectral3d_apply")
        return y

    __call__ = apply

    def update(self, op):
        """Re-derive the background solve from ``op``'s coefficients in place (an
        operator of the same shape and boundary kinds as the one it was made for,
        e.g. the next time step's): nothing is allocated
        (``bella_spectral3d_update`` / ``bella_spectral2d_update``)."""
        upd = (self._lib.bella_spectral2d_update if isinstance(op._op, _lib.Op2D)
               else self._lib.bella_spectral3d_update)
        with torch.cuda.device(self.dev):
            _lib.check(upd(self.handle, ctypes.byref(op._op), self._stream()), "bella_spectral_update")
        self.op = op
        return self

    def launches(self):
        return int(self._lib.bella_spectral3d_launches(self.handle))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self._lib.bella_spectral3d_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
