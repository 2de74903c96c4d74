"""Drop-in ``LinearOperator`` / ``bicgstab`` for the reference's projection solve.

The reference builds its solve as (second_projection.py:175,205,230)::

    lap = lm_lp.stencil_9pt_numba_test(mpv, node, coriolis_params, diag_inv, ud)
    lap = sp.sparse.linalg.LinearOperator((sh, sh), lap)
    p2, _ = sp.sparse.linalg.bicgstab(lap, rhs_inner, tol=ud.tol,
                                      maxiter=ud.max_iterations, callback=counter)

With this package the same three lines read::

    lap = pybella_gb300.laplacian.stencil_9pt_numba_test(mpv, node, coriolis_params, diag_inv, ud)
    lap = pybella_gb300.linalg.LinearOperator((sh, sh), lap)
    p2, _ = pybella_gb300.linalg.bicgstab(lap, rhs_inner, tol=ud.tol,
                                          maxiter=ud.max_iterations, callback=counter)

and the operator and the whole Krylov iteration run on the GPU through
libbella_gb300.  There is no CPU path: a matvec that is not a device nodal
operator is rejected.
"""
import ctypes
import warnings

import numpy as np
import torch

from . import _lib

PRECISIONS = {"fp64": 0, "mixed": 1, "df64": 2}
_INFO = {_lib.BELLA_OK: 0, _lib.BELLA_BREAKDOWN: -10, _lib.BELLA_NONFINITE: -12}


def _device(device):
    if device is None:
        device = torch.cuda.current_device()
    return torch.device("cuda", int(device))


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _to_dev(a, dev, dtype=torch.float64):
    if isinstance(a, torch.Tensor):
        return a.detach().to(device=dev, dtype=dtype).contiguous().reshape(-1)
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a), dtype=np.float64)).to(
        device=dev, dtype=dtype).reshape(-1)


def _all_zero(a):
    if a is None:
        return True
    if isinstance(a, torch.Tensor):
        return bool((a == 0).all().item())
    return not np.any(np.asarray(a))


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class _NodalOperator:
    """Device-resident nodal operator: matvec and solves through libbella_gb300."""

    dev = None
    n = 0
    ws = None

    # -- matvec ------------------------------------------------------------
    def matvec(self, p):
        """``A @ p`` in FP64.  NumPy in -> NumPy out; CUDA tensor in -> CUDA tensor out."""
        is_torch = isinstance(p, torch.Tensor) and p.is_cuda
        x = _to_dev(p, self.dev)
        if x.numel() != self.n:
            raise ValueError("vector has %d entries, operator is %d x %d" % (x.numel(), self.n, self.n))
        y = torch.empty_like(x)
        with torch.cuda.device(self.dev):
            _lib.check(self.ws._lib.bella_apply_f64(self.ws.handle, _ptr(x), _ptr(y), _stream(self.dev)),
                       "bella_apply_f64")
        if is_torch:
            return y
        return y.cpu().numpy()

    __call__ = matvec

    def matvec_f32(self, p):
        """``A @ p`` with the FP32 planes (CUDA float32 tensor in and out)."""
        x = p.detach().to(device=self.dev, dtype=torch.float32).contiguous().reshape(-1)
        y = torch.empty_like(x)
        with torch.cuda.device(self.dev):
            _lib.check(self.ws._lib.bella_apply_f32(self.ws.handle, _ptr(x), _ptr(y), _stream(self.dev)),
                       "bella_apply_f32")
        return y

    # -- solve -------------------------------------------------------------
    def solve(self, b, x0=None, tol=1e-8, atol=0.0, maxiter=6000, precision="fp64", inner_tol=1e-5,
              project_null=True, check_every=16, timeout_s=0.0, out=None, preconditioner=None, max_outer=30,
              method="bicgstab", restart=20):
        """Solve ``A x = b``; returns ``(x, stats)`` with ``x`` a CUDA float64 tensor.

        ``precision='fp64'`` (default) is BiCGStab in FP64 with scipy's
        control flow.  ``'mixed'`` runs FP32 BiCGStab inner solves inside FP64
        iterative refinement (FP64 residuals, FP64 accumulated solution); if an
        inner solve fails (non-finite, breakdown, no progress) the solve is
        finished by double-float BiCGStab with FP64 reliable updates (its convergence
        is accepted only on the FP64 true residual) and ``stats['fallback'] == 1``.
        ``'df64'``
        is double-float BiCGStab with FP64 reliable updates.

        ``preconditioner`` (3D only) selects flexible BiCGStab right-
        preconditioned by a :class:`pybella_gb300.learned.CNN`, a
        :class:`pybella_gb300.spectral.BackgroundSolve` or a
        :class:`pybella_gb300.learned.LearnedPreconditioner` (background solve
        corrected by the network): FP32 inner iterations in FP64 refinement
        (its residual formed in double-float arithmetic, about 1e-14 of
        |A||x|, when ``tol >= 1e-11``), ``precision`` ignored; a failed preconditioned solve is finished by the
        plain double-float method, reported in ``stats['fallback']`` and by a
        warning.  ``method='fgmres'`` runs the preconditioned inner solves as
        flexible GMRES cycles of at most ``restart`` iterations (exact for a
        preconditioner that varies between applications, such as the BF16
        network) instead of flexible BiCGStab.
        """
        bd = _to_dev(b, self.dev)
        if bd.numel() != self.n:
            raise ValueError("rhs has %d entries, operator is %d x %d" % (bd.numel(), self.n, self.n))
        if out is None:
            x = torch.zeros_like(bd) if x0 is None else _to_dev(x0, self.dev).clone()
        else:
            x = out
            if x0 is not None:
                x.copy_(_to_dev(x0, self.dev))
        o = _lib.SolveOpts()
        self.ws._lib.bella_solve_opts_default(ctypes.byref(o))
        o.tol = float(tol)
        o.atol = float(atol or 0.0)
        o.maxiter = int(maxiter)
        o.precision = PRECISIONS[precision]
        o.x0_zero = 1 if x0 is None else 0
        o.project_null = int(bool(project_null))
        o.inner_tol = float(inner_tol)
        o.check_every = int(check_every)
        o.timeout_s = float(timeout_s)
        o.max_outer = int(max_outer)
        st = _lib.SolveStats()
        with torch.cuda.device(self.dev):
            if preconditioner is None:
                _lib.check(self.ws._lib.bella_bicgstab(self.ws.handle, _ptr(bd), _ptr(x), ctypes.byref(o),
                                                       ctypes.byref(st), _stream(self.dev)), "bella_bicgstab")
            else:
                sp, net = _precond_parts(preconditioner)
                if method == "fgmres":
                    _lib.check(self.ws._lib.bella_fgmres_pc(self.ws.handle, sp.handle if sp is not None else None,
                                                            net.handle if net is not None else None,
                                                            int(getattr(preconditioner, "compose", 0)), int(restart),
                                                            _ptr(bd), _ptr(x), ctypes.byref(o), ctypes.byref(st),
                                                            _stream(self.dev)), "bella_fgmres_pc")
                elif method != "bicgstab":
                    raise ValueError("method must be 'bicgstab' or 'fgmres'")
                elif sp is None:
                    _lib.check(self.ws._lib.bella_fbicgstab(self.ws.handle, net.handle, _ptr(bd), _ptr(x),
                                                            ctypes.byref(o), ctypes.byref(st), _stream(self.dev)),
                               "bella_fbicgstab")
                else:
                    _lib.check(self.ws._lib.bella_fbicgstab_pc(self.ws.handle, sp.handle,
                                                               net.handle if net is not None else None,
                                                               int(getattr(preconditioner, "compose", 0)),
                                                               _ptr(bd), _ptr(x), ctypes.byref(o), ctypes.byref(st),
                                                               _stream(self.dev)), "bella_fbicgstab_pc")
                if st.fallback:
                    warnings.warn("preconditioned solve failed; finished by plain BiCGStab "
                                  "(status %d, relres %.3e)" % (st.status, st.relres), RuntimeWarning)
        return x, st.as_dict()


def _precond_parts(pc):
    """(background solve or None, network or None) of a ``preconditioner=`` argument."""
    if hasattr(pc, "background") and hasattr(pc, "network"):
        return pc.background, pc.network
    if getattr(pc, "kind", None) == "background":
        return pc, None
    if not hasattr(pc, "handle"):
        raise TypeError("preconditioner must be a CNN, a BackgroundSolve or a LearnedPreconditioner")
    return None, pc


class NodalHelmholtz2D(_NodalOperator):
    """Device-resident 9-point nodal operator (the reference's ``lap2D_gather_new``).

    Operands are the reference's packed arrays (laplacian.py:517-527):
    ``hplusx, hplusy`` and the four Coriolis coefficient arrays on
    ``(ny+1)*(nx+1)`` cells, ``hcenter`` and ``diag_inv`` on ``ny*nx`` nodes,
    all flattened y-major.  NumPy or torch inputs are accepted; they are copied
    once to the GPU and packed into flux planes (FP64, FP32, double-float).
    ``y_mirror=True`` gives the operator of the reference's ``LAMB_BDRY``
    branch (laplacian.py:531-543, 749-868): x periodic, y padded by mirroring,
    no cell zeroed.
    """

    def __init__(self, hplusx, hplusy, hcenter, coriolis, diag_inv, nx, ny, dx, dy,
                 x_wall, y_wall, device=None, ws=None, y_mirror=False):
        self.dev = _device(device) if ws is None else torch.device("cuda", ws.device)
        self.nx, self.ny = int(nx), int(ny)
        self.n = self.nx * self.ny
        self.shape = (self.n, self.n)
        self.dtype = np.dtype(np.float64)
        cxx, cyy, cxy, cyx = coriolis
        d = self.dev
        self._hx = _to_dev(hplusx, d)
        self._hy = _to_dev(hplusy, d)
        self._hc = None if _all_zero(hcenter) else _to_dev(hcenter, d)
        self._cxx = _to_dev(cxx, d)
        self._cyy = _to_dev(cyy, d)
        self._cxy = None if (_all_zero(cxy) and _all_zero(cyx)) else _to_dev(cxy, d)
        self._cyx = None if self._cxy is None else _to_dev(cyx, d)
        self._dinv = _to_dev(diag_inv, d)
        nc = (self.nx + 1) * (self.ny + 1)
        for t, m, name in ((self._hx, nc, "hplusx"), (self._hy, nc, "hplusy"), (self._cxx, nc, "cxx"),
                           (self._cyy, nc, "cyy"), (self._dinv, self.n, "diag_inv")):
            if t.numel() != m:
                raise ValueError("%s has %d entries, expected %d" % (name, t.numel(), m))
        if y_mirror and x_wall:
            raise ValueError("the mirrored y boundary (LAMB_BDRY) goes with a periodic x axis")
        self.singular = self._hc is None and self._cxy is None and not y_mirror
        self.ws = _lib.Workspace(d.index) if ws is None else ws
        yb = _lib.BELLA_Y_MIRROR if y_mirror else int(bool(y_wall))
        self._op = _lib.Op2D(self.nx, self.ny, int(bool(x_wall)), yb, float(dx), float(dy),
                             _ptr(self._hx), _ptr(self._hy), _ptr(self._hc), _ptr(self._cxx),
                             _ptr(self._cyy), _ptr(self._cxy), _ptr(self._cyx), _ptr(self._dinv))
        with torch.cuda.device(d):
            _lib.check(self.ws._lib.bella_op2d_set(self.ws.handle, ctypes.byref(self._op), _stream(d)),
                       "bella_op2d_set")


class NodalHelmholtz3D(_NodalOperator):
    """Device-resident 27-point nodal operator (the arithmetic of the reference's ``lap3D``).

    Operands: ``hplusx, hplusy, hplusz`` on ``(nx+1)(ny+1)(nz+1)`` cells and
    ``hcenter``, ``diag_inv`` on ``nx*ny*nz`` inner nodes, C order over
    (x, y, z) (second_projection.py:224); ``corrf = dt*coriolis_strength[0]``
    (laplacian.py:894).  Walls per axis; other axes wrap with the duplicated seam.
    """

    def __init__(self, hplusx, hplusy, hplusz, hcenter, diag_inv, nx, ny, nz, dx, dy, dz,
                 walls=(False, True, True), corrf=0.0, device=None, ws=None):
        self.dev = _device(device) if ws is None else torch.device("cuda", ws.device)
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.n = self.nx * self.ny * self.nz
        self.shape = (self.n, self.n)
        self.dtype = np.dtype(np.float64)
        d = self.dev
        self._hx = _to_dev(hplusx, d)
        self._hy = _to_dev(hplusy, d)
        self._hz = _to_dev(hplusz, d)
        self._hc = None if _all_zero(hcenter) else _to_dev(hcenter, d)
        self._dinv = _to_dev(diag_inv, d)
        nc = (self.nx + 1) * (self.ny + 1) * (self.nz + 1)
        for t, m, name in ((self._hx, nc, "hplusx"), (self._hy, nc, "hplusy"), (self._hz, nc, "hplusz"),
                           (self._dinv, self.n, "diag_inv")):
            if t.numel() != m:
                raise ValueError("%s has %d entries, expected %d" % (name, t.numel(), m))
        self.singular = self._hc is None and float(corrf) == 0.0
        self.ws = _lib.Workspace(d.index) if ws is None else ws
        self._op = _lib.Op3D(self.nx, self.ny, self.nz, int(bool(walls[0])), int(bool(walls[1])),
                             int(bool(walls[2])), float(dx), float(dy), float(dz), float(corrf),
                             _ptr(self._hx), _ptr(self._hy), _ptr(self._hz), _ptr(self._hc), _ptr(self._dinv))
        with torch.cuda.device(d):
            _lib.check(self.ws._lib.bella_op3d_set(self.ws.handle, ctypes.byref(self._op), _stream(d)),
                       "bella_op3d_set")


class LinearOperator:
    """``scipy.sparse.linalg.LinearOperator((n, n), matvec)`` for device nodal operators.

    Mirrors the constructor the reference uses (second_projection.py:205).
    Only pybella_gb300 operators are accepted as ``matvec``.
    """

    def __init__(self, shape, matvec, rmatvec=None, matmat=None, dtype=None, rmatmat=None):
        if isinstance(matvec, LinearOperator):
            matvec = matvec.op
        if not hasattr(matvec, "solve") or not hasattr(matvec, "matvec"):
            raise TypeError("pybella_gb300.linalg.LinearOperator wraps device nodal operators "
                            "(NodalHelmholtz2D/3D); got %r" % (matvec,))
        if tuple(shape) != tuple(matvec.shape):
            raise ValueError("shape %s does not match the operator %s" % (shape, matvec.shape))
        self.op = matvec
        self.shape = tuple(shape)
        self.dtype = np.dtype(np.float64) if dtype is None else np.dtype(dtype)

    def matvec(self, x):
        return self.op.matvec(x)

    __call__ = matvec

    def __matmul__(self, x):
        return self.op.matvec(x)


def bicgstab(A, b, x0=None, tol=None, maxiter=None, M=None, callback=None, atol=None, rtol=None,
             *, precision="fp64", stats=None, inner_tol=1e-5):
    """scipy-compatible ``bicgstab`` (scipy 1.7 keyword semantics, which the reference uses).

    Returns ``(x, info)``: ``info == 0`` converged, ``> 0`` iteration count
    without convergence, ``< 0`` breakdown (-10) or non-finite residual (-12).
    ``tol`` (legacy) and ``rtol`` are the same relative tolerance; the stop
    test is ``||b - A x|| <= max(atol, tol*||b||)`` on the FP64 true residual.
    ``callback(xk)``: the reference only counts calls (solver_counter,
    second_projection.py:11-20); it is invoked once per BiCGStab iteration
    after the solve, each time with the final iterate (per-iteration
    iterates stay on the device).  ``M`` (preconditioner, 3D operators) may be
    a :class:`pybella_gb300.learned.CNN`, a
    :class:`pybella_gb300.spectral.BackgroundSolve` or a
    :class:`pybella_gb300.learned.LearnedPreconditioner`; it selects the
    flexible solver.  ``stats`` (a dict) receives iterations, outer refinement
    steps, true relative residual, status and time.
    """
    if M is not None and not (hasattr(M, "train_step") or getattr(M, "kind", None) == "background"
                              or hasattr(M, "background")):
        raise NotImplementedError("bicgstab: M must be a pybella_gb300 CNN, BackgroundSolve or "
                                  "LearnedPreconditioner (flexible BiCGStab)")
    op = A.op if isinstance(A, LinearOperator) else A
    if not hasattr(op, "solve"):
        raise TypeError("bicgstab needs a pybella_gb300 device operator, got %r" % (A,))
    if tol is None:
        tol = 1e-5 if rtol is None else rtol
    n = op.shape[0]
    if maxiter is None:
        maxiter = 10 * n
    is_torch = isinstance(b, torch.Tensor) and b.is_cuda
    x, st = op.solve(b, x0=x0, tol=tol, atol=atol or 0.0, maxiter=maxiter, precision=precision,
                     inner_tol=inner_tol, preconditioner=M)
    status = st["status"]
    if status in (_lib.BELLA_MAXITER, _lib.BELLA_TIMEOUT):
        info = max(int(st["iterations"]), 1)
    else:
        info = _INFO.get(status, -12)
    if stats is not None:
        stats.update(st)
        stats["info"] = info
        stats["fallback_used"] = bool(st["fallback"])
    xo = x if is_torch else x.cpu().numpy()
    if callback is not None:
        for _ in range(int(st["iterations"])):
            callback(xo)
    return xo, info
