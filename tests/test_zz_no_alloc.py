"""GPU test of the allocation-free entry point ``bella_bicgstab2d_noalloc``.

It serves callers that cannot allocate device memory while they run (a host
model that owns the GPU through its own memory pool, or a time loop that
cannot take the stall of a cudaMalloc).  The test calls it through the C ABI
on the rising-bubble projection system (161x81 nodes, tol 1e-10, the
reference's own case) and checks its solution against the workspace entry
point ``bella_bicgstab`` (FP64) on two calls in a row, since every call
reuses the same fixed scratch array.  This file is named to be collected
last.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden, rb_background
from oracle import cases, nodal2d as n2
from oracle.krylov import true_relres

pytestmark = pytest.mark.gpu


def _system():
    d = np.load(golden("rising_bubble_step0.npz"))
    grid, prm, hn, hc, sf = rb_background(d)
    fields = ["rho", "rhou", "rhov", "rhow", "rhoY", "rhoX"]
    Sol = {k: d["full_in_" + k].copy() for k in fields}
    p2 = d["full_p2_in"].copy()
    out = n2.impl_part(Sol, p2, hn["S0"], hc, sf, grid, prm, float(d["full_dt"]))
    return out["op"], out["rhs_inner"], prm.tol


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def test_noalloc_matches_workspace_solver_twice():
    import torch
    from pybella_gb300 import _lib
    from pybella_gb300.linalg import NodalHelmholtz2D
    lib = _lib.load()
    op, b, tol = _system()
    # existing entry point (workspace, FP64)
    A = NodalHelmholtz2D(op["hplusx"], op["hplusy"], op["hcenter"], op["cor"], op["diag_inv"],
                         op["nx"], op["ny"], op["dx"], op["dy"], op["x_wall"], op["y_wall"])
    x_ref, st_ref = A.solve(b, tol=tol, maxiter=6000, precision="fp64")
    assert st_ref["status"] == 0
    x_ref = x_ref.cpu().numpy()
    # allocation-free entry point on the same reference-packed operands
    keep = [_dev(op["hplusx"]), _dev(op["hplusy"]), _dev(op["cor"][0]), _dev(op["cor"][1]),
            _dev(op["diag_inv"])]
    hc = None if not np.any(op["hcenter"]) else _dev(op["hcenter"])
    cxy = None if not (np.any(op["cor"][2]) or np.any(op["cor"][3])) else _dev(op["cor"][2])
    cyx = None if cxy is None else _dev(op["cor"][3])
    o2 = _lib.Op2D(op["nx"], op["ny"], int(op["x_wall"]), int(op["y_wall"]), op["dx"], op["dy"],
                   _ptr(keep[0]), _ptr(keep[1]), _ptr(hc), _ptr(keep[2]), _ptr(keep[3]), _ptr(cxy),
                   _ptr(cyx), _ptr(keep[4]))
    opts = _lib.SolveOpts()
    lib.bella_solve_opts_default(ctypes.byref(opts))
    opts.tol = tol
    opts.maxiter = 6000
    opts.precision = 0
    opts.x0_zero = 1
    bd = _dev(b)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        x = torch.full_like(bd, float("nan"))        # output only: stale contents must not matter
        st = _lib.SolveStats()
        rc = lib.bella_bicgstab2d_noalloc(ctypes.byref(o2), _ptr(bd), _ptr(x), ctypes.byref(opts),
                                          ctypes.byref(st), stream)
        assert rc == 0, (call, rc, lib.bella_last_error())
        torch.cuda.synchronize()
        xn = x.cpu().numpy()
        assert st.iterations == st_ref["iterations"], (call, st.iterations, st_ref["iterations"])
        # same kernels and order of operations as the workspace path
        np.testing.assert_allclose(xn, x_ref, rtol=1e-12, atol=1e-12 * np.abs(x_ref).max())
        assert true_relres(op, xn, b) <= tol


def test_noalloc_rejects_oversized_grid():
    import torch
    from pybella_gb300 import _lib
    lib = _lib.load()
    nx, ny = 513, 257                              # 131841 nodes > 65536
    z = torch.zeros((nx + 1) * (ny + 1), dtype=torch.float64, device="cuda")
    zn = torch.zeros(nx * ny, dtype=torch.float64, device="cuda")
    o2 = _lib.Op2D(nx, ny, 0, 1, 0.01, 0.01, _ptr(z), _ptr(z), _ptr(None), _ptr(z), _ptr(z), _ptr(None),
                   _ptr(None), _ptr(zn))
    st = _lib.SolveStats()
    rc = lib.bella_bicgstab2d_noalloc(ctypes.byref(o2), _ptr(zn), _ptr(zn), None, ctypes.byref(st),
                                      ctypes.c_void_p(0))
    assert rc == _lib.BELLA_EINVAL
    assert b"too large" in lib.bella_last_error()


def test_noalloc_null_opts_takes_the_defaults():
    """opts == NULL: the shared defaults (tol 1e-8, 6000 iterations) in this entry
    point's one precision, FP64; the result meets the default tolerance."""
    import torch
    from pybella_gb300 import _lib
    lib = _lib.load()
    op, b, _ = _system()
    keep = [_dev(op["hplusx"]), _dev(op["hplusy"]), _dev(op["cor"][0]), _dev(op["cor"][1]), _dev(op["diag_inv"])]
    o2 = _lib.Op2D(op["nx"], op["ny"], int(op["x_wall"]), int(op["y_wall"]), op["dx"], op["dy"],
                   _ptr(keep[0]), _ptr(keep[1]), _ptr(None), _ptr(keep[2]), _ptr(keep[3]), _ptr(None),
                   _ptr(None), _ptr(keep[4]))
    bd = _dev(b)
    x = torch.zeros_like(bd)
    st = _lib.SolveStats()
    rc = lib.bella_bicgstab2d_noalloc(ctypes.byref(o2), _ptr(bd), _ptr(x), None, ctypes.byref(st),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, (rc, lib.bella_last_error())
    torch.cuda.synchronize()
    assert st.status == 0 and true_relres(op, x.cpu().numpy(), b) <= 1e-8
