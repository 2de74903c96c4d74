"""GPU BiCGStab parity: the device solve against the reference's scipy path."""
import numpy as np
import pytest

from conftest import golden, rb_background
from oracle import cases, nodal2d as n2
from oracle.krylov import bicgstab_legacy, true_relres

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _op(op):
    from pybella_gb300.linalg import NodalHelmholtz2D
    return NodalHelmholtz2D(op["hplusx"], op["hplusy"], op["hcenter"], op["cor"], op["diag_inv"],
                            op["nx"], op["ny"], op["dx"], op["dy"], op["x_wall"], op["y_wall"])


def _rb_system(tag):
    d = np.load(golden("rising_bubble_step0.npz"))
    grid, prm, hn, hc, sf = rb_background(d)
    fields = ["rho", "rhou", "rhov", "rhow", "rhoY", "rhoX"]
    Sol = {k: d["%s_in_%s" % (tag, k)].copy() for k in fields}
    Sol0 = None
    if ("%s_sol0_rho" % tag) in d:
        Sol0 = {k: d["%s_sol0_%s" % (tag, k)].copy() for k in fields}
    p2 = d[tag + "_p2_in"].copy()
    out = n2.impl_part(Sol, p2, hn["S0"], hc, sf, grid, prm, float(d[tag + "_dt"]), Sol0=Sol0)
    return out["op"], out["rhs_inner"], out["x"], prm.tol


@pytest.mark.parametrize("tag", ["full", "half"])
@pytest.mark.parametrize("precision", ["fp64", "df64", "mixed"])
def test_rising_bubble_solve_matches_reference(tag, precision):
    """Same scaled system and tol (1e-10) as the reference's scipy solve."""
    from pybella_gb300 import linalg
    op, b, x_ref, tol = _rb_system(tag)
    A = linalg.LinearOperator((b.size, b.size), _op(op))
    st = {}
    x, info = linalg.bicgstab(A, b, tol=tol, maxiter=6000, precision=precision, stats=st)
    assert info == 0, st
    assert true_relres(op, x, b) <= tol
    # the reference solution x_ref is the scipy iterate at the same tolerance;
    # both approximate the same Krylov solution in the operator's range
    assert _rel(x, x_ref) < 1e-8, (_rel(x, x_ref), st)


def test_stratified_small_mixed_vs_scipy():
    from pybella_gb300 import linalg
    w = cases.stratified_2d(seed=5, inx=257, iny=129)
    A = _op(w["op"])
    x_ref, info_ref, it_ref = bicgstab_legacy(w["op"], w["b"], 1e-10, 20000)
    x, info = linalg.bicgstab(A, w["b"], tol=1e-10, maxiter=20000, precision="mixed")
    assert info == 0 and info_ref == 0
    assert true_relres(w["op"], x, w["b"]) <= 1e-10
    assert _rel(x, x_ref) < 1e-7


def test_stratified_full_size_fp64_converges():
    """2049x1025, rtol 1e-8: true FP64 residual checked by the oracle."""
    import torch
    w = cases.stratified_2d(seed=0)
    A = _op(w["op"])
    x, st = A.solve(w["b"], tol=1e-8, maxiter=20000, precision="fp64")
    assert st["status"] == 0, st
    xn = x.cpu().numpy()
    assert true_relres(w["op"], xn, w["b"]) <= 1e-8
    assert st["relres"] <= 1e-8
    assert isinstance(x, torch.Tensor) and x.is_cuda


def test_stratified_full_size_df64_converges():
    """Double-float Krylov (FP32 pipe) reaches the FP64 true residual 1e-8."""
    w = cases.stratified_2d(seed=0)
    A = _op(w["op"])
    x, st = A.solve(w["b"], tol=1e-8, maxiter=20000, precision="df64")
    assert st["status"] == 0, st
    xn = x.cpu().numpy()
    assert true_relres(w["op"], xn, w["b"]) <= 1e-8
    x64, s64 = A.solve(w["b"], tol=1e-8, maxiter=20000, precision="fp64")
    assert s64["status"] == 0
    assert _rel(xn, x64.cpu().numpy()) < 1e-6


def test_df64_small_matches_scipy_tight():
    from pybella_gb300 import linalg
    w = cases.stratified_2d(seed=5, inx=257, iny=129)
    A = _op(w["op"])
    x_ref, info_ref, it_ref = bicgstab_legacy(w["op"], w["b"], 1e-11, 20000)
    x, info = linalg.bicgstab(A, w["b"], tol=1e-11, maxiter=20000, precision="df64")
    assert info == 0 and info_ref == 0
    assert true_relres(w["op"], x, w["b"]) <= 1e-11
    assert _rel(x, x_ref) < 1e-8


def test_stratified_full_size_mixed_never_silent():
    """The FP32 inner path either converges or hands over to FP64 -- reported."""
    w = cases.stratified_2d(seed=0)
    A = _op(w["op"])
    x, st = A.solve(w["b"], tol=1e-8, maxiter=30000, precision="mixed")
    assert st["status"] == 0, st
    assert st["fallback"] in (0, 1)
    xn = x.cpu().numpy()
    assert true_relres(w["op"], xn, w["b"]) <= 1e-8
    if not st["fallback"]:
        # x has no component along the null modes (left null vectors z_k = D w e_k)
        wts = cases.null_weights_2d(w["grid"]).T.reshape(-1) / w["op"]["diag_inv"]
        for e in cases.null_modes_2d(w["grid"]):
            z = wts * e.T.reshape(-1)
            assert abs(np.dot(z, xn)) < 1e-9 * np.abs(z * xn).sum()


def test_fp64_and_mixed_agree_full_size():
    w = cases.stratified_2d(seed=7)
    A = _op(w["op"])
    x64, s64 = A.solve(w["b"], tol=1e-9, maxiter=30000, precision="fp64")
    xm, sm = A.solve(w["b"], tol=1e-9, maxiter=30000, precision="mixed")
    assert s64["status"] == 0 and sm["status"] == 0
    assert _rel(xm.cpu().numpy(), x64.cpu().numpy()) < 1e-6


def test_status_codes_are_reported():
    from pybella_gb300 import linalg
    w = cases.stratified_2d(seed=9, inx=129, iny=65)
    A = _op(w["op"])
    # iteration limit -> info > 0, never silent
    _, info = linalg.bicgstab(A, w["b"], tol=1e-12, maxiter=3, precision="fp64")
    assert info > 0
    _, info = linalg.bicgstab(A, w["b"], tol=1e-12, maxiter=3, precision="mixed")
    assert info > 0
    # zero rhs -> x = 0, converged
    x, info = linalg.bicgstab(A, np.zeros_like(w["b"]), tol=1e-8, precision="mixed")
    assert info == 0 and not np.any(x)
    # non-finite rhs -> non-finite status
    b = w["b"].copy()
    b[10] = np.nan
    _, info = linalg.bicgstab(A, b, tol=1e-8, maxiter=50, precision="fp64")
    assert info == -12
    _, info = linalg.bicgstab(A, b, tol=1e-8, maxiter=50, precision="mixed")
    assert info == -12
    _, info = linalg.bicgstab(A, b, tol=1e-8, maxiter=50, precision="df64")
    assert info == -12
    _, info = linalg.bicgstab(A, w["b"], tol=1e-12, maxiter=3, precision="df64")
    assert info > 0


def test_callback_counts_iterations():
    from pybella_gb300 import linalg
    w = cases.stratified_2d(seed=11, inx=129, iny=65)
    A = _op(w["op"])
    cnt = [0]
    st = {}
    linalg.bicgstab(A, w["b"], tol=1e-8, maxiter=5000, precision="fp64",
                    callback=lambda xk: cnt.__setitem__(0, cnt[0] + 1), stats=st)
    assert cnt[0] == st["iterations"] > 0
