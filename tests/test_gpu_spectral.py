"""Background (spectral) solve of the 3D operator on the GPU against the oracle's
FP64 restatement (oracle/spectral3d.py), and the solves it preconditions, checked
by the FP64 true residual and compared with the plain FP64 solve."""
import warnings

import numpy as np
import pytest

from oracle import cases, nodal2d as n2, nodal3d as n3, spectral3d
from oracle.krylov import true_relres

pytestmark = pytest.mark.gpu


def _dev_op(op):
    from pybella_gb300.linalg import NodalHelmholtz3D
    return NodalHelmholtz3D(op["hplusx"], op["hplusy"], op["hplusz"], op["hcenter"], op["diag_inv"],
                            op["nx"], op["ny"], op["nz"], op["dx"], op["dy"], op["dz"],
                            walls=op["walls"], corrf=op["corrf"])


def _seam_consistent(x, shape, walls):
    X = x.reshape(shape).copy()
    for ax, wall in enumerate(walls):
        if not wall:
            lo, hi = [slice(None)] * 3, [slice(None)] * 3
            lo[ax], hi[ax] = 0, -1
            X[tuple(hi)] = X[tuple(lo)]
    return X.reshape(-1)


def _cell_gradients(x, op):
    """The four-edge difference sums of lap3D (laplacian.py:968-985) on every cell
    between walls: the pressure gradient the correction uses, blind to the
    operator's null space."""
    U = n3._pad(np.asarray(x, np.float64).reshape(op["nx"], op["ny"], op["nz"]))
    gx = U[1:] - U[:-1]
    gy = U[:, 1:] - U[:, :-1]
    gz = U[:, :, 1:] - U[:, :, :-1]
    cells = [gx[:, :-1, :-1] + gx[:, :-1, 1:] + gx[:, 1:, :-1] + gx[:, 1:, 1:],
             gy[:-1, :, :-1] + gy[1:, :, :-1] + gy[:-1, :, 1:] + gy[1:, :, 1:],
             gz[:-1, :-1] + gz[:-1, 1:] + gz[1:, :-1] + gz[1:, 1:]]
    inner = tuple(slice(1, -1) if wall else slice(None) for wall in op["walls"])
    return np.concatenate([c[inner].ravel() for c in cells])


@pytest.mark.parametrize("shape,walls,sigma", [
    ((17, 9, 13), (False, True, True), 0.1),
    ((17, 9, 13), (True, True, True), 0.1),
    ((17, 9, 17), (False, True, False), 0.3),
    ((33, 17, 29), (True, True, False), 0.1),
    ((65, 33, 65), (False, True, True), 0.1),
])
def test_background_apply_vs_oracle(shape, walls, sigma):
    import torch
    from pybella_gb300.spectral import BackgroundSolve
    w = cases.stratified_3d(2, *shape, sigma=sigma, walls=walls)
    op = w["op"]
    ref = spectral3d.BackgroundInverse(op)
    bg = BackgroundSolve(_dev_op(op))
    rng = np.random.default_rng(3)
    for r in (w["b"], _seam_consistent(rng.standard_normal(op["nx"] * op["ny"] * op["nz"]), shape, walls)):
        r32 = r.astype(np.float32).astype(np.float64)
        y_ref = ref.apply(r32)
        y = bg.apply(torch.tensor(r32, device="cuda")).double().cpu().numpy()
        assert np.all(np.isfinite(y))
        # FP32 output: the background inverse amplifies the near-null modes by up to
        # 1/lambda_min, and storing those large components in FP32 alone costs
        # `floor` through the operator; the device result stays within a small
        # multiple of that representation floor
        floor = np.linalg.norm(n3.lap3d(y_ref.astype(np.float32).astype(np.float64) - y_ref, op))
        err_a = np.linalg.norm(n3.lap3d(y - y_ref, op))
        assert err_a <= 20.0 * floor + 1e-6 * np.linalg.norm(r32), (err_a, floor)
        err = np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref)
        assert err <= 2e-3, err


@pytest.mark.parametrize("walls", [(False, True, True), (True, True, False)])
def test_background_apply_is_exact_without_lognormal_factor(walls):
    import torch
    from pybella_gb300.spectral import BackgroundSolve
    shape = (33, 17, 33)
    w = cases.stratified_3d(4, *shape, sigma=0.0, walls=walls)
    op = w["op"]
    bg = BackgroundSolve(_dev_op(op))
    x = _seam_consistent(np.random.default_rng(5).standard_normal(int(np.prod(shape))), shape, walls)
    r = n3.lap3d(x, op)
    y = bg.apply(torch.tensor(r, device="cuda")).double().cpu().numpy()
    res = np.linalg.norm(n3.lap3d(y, op) - r) / np.linalg.norm(r)
    assert res <= 2e-5, res


def test_background_apply_with_hcenter_matches_oracle():
    import torch
    from pybella_gb300.spectral import BackgroundSolve
    rng = np.random.default_rng(11)
    nx, ny, nz = 21, 11, 19
    walls = (False, True, True)
    shp = (nx + 1, ny + 1, nz + 1)
    hx, hy, hz = (rng.uniform(0.5, 2.0, shp) for _ in range(3))
    for h in (hx, hy, hz):              # periodic x: duplicated seam cells
        h[0], h[-1] = h[-2], h[1]
    hc = -rng.uniform(0.1, 1.0, (nx, ny, nz))
    dinv = n3.precon_diag_3d(hx, hy, hz, hc, 0.2, 0.3, 0.25)
    op = n3.pack_27pt(hx, hy, hz, hc, dinv, nx, ny, nz, 0.2, 0.3, 0.25, walls=walls)
    ref = spectral3d.BackgroundInverse(op)
    bg = BackgroundSolve(_dev_op(op))
    r = _seam_consistent(rng.standard_normal(nx * ny * nz), (nx, ny, nz), walls).astype(np.float32)
    y = bg.apply(torch.tensor(r, device="cuda")).double().cpu().numpy()
    y_ref = ref.apply(r.astype(np.float64))
    assert np.linalg.norm(y - y_ref) <= 1e-4 * np.linalg.norm(y_ref)


def test_background_preconditioned_solve_converges_in_few_iterations(capsys):
    import torch
    from pybella_gb300 import workloads, learned
    from pybella_gb300.spectral import BackgroundSolve
    shape = (65, 33, 65)
    w = workloads.stratified_3d(1, *shape)
    A = learned.operator_3d(w)
    bg = BackgroundSolve(A)
    xp, sp = A.solve(w["b"], tol=1e-8, maxiter=50000, precision="fp64")
    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        xb, sb = A.solve(w["b"], tol=1e-8, maxiter=2000, preconditioner=bg)
    assert not rec and sb["fallback"] == 0 and sb["status"] == 0, sb
    assert sb["iterations"] <= 20, sb
    assert sb["relres"] <= 1e-8
    r = w["b"] - A.matvec(xb)
    assert float(torch.linalg.norm(r) / torch.linalg.norm(w["b"])) <= 1e-8
    # against the FP64 solve: the cell gradients (the solution modulo the null space)
    op = {k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in w.items()}
    gp = _cell_gradients(xp.cpu().numpy(), op)
    gb = _cell_gradients(xb.cpu().numpy(), op)
    err = np.linalg.norm(gb - gp) / np.linalg.norm(gp)
    assert err <= 1e-6, err
    with capsys.disabled():
        print("\nbackground-preconditioned %s: %d inner iterations, %d outer, %.3f s; FP64 plain %d iterations "
              "%.3f s; gradient error vs FP64 %.2e" % ("x".join(map(str, shape)), sb["iterations"], sb["outer"],
                                                      sb["seconds"], sp["iterations"], sp["seconds"], err))


def test_learned_preconditioner_runs_the_correction_and_scipy_signature():
    import torch
    from pybella_gb300 import learned, linalg, workloads
    from pybella_gb300.spectral import BackgroundSolve
    shape = (41, 21, 41)
    w = workloads.stratified_3d(3, *shape)
    A = learned.operator_3d(w)
    bg = BackgroundSolve(A)
    net = learned.CNN(shape, block=2, mode="linear", skip=0.5)
    net.init(0, last_gain=0.01)
    lp = learned.LearnedPreconditioner(bg, net)
    l0 = net.launches
    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        x, st = A.solve(w["b"], tol=1e-8, maxiter=2000, preconditioner=lp)
    assert st["status"] == 0 and st["fallback"] == 0 and not rec, st
    assert net.launches > l0                    # the network ran inside the solve
    r = w["b"] - A.matvec(x)
    assert float(torch.linalg.norm(r) / torch.linalg.norm(w["b"])) <= 1e-8
    stats = {}
    xs, info = linalg.bicgstab(linalg.LinearOperator(A.shape, A), w["b"], rtol=1e-8, maxiter=2000, M=bg,
                               stats=stats)
    assert info == 0 and stats["fallback"] == 0


@pytest.mark.parametrize("order", ["post", "pre", "sym"])
def test_fgmres_with_every_preconditioner_kind(order):
    """Flexible GMRES with the background solve and the three compositions with a
    network: every solve meets rtol 1e-8 on the FP64 true residual without
    falling back."""
    import torch
    from pybella_gb300 import learned, workloads
    from pybella_gb300.spectral import BackgroundSolve
    shape = (41, 21, 41)
    w = workloads.stratified_3d(5, *shape)
    A = learned.operator_3d(w)
    bg = BackgroundSolve(A)
    net = learned.CNN(shape, block=2, mode="linear", skip=0.5)
    net.init(1, last_gain=0.05)
    pcs = [learned.LearnedPreconditioner(bg, net, order)]
    if order == "post":
        pcs.append(bg)
    for pc in pcs:
        with warnings.catch_warnings(record=True) as rec:
            warnings.simplefilter("always")
            x, st = A.solve(w["b"], tol=1e-8, maxiter=4000, preconditioner=pc, method="fgmres", restart=30)
        assert st["status"] == 0 and st["fallback"] == 0 and not rec, (order, st)
        r = w["b"] - A.matvec(x)
        assert float(torch.linalg.norm(r) / torch.linalg.norm(w["b"])) <= 1e-8


def test_trained_correction_of_the_background_solve(capsys):
    """Train the network on the pairs the background solve leaves (from the
    background-preconditioned solver's own iterates), then solve with and
    without it: the learned solve meets the tolerance on the FP64 true residual,
    never falls back silently, and takes no more flexible-GMRES iterations than
    the same method with the background solve alone; iterations and times of
    both (and of background BiCGStab) are printed -- in time the network's
    application costs more than the iterations it saves."""
    import torch
    from pybella_gb300 import learned, workloads
    from pybella_gb300.spectral import BackgroundSolve
    params, losses = learned.train_preconditioner(shape=(65, 33, 65), seeds=(1, 2), npairs=512, crop=32,
                                                  steps=200, batch=16, background=True, skip=0.7)
    assert np.isfinite(losses[-1][1]) and losses[-1][1] < losses[0][1]
    shape = (65, 33, 65)
    w = workloads.stratified_3d(9, *shape)
    A = learned.operator_3d(w)
    bg = BackgroundSolve(A)
    net = learned.CNN(shape, block=2, mode="linear", skip=0.7)
    net.set_params(params)
    xb, sb = A.solve(w["b"], tol=1e-8, maxiter=4000, preconditioner=bg)
    xf, sf = A.solve(w["b"], tol=1e-8, maxiter=4000, preconditioner=bg, method="fgmres", restart=30)
    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        xl, sl = A.solve(w["b"], tol=1e-8, maxiter=4000, preconditioner=learned.LearnedPreconditioner(bg, net),
                         method="fgmres", restart=30)
    for x, st in ((xb, sb), (xf, sf), (xl, sl)):
        assert st["status"] == 0, st
        r = w["b"] - A.matvec(x)
        assert float(torch.linalg.norm(r) / torch.linalg.norm(w["b"])) <= 1e-8
    assert bool(sl["fallback"]) == any("preconditioned solve failed" in str(m.message) for m in rec)
    assert sl["fallback"] == 0 and sl["iterations"] <= sf["iterations"], (sl, sf)
    with capsys.disabled():
        print("\ntrained correction (%s): background alone: BiCGStab %d iterations %.4f s, FGMRES %d iterations "
              "%.4f s; background + network (FGMRES) %d iterations %.4f s (fallback %d); training loss %.3f -> %.3f"
              % ("x".join(map(str, shape)), sb["iterations"], sb["seconds"], sf["iterations"], sf["seconds"],
                 sl["iterations"], sl["seconds"], sl["fallback"], losses[0][1], losses[-1][1]))


# ---------------------------------------------------------------------------
# the background solve of the 2D 9-point operator
# ---------------------------------------------------------------------------
def test_background_update_equals_a_fresh_set_up():
    """bella_spectral3d_update / bella_spectral2d_update: a background solve made
    for one operator and re-derived in place from another of the same shape (with
    and without an hcenter term) applies exactly as one made for the second;
    another shape, boundary kind or dimension is refused."""
    import torch
    from pybella_gb300 import _lib
    from pybella_gb300.spectral import BackgroundSolve
    rng = np.random.default_rng(5)
    shape, walls = (33, 17, 29), (False, True, True)
    a = cases.stratified_3d(1, *shape, walls=walls)["op"]
    b = cases.stratified_3d(2, *shape, walls=walls)["op"]
    r = torch.tensor(_seam_consistent(rng.standard_normal(int(np.prod(shape))), shape, walls),
                     dtype=torch.float32, device="cuda")
    for hc in (False, True):
        if hc:
            b = dict(b, hcenter=-rng.uniform(0.1, 1.0, shape).reshape(-1))
        A, B = _dev_op(a), _dev_op(b)
        bg = BackgroundSolve(A)
        fresh = BackgroundSolve(B)
        y_up = bg.update(B).apply(r).clone()
        y_new = fresh.apply(r)
        assert torch.equal(y_up, y_new), float((y_up - y_new).abs().max())
    other = _dev_op(cases.stratified_3d(1, 33, 17, 33, walls=walls)["op"])
    with pytest.raises(_lib.BellaError):
        bg.update(other)
    w2 = [cases.stratified_2d(s, 65, 33)["op"] for s in (3, 4)]
    bg2 = BackgroundSolve(_op2d(w2[0]))
    y_up = bg2.update(_op2d(w2[1])).apply(r[: 65 * 33]).clone()
    assert torch.equal(y_up, BackgroundSolve(_op2d(w2[1])).apply(r[: 65 * 33]))
    with pytest.raises(_lib.BellaError):
        bg2.update(A)
    with pytest.raises(_lib.BellaError):
        bg.update(_op2d(w2[0]))


def _op2d(op):
    from pybella_gb300.linalg import NodalHelmholtz2D
    return NodalHelmholtz2D(op["hplusx"], op["hplusy"], op["hcenter"], op["cor"], op["diag_inv"],
                            op["nx"], op["ny"], op["dx"], op["dy"], op["x_wall"], op["y_wall"])


@pytest.mark.parametrize("nx,ny", [(65, 33), (161, 81), (2049, 17)])
def test_background2d_apply_vs_oracle(nx, ny):
    """x transforms by FFT (64, 2048 points) and by GEMM (160): the device apply
    against the oracle, measured through the operator against the FP32 floor."""
    import torch
    from oracle import spectral2d
    from pybella_gb300.spectral import BackgroundSolve
    w = cases.stratified_2d(3, nx, ny)
    op = w["op"]
    ref = spectral2d.BackgroundInverse2D(op)
    bg = BackgroundSolve(_op2d(op))
    rng = np.random.default_rng(6)
    X = rng.standard_normal((ny, nx))
    X[:, -1] = X[:, 0]
    for r in (w["b"], n2.lap2d_gather(X.reshape(-1), op)):
        r32 = r.astype(np.float32).astype(np.float64)
        y_ref = ref.apply(r32)
        y = bg.apply(torch.tensor(r32, device="cuda")).double().cpu().numpy()
        floor = np.linalg.norm(n2.lap2d_gather(y_ref.astype(np.float32).astype(np.float64) - y_ref, op))
        err_a = np.linalg.norm(n2.lap2d_gather(y - y_ref, op))
        assert err_a <= 20.0 * floor + 1e-6 * np.linalg.norm(r32), (err_a, floor)


@pytest.mark.parametrize("tag", ["full", "half"])
def test_background2d_rising_bubble_matches_reference(tag):
    """The reference's rising-bubble systems (tol 1e-10): the background-preconditioned
    solve meets the tolerance on the FP64 true residual and matches the reference's
    scipy solution as the plain solve does."""
    from test_gpu_solver import _rb_system
    from pybella_gb300 import linalg
    from pybella_gb300.spectral import BackgroundSolve
    op, b, x_ref, tol = _rb_system(tag)
    A = _op2d(op)
    st = {}
    x, info = linalg.bicgstab(linalg.LinearOperator(A.shape, A), b, tol=tol, maxiter=6000, M=BackgroundSolve(A),
                              stats=st)
    assert info == 0 and st["fallback"] == 0, st
    assert true_relres(op, x, b) <= tol
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-8
    assert st["iterations"] < 60, st


def test_background2d_full_size_solve(capsys):
    import torch
    from pybella_gb300 import linalg
    from pybella_gb300.spectral import BackgroundSolve
    w = cases.stratified_2d(seed=3, inx=2049, iny=1025)
    A = _op2d(w["op"])
    xp, sp = A.solve(w["b"], tol=1e-8, maxiter=30000, precision="df64")
    bg = BackgroundSolve(A)
    xb, sb = A.solve(w["b"], tol=1e-8, maxiter=2000, preconditioner=bg)
    assert sb["status"] == 0 and sb["fallback"] == 0 and sb["relres"] <= 1e-8, sb
    r = torch.tensor(w["b"], device="cuda") - A.matvec(xb)
    assert float(torch.linalg.norm(r) / np.linalg.norm(w["b"])) <= 1e-8
    err = float(torch.linalg.norm(xb - xp) / torch.linalg.norm(xp))
    assert err < 1e-6, err
    with capsys.disabled():
        print("\n2D 2049x1025: background-preconditioned %d iterations (%d outer) %.4f s; plain double-float %d "
              "iterations %.4f s; difference %.2e" % (sb["iterations"], sb["outer"], sb["seconds"], sp["iterations"],
                                                      sp["seconds"], err))
