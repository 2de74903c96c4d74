"""Self-consistency of the 3D 27-point oracle and of the background inverses.

The operator itself is pinned against the reference's ``lap3D`` outputs in
tests/test_oracle_golden.py; these tests add its relation to the 2D operator
and structural properties (null modes, symmetry).
"""
import numpy as np
import pytest

from oracle import nodal2d as n2
from oracle import nodal3d as n3


def _rand_cells(rng, shape):
    return rng.uniform(0.5, 2.0, shape)


def test_z_invariant_field_reproduces_2d_operator():
    rng = np.random.default_rng(0)
    nx, ny, nz = 9, 7, 5
    dx, dy, dz = 0.3, 0.2, 0.25
    hx2 = _rand_cells(rng, (ny + 1, nx + 1))
    hy2 = _rand_cells(rng, (ny + 1, nx + 1))
    op2 = dict(hplusx=hx2.reshape(-1), hplusy=hy2.reshape(-1), hcenter=np.zeros(nx * ny),
               cor=(np.ones(hx2.size), np.ones(hx2.size), np.zeros(hx2.size), np.zeros(hx2.size)),
               diag_inv=np.ones(nx * ny), nx=nx, ny=ny, dx=dx, dy=dy, x_wall=False, y_wall=True)
    hx3 = np.repeat(hx2.T[:, :, None], nz + 1, axis=2)
    hy3 = np.repeat(hy2.T[:, :, None], nz + 1, axis=2)
    hz3 = _rand_cells(rng, (nx + 1, ny + 1, 1)).repeat(nz + 1, axis=2)
    op3 = n3.pack_27pt(hx3, hy3, hz3, np.zeros(nx * ny * nz), np.ones(nx * ny * nz), nx, ny, nz, dx, dy, dz,
                       walls=(False, True, False), corrf=0.3)
    p2 = rng.standard_normal((ny, nx))
    p3 = np.repeat(p2.T[:, :, None], nz, axis=2)
    y2 = n2.lap2d_gather(p2.reshape(-1), op2).reshape(ny, nx)
    y3 = n3.lap3d(p3.reshape(-1), op3).reshape(nx, ny, nz)
    for k in range(nz):
        np.testing.assert_allclose(y3[:, :, k], y2.T, rtol=1e-12, atol=1e-12 * np.abs(y2).max())


def _op3(rng, nx, ny, nz, walls, corrf=0.0, hc=False):
    shp = (nx + 1, ny + 1, nz + 1)
    hx, hy, hz = (_rand_cells(rng, shp) for _ in range(3))
    for h in (hx, hy, hz):            # periodic copies of the ghost-like cells
        for ax, w in enumerate(walls):
            if not w:
                n = shp[ax] - 1
                sl = [slice(None)] * 3
                src = [slice(None)] * 3
                sl[ax], src[ax] = 0, n - 1
                h[tuple(sl)] = h[tuple(src)]
                sl[ax], src[ax] = n, 1
                h[tuple(sl)] = h[tuple(src)]
    hcen = -rng.uniform(0.1, 1.0, nx * ny * nz) if hc else np.zeros(nx * ny * nz)
    dinv = n3.precon_diag_3d(hx, hy, hz, hcen.reshape(nx, ny, nz), 0.2, 0.3, 0.25)
    return n3.pack_27pt(hx, hy, hz, hcen, dinv, nx, ny, nz, 0.2, 0.3, 0.25, walls=walls, corrf=corrf)


def test_null_modes_of_pseudo_incompressible_3d():
    rng = np.random.default_rng(1)
    nx, ny, nz = 9, 6, 7
    op = _op3(rng, nx, ny, nz, (False, True, True))
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    for e in (np.ones((nx, ny, nz)), (-1.0) ** (i + j), (-1.0) ** (i + k), (-1.0) ** (j + k),
              (-1.0) ** (i + j + k)):
        assert np.abs(n3.lap3d(e.reshape(-1), op)).max() < 1e-12
    assert np.abs(n3.lap3d(((-1.0) ** i).reshape(-1), op)).max() > 1.0


def test_unscaled_operator_is_weighted_symmetric_on_seam_consistent_vectors():
    rng = np.random.default_rng(2)
    nx, ny, nz = 9, 6, 7
    op = _op3(rng, nx, ny, nz, (False, True, True))
    op["diag_inv"] = np.ones(nx * ny * nz)
    w = np.ones((nx, ny, nz))
    w[0] = w[-1] = 0.5
    u = rng.standard_normal((nx, ny, nz))
    v = rng.standard_normal((nx, ny, nz))
    u[-1] = u[0]
    v[-1] = v[0]
    Au = n3.lap3d(u.reshape(-1), op).reshape(u.shape)
    Av = n3.lap3d(v.reshape(-1), op).reshape(v.shape)
    a, b = np.sum(w * v * Au), np.sum(w * u * Av)
    assert abs(a - b) < 1e-11 * (abs(a) + abs(b))


def _seam_consistent(x, shape, walls):
    X = x.reshape(shape).copy()
    for ax, wall in enumerate(walls):
        if not wall:
            lo, hi = [slice(None)] * 3, [slice(None)] * 3
            lo[ax], hi[ax] = 0, -1
            X[tuple(hi)] = X[tuple(lo)]
    return X.reshape(-1)


@pytest.mark.parametrize("walls", [(False, True, True), (True, True, True), (False, True, False),
                                   (True, True, False)])
def test_background_inverse_is_exact_on_horizontally_uniform_coefficients(walls):
    """Coefficients equal to their horizontal means: A (A_bg^+ r) = r for r in the range of A."""
    from oracle import cases, spectral3d
    shape = (17, 9, 13)
    w = cases.stratified_3d(3, *shape, sigma=0.0, walls=walls)
    op = w["op"]
    B = spectral3d.BackgroundInverse(op)
    rng = np.random.default_rng(7)
    x = _seam_consistent(rng.standard_normal(int(np.prod(shape))), shape, walls)
    r = n3.lap3d(x, op)
    assert np.linalg.norm(n3.lap3d(B.apply(r), op) - r) <= 1e-12 * np.linalg.norm(r)


def test_background_inverse_with_uniform_hcenter_on_periodic_axes():
    from oracle import spectral3d
    rng = np.random.default_rng(8)
    nx, ny, nz = 13, 9, 11
    walls = (False, True, False)
    prof = rng.uniform(0.5, 2.0, ny + 1)
    h = np.broadcast_to(prof[None, :, None], (nx + 1, ny + 1, nz + 1)).copy()
    hc = np.broadcast_to(-rng.uniform(0.1, 1.0, ny)[None, :, None], (nx, ny, nz)).copy()
    dinv = n3.precon_diag_3d(h, h, h, hc, 0.2, 0.3, 0.25)
    op = n3.pack_27pt(h, h, h, hc, dinv, nx, ny, nz, 0.2, 0.3, 0.25, walls=walls)
    B = spectral3d.BackgroundInverse(op)
    r = _seam_consistent(rng.standard_normal(nx * ny * nz), (nx, ny, nz), walls)
    assert np.linalg.norm(n3.lap3d(B.apply(r), op) - r) <= 1e-11 * np.linalg.norm(r)


def test_background_inverse_preconditions_lognormal_coefficients():
    """sigma = 0.1 log-normal cells: flexible BiCGStab right-preconditioned by the
    background inverse converges in a handful of iterations where the plain
    method needs hundreds (FP64 restatement, small grid)."""
    from oracle import cases, spectral3d
    from oracle.krylov import bicgstab_legacy
    w = cases.stratified_3d(1, 17, 9, 17)
    op = w["op"]
    b = w["b"]
    B = spectral3d.BackgroundInverse(op)
    A = lambda p: n3.lap3d(p, op)
    x, r, rho, al, om = np.zeros_like(b), b.copy(), 1.0, 1.0, 1.0
    rh, v, p = b.copy(), np.zeros_like(b), np.zeros_like(b)
    it = 0
    while np.linalg.norm(r) > 1e-8 * np.linalg.norm(b) and it < 50:
        it += 1
        rn = rh @ r
        p = r + (rn / rho) * (al / om) * (p - om * v)
        rho = rn
        ph = B.apply(p)
        v = A(ph)
        al = rho / (rh @ v)
        s = r - al * v
        sh = B.apply(s)
        t = A(sh)
        om = (t @ s) / (t @ t)
        x = x + al * ph + om * sh
        r = s - om * t
    assert it <= 8, it
    assert np.linalg.norm(b - A(x)) <= 1e-8 * np.linalg.norm(b) * 1.01
    _, info, it_plain = bicgstab_legacy(A, b, 1e-8, 5000)
    assert info == 0 and it_plain > 10 * it


def test_background2d_inverse_is_exact_without_cross_terms_periodic_x():
    """2D 9-point operator with horizontally uniform coefficients (sigma = 0) and no
    Coriolis cross terms: A (A_bg^+ r) = r for r in the range of A."""
    from oracle import cases, spectral2d
    w = cases.stratified_2d(1, 33, 17, sigma=0.0)
    op = dict(w["op"])
    op["cor"] = (op["cor"][0], op["cor"][1], np.zeros_like(op["cor"][2]), np.zeros_like(op["cor"][3]))
    B = spectral2d.BackgroundInverse2D(op)
    X = np.random.default_rng(0).standard_normal((17, 33))
    X[:, -1] = X[:, 0]                          # duplicated periodic seam
    r = n2.lap2d_gather(X.reshape(-1), op)
    assert np.linalg.norm(n2.lap2d_gather(B.apply(r), op) - r) <= 1e-12 * np.linalg.norm(r)


def _uniform_op2d(rng, nx, ny, x_wall, with_hc):
    prof_x, prof_y = rng.uniform(0.5, 2.0, ny + 1), rng.uniform(0.5, 2.0, ny + 1)
    hx = np.broadcast_to(prof_x[:, None], (ny + 1, nx + 1)).reshape(-1).copy()
    hy = np.broadcast_to(prof_y[:, None], (ny + 1, nx + 1)).reshape(-1).copy()
    hc = (np.broadcast_to(-rng.uniform(0.1, 1.0, ny)[:, None], (ny, nx)).reshape(-1).copy() if with_hc
          else np.zeros(nx * ny))
    nc = (nx + 1) * (ny + 1)
    return dict(hplusx=hx, hplusy=hy, hcenter=hc, cor=(np.ones(nc), np.full(nc, 0.7), np.zeros(nc), np.zeros(nc)),
                diag_inv=-rng.uniform(0.5, 1.5, nx * ny), nx=nx, ny=ny, dx=0.3, dy=0.2, x_wall=x_wall,
                y_wall=True)


@pytest.mark.parametrize("x_wall,with_hc", [(True, False), (False, True)])
def test_background2d_inverse_exact_walls_and_hcenter(x_wall, with_hc):
    """Walls in x (DCT-I with trapezoid weights, exact without hcenter) and a
    periodic x with a row-uniform hcenter (exact): A (A_bg^+ r) = r on the range."""
    from oracle import spectral2d
    rng = np.random.default_rng(4)
    nx, ny = 19, 11
    op = _uniform_op2d(rng, nx, ny, x_wall, with_hc)
    B = spectral2d.BackgroundInverse2D(op)
    X = rng.standard_normal((ny, nx))
    if not x_wall:
        X[:, -1] = X[:, 0]
    r = n2.lap2d_gather(X.reshape(-1), op)
    assert np.linalg.norm(n2.lap2d_gather(B.apply(r), op) - r) <= 1e-11 * np.linalg.norm(r)


def test_3d_step_needs_the_2d_divergence_sign():
    """The reference's 3D divergence_nodes flips the sign of its x term
    (second_projection.py:563).  Four 3D time steps of the warm bubble (17x9x17,
    dt 21.69 ms): with the reference's sign the divergence of the projected
    momenta grows every step and the state turns non-finite; with the 2D
    branch's sign it stays small and the bubble rises smoothly."""
    from oracle import advection3d as a3, cases, step3d
    results = {}
    for x_sign in (-1.0, 1.0):
        grid, prm, Sol, p2, hn, hc, sf = cases.bubble_3d(17, 9, 17, seed=3, tol=1e-12, wind=0.0)
        S0c = np.broadcast_to(hc["S0"][None, :, None], grid.elem_sc).copy()
        flux = a3.new_flux(grid)
        divs = []
        with np.errstate(all="ignore"):
            for step in range(4):
                Sol = step3d.time_step(Sol, p2, flux, step, 0.02169, grid, prm, hn, hc, S0c, sf, x_sign=x_sign)
                check = {k: v.copy() for k, v in Sol.items()}
                divs.append(np.abs(o3_div(check, grid)).max())
        results[x_sign] = (divs, Sol)
    bad, good = results[-1.0], results[1.0]
    assert not np.all(np.isfinite(bad[1]["rhov"])) or bad[0][-1] > 10.0 * bad[0][0], bad[0]
    assert np.all(np.isfinite(good[1]["rhov"])) and good[0][-1] < 1e-2 * good[0][0], good[0]


def o3_div(Sol, grid):
    """The nodal divergence with the 2D branch's sign, away from the walls."""
    from oracle import proj3d as o3
    return o3.divergence_nodes(Sol, grid, x_sign=1.0)[3:-3, 3:-3, 3:-3]
