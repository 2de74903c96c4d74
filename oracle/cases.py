"""Input builders for the projection workloads (oracle; tests, smoke and CPU baseline only).

* :func:`rising_bubble` restates the reference's rising-bubble case:
  ``UserDataInit`` defaults (user_data.py:30-129) overridden by
  ``inputs/rising_bubble.py:5-37``, derived quantities
  (user_data.py:132-183, sim_params.py:11-28), the background
  ``hydrostatics.state`` (hydrostatics.py:79-117) and ``sol_init``
  (rising_bubble.py:42-98).  Pseudo-incompressible regime, tol 1e-10.
* :func:`stratified_2d` / :func:`stratified_3d` build the standalone-solve
  workloads (2049x1025 9-point, 257x129x257 27-point): a stably stratified
  background (N = 0.01 1/s, theta0 = 300 K) times a seeded log-normal factor
  (sigma 0.1) per cell, and a seeded zero-mean Gaussian random RHS with a
  k^-3 power spectrum.  These are synthetic stand-ins with the configured
  shapes and distributions; the reference publishes no such inputs.
"""
import numpy as np

from oracle import nodal2d as n2

# global constants (sim_params.py:11-28)
R_GAS = 287.4
GAMM = 1.4
T_REF = 300.0
H_REF = 10000.0


def _derived(grav, t_ref, h_ref=H_REF, omega=0.0):
    u_ref = h_ref / t_ref                                   # user_data.py:132-134
    Msq = u_ref * u_ref / (R_GAS * T_REF)                   # user_data.py:137-138
    g = grav * h_ref / (R_GAS * T_REF)                      # user_data.py:145
    cor = (omega * t_ref, 0.0, omega * t_ref)               # user_data.py:157-158
    return Msq, g, cor


def hydro_state(grid, prm):
    """``hydrostatics.state`` (hydrostatics.py:79-117): node and cell backgrounds."""
    Gamma = prm.Gamma
    g = prm.g
    Hex = 1.0 / (Gamma * g)
    dy = grid.dy
    out = {}
    for key, y in (("n", grid.node_y), ("c", grid.elem_y)):
        pi_p = np.exp(-(y + 0.5 * dy) / Hex)
        pi_m = np.exp(-(y - 0.5 * dy) / Hex)
        pi = np.exp(-(y) / Hex)
        Y = -Gamma * g * dy / (pi_p - pi_m)
        P = pi ** prm.gm1inv
        p = pi ** prm.Gammainv
        out[key] = dict(p20=pi / prm.Msq, p0=p, rho0=P / Y, rhoY0=P, Y0=Y, S0=1.0 / Y)
    return out["n"], out["c"]


def rising_bubble(inx=161, iny=81, delth=2.0, x0=0.0, y0=0.2, r0=0.2, tol=1e-10):
    """Initial state of the rising bubble (rising_bubble.py:42-98).

    Returns ``(grid, prm, Sol, p2_nodes, hydro_n, hydro_c, strat_fn)``.
    ``x0`` shifts the bubble centre (the reference centres it at 0).
    """
    grid = n2.Grid2D(inx, iny, -1.0, 1.0, 0.0, 1.0, (n2.PERIODIC, n2.WALL))
    Msq, g, cor = _derived(grav=10.0, t_ref=1000.0)
    prm = n2.Params(Msq=Msq, g=g, gamm=GAMM, coriolis=cor, nonhydro=1.0,
                    is_compressible=0, compressibility=0.0, tol=tol, max_iterations=6000)
    hn, hc = hydro_state(grid, prm)
    strat_fn = lambda y: 1.0                                # user_data.py:181-183
    X, Yg = np.meshgrid(grid.elem_x, grid.elem_y)
    r = np.sqrt((X - x0) ** 2 + (Yg - y0) ** 2) / r0
    rhoY = np.repeat(hc["rhoY0"].reshape(1, -1), grid.elem_sc[0], axis=0)
    pert = (delth / 300.0) * (np.cos(0.5 * np.pi * r) ** 2)
    pert[np.where(r > 1.0)] = 0.0
    rho = rhoY / (strat_fn(Yg) + pert.T)
    z = np.zeros(grid.elem_sc)
    Sol = dict(rho=rho, rhou=rho * 0.0, rhov=rho * 0.0, rhow=rho * 0.0, rhoY=rhoY, rhoX=z.copy())
    p2 = np.zeros(grid.node_sc)
    n2.set_explicit_boundary_data(Sol, grid, prm, hc, strat_fn)
    return grid, prm, Sol, p2, hn, hc, strat_fn


def bubble_3d(inx=65, iny=33, inz=65, seed=0, delth=2.0, y0=0.2, r0=0.2, wind=0.05, tol=1e-10,
              bdry=(n2.PERIODIC, n2.WALL, n2.PERIODIC), coriolis=(0.0, 0.0, 0.0), compressible=False):
    """A 3D projection input: the rising bubble's background and warm bubble
    (rising_bubble.py:42-98, centred at x = z = 0) on x, z in [-1, 1], y in
    [0, 1], with seeded smooth momenta (k^-3 spectrum, amplitude ``wind``
    times rho) so that the divergence is not zero.

    Returns ``(grid, prm, Sol, p2_nodes, hydro_n, hydro_c, strat_fn)``.
    """
    from oracle import proj3d as o3
    rng = np.random.default_rng(seed)
    grid = o3.Grid3D(inx, iny, inz, -1.0, 1.0, 0.0, 1.0, -1.0, 1.0, bdry)
    Msq, g, _ = _derived(grav=10.0, t_ref=1000.0)
    prm = n2.Params(Msq=Msq, g=g, gamm=GAMM, coriolis=coriolis, nonhydro=1.0,
                    is_compressible=1 if compressible else 0, compressibility=1.0 if compressible else 0.0,
                    tol=tol, max_iterations=100000)
    g2 = n2.Grid2D(inx, iny, -1.0, 1.0, 0.0, 1.0)
    hn, hc = hydro_state(g2, prm)
    strat_fn = lambda y: 1.0                                # user_data.py:181-183
    ex = -1.0 - 2 * grid.dx + 0.5 * grid.dx + grid.dx * np.arange(grid.elem_sc[0])
    ez = -1.0 - 2 * grid.dz + 0.5 * grid.dz + grid.dz * np.arange(grid.elem_sc[2])
    X, Yg, Z = np.meshgrid(ex, grid.elem_y, ez, indexing="ij")
    r = np.sqrt(X ** 2 + (Yg - y0) ** 2 + Z ** 2) / r0
    pert = (delth / 300.0) * (np.cos(0.5 * np.pi * r) ** 2)
    pert[np.where(r > 1.0)] = 0.0
    rhoY = np.broadcast_to(hc["rhoY0"][None, :, None], grid.elem_sc).copy()
    rho = rhoY / (strat_fn(Yg) + pert)
    mom = [wind * rho * _kminus3_field(grid.elem_sc, rng) for _ in range(3)]
    Sol = dict(rho=rho, rhou=mom[0], rhov=mom[1], rhow=mom[2], rhoY=rhoY, rhoX=np.zeros(grid.elem_sc))
    p2 = np.zeros(grid.node_sc)
    o3.set_explicit_boundary_data(Sol, grid, prm, hc, strat_fn)
    return grid, prm, Sol, p2, hn, hc, strat_fn


# --------------------------------------------------------------------------
# standalone solves on a stratified background
# --------------------------------------------------------------------------
def _kminus3_field(shape, rng, power=3.0):
    """Zero-mean Gaussian random field with power spectrum ~ k^-power (k=0 removed)."""
    white = rng.standard_normal(shape)
    F = np.fft.rfftn(white)
    ks = [np.fft.fftfreq(n) * n for n in shape[:-1]] + [np.fft.rfftfreq(shape[-1]) * shape[-1]]
    K = np.sqrt(sum(np.meshgrid(*[k ** 2 for k in ks], indexing="ij")))
    amp = np.zeros_like(K)
    nz = K > 0
    amp[nz] = K[nz] ** (-0.5 * power)
    f = np.fft.irfftn(F * amp, s=shape, axes=tuple(range(len(shape))))
    f -= f.mean()
    return f / f.std()


def _stratified_profile(y_nd, prm, N=0.01, theta0=300.0, grav=9.81):
    """theta(y)/theta0 = exp(N^2 z / g) and hydrostatic rhoY (P = pi^(1/(gamma-1)))."""
    Y = np.exp(N * N * (y_nd * H_REF) / grav)
    # hydrostatic Exner pressure d(pi)/dy = -Gamma g / Y, pi(0) = 1
    yy = np.asarray(y_nd, dtype=np.float64)
    # exact integral of 1/Y: (1 - exp(-a y)) / a with a = N^2 h_ref / grav
    a = N * N * H_REF / grav
    pi = 1.0 - prm.Gamma * prm.g * (1.0 - np.exp(-a * yy)) / a
    P = pi ** prm.gm1inv
    return Y, P


def stratified_2d(seed, inx=2049, iny=1025, sigma=0.1, dt=0.01, compressible=False):
    """Operands of one 2049x1025 9-point solve (flattened y-major, FP64).

    Returns a dict with ``op`` (packed operator for :func:`nodal2d.lap2d_gather`),
    ``b`` (Jacobi-scaled RHS), ``b_unscaled`` and the grid.
    """
    rng = np.random.default_rng(seed)
    grid = n2.Grid2D(inx, iny, -1.0, 1.0, 0.0, 1.0, (n2.PERIODIC, n2.WALL))
    Msq, g, cor = _derived(grav=9.81, t_ref=1000.0)
    prm = n2.Params(Msq=Msq, g=g, gamm=GAMM, coriolis=cor, nonhydro=1.0,
                    is_compressible=1 if compressible else 0, compressibility=1.0 if compressible else 0.0)
    Yc, Pc = _stratified_profile(grid.elem_y, prm)
    Yn, _ = _stratified_profile(grid.node_y, prm)
    rhoY = np.repeat(Pc[None, :], grid.elem_sc[0], axis=0)
    rho = rhoY / Yc[None, :]
    # seeded log-normal factor per cell; periodic in x over the inner cells
    fac = np.exp(sigma * rng.standard_normal(grid.elem_sc))
    fac[:2, :] = fac[-4:-2, :]
    fac[-2:, :] = fac[2:4, :]
    Sol = dict(rho=rho, rhoY=rhoY)
    wplus, wcenter, nu = n2.operator_coefficients_nodes(Sol, 1.0 / Yn, grid, prm, dt)
    wplus = wplus * fac[None]
    if not compressible:
        wcenter = wcenter * 0.0
    cor = n2.coriolis_params(Sol, 1.0 / Yn, grid, prm, dt)
    diag_inv = n2.precon_diag_prepare(wplus, wcenter, grid.dx, grid.dy)
    op = n2.pack_9pt(wplus, wcenter, cor, diag_inv, grid)
    # RHS on the physical periodic grid (inx-1 distinct columns), seam duplicated
    f = _kminus3_field((inx - 1, 2 * (iny - 1)), rng)[:, :iny]
    b = np.concatenate([f, f[:1]], axis=0)          # (inx, iny), col inx-1 == col 0
    b = project_out_null_2d(b, grid)
    b_flat = b.T.reshape(-1)
    bs = b_flat * op["diag_inv"]
    return dict(grid=grid, prm=prm, op=op, b=bs, b_unscaled=b_flat, dt=dt,
                wplus=wplus, wcenter=wcenter, cor=cor, diag_inv=diag_inv, seed=seed)


def null_modes_2d(grid):
    """Null vectors of the pseudo-incompressible 9-point operator, shape (k, inx, iny).

    Constants always; the checkerboard (-1)^(i+j) too, because the operator
    differences are averaged over the two rows/columns of a cell
    (laplacian.py:721-729), so the checkerboard has zero cell gradients.  On a
    periodic axis the checkerboard must be consistent with the wrap, i.e. the
    period n-1 must be even.
    """
    i = np.arange(grid.inx)[:, None]
    j = np.arange(grid.iny)[None, :]
    modes = [np.ones((grid.inx, grid.iny))]
    ok = True
    if grid.bdry[0] == n2.PERIODIC and (grid.inx - 1) % 2:
        ok = False
    if grid.bdry[1] == n2.PERIODIC and (grid.iny - 1) % 2:
        ok = False
    if ok:
        modes.append(((-1.0) ** (i + j)) * np.ones((grid.inx, grid.iny)))
    return np.stack(modes)


def project_out_null_2d(b, grid):
    """Make a seam-consistent node field b (inx, iny) compatible: <w e_k, b> = 0 for every null mode."""
    w = null_weights_2d(grid)
    E = null_modes_2d(grid)
    G = np.array([[np.sum(w * ek * el) for el in E] for ek in E])
    r = np.array([np.sum(w * ek * b) for ek in E])
    c = np.linalg.solve(G, r)
    return b - np.tensordot(c, E, axes=1)


def null_weights_2d(grid):
    """Left null vector of the unscaled pseudo-incompressible 2D operator, shape (inx, iny).

    The periodic seam node is duplicated (wrap distance n-1), so the
    duplicated seam columns carry weight 1/2; wall directions weight 1.
    """
    wx = np.ones(grid.inx)
    wy = np.ones(grid.iny)
    if grid.bdry[0] == n2.PERIODIC:
        wx[0] = wx[-1] = 0.5
    if grid.bdry[1] == n2.PERIODIC:
        wy[0] = wy[-1] = 0.5
    return np.outer(wx, wy)


# --------------------------------------------------------------------------
# 3D standalone solve (27-point), same construction as the 2D case
# --------------------------------------------------------------------------
SIGN_MODES_3D = ((1, 1, 1), (-1, -1, 1), (-1, 1, -1), (1, -1, -1), (-1, -1, -1))


def null_modes_3d(shape, periodic):
    """Sign-pattern null vectors of the pseudo-incompressible 27-point operator."""
    nx, ny, nz = shape
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    out = []
    for sx, sy, sz in SIGN_MODES_3D:
        ok = all(not (per and s < 0 and (n - 1) % 2) for per, s, n in zip(periodic, (sx, sy, sz), shape))
        if ok:
            e = np.ones(shape)
            if sx < 0:
                e = e * (-1.0) ** i
            if sy < 0:
                e = e * (-1.0) ** j
            if sz < 0:
                e = e * (-1.0) ** k
            out.append(e)
    return np.stack(out)


def trapezoid_weights(shape, periodic):
    ws = []
    for n, per in zip(shape, periodic):
        w = np.ones(n)
        if per:
            w[0] = w[-1] = 0.5
        ws.append(w)
    return np.einsum("i,j,k->ijk", *ws)


def stratified_3d(seed, nx=257, ny=129, nz=257, sigma=0.1, walls=(False, True, True)):
    """Operands of one 3D 27-point pseudo-incompressible solve (C order, z fastest)."""
    from oracle import nodal3d as n3
    rng = np.random.default_rng(seed)
    Msq, g, cor = _derived(grav=9.81, t_ref=1000.0)
    prm = n2.Params(Msq=Msq, g=g, gamm=GAMM)
    dx, dy, dz = 2.0 / (nx - 1), 1.0 / (ny - 1), 2.0 / (nz - 1)
    yc = (np.arange(ny + 1) - 0.5) * dy
    Yc, Pc = _stratified_profile(yc, prm)
    coeff = prm.Gammainv * Pc * Yc
    fac = np.exp(sigma * rng.standard_normal((nx + 1, ny + 1, nz + 1)))
    for ax, wall in enumerate(walls):
        if not wall:
            n = fac.shape[ax] - 1
            sl, src = [slice(None)] * 3, [slice(None)] * 3
            sl[ax], src[ax] = 0, n - 1
            fac[tuple(sl)] = fac[tuple(src)]
            sl[ax], src[ax] = n, 1
            fac[tuple(sl)] = fac[tuple(src)]
    h = coeff[None, :, None] * fac
    hc = np.zeros((nx, ny, nz))
    dinv = n3.precon_diag_3d(h, h, h, hc, dx, dy, dz)
    periodic = tuple(not w for w in walls)
    # right-hand side: nodal divergence of a seeded Gaussian cell flux field
    # with power ~k^-5 per component, so the divergence has ~k^-3 power; the
    # divergence form makes it compatible with the operator's large null space
    cshape = (nx + 1, ny + 1, nz + 1)
    F = []
    for _ in range(3):
        f = _kminus3_field(cshape, rng, power=5.0)
        for ax, per in enumerate(periodic):
            if per:
                n = cshape[ax] - 1
                sl, src = [slice(None)] * 3, [slice(None)] * 3
                sl[ax], src[ax] = 0, n - 1
                f[tuple(sl)] = f[tuple(src)]
                sl[ax], src[ax] = n, 1
                f[tuple(sl)] = f[tuple(src)]
        F.append(f)
    b = n3.node_divergence(F[0], F[1], F[2], walls)
    b = b / np.sqrt(np.mean(b * b))
    op = n3.pack_27pt(h, h, h, hc, dinv, nx, ny, nz, dx, dy, dz, walls=walls)
    return dict(op=op, b=b.reshape(-1) * dinv.reshape(-1), b_unscaled=b.reshape(-1), walls=walls,
                periodic=periodic, seed=seed)
