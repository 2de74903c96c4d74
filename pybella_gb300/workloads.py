"""Synthetic inputs of the standalone solve workloads, generated on the GPU.

``stratified_2d`` builds the operands of one 2049x1025 9-point solve in the
reference's packed layout (laplacian.py:517-527): a stably stratified
background (Brunt-Vaisala N = 0.01 1/s, theta0 = 300 K, hydrostatic Exner
pressure) gives the pseudo-incompressible coefficients of
``operator_coefficients_nodes`` (second_projection.py:308-356) and the
Coriolis/buoyancy factors of ``multiply_inverse_coriolis``
(second_projection.py:604-652); every cell coefficient is multiplied by a
seeded log-normal factor (sigma 0.1).  The right-hand side is a seeded
zero-mean Gaussian random field with a k^-3 power spectrum, made compatible
with the singular operator (no component along its null modes) and scaled by
the Jacobi diagonal ``precon_diag_prepare`` (laplacian.py:1284-1356).

These stand in for the reference's configuration; the reference ships no
such input data.  Values are drawn with torch's CUDA generator, so they are
reproducible per seed on a given torch build.
"""
import numpy as np
import torch

R_GAS, GAMM, T_REF, H_REF = 287.4, 1.4, 300.0, 10000.0


def _consts(grav=9.81, t_ref=1000.0):
    u_ref = H_REF / t_ref
    Msq = u_ref * u_ref / (R_GAS * T_REF)
    g = grav * H_REF / (R_GAS * T_REF)
    return Msq, g


def _profile(y, g, N=0.01, grav=9.81):
    a = N * N * H_REF / grav
    Gamma = (GAMM - 1.0) / GAMM
    Y = torch.exp(a * y)
    pi = 1.0 - Gamma * g * (1.0 - torch.exp(-a * y)) / a
    P = pi ** (1.0 / (GAMM - 1.0))
    return Y, P


def _kminus3(shape, gen, device):
    white = torch.randn(shape, generator=gen, device=device, dtype=torch.float64)
    F = torch.fft.rfftn(white)
    kx = torch.fft.fftfreq(shape[0], device=device, dtype=torch.float64) * shape[0]
    ky = torch.fft.rfftfreq(shape[1], device=device, dtype=torch.float64) * shape[1]
    K = torch.sqrt(kx[:, None] ** 2 + ky[None, :] ** 2)
    amp = torch.where(K > 0, K.clamp_min(1e-30) ** -1.5, torch.zeros_like(K))
    f = torch.fft.irfftn(F * amp, s=shape)
    f = f - f.mean()
    return f / f.std()


def null_modes_2d(nx, ny, x_periodic, y_periodic, device):
    """Constant and checkerboard null modes (shape (k, nx, ny)) and trapezoid weights."""
    i = torch.arange(nx, device=device)[:, None]
    j = torch.arange(ny, device=device)[None, :]
    modes = [torch.ones(nx, ny, dtype=torch.float64, device=device)]
    if not ((x_periodic and (nx - 1) % 2) or (y_periodic and (ny - 1) % 2)):
        modes.append((1.0 - 2.0 * ((i + j) % 2)).to(torch.float64).expand(nx, ny).clone())
    wx = torch.ones(nx, dtype=torch.float64, device=device)
    wy = torch.ones(ny, dtype=torch.float64, device=device)
    if x_periodic:
        wx[0] = wx[-1] = 0.5
    if y_periodic:
        wy[0] = wy[-1] = 0.5
    return torch.stack(modes), wx[:, None] * wy[None, :]


def stratified_2d(seed, nx=2049, ny=1025, sigma=0.1, dt=0.01, device="cuda"):
    """Operands of one pseudo-incompressible 9-point solve (flat, reference packing)."""
    dev = torch.device(device)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    Msq, g = _consts()
    dx = 2.0 / (nx - 1)
    dy = 1.0 / (ny - 1)
    ecx, ecy = nx + 3, ny + 3
    ey = -2 * dy + 0.5 * dy + dy * torch.arange(ecy, device=dev, dtype=torch.float64)
    ny_ = -2 * dy + dy * torch.arange(ny + 4, device=dev, dtype=torch.float64)
    Yc, Pc = _profile(ey, g)
    Yn, _ = _profile(ny_, g)
    Gammainv = GAMM / (GAMM - 1.0)
    coeff = (Gammainv * Pc * Yc)[None, :].expand(ecx, ecy)
    fac = torch.exp(sigma * torch.randn(ecx, ecy, generator=gen, device=dev, dtype=torch.float64))
    fac[:2] = fac[-4:-2].clone()
    fac[-2:] = fac[2:4].clone()
    wplus = coeff * fac                                     # (ecx, ecy), both directions
    S0 = 1.0 / Yn
    dSdy = (S0[1:] - S0[:-1]) / dy                          # cell rows
    nu = -dt * dt * (g / Msq) * dSdy * Yc                   # (ecy,)
    cxx = torch.ones(ecy, ecx, dtype=torch.float64, device=dev)
    cyy = (1.0 / (nu + 1.0))[:, None].expand(ecy, ecx)
    box = wplus[:-1, :-1] + wplus[1:, :-1] + wplus[:-1, 1:] + wplus[1:, 1:]
    c = 0.75
    diag = -(c / dx ** 2) * box - (c / dy ** 2) * box - (c / (dx * dy)) * box - (c / (dy * dx)) * box
    diag_inv = 1.0 / diag                                    # node.isc (nx+2, ny+2)
    s = (slice(1, -1), slice(1, -1))
    hplus = wplus[s].T.contiguous().reshape(-1)
    dinv = diag_inv[s].T.contiguous().reshape(-1)
    f = _kminus3((nx - 1, 2 * (ny - 1)), gen, dev)[:, :ny]
    b = torch.cat([f, f[:1]], dim=0)                        # seam column duplicated
    E, w = null_modes_2d(nx, ny, True, False, dev)
    # tiny Gram system solved on the host (no device linear-algebra library needed)
    G = torch.stack([torch.stack([(w * ek * el).sum() for el in E]) for ek in E]).cpu().numpy()
    r = torch.stack([(w * ek * b).sum() for ek in E]).cpu().numpy()
    cf = torch.from_numpy(np.linalg.solve(G, r)).to(dev)
    b = b - torch.tensordot(cf, E, dims=1)
    b_flat = b.T.contiguous().reshape(-1)
    return dict(hplusx=hplus, hplusy=hplus.clone(), hcenter=None,
                cor=(cxx[s].contiguous().reshape(-1), cyy[s].contiguous().reshape(-1), None, None),
                diag_inv=dinv, b=b_flat * dinv, nx=nx, ny=ny, dx=dx, dy=dy, x_wall=False, y_wall=True,
                seed=int(seed))


def operator_bytes_2d(w):
    """Host<->device bytes of the operands of one solve (FP64)."""
    n = w["nx"] * w["ny"]
    nc = (w["nx"] + 1) * (w["ny"] + 1)
    return 8 * (4 * nc + 2 * n)


def _power_field(shape, power, gen, device):
    """Zero-mean Gaussian random field with power spectrum ~ k^-power (k = 0 removed)."""
    white = torch.randn(shape, generator=gen, device=device, dtype=torch.float64)
    F = torch.fft.rfftn(white)
    ks = [torch.fft.fftfreq(n, device=device, dtype=torch.float64) * n for n in shape[:-1]]
    ks.append(torch.fft.rfftfreq(shape[-1], device=device, dtype=torch.float64) * shape[-1])
    grids = torch.meshgrid(*ks, indexing="ij")
    K = torch.sqrt(sum(g * g for g in grids))
    amp = torch.where(K > 0, K.clamp_min(1e-30) ** (-0.5 * power), torch.zeros_like(K))
    f = torch.fft.irfftn(F * amp, s=shape)
    f = f - f.mean()
    return f / f.std()


def _box3(a):
    return (a[:-1, :-1, :-1] + a[1:, :-1, :-1] + a[:-1, 1:, :-1] + a[1:, 1:, :-1]
            + a[:-1, :-1, 1:] + a[1:, :-1, 1:] + a[:-1, 1:, 1:] + a[1:, 1:, 1:])


def stratified_3d(seed, nx=257, ny=129, nz=257, sigma=0.1, walls=(False, True, True), device="cuda"):
    """Operands of one 3D 27-point solve (257x129x257 by default), C order (z fastest).

    Cells carry the stratified pseudo-incompressible coefficient (same
    background as :func:`stratified_2d`) times a seeded log-normal factor;
    the right-hand side is the nodal divergence (the operator's own node sums)
    of three seeded Gaussian cell flux fields with power ~k^-5, i.e. a field
    with ~k^-3 power that is compatible with the 27-point operator's null
    space (constants and hourglass modes).  Scaled by the 3D Jacobi diagonal
    of ``precon_diag_prepare`` (laplacian.py:1323-1356).
    """
    dev = torch.device(device)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    Msq, g = _consts()
    dx, dy, dz = 2.0 / (nx - 1), 1.0 / (ny - 1), 2.0 / (nz - 1)
    yc = (torch.arange(ny + 1, device=dev, dtype=torch.float64) - 0.5) * dy
    Yc, Pc = _profile(yc, g)
    coeff = GAMM / (GAMM - 1.0) * Pc * Yc
    cshape = (nx + 1, ny + 1, nz + 1)

    def periodic_copy(f):
        for ax, wall in enumerate(walls):
            if not wall:
                n = cshape[ax] - 1
                f.index_copy_(ax, torch.tensor([0, n], device=dev),
                              f.index_select(ax, torch.tensor([n - 1, 1], device=dev)))
        return f

    fac = periodic_copy(torch.exp(sigma * torch.randn(cshape, generator=gen, device=dev, dtype=torch.float64)))
    h = (coeff[None, :, None] * fac).contiguous()
    c = 0.0625
    S = _box3(h)
    diag = -(c / dx ** 2) * S - (c / dy ** 2) * S - (c / (dx * dy)) * S - (c / (dy * dx)) * S - (c / dz ** 2) * S
    dinv = 1.0 / diag
    F = []
    for _ in range(3):
        f = periodic_copy(_power_field(cshape, 5.0, gen, dev))
        for ax, wall in enumerate(walls):
            if wall:
                f.index_fill_(ax, torch.tensor([0, cshape[ax] - 1], device=dev), 0.0)
        F.append(f)
    fx, fy, fz = F
    xs = (fx[1:, :-1, :-1] + fx[1:, :-1, 1:] + fx[1:, 1:, :-1] + fx[1:, 1:, 1:]) - \
         (fx[:-1, :-1, :-1] + fx[:-1, :-1, 1:] + fx[:-1, 1:, :-1] + fx[:-1, 1:, 1:])
    ys = (fy[:-1, 1:, :-1] + fy[1:, 1:, :-1] + fy[:-1, 1:, 1:] + fy[1:, 1:, 1:]) - \
         (fy[:-1, :-1, :-1] + fy[1:, :-1, :-1] + fy[:-1, :-1, 1:] + fy[1:, :-1, 1:])
    zs = (fz[:-1, :-1, 1:] + fz[:-1, 1:, 1:] + fz[1:, :-1, 1:] + fz[1:, 1:, 1:]) - \
         (fz[:-1, :-1, :-1] + fz[:-1, 1:, :-1] + fz[1:, :-1, :-1] + fz[1:, 1:, :-1])
    b = xs + ys + zs
    b = b / torch.sqrt(torch.mean(b * b))
    dflat = dinv.reshape(-1).contiguous()
    hf = h.reshape(-1)
    return dict(hplusx=hf, hplusy=hf, hplusz=hf, hcenter=None, diag_inv=dflat,
                b=(b.reshape(-1) * dflat).contiguous(), nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz,
                walls=tuple(walls), corrf=0.0, seed=int(seed))


def operator_2d(w, ws=None):
    """Device 9-point operator of a 2D workload dict (its own workspace unless ``ws``)."""
    from .linalg import NodalHelmholtz2D
    return NodalHelmholtz2D(w["hplusx"], w["hplusy"], w["hcenter"], w["cor"], w["diag_inv"], w["nx"], w["ny"],
                            w["dx"], w["dy"], x_wall=w["x_wall"], y_wall=w["y_wall"], ws=ws)


ENSEMBLE_GRIDS = ((160, 80), (320, 160), (640, 320))


def rising_bubble_member(cells, amplitude_K, centre_x, grav=10.0, r0=0.2, z0=0.2, device="cuda"):
    """Operands of one pseudo-incompressible rising-bubble projection solve.

    The rising-bubble set-up (inputs/rising_bubble.py:5-98): x in [-1, 1]
    (periodic), z in [0, 1] (walls) in units of h_ref = 10 km, isentropic
    background theta = 300 K with hydrostatic pressure, g = 10, and a warm
    bubble theta' = amplitude * cos^2(pi r / 2), r = |(x, z) - (centre_x, z0)| / r0.
    Cell coefficients as operator_coefficients_nodes (second_projection.py:
    308-356): hplus = Gamma^-1 P theta (P the background rho*theta); isentropic,
    so the buoyancy factor of multiply_inverse_coriolis is 1.  The right-hand
    side is the nodal divergence of the bubble's buoyancy flux (0, P theta' g dt)
    on cells (none through the walls), cleared of the operator's null modes and
    scaled by the Jacobi diagonal of precon_diag_prepare (laplacian.py:1284-1356).
    """
    dev = torch.device(device)
    cx, cz = cells
    nx, ny = cx + 1, cz + 1
    dx, dy = 2.0 / cx, 1.0 / cz
    Msq, g = _consts(grav=grav)
    Gamma = (GAMM - 1.0) / GAMM
    # cell centres of the (nx+1) x (ny+1) cells around the inner nodes; x wraps
    xc = -1.0 + (torch.arange(nx + 1, device=dev, dtype=torch.float64) - 0.5) * dx
    xc = torch.remainder(xc + 1.0, 2.0) - 1.0
    zc = (torch.arange(ny + 1, device=dev, dtype=torch.float64) - 0.5) * dy
    X, Z = torch.meshgrid(xc, zc, indexing="ij")
    pi = 1.0 - Gamma * g * Z                                # isentropic Exner pressure, theta = 1
    P = pi.clamp_min(1e-6) ** (1.0 / (GAMM - 1.0))
    r = torch.sqrt((X - centre_x) ** 2 + (Z - z0) ** 2) / r0
    dth = torch.where(r < 1.0, (amplitude_K / T_REF) * torch.cos(0.5 * np.pi * r) ** 2, torch.zeros_like(r))
    theta = 1.0 + dth
    wplus = P * theta / Gamma                               # (nx+1, ny+1)
    box = wplus[:-1, :-1] + wplus[1:, :-1] + wplus[:-1, 1:] + wplus[1:, 1:]
    c = 0.75
    diag = -(c / dx ** 2) * box - (c / dy ** 2) * box - (c / (dx * dy)) * box - (c / (dy * dx)) * box
    dinv = 1.0 / diag                                       # (nx, ny)
    dt = 0.5 * dx
    Fy = P * dth * g * dt
    Fy[:, 0] = 0.0
    Fy[:, -1] = 0.0
    b = 0.5 * ((Fy[:-1, 1:] + Fy[1:, 1:]) - (Fy[:-1, :-1] + Fy[1:, :-1])) / dy
    E, w = null_modes_2d(nx, ny, True, False, dev)
    G = torch.stack([torch.stack([(w * ek * el).sum() for el in E]) for ek in E]).cpu().numpy()
    rr = torch.stack([(w * ek * b).sum() for ek in E]).cpu().numpy()
    cf = torch.from_numpy(np.linalg.solve(G, rr)).to(dev)
    b = b - torch.tensordot(cf, E, dims=1)
    ones = torch.ones(ny + 1, nx + 1, dtype=torch.float64, device=dev).reshape(-1)
    hplus = wplus.T.contiguous().reshape(-1)
    dflat = dinv.T.contiguous().reshape(-1)
    return dict(hplusx=hplus, hplusy=hplus.clone(), hcenter=None, cor=(ones, ones.clone(), None, None),
                diag_inv=dflat, b=b.T.contiguous().reshape(-1) * dflat, nx=nx, ny=ny, dx=dx, dy=dy,
                x_wall=False, y_wall=True, amplitude_K=float(amplitude_K), centre_x=float(centre_x))


def rising_bubble_ensemble(seed, per_grid=16, grids=ENSEMBLE_GRIDS, device="cuda"):
    """48 members (16 per grid by default): amplitude ~ N(2 K, 0.2 K), centre ~ N(0, 200 m), seeded."""
    rng = np.random.default_rng(int(seed))
    members = []
    for cells in grids:
        for _ in range(per_grid):
            amp = rng.normal(2.0, 0.2)
            x0 = rng.normal(0.0, 200.0 / H_REF)
            members.append(rising_bubble_member(cells, amp, x0, device=device))
    return members


def bubble_3d_state(nx, ny, nz, seed=0, delth=2.0, y0=0.2, r0=0.2, grav=10.0, t_ref=1000.0):
    """The state of a 3D warm-bubble run in the reference's objects (host NumPy
    arrays): the rising bubble's set-up (inputs/rising_bubble.py:42-98) on x, z in
    [-1, 1] (periodic), y in [0, 1] (walls), nx x ny x nz nodes, the bubble centred
    at x = z = 0 (its amplitude shifted by ``seed`` * 1e-3 K so that replicas differ),
    the isentropic hydrostatic background of hydrostatics.state (hydrostatics.py:
    79-117), fluid at rest.  Returns a dict with ``Sol``, ``mpv``, ``elem``,
    ``node``, ``ud``, ``th`` for :class:`pybella_gb300.time_update.DeviceStep3D`."""
    from types import SimpleNamespace as NS
    ig = 2
    u_ref = H_REF / t_ref
    Msq = u_ref * u_ref / (R_GAS * T_REF)
    g = grav * H_REF / (R_GAS * T_REF)
    Gamma, gm1inv = (GAMM - 1.0) / GAMM, 1.0 / (GAMM - 1.0)
    dx, dy, dz = 2.0 / (nx - 1.0), 1.0 / (ny - 1.0), 2.0 / (nz - 1.0)
    sc = (nx - 1 + 2 * ig, ny - 1 + 2 * ig, nz - 1 + 2 * ig)
    ex = -1.0 - ig * dx + 0.5 * dx + dx * np.arange(sc[0])
    ey = 0.0 - ig * dy + 0.5 * dy + dy * np.arange(sc[1])
    ez = -1.0 - ig * dz + 0.5 * dz + dz * np.arange(sc[2])
    ny_ = 0.0 - ig * dy + dy * np.arange(ny + 2 * ig)
    Hex = 1.0 / (Gamma * g)

    def column(y):
        pi_p, pi_m, pi = np.exp(-(y + 0.5 * dy) / Hex), np.exp(-(y - 0.5 * dy) / Hex), np.exp(-y / Hex)
        Y = -Gamma * g * dy / (pi_p - pi_m)
        return pi ** gm1inv, Y                           # rhoY0 and Y0 (hydrostatics.py:92-112)
    rhoY0_c, _ = column(ey)
    _, Y0_n = column(ny_)
    X, Yg, Z = np.meshgrid(ex, ey, ez, indexing="ij")
    r = np.sqrt(X ** 2 + (Yg - y0) ** 2 + Z ** 2) / r0
    pert = ((delth + 1e-3 * seed) / 300.0) * np.cos(0.5 * np.pi * r) ** 2
    pert[r > 1.0] = 0.0
    rhoY = np.broadcast_to(rhoY0_c[None, :, None], sc).copy()
    rho = rhoY / (1.0 + pert)
    z = np.zeros(sc)
    Sol = NS(rho=rho, rhou=z.copy(), rhov=z.copy(), rhow=z.copy(), rhoY=rhoY, rhoX=z.copy())
    S0c = np.broadcast_to((1.0 / column(ey)[1])[None, :, None], sc).copy()
    mpv = NS(p2_nodes=np.zeros((nx + 2 * ig, ny + 2 * ig, nz + 2 * ig)),
             HydroState=NS(rhoY0=rhoY0_c, get_S0c=lambda elem: S0c), HydroState_n=NS(S0=1.0 / Y0_n))
    elem = NS(ndim=3, y=ey)
    node = NS(iicx=nx, iicy=ny, iicz=nz, dx=dx, dy=dy, dz=dz)
    ud = NS(bdry_type=["wrap", "symmetric", "wrap"], gravity_strength=[0.0, g, 0.0], Msq=Msq, nonhydrostasy=1.0,
            compressibility=0.0, is_compressible=0, coriolis_strength=np.zeros(3), u_wind_speed=0.0,
            v_wind_speed=0.0, w_wind_speed=0.0, stratification=lambda y: 1.0, tol=1e-10, max_iterations=1000)
    return dict(Sol=Sol, mpv=mpv, elem=elem, node=node, ud=ud, th=NS(gamm=GAMM))


def bubble_2d_state(inx=161, iny=81, delth=2.0, y0=0.2, r0=0.2, grav=10.0, t_ref=1000.0, x0=0.0):
    """The rising bubble's initial state (inputs/rising_bubble.py:42-98) in the
    reference's objects (host NumPy arrays): inx x iny nodes on x in [-1, 1]
    (periodic), y in [0, 1] (walls), isentropic hydrostatic background
    (hydrostatics.py:79-117), the warm bubble at (x0, y0), fluid at rest, the
    reference's boundary data applied by the first step.  Returns a dict with
    ``Sol``, ``mpv``, ``elem``, ``node``, ``ud``, ``th`` for
    :class:`pybella_gb300.time_update.DeviceStep2D`."""
    from types import SimpleNamespace as NS
    ig = 2
    u_ref = H_REF / t_ref
    Msq = u_ref * u_ref / (R_GAS * T_REF)
    g = grav * H_REF / (R_GAS * T_REF)
    Gamma, gm1inv = (GAMM - 1.0) / GAMM, 1.0 / (GAMM - 1.0)
    dx, dy = 2.0 / (inx - 1.0), 1.0 / (iny - 1.0)
    sc = (inx - 1 + 2 * ig, iny - 1 + 2 * ig)
    ex = -1.0 - ig * dx + 0.5 * dx + dx * np.arange(sc[0])
    ey = 0.0 - ig * dy + 0.5 * dy + dy * np.arange(sc[1])
    ny_ = 0.0 - ig * dy + dy * np.arange(iny + 2 * ig)
    Hex = 1.0 / (Gamma * g)

    def column(y):
        pi_p, pi_m, pi = np.exp(-(y + 0.5 * dy) / Hex), np.exp(-(y - 0.5 * dy) / Hex), np.exp(-y / Hex)
        return pi ** gm1inv, -Gamma * g * dy / (pi_p - pi_m)
    rhoY0_c, Y0_c = column(ey)
    _, Y0_n = column(ny_)
    X, Yg = np.meshgrid(ex, ey, indexing="ij")
    r = np.sqrt((X - x0) ** 2 + (Yg - y0) ** 2) / r0
    pert = (delth / 300.0) * np.cos(0.5 * np.pi * r) ** 2
    pert[r > 1.0] = 0.0
    rhoY = np.broadcast_to(rhoY0_c[None, :], sc).copy()
    rho = rhoY / (1.0 + pert)
    z = np.zeros(sc)
    Sol = NS(rho=rho, rhou=z.copy(), rhov=z.copy(), rhow=z.copy(), rhoY=rhoY, rhoX=z.copy())
    S0c = np.broadcast_to((1.0 / Y0_c)[None, :], sc).copy()
    mpv = NS(p2_nodes=np.zeros((inx + 2 * ig, iny + 2 * ig)),
             HydroState=NS(rhoY0=rhoY0_c, get_S0c=lambda elem: S0c), HydroState_n=NS(S0=1.0 / Y0_n))
    elem = NS(ndim=2, y=ey)
    node = NS(iicx=inx, iicy=iny, dx=dx, dy=dy)
    ud = NS(bdry_type=["wrap", "symmetric", "symmetric"], gravity_strength=[0.0, g, 0.0], Msq=Msq,
            nonhydrostasy=1.0, compressibility=0.0, is_compressible=0, coriolis_strength=np.zeros(3),
            u_wind_speed=0.0, v_wind_speed=0.0, w_wind_speed=0.0, stratification=lambda y: 1.0, tol=1e-10,
            max_iterations=6000, t_ref=t_ref)
    return dict(Sol=Sol, mpv=mpv, elem=elem, node=node, ud=ud, th=NS(gamm=GAMM))


def bubble_ensemble_states(seed, per_grid=16, grids=ENSEMBLE_GRIDS):
    """The 48-member rising-bubble ensemble as time-step states: ``per_grid``
    members on each of ``grids`` (cells), bubble amplitude ~ N(2 K, 0.2 K) and
    x-centre ~ N(0, 200 m) (units of h_ref = 10 km), seeded; each entry is a
    :func:`bubble_2d_state` dict."""
    rng = np.random.default_rng(int(seed))
    out = []
    for (cx, cy) in grids:
        for _ in range(per_grid):
            out.append(bubble_2d_state(inx=cx + 1, iny=cy + 1, delth=float(rng.normal(2.0, 0.2)),
                                       x0=float(rng.normal(0.0, 200.0 / H_REF))))
    return out
