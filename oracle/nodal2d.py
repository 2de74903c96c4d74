"""FP64 NumPy restatement of the reference's 2D nodal projection (oracle; tests only).

Every function names the reference file:line (paths inside the pyBELLA
repository) whose arithmetic it restates.  Array conventions are the
reference's:

* cell arrays have shape ``elem.sc = (inx-1+4, iny-1+4)`` (two ghost layers),
* node arrays ``node.sc = (inx+4, iny+4)``; ``node.isc = (inx+2, iny+2)``
  (``rhs``, ``wcenter``, ``diag_inv``); inner unknowns ``node.iisc = (inx, iny)``,
* the solver vector is the inner node block flattened y-major
  (``rhs[1:-1,1:-1].T.ravel()``, second_projection.py:214), i.e.
  ``idx = j * inx + i``.
"""
import numpy as np
from scipy.signal import fftconvolve

PERIODIC = "periodic"
WALL = "wall"
RAYLEIGH = "rayleigh"


# --------------------------------------------------------------------------
# grid (grid.py:39-298, 2D part)
# --------------------------------------------------------------------------
class Grid2D:
    """Cell and node grid sizes of ``grid.py:111-298`` for a 2D domain."""

    def __init__(self, inx, iny, xmin, xmax, ymin, ymax, bdry=(PERIODIC, WALL)):
        ig = 2
        self.inx, self.iny = inx, iny
        self.dx = (xmax - xmin) / (inx - 1.0)            # grid.py:84
        self.dy = (ymax - ymin) / (iny - 1.0)            # grid.py:85
        self.igs = (ig, ig)
        self.elem_sc = (inx - 1 + 2 * ig, iny - 1 + 2 * ig)   # grid.py:142-153
        self.node_sc = (inx + 2 * ig, iny + 2 * ig)           # grid.py:259-273
        self.node_isc = (inx + ig, iny + ig)
        self.node_iisc = (inx, iny)
        self.elem_x = xmin - ig * self.dx + 0.5 * self.dx + self.dx * np.arange(self.elem_sc[0])
        self.elem_y = ymin - ig * self.dy + 0.5 * self.dy + self.dy * np.arange(self.elem_sc[1])
        self.node_x = xmin - ig * self.dx + self.dx * np.arange(self.node_sc[0])
        self.node_y = ymin - ig * self.dy + self.dy * np.arange(self.node_sc[1])
        self.bdry = tuple(bdry)

    @property
    def x_wall(self):
        return self.bdry[0] in (WALL, RAYLEIGH)

    @property
    def y_wall(self):
        return self.bdry[1] in (WALL, RAYLEIGH)


def box2(a):
    """2x2 box sum, ``fftconvolve(a, ones((2,2)), 'valid')`` (second_projection.py:345).

    Evaluated with the same SciPy routine as the reference so that the
    oracle reproduces its FFT round-off bit for bit.
    """
    return fftconvolve(a, np.ones((2, 2)), mode="valid")


def box2_direct(a):
    """Exact 2x2 box sum (what the FFT form approximates to ~1e-16 relative)."""
    return a[:-1, :-1] + a[1:, :-1] + a[:-1, 1:] + a[1:, 1:]


# --------------------------------------------------------------------------
# operator (laplacian.py:496-528, 546-746, 1284-1356)
# --------------------------------------------------------------------------
def pack_9pt(wplus, wcenter, coriolis, diag_inv, grid):
    """Operand packing of ``stencil_9pt_numba_test`` (laplacian.py:496-528).

    ``coriolis`` is the 4-tuple returned by ``multiply_inverse_coriolis(...,
    get_coeffs=True)`` (already transposed, second_projection.py:651).
    Returns the flat operands consumed by :func:`lap2d_gather`.
    """
    s = (slice(1, -1), slice(1, -1))
    hplusx = wplus[0][s].T.reshape(-1)
    hplusy = wplus[1][s].T.reshape(-1)
    hcenter = wcenter[s].T.reshape(-1)
    cor = tuple(c[s].reshape(-1) for c in coriolis)
    dinv = diag_inv[s].T.reshape(-1)
    return dict(hplusx=hplusx, hplusy=hplusy, hcenter=hcenter, cor=cor, diag_inv=dinv,
                nx=grid.inx, ny=grid.iny, dx=grid.dx, dy=grid.dy,
                x_wall=grid.x_wall, y_wall=grid.y_wall)


def _wrap_index(n):
    """Neighbour indices with the reference's periodic wrap (laplacian.py:595-638).

    Left/top neighbour of index 0 is ``n-2`` and right/bottom neighbour of
    ``n-1`` is ``1``: the seam node is duplicated, so the wrap distance is
    ``n-1``.
    """
    i = np.arange(n)
    lo = i - 1
    hi = i + 1
    lo[0] += n - 1
    hi[-1] -= n - 1
    return lo, hi


def lap2d_gather(p, op):
    """Vectorised restatement of ``lap2D_gather_new`` (laplacian.py:546-746).

    Same operation order as the reference loop body, so results agree to the
    last bit with the reference run un-jitted.
    """
    nx, ny = op["nx"], op["ny"]
    P = np.asarray(p, dtype=np.float64).reshape(ny, nx)
    jlo, jhi = _wrap_index(ny)
    ilo, ihi = _wrap_index(nx)

    topleft = P[jlo][:, ilo]
    topmid = P[jlo]
    topright = P[jlo][:, ihi]
    midleft = P[:, ilo]
    midmid = P
    midright = P[:, ihi]
    botleft = P[jhi][:, ilo]
    botmid = P[jhi]
    botright = P[jhi][:, ihi]

    def corners(flat):
        a = flat.reshape(ny + 1, nx + 1)
        return (a[:-1, :-1].copy(), a[:-1, 1:].copy(), a[1:, :-1].copy(), a[1:, 1:].copy())

    hx_tl, hx_tr, hx_bl, hx_br = corners(op["hplusx"])
    hy_tl, hy_tr, hy_bl, hy_br = corners(op["hplusy"])
    cxx, cyy, cxy, cyx = op["cor"]
    cxx_tl, cxx_tr, cxx_bl, cxx_br = corners(cxx)
    cyy_tl, cyy_tr, cyy_bl, cyy_br = corners(cyy)
    cxy_tl, cxy_tr, cxy_bl, cxy_br = corners(cxy)
    cyx_tl, cyx_tr, cyx_bl, cyx_br = corners(cyx)

    # wall zeroing (laplacian.py:691-713)
    if op["x_wall"]:
        for a in (hx_tl, hy_tl, hx_bl, hy_bl):
            a[:, 0] = 0.0
        for a in (hx_tr, hy_tr, hx_br, hy_br):
            a[:, -1] = 0.0
    if op["y_wall"]:
        for a in (hx_tl, hy_tl, hx_tr, hy_tr):
            a[0, :] = 0.0
        for a in (hx_bl, hy_bl, hx_br, hy_br):
            a[-1, :] = 0.0

    oodx = 1.0 / op["dx"]
    oody = 1.0 / op["dy"]
    # laplacian.py:721-729
    Dx_tl = 0.5 * (topmid - topleft + midmid - midleft) * hx_tl
    Dx_tr = 0.5 * (topright - topmid + midright - midmid) * hx_tr
    Dx_bl = 0.5 * (botmid - botleft + midmid - midleft) * hx_bl
    Dx_br = 0.5 * (botright - botmid + midright - midmid) * hx_br
    Dy_tl = 0.5 * (midmid - topmid + midleft - topleft) * hy_tl
    Dy_tr = 0.5 * (midright - topright + midmid - topmid) * hy_tr
    Dy_bl = 0.5 * (botmid - midmid + botleft - midleft) * hy_bl
    Dy_br = 0.5 * (botright - midright + botmid - midmid) * hy_br
    # laplacian.py:731-739
    fac = 1.0
    Dxx = 0.5 * (cxx_tr * Dx_tr - cxx_tl * Dx_tl + cxx_br * Dx_br - cxx_bl * Dx_bl) * oodx * oodx * fac
    Dyy = 0.5 * (cyy_br * Dy_br - cyy_tr * Dy_tr + cyy_bl * Dy_bl - cyy_tl * Dy_tl) * oody * oody * fac
    Dyx = 0.5 * (cxy_br * Dy_br - cxy_bl * Dy_bl + cxy_tr * Dy_tr - cxy_tl * Dy_tl) * oody * oodx * fac
    Dxy = 0.5 * (cyx_br * Dx_br - cyx_tr * Dx_tr + cyx_bl * Dx_bl - cyx_tl * Dx_tl) * oodx * oody * fac
    hc = op["hcenter"].reshape(ny, nx)
    lap = Dxx + Dyy + Dyx + Dxy + hc * midmid
    lap = lap * op["diag_inv"].reshape(ny, nx)
    return lap.reshape(-1)


def lap2d_lamb(p, op):
    """The ``LAMB_BDRY`` branch of ``stencil_9pt_numba_test``: ``lap2D_numba_test``
    (laplacian.py:531-543) with its padding ``periodic`` (:858-868) and the
    ``kernel_9pt`` stencil (:749-856).

    The inner nodes are padded by one node: x wraps with the duplicated seam
    (column 0 <- column n-2, column n+1 <- column 1), then y mirrors (row 0 <- row
    2, last <- third last); no cell coefficient is zeroed at a boundary.  With the
    operands packed as :func:`pack_9pt` packs them (the reference's factory passes
    the same arrays transposed), node (j, i) reads the cells (j, i), (j, i+1) below
    it and (j+1, i), (j+1, i+1) above it, and y grows towards "top".  Same
    operation order as ``kernel_9pt``.
    """
    nx, ny = op["nx"], op["ny"]
    a = np.zeros((ny + 2, nx + 2))
    a[1:-1, 1:-1] = np.asarray(p, dtype=np.float64).reshape(ny, nx)
    a[:, 0] = a[:, -3]
    a[:, -1] = a[:, 2]
    a[0, :] = a[2, :]
    a[-1, :] = a[-3, :]
    c = slice(1, -1)
    topleft, topmid, topright = a[2:, :-2], a[2:, c], a[2:, 2:]
    midleft, midmid, midright = a[c, :-2], a[c, c], a[c, 2:]
    botleft, botmid, botright = a[:-2, :-2], a[:-2, c], a[:-2, 2:]

    def cells(flat):
        q = np.asarray(flat, dtype=np.float64).reshape(ny + 1, nx + 1)
        return q[1:, :-1], q[1:, 1:], q[:-1, :-1], q[:-1, 1:]         # tl, tr, bl, br
    hpx_tl, hpx_tr, hpx_bl, hpx_br = cells(op["hplusx"])
    hpy_tl, hpy_tr, hpy_bl, hpy_br = cells(op["hplusy"])
    cxx, cyy, cxy, cyx = op["cor"]
    cxx_tl, cxx_tr, cxx_bl, cxx_br = cells(cxx)
    cyy_tl, cyy_tr, cyy_bl, cyy_br = cells(cyy)
    cxy_tl, cxy_tr, cxy_bl, cxy_br = cells(cxy)
    cyx_tl, cyx_tr, cyx_bl, cyx_br = cells(cyx)
    oodx, oody = 1.0 / op["dx"], 1.0 / op["dy"]
    Dx_tl = 0.5 * (topmid - topleft + midmid - midleft) * hpx_tl
    Dx_tr = 0.5 * (topright - topmid + midright - midmid) * hpx_tr
    Dx_bl = 0.5 * (botmid - botleft + midmid - midleft) * hpx_bl
    Dx_br = 0.5 * (botright - botmid + midright - midmid) * hpx_br
    Dy_tl = 0.5 * (topmid - midmid + topleft - midleft) * hpy_tl
    Dy_tr = 0.5 * (topright - midright + topmid - midmid) * hpy_tr
    Dy_bl = 0.5 * (midmid - botmid + midleft - botleft) * hpy_bl
    Dy_br = 0.5 * (midright - botright + midmid - botmid) * hpy_br
    Dxx = 0.5 * (cxx_tr * Dx_tr - cxx_tl * Dx_tl + cxx_br * Dx_br - cxx_bl * Dx_bl) * oodx * oodx
    Dyy = 0.5 * (cyy_tr * Dy_tr - cyy_br * Dy_br + cyy_tl * Dy_tl - cyy_bl * Dy_bl) * oody * oody
    Dyx = 0.5 * (cxy_br * Dy_br - cxy_bl * Dy_bl + cxy_tr * Dy_tr - cxy_tl * Dy_tl) * oody * oodx
    Dxy = 0.5 * (cyx_tr * Dx_tr - cyx_br * Dx_br + cyx_tl * Dx_tl - cyx_bl * Dx_bl) * oodx * oody
    hc = np.asarray(op["hcenter"], dtype=np.float64).reshape(ny, nx)
    dinv = np.asarray(op["diag_inv"], dtype=np.float64).reshape(ny, nx)
    return (((Dxx + Dyy + Dyx + Dxy) + hc * midmid) * dinv).reshape(-1)


def precon_diag_prepare(wplus, wcenter, dx, dy, dz=None):
    """Approximate Jacobi diagonal, ``precon_diag_prepare`` (laplacian.py:1284-1356).

    Returns ``diag_inv`` with the shape of ``wcenter`` (node.isc).  The
    2x2(x2) box sums use the same ``fftconvolve(..., 'valid')`` as the
    reference, so the result is bit-identical.
    """
    ndim = wcenter.ndim
    if ndim == 2:
        coeff = 1.0 - 0.5 * 0.5                          # laplacian.py:1318-1321
        S = box2
    else:
        coeff = 0.0625                                   # laplacian.py:1323
        S = box3
    wxx = coeff / dx ** 2
    wyy = coeff / dy ** 2
    wxy = coeff / (dx * dy)
    wyx = coeff / (dy * dx)
    diag = -wxx * S(wplus[0])
    diag = diag - wyy * S(wplus[1])
    diag = diag - wxy * S(wplus[0])                       # hplusxy = wplus[0] (:1313)
    diag = diag - wyx * S(wplus[1])                       # hplusyx = wplus[1] (:1314)
    if ndim == 3:
        wzz = coeff / dz ** 2
        diag = diag - wzz * S(wplus[2])
    diag = diag + wcenter
    return 1.0 / diag


def box3(a):
    """2x2x2 box sum, ``fftconvolve(a, ones((2,2,2)), 'valid')`` (laplacian.py:1346-1351)."""
    return fftconvolve(a, np.ones((2, 2, 2)), mode="valid")


def box3_direct(a):
    """Exact 2x2x2 box sum."""
    return (a[:-1, :-1, :-1] + a[1:, :-1, :-1] + a[:-1, 1:, :-1] + a[1:, 1:, :-1]
            + a[:-1, :-1, 1:] + a[1:, :-1, 1:] + a[:-1, 1:, 1:] + a[1:, 1:, 1:])


# --------------------------------------------------------------------------
# physics pieces of the projection (second_projection.py)
# --------------------------------------------------------------------------
class Params:
    """Scalars the projection reads from ``ud`` and ``th``.

    ``g`` is ``ud.gravity_strength[1]``, ``coriolis`` is
    ``ud.coriolis_strength`` (3 entries), ``gamm`` the ratio of specific
    heats (thermodynamic.py:14-20).
    """

    def __init__(self, Msq, g, gamm=1.4, coriolis=(0.0, 0.0, 0.0), nonhydro=1.0,
                 is_compressible=0, compressibility=0.0, tol=1e-10, max_iterations=6000):
        self.Msq = Msq
        self.g = g
        self.gamm = gamm
        self.gm1 = gamm - 1.0
        self.gm1inv = 1.0 / (gamm - 1.0)
        self.Gamma = (gamm - 1.0) / gamm
        self.Gammainv = gamm / (gamm - 1.0)
        self.coriolis = np.asarray(coriolis, dtype=np.float64)
        self.nonhydro = nonhydro
        self.is_compressible = is_compressible
        self.compressibility = compressibility
        self.tol = tol
        self.max_iterations = max_iterations


def get_dSdy(S0_nodes, grid):
    """Cell field ``dS/dy`` from the node background ``S0`` (variable.py:162-177)."""
    d = (S0_nodes[1:] - S0_nodes[:-1]) / grid.dy
    return np.repeat(d[None, :], grid.elem_sc[0], axis=0)


def operator_coefficients_nodes(Sol, S0n, grid, prm, dt):
    """``operator_coefficients_nodes`` (second_projection.py:308-356).

    Returns ``(wplus, wcenter, nu_c)``; ``wcenter`` is already scaled by 0.5
    on wall node rows (``scale_wall_node_values``, :356).
    """
    ccenter = -prm.Msq * prm.gm1inv / dt ** 2
    cexp = 2.0 - prm.gamm
    strat = get_dSdy(S0n, grid)
    Y = Sol["rhoY"] / Sol["rho"]
    coeff = prm.Gammainv * Sol["rhoY"] * Y
    nu = -dt ** 2 * (prm.g / prm.Msq) * strat * Y
    wplus = np.stack([coeff, coeff])
    wcenter = ccenter * box2(Sol["rhoY"] ** cexp) / 4.0
    scale_wall_node_values(wcenter, grid, 0.5)
    return wplus, wcenter, nu


def scale_wall_node_values(a, grid, factor=0.5):
    """``scale_wall_node_values`` (second_projection.py:433-474) on a node.isc array (2D or 3D).

    The index starts as ``[igs:-igs]`` on every axis; each wall axis in turn is
    set to row -2, then row 1, and scaled there -- and is left at row 1, so a
    later wall axis scales only the entries on row 1 of the earlier ones (with
    walls in x and y, the y-wall rows are scaled at x row 1 alone).
    """
    ig = grid.igs
    nd = a.ndim
    idx = [slice(ig[d], -ig[d]) for d in range(nd)]
    for dim in range(nd):
        if grid.bdry[dim] in (WALL, RAYLEIGH):
            for direction in (-1, 1):
                idx[dim] = (ig[dim] - 1) * direction
                if direction == -1:
                    idx[dim] -= 1
                a[tuple(idx)] *= factor


def coriolis_coefficients(Sol, S0n, grid, prm, dt):
    """Coefficients of ``multiply_inverse_coriolis`` (second_projection.py:604-633).

    Returns the 3x3 coefficient fields (already multiplied by ``denom``) as a
    dict with keys ``uu, uv, uw, vu, vv, vw, wu, wv, ww``.
    """
    nonhydro = prm.nonhydro
    wh1, wv, wh2 = dt * prm.coriolis
    strat = get_dSdy(S0n, grid)
    Y = Sol["rhoY"] / Sol["rho"]
    nu = -dt ** 2 * (prm.g / prm.Msq) * strat * Y
    denom = 1.0 / (wh1 ** 2 + wh2 ** 2 + (nu + nonhydro) * (wv ** 2 + 1.0))
    c = dict(
        uu=(wh1 ** 2 + nu + nonhydro), uv=nonhydro * (wh1 * wv + wh2), uw=(wh1 * wh2 - (nu + nonhydro) * wv),
        vu=(wh1 * wv - wh2), vv=nonhydro * (1 + wv ** 2), vw=(wh2 * wv + wh1),
        wu=(wh1 * wh2 + (nu + nonhydro) * wv), wv=nonhydro * (wh2 * wv - wh1), ww=(nu + nonhydro + wh2 ** 2))
    return c, denom


def multiply_inverse_coriolis(U, V, W, Sol, S0n, grid, prm, dt):
    """Vector form of ``multiply_inverse_coriolis`` (second_projection.py:604-646)."""
    c, denom = coriolis_coefficients(Sol, S0n, grid, prm, dt)
    U2 = denom * (c["uu"] * U + c["uv"] * V + c["uw"] * W)
    V2 = denom * (c["vu"] * U + c["vv"] * V + c["vw"] * W)
    W2 = denom * (c["wu"] * U + c["wv"] * V + c["ww"] * W)
    return U2, V2, W2


def coriolis_params(Sol, S0n, grid, prm, dt):
    """``get_coeffs=True`` return value (second_projection.py:649-652): transposed cell arrays."""
    c, denom = coriolis_coefficients(Sol, S0n, grid, prm, dt)
    shp = Sol["rho"].shape
    f = lambda a: np.broadcast_to(a * denom, shp).T.copy()
    return (f(c["uu"]), f(c["vv"]), f(c["uv"]), f(c["vu"]))


def grad_nodes(p, dx, dy):
    """2D ``grad_nodes`` (second_projection.py:496-521): cell gradient of a node field."""
    a00 = p[:-1, :-1]   # (slice(0,-1), slice(0,-1))
    a01 = p[:-1, 1:]
    a10 = p[1:, :-1]
    a11 = p[1:, 1:]
    Dpx = 0.0
    Dpy = 0.0
    for s_x, s_y, a in ((-1., -1., a00), (-1., +1., a01), (+1., -1., a10), (+1., +1., a11)):
        Dpx = Dpx + s_x * a
        Dpy = Dpy + s_y * a
    Dpx = Dpx * (0.5 / dx)
    Dpy = Dpy * (0.5 / dy)
    return Dpx, Dpy


def correction_nodes(Sol, p, S0n, grid, prm, dt, updt_chi):
    """``correction_nodes`` (second_projection.py:280-306), 2D; updates ``Sol`` in place."""
    dSdy = get_dSdy(S0n, grid)
    Dpx, Dpy = grad_nodes(p, grid.dx, grid.dy)
    thinv = Sol["rho"] / Sol["rhoY"]
    Y = Sol["rhoY"] / Sol["rho"]
    coeff = prm.Gammainv * Sol["rhoY"] * Y
    u = -dt * coeff * Dpx
    v = -dt * coeff * Dpy
    w = -dt * coeff * 0.0
    u, v, w = multiply_inverse_coriolis(u, v, w, Sol, S0n, grid, prm, dt)
    Sol["rhou"] = Sol["rhou"] + thinv * u
    Sol["rhov"] = Sol["rhov"] + thinv * v
    Sol["rhow"] = Sol["rhow"] + 0.0
    Sol["rhoX"] = Sol["rhoX"] + (-updt_chi * dt * dSdy * Sol["rhov"])
    return u, v, w


def divergence_nodes(Sol, grid):
    """2D ``divergence_nodes`` (second_projection.py:525-575).

    Zeroes the momenta in the two ghost rows of a y-wall in place (:542-551)
    and returns the node.isc divergence.
    """
    if grid.y_wall:
        for k in ("rhou", "rhov", "rhow"):
            Sol[k][:, :2] = 0.0
            Sol[k][:, -2:] = 0.0
    Y = Sol["rhoY"] / Sol["rho"]
    Ux = np.diff(Sol["rhou"] * Y, axis=0) / grid.dx
    Ux = 0.5 * (Ux[:, :-1] + Ux[:, 1:])
    Vy = np.diff(Sol["rhov"] * Y, axis=1) / grid.dy
    Vy = 0.5 * (Vy[:-1, :] + Vy[1:, :])
    return Ux + Vy


def set_ghostnodes_p2(p, grid):
    """``set_ghostnodes_p2`` (boundary.py:296-310) incl. ``periodic_plus_one`` (:348-369)."""
    ig = 2
    for dim in range(2):
        inner = [slice(None)] * 2
        inner[dim] = slice(ig, -ig)
        pad = [(0, 0), (0, 0)]
        pad[dim] = (ig, ig)
        core = p[tuple(inner)]
        if grid.bdry[dim] == PERIODIC:
            q = np.pad(core, pad, mode="constant")
            q = np.moveaxis(q, dim, 0).copy()
            n = q.shape[0]
            head = q[n - 2 * ig - 1:n - ig].copy()
            tail = q[ig:2 * ig + 1].copy()
            q[:ig + 1] = head
            q[n - ig - 1:] = tail
            p[...] = np.moveaxis(q, 0, dim)
        else:
            p[...] = np.pad(core, pad, mode="reflect")
    return p


def set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn):
    """2D ``set_explicit_boundary_data`` (boundary.py:7-132) for gravity along y.

    ``hydro_c`` holds the cell background ``rhoY0`` (``mpv.HydroState``) and
    ``strat_fn`` is ``ud.stratification``.  x is handled by
    ``set_boundary`` (wrap or symmetric, boundary.py:135-216); y (gravity
    axis) by the hydrostatic reflection (boundary.py:56-132).
    """
    ig = 2
    dims = (0, 1)
    for dim in dims:
        inner = [slice(None)] * 2
        inner[dim] = slice(ig, -ig)
        inner = tuple(inner)
        pad = [(0, 0), (0, 0)]
        pad[dim] = (ig, ig)
        g_dim = prm.g if dim == 1 else 0.0
        if g_dim == 0.0:
            bt = grid.bdry[dim]
            if bt == PERIODIC:
                for k in Sol:
                    Sol[k] = np.pad(Sol[k][inner], pad, mode="wrap")
            elif bt == WALL:
                Sol["rho"] = np.pad(Sol["rho"][inner], pad, mode="symmetric")
                Sol["rhov"] = _neg_symmetric(Sol["rhov"][inner], pad, dim)
                Sol["rhou"] = np.pad(Sol["rhou"][inner], pad, mode="symmetric")
                Sol["rhoY"] = np.pad(Sol["rhoY"][inner], pad, mode="symmetric")
                Sol["rhoX"] = np.pad(Sol["rhoX"][inner], pad, mode="symmetric")
            else:
                raise ValueError("Rayleigh boundary not defined on x-direction")
        else:
            _gravity_ghosts(Sol, grid, prm, hydro_c, strat_fn)


def _neg_symmetric(core, pad, dim):
    """``negative_symmetric`` padding (boundary.py:219-245)."""
    q = np.pad(core, pad, mode="constant")
    q = np.moveaxis(q, dim, 0)
    w = pad[dim][0]
    q[:w] = -q[w:2 * w][::-1]
    q[-w:] = -q[-2 * w:-w][::-1]
    return np.moveaxis(q, 0, dim).copy()


def _gravity_ghosts(Sol, grid, prm, hydro_c, strat_fn):
    """Hydrostatic ghost rows along y (boundary.py:56-132, non-Lamb branch)."""
    icy = grid.elem_sc[1]
    igy = 2
    dy = grid.dy
    direction = -1.0
    offset = 0
    for side in (igy, igy):
        direction *= -1
        for cur in range(side)[::-1]:
            # get_gravity_padding (boundary.py:248-281)
            cur_i = cur
            cur_idx = cur + offset * ((icy - 1) - 2 * cur)
            nlast = int(cur_idx + direction)
            nsource = int(offset * icy + direction * (2 * igy - (1 - offset) - cur_i))
            nimage = int(cur_idx)
            Y_last = Sol["rhoY"][:, nlast] / Sol["rho"][:, nlast]
            rhoYv_image = -Sol["rhov"][:, nsource] * Sol["rhoY"][:, nsource] / Sol["rho"][:, nsource]
            S = 1.0 / strat_fn(grid.elem_y[nimage])
            dpi = direction * (prm.Gamma * prm.g) * 0.5 * dy * (1.0 / Y_last + S)
            if prm.is_compressible == 1:
                rhoY = ((Sol["rhoY"][:, nlast] ** prm.gm1) + dpi) ** prm.gm1inv
            else:
                rhoY = hydro_c["rhoY0"][nimage] * np.ones_like(Y_last)
            rho = rhoY * S
            v = rhoYv_image / rhoY
            u = Sol["rhou"][:, nsource] / Sol["rho"][:, nsource]
            w = Sol["rhow"][:, nsource] / Sol["rho"][:, nsource]
            X = Sol["rhoX"][:, nsource] / Sol["rho"][:, nsource]
            Sol["rho"][:, nimage] = rho
            Sol["rhou"][:, nimage] = rho * u * 1.0
            Sol["rhov"][:, nimage] = rho * v
            Sol["rhow"][:, nimage] = rho * w * 1.0
            Sol["rhoY"][:, nimage] = rhoY
            Sol["rhoX"][:, nimage] = rho * X
        offset += 1


# --------------------------------------------------------------------------
# the whole projection (second_projection.py:97-277), 2D, non-Lamb
# --------------------------------------------------------------------------
def projection_operator(Sol_coef, S0n, grid, prm, dt, scaled=True):
    """Coefficients, Coriolis params, diagonal and packed operator of one projection.

    Follows second_projection.py:113-118 (coefficients from ``Sol_coef``),
    :151 (``wcenter *= compressibility`` in the pseudo-incompressible
    regime), :165-175 (Coriolis params, diagonal, packing).
    """
    wplus, wcenter, nu = operator_coefficients_nodes(Sol_coef, S0n, grid, prm, dt)
    if prm.is_compressible == 0:
        wcenter = wcenter * prm.compressibility
    return wplus, wcenter, nu


def impl_part(Sol, p2_nodes, S0n, hydro_c, strat_fn, grid, prm, dt, Sol0=None, solver=None):
    """Restatement of ``euler_backward_non_advective_impl_part`` (second_projection.py:97-277).

    ``Sol`` is a dict of cell arrays and is updated in place (as is
    ``p2_nodes``).  ``solver(op, rhs_inner, tol, maxiter) -> (x, info, niter)``
    defaults to :func:`oracle.krylov.bicgstab_legacy`.  Returns a dict of the
    intermediate fields (rhs, diag_inv, packed operator, solution).
    """
    from oracle.krylov import bicgstab_legacy
    if solver is None:
        solver = bicgstab_legacy
    coefsrc = Sol0 if Sol0 is not None else Sol
    set_explicit_boundary_data(coefsrc, grid, prm, hydro_c, strat_fn)       # :114 / :117
    wplus, wcenter, nu = operator_coefficients_nodes(coefsrc, S0n, grid, prm, dt)  # :115 / :118

    set_ghostnodes_p2(p2_nodes, grid)                                      # :130
    correction_nodes(Sol, p2_nodes, S0n, grid, prm, dt, 0)                 # :131
    set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)          # :132
    rhs = divergence_nodes(Sol, grid)                                      # :134
    rhs = rhs / dt                                                         # :139
    if prm.is_compressible == 1:
        rhs = rhs + 0.0 * (wcenter * p2_nodes[1:-1, 1:-1])                 # :142, :578-601
    else:
        rhs_new = rhs + 0.0 * (wcenter * p2_nodes[1:-1, 1:-1])
        rhs = prm.compressibility * rhs_new + (1.0 - prm.compressibility) * rhs   # :149-150
        wcenter = wcenter * prm.compressibility                            # :151
    mpv_rhs = rhs.copy()                                                   # :158
    cor = coriolis_params(Sol, S0n, grid, prm, dt)                         # :165
    diag_inv = precon_diag_prepare(wplus, wcenter, grid.dx, grid.dy)       # :169
    rhs = rhs * diag_inv                                                   # :170
    op = pack_9pt(wplus, wcenter, cor, diag_inv, grid)                     # :175
    rhs_inner = rhs[1:-1, 1:-1].T.ravel()                                  # :214
    x, info, niter = solver(op, rhs_inner, prm.tol, prm.max_iterations)    # :230
    p2_full = np.zeros(grid.node_sc)
    p2_full[2:-2, 2:-2] = x.reshape(grid.iny, grid.inx).T                  # :245
    set_ghostnodes_p2(p2_full, grid)                                       # :272
    correction_nodes(Sol, p2_full, S0n, grid, prm, dt, 1)                  # :273
    p2_nodes += p2_full                                                    # :275
    set_ghostnodes_p2(p2_nodes, grid)                                      # :276
    set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)          # :277
    return dict(rhs=mpv_rhs, rhs_inner=rhs_inner, diag_inv=diag_inv, op=op, x=x, info=info,
                niter=niter, wplus=wplus, wcenter=wcenter, nu_c=nu)


# --------------------------------------------------------------------------
# explicit parts of the projection (second_projection.py:22-92)
# --------------------------------------------------------------------------
def mod_bg_wind(Sol, wind, fac):
    """``Vars.mod_bg_wind`` (variable.py:109-116)."""
    u0, v0, w0 = wind
    Sol["rhou"] = Sol["rhou"] + fac * u0 * Sol["rho"]
    Sol["rhov"] = Sol["rhov"] + fac * v0 * Sol["rho"]
    Sol["rhow"] = Sol["rhow"] + fac * w0 * Sol["rho"]


def euler_forward_non_advective(Sol, p2, S0c, S0n, grid, prm, dt, hydro_c, strat_fn, wind=(0.0, 0.0, 0.0),
                                is_ArakawaKonor=0):
    """2D ``euler_forward_non_advective`` (second_projection.py:22-74).

    Updates ``Sol`` and ``p2`` in place and returns ``mpv.rhs`` (the node
    divergence, wall rows doubled by ``scale_wall_node_values``, :41-42).
    ``S0c`` is ``mpv.HydroState.get_S0c(elem)`` (cells), ``S0n`` the node
    background of ``mpv.HydroState_n``.
    """
    corr_h1, corr_v, corr_h2 = prm.coriolis
    u0, v0, w0 = wind
    p2n = np.copy(p2)
    dp2n = np.zeros_like(p2n)
    dSdy = get_dSdy(S0n, grid)
    div = divergence_nodes(Sol, grid)                                          # :39
    scale_wall_node_values(div, grid, 2.0)                                     # :40
    rhoY = Sol["rhoY"] ** (prm.gamm - 2.0)                                     # :45-47
    kern = np.ones((2, 2))
    dpidP = (prm.gm1 / prm.Msq) * fftconvolve(rhoY, kern, mode="valid") / kern.sum()
    rhoYovG = prm.Gammainv * Sol["rhoY"]                                       # :49
    dbuoy = Sol["rhoY"] * (Sol["rhoX"] / Sol["rho"])
    dpdx, dpdy = grad_nodes(p2n, grid.dx, grid.dy)                             # :51
    drhou = Sol["rhou"] - u0 * Sol["rho"]                                      # :53-56
    drhov = Sol["rhov"] - v0 * Sol["rho"]
    drhow = Sol["rhow"] - w0 * Sol["rho"]
    v = Sol["rhov"] / Sol["rho"]
    Sol["rhou"] = Sol["rhou"] - dt * (rhoYovG * dpdx - corr_h2 * drhov + corr_v * drhow)          # :58
    Sol["rhov"] = Sol["rhov"] - dt * (rhoYovG * dpdy + (prm.g / prm.Msq) * dbuoy * prm.nonhydro
                                      - corr_h1 * drhow + corr_h2 * drhou) * (1 - is_ArakawaKonor)  # :60
    # :62 is multiplied by (ndim == 3): rhow is unchanged in 2D
    Sol["rhoX"] = (Sol["rho"] * (Sol["rho"] / Sol["rhoY"] - S0c)) - dt * (v * dSdy) * Sol["rho"]  # :64
    dp2n[1:-1, 1:-1] -= dt * dpidP * div                                       # :66
    p2 += prm.compressibility * dp2n                                           # :68-69
    set_ghostnodes_p2(p2, grid)                                                # :71
    set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)              # :72
    return div


def euler_backward_non_advective_expl_part(Sol, S0n, grid, prm, dt, hydro_c, strat_fn, wind=(0.0, 0.0, 0.0)):
    """``euler_backward_non_advective_expl_part`` (second_projection.py:77-92); updates ``Sol``."""
    dbuoy = Sol["rhoY"] * (Sol["rhoX"] / Sol["rho"])                           # :82
    Sol["rhov"] = (prm.nonhydro * Sol["rhov"]) - dt * (prm.g / prm.Msq) * dbuoy  # :83
    mod_bg_wind(Sol, wind, -1.0)                                               # :86
    U, V, W = multiply_inverse_coriolis(Sol["rhou"], Sol["rhov"], Sol["rhow"], Sol, S0n, grid, prm, dt)  # :88
    Sol["rhou"], Sol["rhov"], Sol["rhow"] = U, V, W
    mod_bg_wind(Sol, wind, +1.0)                                               # :90
    set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)              # :92
