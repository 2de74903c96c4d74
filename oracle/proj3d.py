"""FP64 NumPy restatement of the reference's 3D projection pieces, and the 3D
projection step assembled from them (oracle; tests only).

The pieces of ``euler_backward_non_advective_impl_part`` are dimension-generic
in the reference and run in 3D; tests/golden/make_golden.py records them on a
small 3D state (``proj3d_kat.npz``) and tests/test_oracle_golden.py pins each
function below against them:

* ``set_explicit_boundary_data`` (boundary.py:7-216): wrap / symmetric along x
  and z, hydrostatic reflection along y (gravity);
* ``operator_coefficients_nodes`` (second_projection.py:308-356): ``wplus`` on
  all three axes, ``wcenter`` = 2x2x2 box of ``rhoY^(2-gamma)`` / 8, wall rows
  halved (``scale_wall_node_values``);
* ``divergence_nodes`` (:525-575), 3D branch -- including the reference's
  ``Ux = -0.5 * (...)`` (:563), which flips the sign of the x term in 3D;
* ``grad_nodes`` (:496-521) and ``correction_nodes`` (:280-306) with the
  3D ``multiply_inverse_coriolis`` (:604-646) and ``get_dSdy`` (variable.py:162-177);
* ``set_ghostnodes_p2`` (boundary.py:296-310, ``periodic_plus_one`` :348-369).

The step itself cannot run in the reference (second_projection.py:183-203 use
``diag_inv`` and ``p2`` before assignment, ``stencil_27pt`` slices cell
arrays one plane short of ``lap3D``'s, and ``rhs_from_p_old`` adds a node.isc
array to a node.sc one).  ``impl_part`` below assembles it with the
conventions of the reference's working 2D branch: unknowns are the inner nodes
``node.i2``, ``hplus`` the cells around them, ``hcenter`` and ``diag_inv``
(the 3D ``precon_diag_prepare``) at those nodes, the right-hand side the
divergence on node.isc scaled by ``1/dt`` and ``diag_inv``, the vector in C
order over (x, y, z) (second_projection.py:224), and ``corrf =
dt * coriolis_strength[0]`` (laplacian.py:894).
"""
import numpy as np
from scipy.signal import fftconvolve

from oracle import nodal3d as n3
from oracle.nodal2d import PERIODIC, RAYLEIGH, WALL, scale_wall_node_values


class Grid3D:
    """Cell and node grid sizes of ``grid.py`` for a 3D domain (two ghost layers)."""

    def __init__(self, inx, iny, inz, xmin, xmax, ymin, ymax, zmin, zmax, bdry=(PERIODIC, WALL, PERIODIC)):
        ig = 2
        self.inx, self.iny, self.inz = inx, iny, inz
        self.dx = (xmax - xmin) / (inx - 1.0)
        self.dy = (ymax - ymin) / (iny - 1.0)
        self.dz = (zmax - zmin) / (inz - 1.0)
        self.igs = (ig, ig, ig)
        self.elem_sc = (inx - 1 + 2 * ig, iny - 1 + 2 * ig, inz - 1 + 2 * ig)
        self.node_sc = (inx + 2 * ig, iny + 2 * ig, inz + 2 * ig)
        self.node_isc = (inx + ig, iny + ig, inz + ig)
        self.elem_y = ymin - ig * self.dy + 0.5 * self.dy + self.dy * np.arange(self.elem_sc[1])
        self.bdry = tuple(bdry)

    def wall(self, dim):
        return self.bdry[dim] in (WALL, RAYLEIGH)


def get_dSdy(S0n, grid):
    """Cell field ``dS/dy`` (variable.py:162-177): node differences along y, repeated along x and z."""
    d = (S0n[1:] - S0n[:-1]) / grid.dy
    return np.broadcast_to(d[None, :, None], grid.elem_sc).copy()


def operator_coefficients_nodes(Sol, S0n, grid, prm, dt):
    """3D ``operator_coefficients_nodes`` (second_projection.py:308-356): ``(wplus, wcenter, nu)``."""
    ccenter = -prm.Msq * prm.gm1inv / dt ** 2
    cexp = 2.0 - prm.gamm
    strat = get_dSdy(S0n, grid)
    Y = Sol["rhoY"] / Sol["rho"]
    coeff = prm.Gammainv * Sol["rhoY"] * Y
    nu = -dt ** 2 * (prm.g / prm.Msq) * strat * Y
    wplus = np.stack([coeff, coeff, coeff])
    kernel = np.ones((2, 2, 2))
    wcenter = ccenter * fftconvolve(Sol["rhoY"] ** cexp, kernel, mode="valid") / kernel.sum()
    scale_wall_node_values(wcenter, grid, 0.5)
    return wplus, wcenter, nu


def divergence_nodes(Sol, grid, x_sign=-1.0):
    """3D ``divergence_nodes`` (second_projection.py:525-575) on a node.sc array.

    Zeroes the momenta in the two ghost rows of a y wall in place (:542-551).
    The x term carries the reference's 3D sign, ``Ux = -0.5 * (...)`` (:563),
    unless ``x_sign = +1``: the sign of the 2D branch, with which the 3D time step
    stays bounded (with the reference's sign it blows up within a few steps,
    tests/test_oracle_3d.py).
    """
    if grid.wall(1):
        for k in ("rhou", "rhov", "rhow"):
            Sol[k][:, :2, ...] = 0.0
            Sol[k][:, -2:, ...] = 0.0
    Y = Sol["rhoY"] / Sol["rho"]
    Ux = np.diff(Sol["rhou"] * Y, axis=0) / grid.dx
    Ux = 0.5 * (Ux[:, :-1, ...] + Ux[:, 1:, ...])
    Vy = np.diff(Sol["rhov"] * Y, axis=1) / grid.dy
    Vy = 0.5 * (Vy[:-1, ...] + Vy[1:, ...])
    Ux = (0.5 * x_sign) * (Ux[..., :-1] + Ux[..., 1:])
    Vy = 0.5 * (Vy[..., :-1] + Vy[..., 1:])
    Wz = np.diff(Sol["rhow"] * Y, axis=2) / grid.dz
    Wz = 0.5 * (Wz[:-1, ...] + Wz[1:, ...])
    Wz = 0.5 * (Wz[:, :-1, ...] + Wz[:, 1:, ...])
    rhs = np.zeros(grid.node_sc)
    rhs[1:-1, 1:-1, 1:-1] = (Ux + Vy + Wz)
    return rhs


def grad_nodes(p, dx, dy, dz):
    """3D ``grad_nodes`` (second_projection.py:496-521): cell gradient from the 8 corner nodes."""
    lo, hi = slice(0, -1), slice(1, None)
    corners = [(a, b, c) for a in (lo, hi) for b in (lo, hi) for c in (lo, hi)]
    sx = (-1., -1., -1., -1., +1., +1., +1., +1.)
    sy = (-1., -1., +1., +1., -1., -1., +1., +1.)
    sz = (-1., +1., -1., +1., -1., +1., -1., +1.)
    Dpx, Dpy, Dpz = 0., 0., 0.
    for n, idx in enumerate(corners):
        Dpx = Dpx + sx[n] * p[idx]
        Dpy = Dpy + sy[n] * p[idx]
        Dpz = Dpz + sz[n] * p[idx]
    Dpx = Dpx * (0.5 ** 2 / dx)
    Dpy = Dpy * (0.5 ** 2 / dy)
    Dpz = Dpz * (0.5 ** 2 / dz)
    return Dpx, Dpy, Dpz


def multiply_inverse_coriolis(U, V, W, Sol, S0n, grid, prm, dt):
    """``multiply_inverse_coriolis`` (second_projection.py:604-646) with the 3D ``dS/dy``."""
    nonhydro = prm.nonhydro
    wh1, wv, wh2 = dt * prm.coriolis
    strat = get_dSdy(S0n, grid)
    Y = Sol["rhoY"] / Sol["rho"]
    nu = -dt ** 2 * (prm.g / prm.Msq) * strat * Y
    denom = 1.0 / (wh1 ** 2 + wh2 ** 2 + (nu + nonhydro) * (wv ** 2 + 1.0))
    uu, uv, uw = (wh1 ** 2 + nu + nonhydro), nonhydro * (wh1 * wv + wh2), (wh1 * wh2 - (nu + nonhydro) * wv)
    vu, vv, vw = (wh1 * wv - wh2), nonhydro * (1 + wv ** 2), (wh2 * wv + wh1)
    wu, wv_, ww = (wh1 * wh2 + (nu + nonhydro) * wv), nonhydro * (wh2 * wv - wh1), (nu + nonhydro + wh2 ** 2)
    U2 = denom * (uu * U + uv * V + uw * W)
    V2 = denom * (vu * U + vv * V + vw * W)
    W2 = denom * (wu * U + wv_ * V + ww * W)
    return U2, V2, W2


def correction_nodes(Sol, p, S0n, grid, prm, dt, updt_chi):
    """3D ``correction_nodes`` (second_projection.py:280-306); updates ``Sol`` in place."""
    dSdy = get_dSdy(S0n, grid)
    Dpx, Dpy, Dpz = grad_nodes(p, grid.dx, grid.dy, grid.dz)
    thinv = Sol["rho"] / Sol["rhoY"]
    Y = Sol["rhoY"] / Sol["rho"]
    coeff = prm.Gammainv * Sol["rhoY"] * Y
    u = -dt * coeff * Dpx
    v = -dt * coeff * Dpy
    w = -dt * coeff * Dpz
    u, v, w = multiply_inverse_coriolis(u, v, w, Sol, S0n, grid, prm, dt)
    Sol["rhou"] = Sol["rhou"] + thinv * u
    Sol["rhov"] = Sol["rhov"] + thinv * v
    Sol["rhow"] = Sol["rhow"] + thinv * w
    Sol["rhoX"] = Sol["rhoX"] + (-updt_chi * dt * dSdy * Sol["rhov"])
    return u, v, w


def _axis_pad(core, dim, ig):
    pad = [(0, 0)] * core.ndim
    pad[dim] = (ig, ig)
    return pad


def set_ghostnodes_p2(p, grid):
    """``set_ghostnodes_p2`` (boundary.py:296-310): ``periodic_plus_one`` (:348-369) or
    ``reflect`` along each axis in turn."""
    ig = 2
    for dim in range(3):
        inner = [slice(None)] * 3
        inner[dim] = slice(ig, -ig)
        core = p[tuple(inner)]
        if grid.bdry[dim] == PERIODIC:
            q = np.moveaxis(np.pad(core, _axis_pad(core, dim, ig), mode="constant"), dim, 0).copy()
            n = q.shape[0]
            head = q[n - 2 * ig - 1:n - ig].copy()
            tail = q[ig:2 * ig + 1].copy()
            q[:ig + 1] = head
            q[n - ig - 1:] = tail
            p[...] = np.moveaxis(q, 0, dim)
        else:
            p[...] = np.pad(core, _axis_pad(core, dim, ig), mode="reflect")
    return p


def _neg_symmetric(core, dim, ig):
    """``negative_symmetric`` padding (boundary.py:219-245) along ``dim``."""
    q = np.moveaxis(np.pad(core, _axis_pad(core, dim, ig), mode="constant"), dim, 0).copy()
    q[:ig] = -q[ig:2 * ig][::-1]
    q[-ig:] = -q[-2 * ig:-ig][::-1]
    return np.moveaxis(q, 0, dim).copy()


def set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn):
    """3D ``set_explicit_boundary_data`` (boundary.py:7-216), gravity along y.

    x and z: ``set_boundary`` with 'wrap' (periodic) or 'symmetric' (wall:
    ``rhov`` negative-symmetric, ``rhow`` left as it is, boundary.py:156-166);
    y: the hydrostatic reflection (boundary.py:56-132, non-Lamb branch).
    """
    ig = 2
    for dim in range(3):
        if dim == 1 and prm.g != 0.0:
            _gravity_ghosts(Sol, grid, prm, hydro_c, strat_fn)
            continue
        inner = [slice(None)] * 3
        inner[dim] = slice(ig, -ig)
        inner = tuple(inner)
        if grid.bdry[dim] == PERIODIC:
            for k in Sol:
                Sol[k] = np.pad(Sol[k][inner], _axis_pad(Sol[k][inner], dim, ig), mode="wrap")
        elif grid.bdry[dim] == WALL:
            sym = lambda a: np.pad(a[inner], _axis_pad(a[inner], dim, ig), mode="symmetric")
            Sol["rho"] = sym(Sol["rho"])
            Sol["rhov"] = _neg_symmetric(Sol["rhov"][inner], dim, ig)
            Sol["rhou"] = sym(Sol["rhou"])
            Sol["rhoY"] = sym(Sol["rhoY"])
            Sol["rhoX"] = sym(Sol["rhoX"])
        else:
            raise ValueError("Rayleigh boundary not defined off the gravity axis")


def _gravity_ghosts(Sol, grid, prm, hydro_c, strat_fn):
    """Hydrostatic ghost planes along y (boundary.py:56-132 with get_gravity_padding :248-281)."""
    icy = grid.elem_sc[1]
    igy = 2
    direction = -1.0
    offset = 0
    for side in (igy, igy):
        direction *= -1
        for cur in range(side)[::-1]:
            cur_idx = cur + offset * ((icy - 1) - 2 * cur)
            nlast = int(cur_idx + direction)
            nsource = int(offset * icy + direction * (2 * igy - (1 - offset) - cur))
            nimage = int(cur_idx)
            at = lambda k, j: Sol[k][:, j, :]
            Y_last = at("rhoY", nlast) / at("rho", nlast)
            rhoYv_image = -at("rhov", nsource) * at("rhoY", nsource) / at("rho", nsource)
            S = 1.0 / strat_fn(grid.elem_y[nimage])
            dpi = direction * (prm.Gamma * prm.g) * 0.5 * grid.dy * (1.0 / Y_last + S)
            if prm.is_compressible == 1:
                rhoY = ((at("rhoY", nlast) ** prm.gm1) + dpi) ** prm.gm1inv
            else:
                rhoY = hydro_c["rhoY0"][nimage] * np.ones_like(Y_last)
            rho = rhoY * S
            v = rhoYv_image / rhoY
            u = at("rhou", nsource) / at("rho", nsource)
            w = at("rhow", nsource) / at("rho", nsource)
            X = at("rhoX", nsource) / at("rho", nsource)
            Sol["rho"][:, nimage, :] = rho
            Sol["rhou"][:, nimage, :] = rho * u * 1.0
            Sol["rhov"][:, nimage, :] = rho * v
            Sol["rhow"][:, nimage, :] = rho * w * 1.0
            Sol["rhoY"][:, nimage, :] = rhoY
            Sol["rhoX"][:, nimage, :] = rho * X
        offset += 1


def impl_part(Sol, p2_nodes, S0n, hydro_c, strat_fn, grid, prm, dt, Sol0=None, solver=None, x_sign=-1.0):
    """The 3D projection step from the pinned pieces, with the glue of the 2D branch.

    Same order as second_projection.py:113-277.  ``Sol`` (dict of cell arrays)
    and ``p2_nodes`` are updated in place.  ``solver(op, b, tol, maxiter) ->
    (x, info, niter)`` defaults to :func:`oracle.krylov.bicgstab_legacy`.
    """
    from oracle.krylov import bicgstab_legacy
    if solver is None:
        solver = bicgstab_legacy
    coefsrc = Sol0 if Sol0 is not None else Sol
    set_explicit_boundary_data(coefsrc, grid, prm, hydro_c, strat_fn)        # :114 / :117
    wplus, wcenter, nu = operator_coefficients_nodes(coefsrc, S0n, grid, prm, dt)   # :115 / :118
    set_ghostnodes_p2(p2_nodes, grid)                                       # :130
    correction_nodes(Sol, p2_nodes, S0n, grid, prm, dt, 0)                  # :131
    set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)           # :132
    rhs = divergence_nodes(Sol, grid, x_sign)[1:-1, 1:-1, 1:-1]             # :134, on node.isc
    rhs = rhs / dt                                                          # :139
    i1 = (slice(1, -1),) * 3
    if prm.is_compressible == 1:
        rhs = rhs + 0.0 * (wcenter * p2_nodes[i1])                          # :142, :578-601
    else:
        rhs_new = rhs + 0.0 * (wcenter * p2_nodes[i1])
        rhs = prm.compressibility * rhs_new + (1.0 - prm.compressibility) * rhs   # :149-150
        wcenter = wcenter * prm.compressibility                             # :151
    mpv_rhs = rhs.copy()                                                    # :158
    diag_inv = n3.precon_diag_3d(wplus[0], wplus[1], wplus[2], wcenter, grid.dx, grid.dy, grid.dz)
    rhs = rhs * diag_inv
    op = n3.pack_27pt(wplus[0][i1], wplus[1][i1], wplus[2][i1], wcenter[i1], diag_inv[i1],
                      grid.inx, grid.iny, grid.inz, grid.dx, grid.dy, grid.dz,
                      walls=tuple(grid.wall(d) for d in range(3)), corrf=dt * prm.coriolis[0])
    b = rhs[i1].ravel()                                                     # :224
    x, info, niter = solver(op, b, prm.tol, prm.max_iterations)            # :230
    p2_full = np.zeros(grid.node_sc)
    p2_full[2:-2, 2:-2, 2:-2] = x.reshape(grid.inx, grid.iny, grid.inz)     # :265-266
    set_ghostnodes_p2(p2_full, grid)                                        # :272
    correction_nodes(Sol, p2_full, S0n, grid, prm, dt, 1)                   # :273
    p2_nodes += p2_full                                                     # :275
    set_ghostnodes_p2(p2_nodes, grid)                                       # :276
    set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)           # :277
    return dict(rhs=mpv_rhs, b=b, diag_inv=diag_inv, op=op, x=x, info=info, niter=niter,
                wplus=wplus, wcenter=wcenter, nu_c=nu)


# --------------------------------------------------------------------------
# explicit parts of the projection (second_projection.py:22-92), 3D
# --------------------------------------------------------------------------
def mod_bg_wind(Sol, wind, fac):
    """``Vars.mod_bg_wind`` (variable.py:109-116)."""
    u0, v0, w0 = wind
    Sol["rhou"] = Sol["rhou"] + fac * u0 * Sol["rho"]
    Sol["rhov"] = Sol["rhov"] + fac * v0 * Sol["rho"]
    Sol["rhow"] = Sol["rhow"] + fac * w0 * Sol["rho"]


def euler_backward_non_advective_expl_part(Sol, S0n, grid, prm, dt, hydro_c, strat_fn, wind=(0.0, 0.0, 0.0)):
    """``euler_backward_non_advective_expl_part`` (second_projection.py:77-92) in 3D;
    updates ``Sol``.  Dimension-generic in the reference; pinned by proj3d_kat.npz."""
    dbuoy = Sol["rhoY"] * (Sol["rhoX"] / Sol["rho"])                        # :82
    Sol["rhov"] = (prm.nonhydro * Sol["rhov"]) - dt * (prm.g / prm.Msq) * dbuoy  # :83
    mod_bg_wind(Sol, wind, -1.0)                                             # :86
    U, V, W = multiply_inverse_coriolis(Sol["rhou"], Sol["rhov"], Sol["rhow"], Sol, S0n, grid, prm, dt)  # :88
    Sol["rhou"], Sol["rhov"], Sol["rhow"] = U, V, W
    mod_bg_wind(Sol, wind, +1.0)                                             # :90
    set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)            # :92


def euler_forward_non_advective(Sol, p2, S0c, S0n, grid, prm, dt, hydro_c, strat_fn, wind=(0.0, 0.0, 0.0),
                                is_ArakawaKonor=0, x_sign=-1.0):
    """``euler_forward_non_advective`` (second_projection.py:22-74) in 3D with the
    2D branch's glue: the divergence on node.isc (the reference's 3D call writes
    divergence_nodes' node.sc result into the node.isc ``mpv.rhs`` and cannot
    run), wall rows doubled there, ``dp2n[node.i1] -= dt * dpidP * div``.
    Updates ``Sol`` and ``p2`` in place; returns the divergence (``mpv.rhs``)."""
    corr_h1, corr_v, corr_h2 = prm.coriolis
    u0, v0, w0 = wind
    p2n = np.copy(p2)
    dp2n = np.zeros_like(p2n)
    dSdy = get_dSdy(S0n, grid)
    div = divergence_nodes(Sol, grid, x_sign)[1:-1, 1:-1, 1:-1]               # :39
    scale_wall_node_values(div, grid, 2.0)                                   # :40
    rhoY = Sol["rhoY"] ** (prm.gamm - 2.0)                                   # :45-47
    kern = np.ones((2, 2, 2))
    dpidP = (prm.gm1 / prm.Msq) * fftconvolve(rhoY, kern, mode="valid") / kern.sum()
    rhoYovG = prm.Gammainv * Sol["rhoY"]                                     # :49
    dbuoy = Sol["rhoY"] * (Sol["rhoX"] / Sol["rho"])
    dpdx, dpdy, dpdz = grad_nodes(p2n, grid.dx, grid.dy, grid.dz)            # :51
    drhou = Sol["rhou"] - u0 * Sol["rho"]                                    # :53-56
    drhov = Sol["rhov"] - v0 * Sol["rho"]
    drhow = Sol["rhow"] - w0 * Sol["rho"]
    v = Sol["rhov"] / Sol["rho"]
    Sol["rhou"] = Sol["rhou"] - dt * (rhoYovG * dpdx - corr_h2 * drhov + corr_v * drhow)          # :58
    Sol["rhov"] = Sol["rhov"] - dt * (rhoYovG * dpdy + (prm.g / prm.Msq) * dbuoy * prm.nonhydro
                                      - corr_h1 * drhow + corr_h2 * drhou) * (1 - is_ArakawaKonor)  # :60
    Sol["rhow"] = Sol["rhow"] - dt * (rhoYovG * dpdz - corr_v * drhou + corr_h1 * drhov) * True     # :62
    Sol["rhoX"] = (Sol["rho"] * (Sol["rho"] / Sol["rhoY"] - S0c)) - dt * (v * dSdy) * Sol["rho"]  # :64
    dp2n[1:-1, 1:-1, 1:-1] -= dt * dpidP * div                               # :66
    p2 += prm.compressibility * dp2n                                         # :68-69
    set_ghostnodes_p2(p2, grid)                                              # :71
    set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)            # :72
    return div
