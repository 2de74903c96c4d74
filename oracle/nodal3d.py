"""FP64 NumPy restatement of the reference's 3D 27-point nodal operator (oracle; tests only).

Pinned against the reference itself: ``lap3D`` (laplacian.py:898-1026) is a
pure function of its operands, so tests/golden/make_golden.py calls it on
random operands (periodic/wall mixes, Coriolis cross terms) and
tests/test_oracle_golden.py checks that ``lap3d`` below reproduces its inner
nodes bit for bit, and ``precon_diag_3d`` its 3D ``precon_diag_prepare``.
What cannot be pinned is the 3D projection glue, which cannot run as shipped
(second_projection.py:183-203 uses ``diag_inv`` and ``p2`` before
assignment); this module defines it with the conventions of the reference's
working 2D path (laplacian.py:546-746): the unknowns are the inner nodes, a
periodic axis wraps with the duplicated seam (wrap distance n-1), a wall
zeroes the ``hplus`` of the outer cell planes (laplacian.py:933-965).  Two
properties of ``lap3D`` the glue leaves behind: it takes the vector with a
one-node halo and returns zeros on that shell, and along a periodic axis it
overwrites inner node 0 with inner node n-1 before differencing
(laplacian.py:927-960), so it equals ``lap3d`` on vectors whose duplicated
seam values agree.  ``lap3D`` reshapes its vector as (z, y, x) but indexes
its coefficients (x, y, z), consistent only for nx == nz (laplacian.py:901);
vector order here is C order over (x, y, z), z fastest
(second_projection.py:224).
"""
import numpy as np

from oracle.nodal2d import _wrap_index, box3


def pack_27pt(hplusx, hplusy, hplusz, hcenter, diag_inv, nx, ny, nz, dx, dy, dz,
              walls=(False, True, True), corrf=0.0):
    """Operands of the 3D operator: cells (nx+1, ny+1, nz+1), nodes (nx, ny, nz), flat C order."""
    return dict(hplusx=np.asarray(hplusx, np.float64).reshape(-1), hplusy=np.asarray(hplusy, np.float64).reshape(-1),
                hplusz=np.asarray(hplusz, np.float64).reshape(-1),
                hcenter=np.asarray(hcenter, np.float64).reshape(-1),
                diag_inv=np.asarray(diag_inv, np.float64).reshape(-1),
                nx=int(nx), ny=int(ny), nz=int(nz), dx=float(dx), dy=float(dy), dz=float(dz),
                walls=tuple(bool(w) for w in walls), corrf=float(corrf))


def _pad(P):
    """Inner nodes (nx,ny,nz) -> one-node halo with the duplicated-seam wrap."""
    nx, ny, nz = P.shape
    lo = [_wrap_index(n)[0][0] for n in (nx, ny, nz)]
    hi = [_wrap_index(n)[1][-1] for n in (nx, ny, nz)]
    ix = np.r_[lo[0], np.arange(nx), hi[0]]
    iy = np.r_[lo[1], np.arange(ny), hi[1]]
    iz = np.r_[lo[2], np.arange(nz), hi[2]]
    return P[np.ix_(ix, iy, iz)]


def lap3d(p, op):
    """27-point operator of lap3D (laplacian.py:898-1026) on the inner nodes."""
    nx, ny, nz = op["nx"], op["ny"], op["nz"]
    P = np.asarray(p, np.float64).reshape(nx, ny, nz)
    U = _pad(P)                                                   # (nx+2, ny+2, nz+2)
    shp = (nx + 1, ny + 1, nz + 1)
    hx = op["hplusx"].reshape(shp).copy()
    hy = op["hplusy"].reshape(shp).copy()
    hz = op["hplusz"].reshape(shp).copy()
    for axis, wall in enumerate(op["walls"]):                     # laplacian.py:933-965
        if wall:
            for h in (hx, hy, hz):
                idx = [slice(None)] * 3
                idx[axis] = 0
                h[tuple(idx)] = 0.0
                idx[axis] = -1
                h[tuple(idx)] = 0.0
    # edge differences (laplacian.py:968-981)
    z_fluxes = U[:, :, 1:] - U[:, :, :-1]
    y_fluxes = U[:, 1:, :] - U[:, :-1, :]
    x_fluxes = U[1:, :, :] - U[:-1, :, :]
    # four-edge sums per cell (laplacian.py:983-985; corner slices :907-923)
    x_flx = x_fluxes[:, :-1, :-1] + x_fluxes[:, :-1, 1:] + x_fluxes[:, 1:, :-1] + x_fluxes[:, 1:, 1:]
    y_flx = y_fluxes[:-1, :, :-1] + y_fluxes[1:, :, :-1] + y_fluxes[:-1, :, 1:] + y_fluxes[1:, :, 1:]
    z_flx = z_fluxes[:-1, :-1, :] + z_fluxes[:-1, 1:, :] + z_fluxes[1:, :-1, :] + z_fluxes[1:, 1:, :]

    def sum_x(c):    # four cells in the (y,z) plane around each node, cells shifted in x already
        return c[:, :-1, :-1] + c[:, :-1, 1:] + c[:, 1:, :-1] + c[:, 1:, 1:]

    def sum_y(c):
        return c[:-1, :, :-1] + c[1:, :, :-1] + c[:-1, :, 1:] + c[1:, :, 1:]

    def sum_z(c):
        return c[:-1, :-1, :] + c[:-1, 1:, :] + c[1:, :-1, :] + c[1:, 1:, :]

    hxzp = hx * z_flx                                             # laplacian.py:987-991
    hxzpm = sum_x(hxzp[:-1, :, :])
    hxzpp = sum_x(hxzp[1:, :, :])
    hzxp = hz * x_flx                                             # :993-997
    hzxpm = sum_z(hzxp[:, :, :-1])
    hzxpp = sum_z(hzxp[:, :, 1:])
    x_flx = hx * x_flx                                            # :999-1003
    x_flxm = sum_x(x_flx[:-1, :, :])
    x_flxp = sum_x(x_flx[1:, :, :])
    y_flx = hy * y_flx                                            # :1005-1009
    y_flxm = sum_y(y_flx[:, :-1, :])
    y_flxp = sum_y(y_flx[:, 1:, :])
    z_flx = hz * z_flx                                            # :1011-1015
    z_flxm = sum_z(z_flx[:, :, :-1])
    z_flxp = sum_z(z_flx[:, :, 1:])
    coeff = 1.0 / 16
    oodx2, oody2, oodz2 = 1.0 / op["dx"] ** 2, 1.0 / op["dy"] ** 2, 1.0 / op["dz"] ** 2
    odx, odz = 1.0 / op["dx"], 1.0 / op["dz"]
    corrf = op["corrf"]
    hc = op["hcenter"].reshape(nx, ny, nz)
    lap = oodx2 * coeff * (-x_flxm + x_flxp) + \
        oody2 * coeff * (-y_flxm + y_flxp) + \
        oodz2 * coeff * (-z_flxm + z_flxp) + \
        +1.0 * odx * odz * coeff * corrf * (hxzpp - hxzpm) + \
        -1.0 * odx * odz * coeff * corrf * (hzxpp - hzxpm) + \
        hc * P                                                    # :1017-1022
    lap = lap * op["diag_inv"].reshape(nx, ny, nz)                # :1024
    return lap.reshape(-1)


def precon_diag_3d(hplusx, hplusy, hplusz, hcenter, dx, dy, dz):
    """3D branch of ``precon_diag_prepare`` (laplacian.py:1284-1356) on inner cells/nodes.

    coeff = 0.0625; the x-y cross terms of the reference (``wxy``/``wyx`` with
    ``hplusx``/``hplusy``, :1348-1349) are kept as the reference computes them.
    """
    c = 0.0625
    Sx, Sy, Sz = box3(hplusx), box3(hplusy), box3(hplusz)
    diag = -(c / dx ** 2) * Sx
    diag = diag - (c / dy ** 2) * Sy
    diag = diag - (c / (dx * dy)) * Sx
    diag = diag - (c / (dy * dx)) * Sy
    diag = diag - (c / dz ** 2) * Sz
    diag = diag + hcenter
    return 1.0 / diag


def node_divergence(Fx, Fy, Fz, walls):
    """Nodal divergence of cell fluxes with the operator's own node sums.

    b = sum over the four cells on the + side minus the four on the - side,
    per axis (the node-sum step of lap3D, laplacian.py:999-1015).  Any b of
    this form lies in the range of the 27-point operator, whose null space
    (constants and the hourglass modes f(i)(-1)^(j+k), g(j)(-1)^(i+k),
    h(k)(-1)^(i+j)) it is orthogonal to; wall cell planes carry no flux.
    Fx, Fy, Fz have shape (nx+1, ny+1, nz+1); returns (nx, ny, nz).
    """
    F = [np.array(f, np.float64) for f in (Fx, Fy, Fz)]
    for axis, wall in enumerate(walls):
        if wall:
            for f in F:
                idx = [slice(None)] * 3
                idx[axis] = 0
                f[tuple(idx)] = 0.0
                idx[axis] = -1
                f[tuple(idx)] = 0.0
    fx, fy, fz = F
    xs = (fx[1:, :-1, :-1] + fx[1:, :-1, 1:] + fx[1:, 1:, :-1] + fx[1:, 1:, 1:]) - \
         (fx[:-1, :-1, :-1] + fx[:-1, :-1, 1:] + fx[:-1, 1:, :-1] + fx[:-1, 1:, 1:])
    ys = (fy[:-1, 1:, :-1] + fy[1:, 1:, :-1] + fy[:-1, 1:, 1:] + fy[1:, 1:, 1:]) - \
         (fy[:-1, :-1, :-1] + fy[1:, :-1, :-1] + fy[:-1, :-1, 1:] + fy[1:, :-1, 1:])
    zs = (fz[:-1, :-1, 1:] + fz[:-1, 1:, 1:] + fz[1:, :-1, 1:] + fz[1:, 1:, 1:]) - \
         (fz[:-1, :-1, :-1] + fz[:-1, 1:, :-1] + fz[1:, :-1, :-1] + fz[1:, 1:, :-1])
    return xs + ys + zs
