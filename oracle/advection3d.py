"""FP64 NumPy restatement of the reference's 3D advection (oracle; tests only).

The same routines as oracle/advection2d.py in three dimensions: face mass fluxes
with the 2x3x3 weighted boxes of ``recompute_advective_fluxes``
(numerical_flux.py:5-46, 3D branch), Strang-split ``advect`` (explicit.py:5-74)
and first-order ``advect_rk`` (explicit.py:160-257) whose sweeps rotate the
arrays with ``Vars.flip_forward`` / ``flip_backward`` (variable.py:89-97:
moveaxis 0 -> -1 and back, so the sweep axis is last: x in (y, z, x), y in
(z, x, y), z in (x, y, z)).  Recovery, upwind flux and update are
oracle/advection2d.py's, which work along the last axis in any dimension.
Boundary data along a sweep follows boundary.py:7-216 with ``step``: the sweep
axis is padded, with the hydrostatic reflection when it is y (gravity).
Pinned bit for bit against the reference (tests/golden/advect3d_kat.npz).
"""
import numpy as np
from scipy.signal import fftconvolve

from oracle import proj3d as o3
from oracle.advection2d import FIELDS, _hll, _recovery, _update
from oracle.nodal2d import PERIODIC, WALL


def recompute_advective_fluxes(Sol, flux):
    """Face mass fluxes rhoY u, rhoY v, rhoY w in place (numerical_flux.py:5-46, 3D)."""
    inner = (slice(1, -1),) * 3
    kernel_u = np.array([[[1, 2, 1], [2, 4, 2], [1, 2, 1]], [[1, 2, 1], [2, 4, 2], [1, 2, 1]]])
    kernel_v = np.swapaxes(kernel_u, 1, 0)
    kernel_w = np.swapaxes(kernel_u, 2, 0)
    rhoYw = Sol["rhoY"] * Sol["rhow"] / Sol["rho"]
    flux[2]["rhoY"][inner] = fftconvolve(rhoYw, kernel_w, mode="valid") / kernel_w.sum()
    rhoYu = Sol["rhoY"] * Sol["rhou"] / Sol["rho"]
    flux[0]["rhoY"][inner] = np.moveaxis(fftconvolve(rhoYu, kernel_u, mode="valid") / kernel_u.sum(), 0, -1)
    rhoYv = Sol["rhoY"] * Sol["rhov"] / Sol["rho"]
    flux[1]["rhoY"][inner] = np.moveaxis(fftconvolve(rhoYv, kernel_v, mode="valid") / kernel_v.sum(), -1, 0)


def new_flux(grid):
    """Zeroed face containers ``elem.sfx = (icy, icz, icx+1)``, ``sfy = (icz, icx, icy+1)``,
    ``sfz = (icx, icy, icz+1)`` (grid.py:164-166)."""
    icx, icy, icz = grid.elem_sc
    shapes = [(icy, icz, icx + 1), (icz, icx, icy + 1), (icx, icy, icz + 1)]
    return [{k: np.zeros(s) for k in FIELDS} for s in shapes]


def _flip_forward(Sol):
    for k in FIELDS:
        Sol[k] = np.moveaxis(Sol[k], 0, -1)


def _flip_backward(Sol):
    for k in FIELDS:
        Sol[k] = np.moveaxis(Sol[k], -1, 0)


def _neg_symmetric_last(core, ig):
    q = np.pad(core, [(0, 0)] * (core.ndim - 1) + [(ig, ig)], mode="constant")
    q[..., :ig] = -q[..., ig:2 * ig][..., ::-1]
    q[..., -ig:] = -q[..., -2 * ig:-ig][..., ::-1]
    return q


def _gravity_last(Sol, grid, prm, hydro_c, strat_fn):
    """The hydrostatic ghost cells of boundary.py:56-132 along the last axis (y in the y sweep)."""
    moved = {k: np.moveaxis(Sol[k], -1, 1) for k in FIELDS}          # (z, x, y) -> (z, y, x): y on axis 1
    o3._gravity_ghosts(moved, grid, prm, hydro_c, strat_fn)
    for k in FIELDS:
        Sol[k] = np.moveaxis(moved[k], 1, -1)


def _boundary_step(Sol, grid, prm, hydro_c, strat_fn, split):
    """``set_explicit_boundary_data(..., step=split)``: ghost cells along the last axis."""
    ig = 2
    if split == 1 and prm.g != 0.0:
        _gravity_last(Sol, grid, prm, hydro_c, strat_fn)
        return
    pad = [(0, 0), (0, 0), (ig, ig)]
    inner = (Ellipsis, slice(ig, -ig))
    if grid.bdry[split] == PERIODIC:
        for k in FIELDS:
            Sol[k] = np.pad(Sol[k][inner], pad, mode="wrap")
    elif grid.bdry[split] == WALL:
        Sol["rho"] = np.pad(Sol["rho"][inner], pad, mode="symmetric")
        Sol["rhov"] = _neg_symmetric_last(Sol["rhov"][inner], ig)
        Sol["rhou"] = np.pad(Sol["rhou"][inner], pad, mode="symmetric")
        Sol["rhoY"] = np.pad(Sol["rhoY"][inner], pad, mode="symmetric")
        Sol["rhoX"] = np.pad(Sol["rhoX"][inner], pad, mode="symmetric")
    else:
        raise ValueError("Rayleigh boundary not defined off the gravity axis")


def explicit_step_and_flux(Sol, flux, lmbda, split, grid, prm, hydro_c, strat_fn, rk=False):
    """One sweep (explicit.py:77-158) on the sweep's layout; ``rk``: fluxes only."""
    _boundary_step(Sol, grid, prm, hydro_c, strat_fn, split)
    Lefts, Rights = _recovery(Sol, flux, 0.0 if rk else lmbda, split)
    _hll(flux, Lefts, Rights)
    if not rk:
        _update(Sol, flux, lmbda)
    _boundary_step(Sol, grid, prm, hydro_c, strat_fn, split)


def advect(Sol, flux, dt, odd, grid, prm, hydro_c, strat_fn):
    """Strang-split advection over ``dt`` (explicit.py:5-74), in place."""
    h = 0.5 * dt
    dxyz = (grid.dx, grid.dy, grid.dz)
    step = lambda s: explicit_step_and_flux(Sol, flux[s], h / dxyz[s], s, grid, prm, hydro_c, strat_fn)
    if odd:
        for s in (0, 1, 2):
            _flip_forward(Sol)
            step(s)
        for s in (2, 1, 0):
            step(s)
            _flip_backward(Sol)
    else:
        for s in (2, 1, 0):
            step(s)
            _flip_backward(Sol)
        for s in (0, 1, 2):
            _flip_forward(Sol)
            step(s)
    o3.set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)


def advect_rk(Sol, flux, dt, grid, prm, hydro_c, strat_fn):
    """First-order advection over ``dt`` (explicit.py:160-257), in place; returns the
    y sweep's rhoX update ``Sol.pwchi`` (set on ``Sol`` during the y sweep, so the
    z sweep's flip turns it back to the (x, y, z) layout)."""
    dxyz = (grid.dx, grid.dy, grid.dz)
    for s in (0, 1, 2):
        _flip_forward(Sol)
        explicit_step_and_flux(Sol, flux[s], dt / dxyz[s], s, grid, prm, hydro_c, strat_fn, rk=True)
    L, R = (Ellipsis, slice(0, -1)), (Ellipsis, slice(1, None))
    pwchi = None
    for s in (0, 1, 2):
        lmbda = dt / dxyz[s]
        _flip_forward(Sol)
        if pwchi is not None:                 # an attribute of Sol: flipped with it
            pwchi = np.moveaxis(pwchi, 0, -1)
        _update(Sol, flux[s], lmbda)
        if s == 1:
            pwchi = lmbda * (flux[s]["rhoX"][L] - flux[s]["rhoX"][R])
    o3.set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)
    return pwchi
