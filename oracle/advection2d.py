"""FP64 NumPy restatement of the reference's 2D advection (oracle; tests only).

The gas-dynamics half of a pyBELLA time step, the row after the projection in
the hot path's widening order: the face mass fluxes
(``recompute_advective_fluxes``, numerical_flux.py:5-46), the Strang-split
sweeps of ``advect`` (explicit.py:5-74) and the first-order ``advect_rk``
(explicit.py:160-257), each sweep being ``explicit_step_and_flux``
(explicit.py:77-158): boundary data along the sweep axis, the limited
reconstruction of ``recovery.do`` (recovery.py:6-141, limiter NONE), the
upwind flux of ``hll_solver`` (numerical_flux.py:48-99) and the conservative
update.  Pinned bit for bit against the reference's own outputs
(tests/golden/advect_kat.npz, tests/test_oracle_golden.py).

Layout: the reference's arrays are C order over (x, y) with two ghost layers;
a sweep works on the array with the sweep axis last (``Vars.flip_forward`` /
``flip_backward``, variable.py:89-97, are transposes in 2D), and the face
arrays of sweep ``s`` are ``(n_other, n_s + 1)`` (``elem.sfx``, ``elem.sfy``).
State dicts hold ``rho, rhou, rhov, rhow, rhoY, rhoX``.
"""
import numpy as np
from scipy.signal import fftconvolve

from oracle.nodal2d import PERIODIC, WALL, _gravity_ghosts, _neg_symmetric

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")


def recompute_advective_fluxes(Sol, flux):
    """Face mass fluxes ``rhoY u`` (x faces) and ``rhoY v`` (y faces) in place
    (numerical_flux.py:5-46, 2D): 2x3 and 3x2 weighted box averages."""
    inner = (slice(1, -1), slice(1, -1))
    kernel_u = np.array([[0.5, 1., 0.5], [0.5, 1., 0.5]])
    kernel_v = kernel_u.T
    rhoYu = Sol["rhoY"] * Sol["rhou"] / Sol["rho"]
    flux[0]["rhoY"][inner] = np.moveaxis(fftconvolve(rhoYu, kernel_u, mode="valid") / kernel_u.sum(), 0, -1)
    rhoYv = Sol["rhoY"] * Sol["rhov"] / Sol["rho"]
    flux[1]["rhoY"][inner] = fftconvolve(rhoYv, kernel_v, mode="valid") / kernel_v.sum()


def new_flux(grid):
    """Zeroed face containers of the two sweeps (``States(elem.sfx)``, ``States(elem.sfy)``)."""
    icx, icy = grid.elem_sc
    return [{k: np.zeros((icy, icx + 1)) for k in FIELDS}, {k: np.zeros((icx, icy + 1)) for k in FIELDS}]


def _flip(Sol):
    for k in FIELDS:
        Sol[k] = Sol[k].T


def _boundary_step(Sol, grid, prm, hydro_c, strat_fn, split):
    """``set_explicit_boundary_data(..., step=split)`` (boundary.py:7-132): ghost
    cells along the last axis of the sweep's layout."""
    ig = 2
    pad = ((0, 0), (ig, ig))
    inner = (slice(None), slice(ig, -ig))
    g = prm.g if split == 1 else 0.0
    if g != 0.0:
        _gravity_ghosts(Sol, grid, prm, hydro_c, strat_fn)          # the last axis is y here
        return
    if grid.bdry[split] == PERIODIC:
        for k in FIELDS:
            Sol[k] = np.pad(Sol[k][inner], pad, mode="wrap")
    elif grid.bdry[split] == WALL:
        Sol["rho"] = np.pad(Sol["rho"][inner], pad, mode="symmetric")
        Sol["rhov"] = _neg_symmetric(Sol["rhov"][inner], pad, 1)
        Sol["rhou"] = np.pad(Sol["rhou"][inner], pad, mode="symmetric")
        Sol["rhoY"] = np.pad(Sol["rhoY"][inner], pad, mode="symmetric")
        Sol["rhoX"] = np.pad(Sol["rhoX"][inner], pad, mode="symmetric")
    else:
        raise ValueError("Rayleigh boundary not defined on x-direction")


def _primitives(U):
    """``Vars.primitives`` (variable.py:56-86): u, v, w, Y, X where rho != 0, else 0."""
    nz = np.nonzero(U["rho"])
    out = {}
    for name, k in (("u", "rhou"), ("v", "rhov"), ("w", "rhow"), ("Y", "rhoY"), ("X", "rhoX")):
        a = np.zeros_like(U[k])
        a[nz] = U[k][nz] / U["rho"][nz]
        out[name] = a
    return out


def _recovery(Sol, flux, lmbda, split):
    """``recovery.do`` (recovery.py:6-141) with limiter NONE: interface states
    along the last axis (2D or 3D)."""
    P = _primitives(Sol)
    L, R = (Ellipsis, slice(0, -1)), (Ellipsis, slice(1, None))
    inner = (slice(1, -1),) * Sol["rho"].ndim
    u = np.zeros_like(Sol["rhoY"])
    fr = flux["rhoY"][inner]
    u[inner] = 0.5 * (fr[L] + fr[R]) / Sol["rhoY"][inner]
    shape = P["u"].shape
    diffs = {}
    for q in ("u", "v", "w", "X"):
        d = np.zeros(shape)
        d[..., :-1] = P[q][R] - P[q][L]
        diffs[q] = d
    d = np.zeros(shape)
    d[..., :-1] = 1.0 / P["Y"][R] - 1.0 / P["Y"][L]
    diffs["Y"] = d
    slopes = {}
    for q in ("u", "v", "w", "X", "Y"):                               # recovery.py:144-209, limiters :212-238
        s = np.zeros(shape)
        s[..., 1:-1] = 0.5 * (diffs[q][L][L] + diffs[q][L][R])
        slopes[q] = s
    sides = []
    for sign in (1.0, -1.0):
        amp = {q: sign * 0.5 * slopes[q] * (1. - sign * lmbda * u) for q in slopes}
        S = {k: np.zeros(shape) for k in FIELDS}
        S["u"] = P["u"] + 1 * amp["u"]
        S["v"] = P["v"] + 1 * amp["v"]
        S["w"] = P["w"] + 1 * amp["w"]
        S["X"] = P["X"] + 1 * amp["X"]
        S["Y"] = 1.0 / (1.0 / P["Y"] + 1 * amp["Y"])
        sides.append(S)
    Lefts, Rights = sides
    vel = [P["u"], P["v"], P["w"]][split]
    face = 0.5 * (Sol["rhoY"][L] + Sol["rhoY"][R]) - 1 * 0.5 * lmbda * (vel[R] * Sol["rhoY"][R] - vel[L] * Sol["rhoY"][L])
    Lefts["rhoY"][L] = face
    Rights["rhoY"][R] = face
    for U in (Rights, Lefts):                                         # get_conservatives, recovery.py:241-262
        U["rho"] = U["rhoY"] / U["Y"]
        U["rhou"] = U["u"] * U["rho"]
        U["rhov"] = U["v"] * U["rho"]
        U["rhow"] = U["w"] * U["rho"]
        U["rhoY"] = U["Y"] * U["rho"]
        U["rhoX"] = U["X"] * U["rho"]
    return Lefts, Rights


def _hll(flux, Lefts, Rights):
    """``hll_solver`` (numerical_flux.py:48-99): upwind by the sign of the face mass flux."""
    L, R, mid = (Ellipsis, slice(0, -1)), (Ellipsis, slice(1, None)), (Ellipsis, slice(1, -1))
    PL, PR = _primitives(Lefts), _primitives(Rights)
    upwind = 0.5 * (1.0 + np.sign(flux["rhoY"]))
    upl = upwind[R]
    upr = (1.0 - upwind[L])
    f = flux["rhoY"][mid]
    a, b = upl[L] / PL["Y"][L], upr[R] / PR["Y"][R]
    flux["rhou"][mid] = f * (upl[L] / PL["Y"][L] * PL["u"][L] + upr[R] / PR["Y"][R] * PR["u"][R])
    flux["rho"][mid] = f * (a * 1.0 + b * 1.0)
    flux["rhov"][mid] = f * (upl[L] / PL["Y"][L] * PL["v"][L] + upr[R] / PR["Y"][R] * PR["v"][R])
    flux["rhow"][mid] = f * (upl[L] / PL["Y"][L] * PL["w"][L] + upr[R] / PR["Y"][R] * PR["w"][R])
    flux["rhoX"][mid] = f * (upl[L] / PL["Y"][L] * PL["X"][L] + upr[R] / PR["Y"][R] * PR["X"][R])


def _update(Sol, flux, lmbda):
    L, R = (Ellipsis, slice(0, -1)), (Ellipsis, slice(1, None))
    for k in ("rho", "rhou", "rhov", "rhow", "rhoX", "rhoY"):
        Sol[k] = Sol[k] + lmbda * (flux[k][L] - flux[k][R])


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
    from oracle.nodal2d import set_explicit_boundary_data
    h = 0.5 * dt
    dxy = (grid.dx, grid.dy)
    step = lambda s: explicit_step_and_flux(Sol, flux[s], h / dxy[s], s, grid, prm, hydro_c, strat_fn)
    if odd:
        for s in (0, 1):
            _flip(Sol)
            step(s)
        for s in (1, 0):
            step(s)
            _flip(Sol)
    else:
        for s in (1, 0):
            step(s)
            _flip(Sol)
        for s in (0, 1):
            _flip(Sol)
            step(s)
    set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)


def advect_rk(Sol, flux, dt, grid, prm, hydro_c, strat_fn):
    """First-order advection over ``dt`` (explicit.py:160-257), in place; returns
    the y-sweep's rhoX update (``Sol.pwchi``)."""
    from oracle.nodal2d import set_explicit_boundary_data
    dxy = (grid.dx, grid.dy)
    for s in (0, 1):
        _flip(Sol)
        explicit_step_and_flux(Sol, flux[s], dt / dxy[s], s, grid, prm, hydro_c, strat_fn, rk=True)
    L, R = (slice(None), slice(0, -1)), (slice(None), slice(1, None))
    pwchi = None
    for s in (0, 1):
        lmbda = dt / dxy[s]
        _flip(Sol)
        _update(Sol, flux[s], lmbda)
        if s == 1:
            pwchi = lmbda * (flux[s]["rhoX"][L] - flux[s]["rhoX"][R])
    set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)
    return pwchi
