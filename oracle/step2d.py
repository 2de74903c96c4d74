"""FP64 NumPy restatement of one pyBELLA time step in 2D (oracle; tests only).

``time_update.do`` (time_update.py:129-708) for the pseudo-incompressible
case without blending, data assimilation or Rayleigh damping, composed from
the pinned pieces: boundary data, face mass fluxes and first-order advection
over dt/2 (``advect_rk``), the explicit and implicit halves of the projection
with the coefficients of the step's start (``Sol0``), fluxes from that
half-step state, then from the start state again the forward explicit part,
Strang-split advection over dt and both projection halves.  Pinned bit for bit
against the reference's ``do`` after one and two steps of the 64x32 rising
bubble (tests/golden/step_kat.npz); ``dynamic_timestep`` and ``run`` add the
CFL time step and the loop, pinned over a run to tout (two steps with the fixed
dt of 'CFLfixed', a third whose CFL step is cut to reach tout).
"""
import copy

import numpy as np

from oracle import advection2d as adv
from oracle import nodal2d as n2

MACHINE_EPSILON = np.finfo(float).eps


def time_step(Sol, p2, flux, step, dt, grid, prm, hydro_n, hydro_c, S0c, strat_fn):
    """One step of ``do`` (time_update.py:129-489); returns the new ``Sol`` (p2 and flux in place)."""
    if prm.is_compressible != 0:
        raise NotImplementedError("the pseudo-incompressible step only")
    S0n = hydro_n["S0"]
    n2.set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)              # :130
    Sol0 = copy.deepcopy(Sol)                                                     # :205
    adv.recompute_advective_fluxes(Sol, flux)                                     # :212
    adv.advect_rk(Sol, flux, 0.5 * dt, grid, prm, hydro_c, strat_fn)             # :224-237
    n2.euler_backward_non_advective_expl_part(Sol, S0n, grid, prm, 0.5 * dt, hydro_c, strat_fn)   # :247
    n2.impl_part(Sol, p2, S0n, hydro_c, strat_fn, grid, prm, 0.5 * dt, Sol0=Sol0)   # :251-263
    adv.recompute_advective_fluxes(Sol, flux)                                     # :337
    Sol = copy.deepcopy(Sol0)                                                     # :376-377
    n2.euler_forward_non_advective(Sol, p2, S0c, S0n, grid, prm, 0.5 * dt, hydro_c, strat_fn)   # :419-429
    adv.advect(Sol, flux, dt, step % 2, grid, prm, hydro_c, strat_fn)            # :434-446
    n2.euler_backward_non_advective_expl_part(Sol, S0n, grid, prm, 0.5 * dt, hydro_c, strat_fn)   # :455
    n2.impl_part(Sol, p2, S0n, hydro_c, strat_fn, grid, prm, 0.5 * dt)           # :462-473
    return Sol


def dynamic_timestep(Sol, time, time_output, grid, prm, step, CFL=0.5, dtfixed0=100.0, dtfixed=100.0,
                     acoustic_timestep=0):
    """``dynamic_timestep`` (cfl.py:5-74) in 2D (elem.dz = 1, grid.py:110, 171);
    returns ``dt`` (and, in the advective branch, ``cfl``, ``cfl_ac`` as the reference does)."""
    Minv = 1.0 / np.sqrt(prm.Msq)
    p = Sol["rhoY"] ** prm.gamm
    c = np.sqrt(prm.gamm * p / Sol["rho"]) * Minv
    u = np.abs(Sol["rhou"] / Sol["rho"])
    v = np.abs(Sol["rhov"] / Sol["rho"])
    w = np.abs(Sol["rhow"] / Sol["rho"])
    eps = MACHINE_EPSILON
    u_max, v_max, w_max = max(u.max(), eps), max(v.max(), eps), max(w.max(), eps)
    upc_max, vpc_max, wpc_max = max((u + c).max(), eps), max((v + c).max(), eps), max((w + c).max(), eps)
    dx, dy, dz = grid.dx, grid.dy, 1.0
    if acoustic_timestep == 1:
        dt_cfl = min(min(CFL * dx / upc_max, CFL * dy / vpc_max), CFL * dz / wpc_max)
        dt = min(dt_cfl, dtfixed0 + min(step, 1.) * (dtfixed - dtfixed0))
        if dt > (time_output - time):
            dt = (time_output - time) + eps
        return dt
    dt_cfl = min(min(CFL * dx / u_max, CFL * dy / v_max), CFL * dz / w_max)
    dt = min(dt_cfl, dtfixed0 + min(step, 1.) * (dtfixed - dtfixed0))
    dt *= min(float(step + 1), 1.0)
    if dt > (time_output - time):
        dt = (time_output - time)
    cfl = CFL * dt / dt_cfl
    cfl_ac = max(dt * upc_max / dx, dt * vpc_max / dy, dt * wpc_max / dz)
    return dt, cfl, cfl_ac


def run(Sol, p2, t, tout, nsteps, grid, prm, hydro_n, hydro_c, S0c, strat_fn, t_ref, cfl_fixed=True, step=0,
        flux=None):
    """The loop of ``do`` (time_update.py:129-140, 686-708): the CFL time step
    ('CFLfixed': 21.69 / t_ref while the global step index is below 2), then
    :func:`time_step`, until ``tout`` or until the global step index reaches
    ``nsteps`` (the reference's ``stepmax``).  ``step`` is the global index the
    run starts from (``do`` receives it in ``steps`` and returns it), so calls for
    consecutive output times continue one run.  Returns ``(Sol, t, dts, step)``."""
    flux = adv.new_flux(grid) if flux is None else flux
    dts = []
    while t < tout and step < nsteps:
        n2.set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)
        dt, _, _ = dynamic_timestep(Sol, t, tout, grid, prm, step)
        if cfl_fixed and step < 2:
            dt = 21.69 / t_ref
        Sol = time_step(Sol, p2, flux, step, dt, grid, prm, hydro_n, hydro_c, S0c, strat_fn)
        dts.append(dt)
        t += dt
        step += 1
    return Sol, t, dts, step


def run_outputs(Sol, p2, touts, stepmax, grid, prm, hydro_n, hydro_c, S0c, strat_fn, t_ref, t=0.0,
                on_output=None):
    """The output loop of the reference's driver for one member (__main__.py:198-393):
    one :func:`run` per output time, the step index carried across them, and
    ``t`` set to the output time rounded to three decimals after each
    (__main__.py:266, 388).  ``on_output(tout, Sol, p2, step)`` is called at
    every output time.  Returns ``(Sol, t, step)``."""
    flux = adv.new_flux(grid)
    step = 0
    for tout in touts:
        Sol, t, _, step = run(Sol, p2, t, tout, stepmax, grid, prm, hydro_n, hydro_c, S0c, strat_fn, t_ref,
                              step=step, flux=flux)
        t = float(np.around(tout, 3))
        if on_output is not None:
            on_output(t, Sol, p2, step)
    return Sol, t, step
