"""FP64 NumPy restatement of one pyBELLA time step in 2D (oracle; tests only).

``time_update.do`` (time_update.py:129-708) for the pseudo-incompressible
case without blending, data assimilation or Rayleigh damping, composed from
the pinned pieces: boundary data, face mass fluxes and first-order advection
over dt/2 (``advect_rk``), the explicit and implicit halves of the projection
with the coefficients of the step's start (``Sol0``), fluxes from that
half-step state, then from the start state again the forward explicit part,
Strang-split advection over dt and both projection halves.  Pinned bit for bit
against the reference's ``do`` after one and two steps of the 64x32 rising
bubble (tests/golden/step_kat.npz).
"""
import copy

from oracle import advection2d as adv
from oracle import nodal2d as n2


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
