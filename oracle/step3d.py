"""FP64 NumPy restatement of one 3D time step (oracle; tests only).

``time_update.do`` (time_update.py:129-489) composed from the 3D pieces: the
advection of oracle/advection3d.py and the projection parts of oracle/proj3d.py
(boundary data, backward explicit part and the pieces of the implicit step are
the reference's and pinned against it; the implicit step and the forward
explicit part use the glue of the reference's 2D branch, whose 3D code cannot
run).  Same order as oracle/step2d.py: boundary data, Sol0, fluxes, first-order
advection over dt/2, both projection halves with Sol0's coefficients, fluxes of
the half-step state, back to Sol0 (p2 kept), the forward explicit part,
Strang-split advection over dt, both projection halves.  The divergence takes
the 2D branch's sign on its x term (``x_sign = +1``): with the reference's 3D
sign (second_projection.py:563) the step blows up within a few steps.
"""
import copy

from oracle import advection3d as a3
from oracle import proj3d as o3


def time_step(Sol, p2, flux, step, dt, grid, prm, hydro_n, hydro_c, S0c, strat_fn, wind=(0.0, 0.0, 0.0),
              solver=None, x_sign=1.0):
    if prm.is_compressible != 0:
        raise NotImplementedError("the pseudo-incompressible step only")
    S0n = hydro_n["S0"]
    o3.set_explicit_boundary_data(Sol, grid, prm, hydro_c, strat_fn)
    Sol0 = copy.deepcopy(Sol)
    a3.recompute_advective_fluxes(Sol, flux)
    a3.advect_rk(Sol, flux, 0.5 * dt, grid, prm, hydro_c, strat_fn)
    o3.euler_backward_non_advective_expl_part(Sol, S0n, grid, prm, 0.5 * dt, hydro_c, strat_fn, wind)
    o3.impl_part(Sol, p2, S0n, hydro_c, strat_fn, grid, prm, 0.5 * dt, Sol0=Sol0, solver=solver, x_sign=x_sign)
    a3.recompute_advective_fluxes(Sol, flux)
    Sol = copy.deepcopy(Sol0)
    o3.euler_forward_non_advective(Sol, p2, S0c, S0n, grid, prm, 0.5 * dt, hydro_c, strat_fn, wind, x_sign=x_sign)
    a3.advect(Sol, flux, dt, step % 2, grid, prm, hydro_c, strat_fn)
    o3.euler_backward_non_advective_expl_part(Sol, S0n, grid, prm, 0.5 * dt, hydro_c, strat_fn, wind)
    o3.impl_part(Sol, p2, S0n, hydro_c, strat_fn, grid, prm, 0.5 * dt, solver=solver, x_sign=x_sign)
    return Sol
