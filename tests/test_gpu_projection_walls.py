"""The whole 2D projection step on the device against the reference on the
33x17 states of tests/golden/step2d_kat.npz: walls in x and y (the wall-scaling
index carry-over, x-wall ghost cells and nodes), and periodic x with Coriolis
cross terms, both in the compressible regime; the bar of the rising-bubble
calls in tests/test_gpu_projection.py."""
import types

import numpy as np
import pytest

from conftest import golden
from oracle import nodal2d as n2
from oracle.krylov import bicgstab_legacy

pytestmark = pytest.mark.gpu
FIELDS = ["rho", "rhou", "rhov", "rhow", "rhoY", "rhoX"]


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("tag", ["ww", "cor"])
def test_device_projection_walls_and_coriolis(tag):
    """The whole 2D step against the reference on 33x17 states it records in
    step2d_kat.npz: walls in x and y, and periodic x with Coriolis cross terms,
    both in the compressible regime; the same bar as the rising-bubble calls."""
    from pybella_gb300.second_projection import euler_backward_non_advective_impl_part
    from conftest import step2d_case
    d = np.load(golden("step2d_kat.npz"))
    grid, prm, dt, hn, hc, sf = step2d_case(d, tag)
    Sol = types.SimpleNamespace(**{k: d["%s_in_%s" % (tag, k)].copy() for k in FIELDS})
    mpv = types.SimpleNamespace(p2_nodes=d[tag + "_p2_in"].copy(), rhs=np.zeros(grid.node_isc),
                                HydroState=types.SimpleNamespace(rhoY0=hc["rhoY0"]),
                                HydroState_n=types.SimpleNamespace(S0=hn["S0"]))
    elem = types.SimpleNamespace(ndim=2, y=grid.elem_y, dx=grid.dx, dy=grid.dy)
    node = types.SimpleNamespace(iicx=grid.inx, iicy=grid.iny, dx=grid.dx, dy=grid.dy, isc=grid.node_isc)
    ud = types.SimpleNamespace(bdry_type=["symmetric" if grid.x_wall else "wrap", "symmetric", "symmetric"],
                               Msq=prm.Msq, gravity_strength=np.array([0.0, prm.g, 0.0]),
                               coriolis_strength=np.asarray(prm.coriolis, dtype=np.float64), nonhydrostasy=1.0,
                               compressibility=prm.compressibility, is_compressible=prm.is_compressible,
                               tol=1e-10, max_iterations=6000, stratification=sf)
    st = {}
    euler_backward_non_advective_impl_part(Sol, mpv, elem, node, ud, types.SimpleNamespace(gamm=prm.gamm), 0.0,
                                           dt, 1.0, precision="fp64", stats=st)
    assert st["status"] == 0 and st["relres"] <= 1e-10, st
    np.testing.assert_allclose(mpv.rhs, d[tag + "_rhs"], rtol=1e-12, atol=1e-12 * np.abs(d[tag + "_rhs"]).max())
    Sc = {k: d["%s_in_%s" % (tag, k)].copy() for k in FIELDS}
    pc = d[tag + "_p2_in"].copy()
    n2.impl_part(Sc, pc, hn["S0"], hc, sf, grid, prm, dt,
                 solver=lambda op, b, tol, maxiter: bicgstab_legacy(op, b, 1e-13, 20000))
    for name, mine, ref, conv in [("p2", mpv.p2_nodes, d[tag + "_p2_out"], pc)] + \
            [(k, getattr(Sol, k), d["%s_out_%s" % (tag, k)], Sc[k]) for k in ("rhou", "rhov", "rhoX")]:
        ref_err = _rel(ref, conv)
        my_err = _rel(mine, conv)
        assert my_err <= max(1e-8, 3.0 * ref_err), (name, my_err, ref_err)
