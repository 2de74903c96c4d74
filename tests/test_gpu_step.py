"""The device-resident 2D time step (pybella_gb300.time_update.DeviceStep2D:
advection, explicit and implicit projection halves, all on the GPU) against two
steps of the reference's time_update.do on the 64x32 rising bubble
(tests/golden/step_kat.npz)."""
from types import SimpleNamespace as NS

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_device_time_step_matches_reference():
    """State after each of two steps as close to the converged answer (the
    oracle's step with its solves at 1e-13) as the reference's own tol=1e-10
    result is, or within 1e-8 of it; rho and rhoY, which the solves' error reaches
    only through the next advection, within 1e-10."""
    from oracle import advection2d as adv, cases, step2d
    from pybella_gb300.time_update import DeviceStep2D
    d = np.load(golden("step_kat.npz"))
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble(inx=64, iny=32)
    hn, hc = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"])
    dt = float(d["meta"][2])
    S0c = d["S0c"]
    Sol = NS(**{k: d["in_" + k].copy() for k in FIELDS})
    mpv = NS(p2_nodes=d["p2_in"].copy(), HydroState=NS(rhoY0=hc["rhoY0"], get_S0c=lambda elem: S0c),
             HydroState_n=NS(S0=hn["S0"]))
    elem = NS(ndim=2, y=grid.elem_y)
    node = NS(iicx=grid.inx, iicy=grid.iny, dx=grid.dx, dy=grid.dy)
    ud = NS(bdry_type=["wrap", "symmetric", "symmetric"], gravity_strength=[0.0, prm.g, 0.0], Msq=prm.Msq,
            nonhydrostasy=1.0, compressibility=0.0, is_compressible=0, coriolis_strength=np.zeros(3),
            u_wind_speed=0.0, v_wind_speed=0.0, w_wind_speed=0.0, stratification=sf, tol=1e-10,
            max_iterations=6000)
    run = DeviceStep2D(Sol, mpv, elem, node, ud, NS(gamm=prm.gamm))
    prm_c = cases.n2.Params(Msq=prm.Msq, g=prm.g, gamm=prm.gamm, tol=1e-13, max_iterations=20000)
    Sc = {k: d["in_" + k].copy() for k in FIELDS}
    pc = d["p2_in"].copy()
    flux = adv.new_flux(grid)
    for step in (0, 1):
        run.step(step, dt, precision="fp64")
        run.download(Sol, mpv)
        Sc = step2d.time_step(Sc, pc, flux, step, dt, grid, prm_c, hn, hc, S0c, sf)
        for st in run.stats[-2:]:
            assert st["status"] == 0 and st["relres"] <= 1e-10, st
        tag = "s%d_" % (step + 1)
        for name, mine, ref, conv in [("p2", mpv.p2_nodes, d[tag + "p2"], pc)] + \
                [(k, getattr(Sol, k), d[tag + k], Sc[k]) for k in ("rhou", "rhov", "rhoX")]:
            ref_err, my_err = _rel(ref, conv), _rel(mine, conv)
            assert my_err <= max(1e-8, 3.0 * ref_err), (step, name, my_err, ref_err)
        for k in ("rho", "rhoY"):
            assert _rel(getattr(Sol, k), d[tag + k]) < 1e-10, (step, k)


def test_device_run_to_tout_matches_reference():
    """DeviceStep2D.run: dt from the CFL maxima of the device state
    (bella_cfl_maxima) and the loop of time_update.do, to tout = 0.1 (two fixed
    steps, a third cut to tout), against the reference's run (step_kat.npz)."""
    from oracle import cases
    from pybella_gb300.time_update import DeviceStep2D
    d = np.load(golden("step_kat.npz"))
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble(inx=64, iny=32)
    hn, hc = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"])
    S0c = d["S0c"]
    Sol = NS(**{k: d["in_" + k].copy() for k in FIELDS})
    mpv = NS(p2_nodes=d["p2_in"].copy(), HydroState=NS(rhoY0=hc["rhoY0"], get_S0c=lambda elem: S0c),
             HydroState_n=NS(S0=hn["S0"]))
    ud = NS(bdry_type=["wrap", "symmetric", "symmetric"], gravity_strength=[0.0, prm.g, 0.0], Msq=prm.Msq,
            nonhydrostasy=1.0, compressibility=0.0, is_compressible=0, coriolis_strength=np.zeros(3),
            u_wind_speed=0.0, v_wind_speed=0.0, w_wind_speed=0.0, stratification=sf, tol=1e-10,
            max_iterations=6000)
    run = DeviceStep2D(Sol, mpv, NS(ndim=2, y=grid.elem_y), NS(iicx=grid.inx, iicy=grid.iny, dx=grid.dx, dy=grid.dy),
                       ud, NS(gamm=prm.gamm))
    t, dts, nstep = run.run(0.0, float(d["meta"][7]), 4, t_ref=float(d["meta"][6]))
    run.download(Sol, mpv)
    assert len(dts) == 3 and abs(t - float(d["meta"][7])) < 1e-12
    for st in run.stats:
        assert st["status"] == 0 and st["relres"] <= 1e-10, st
    for k in ("rho", "rhoY"):
        assert _rel(getattr(Sol, k), d["s4_" + k]) < 1e-10, k
    for k in ("rhou", "rhov", "rhoX"):
        assert _rel(getattr(Sol, k), d["s4_" + k]) < 1e-6, (k, _rel(getattr(Sol, k), d["s4_" + k]))
