"""The device-resident 3D time step (pybella_gb300.time_update.DeviceStep3D) against
the oracle's 3D step (oracle/step3d.py: the reference's 3D pieces with the 2D
branch's glue and divergence sign; the reference's own 3D step cannot run), and
its time per step at 257x129x257 with the background-preconditioned projections."""
from types import SimpleNamespace as NS

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")


def _objects(grid, prm, Sol, p2, hn, hc, tol):
    S0c = np.broadcast_to(hc["S0"][None, :, None], grid.elem_sc).copy()
    S = NS(**{k: Sol[k].copy() for k in FIELDS})
    mpv = NS(p2_nodes=p2.copy(), HydroState=NS(rhoY0=hc["rhoY0"], get_S0c=lambda elem: S0c),
             HydroState_n=NS(S0=hn["S0"]))
    elem = NS(ndim=3, y=grid.elem_y)
    node = NS(iicx=grid.inx, iicy=grid.iny, iicz=grid.inz, dx=grid.dx, dy=grid.dy, dz=grid.dz)
    ud = NS(bdry_type=["symmetric" if grid.wall(d) else "wrap" for d in range(3)],
            gravity_strength=[0.0, prm.g, 0.0], Msq=prm.Msq, nonhydrostasy=1.0, compressibility=0.0,
            is_compressible=0, coriolis_strength=np.zeros(3), u_wind_speed=0.0, v_wind_speed=0.0,
            w_wind_speed=0.0, stratification=lambda y: 1.0, tol=tol, max_iterations=20000)
    return S, mpv, elem, node, ud, NS(gamm=prm.gamm), S0c


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_device_step3d_matches_oracle():
    """Two steps of the 17x9x17 warm bubble: momenta and rhoX within 1e-8, rho and
    rhoY within 1e-10 (relative L2) of the oracle's step with its solves at 1e-13;
    the device solves at 1e-12 in FP64."""
    from oracle import advection3d as a3, cases, step3d
    from oracle.krylov import bicgstab_legacy
    from pybella_gb300.time_update import DeviceStep3D
    grid, prm, Sol, p2, hn, hc, sf = cases.bubble_3d(17, 9, 17, seed=3, wind=0.0)
    S, mpv, elem, node, ud, th, S0c = _objects(grid, prm, Sol, p2, hn, hc, 1e-12)
    run = DeviceStep3D(S, mpv, elem, node, ud, th)
    Sc = {k: v.copy() for k, v in Sol.items()}
    pc = p2.copy()
    flux = a3.new_flux(grid)
    solver = lambda op, b, tol, maxiter: bicgstab_legacy(op, b, 1e-13, 20000)
    dt = 0.02169
    for step in (0, 1):
        run.step(step, dt, precision="fp64")
        run.download(S, mpv)
        Sc = step3d.time_step(Sc, pc, flux, step, dt, grid, prm, hn, hc, S0c, sf, solver=solver)
        for st in run.stats[-2:]:
            assert st["status"] == 0 and st["relres"] <= 1e-12, st
        for k in ("rhou", "rhov", "rhow", "rhoX"):
            assert _rel(getattr(S, k), Sc[k]) < 1e-8, (step, k, _rel(getattr(S, k), Sc[k]))
        for k in ("rho", "rhoY"):
            assert _rel(getattr(S, k), Sc[k]) < 1e-10, (step, k)


def test_device_step3d_full_size(capsys):
    """Three steps of the 257x129x257 warm bubble with background-preconditioned
    projections: every solve converged, the state finite; device time per step."""
    import torch
    from oracle import cases
    from pybella_gb300.time_update import DeviceStep3D
    grid, prm, Sol, p2, hn, hc, sf = cases.bubble_3d(257, 129, 257, seed=11, wind=0.0)
    S, mpv, elem, node, ud, th, _ = _objects(grid, prm, Sol, p2, hn, hc, 1e-10)
    run = DeviceStep3D(S, mpv, elem, node, ud, th, preconditioner="background")
    run.step(0, 0.02169)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for step in (1, 2):
        run.step(step, 0.02169)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 2
    for st in run.stats:
        assert st["status"] == 0 and st["relres"] <= 1e-10, st
    run.download(S, mpv)
    assert all(np.all(np.isfinite(getattr(S, k))) for k in FIELDS)
    with capsys.disabled():
        print("\n3D time step 257x129x257 (background-preconditioned projections): %.1f ms per step, "
              "iterations per solve %s" % (ms, [st["iterations"] for st in run.stats]))
