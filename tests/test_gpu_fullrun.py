"""The rising bubble run to its end on the GPU: 160x80 cells, pseudo-incompressible,
CFL 0.5, BiCGStab tol 1e-10 in every projection, output times 0.1 ... 1.0 (units
of t_ref = 1000 s) every 0.01 (inputs/rising_bubble.py:5-98), 216 time steps with
the whole state resident on the device (DeviceStep2D.run_outputs, the output loop
of the reference's driver, __main__.py:198-393).

theta = rhoY / rho is compared every 0.1 against

* the oracle's run of the same case (``fullrun_oracle_kat.npz``; the oracle's
  step and loop are pinned bit for bit to the reference's ``do``), and
* the reference's own run (``fullrun_kat.npz``, generated by running pyBELLA
  as plain Python through ``tests/golden/make_fullrun.py``: all ten output times
  0.1 ... 1.0, 216 steps, about five hours on the host).

The bar is relative L2 <= 1e-6 at every output time, t_end included; the
errors are also printed relative to the bubble's perturbation theta - 1.
"""
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")
BAR = 1e-6


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _device_run(d, precision):
    from types import SimpleNamespace as NS
    from oracle import cases
    from pybella_gb300.time_update import DeviceStep2D
    grid, prm, _, _, _, _, sf = cases.rising_bubble()
    Sol = NS(**{k: d["in_" + k].copy() for k in FIELDS})
    S0c = d["S0c"]
    mpv = NS(p2_nodes=d["p2_in"].copy(), HydroState=NS(rhoY0=d["rhoY0"], get_S0c=lambda elem: S0c),
             HydroState_n=NS(S0=d["S0n"]))
    ud = NS(bdry_type=["wrap", "symmetric", "symmetric"], gravity_strength=[0.0, prm.g, 0.0], Msq=prm.Msq,
            nonhydrostasy=1.0, compressibility=0.0, is_compressible=0, coriolis_strength=np.zeros(3),
            u_wind_speed=0.0, v_wind_speed=0.0, w_wind_speed=0.0, stratification=sf, tol=1e-10,
            max_iterations=6000)
    run = DeviceStep2D(Sol, mpv, NS(ndim=2, y=grid.elem_y),
                       NS(iicx=grid.inx, iicy=grid.iny, dx=grid.dx, dy=grid.dy), ud, NS(gamm=prm.gamm))
    snaps = {}

    def on_output(t, step):
        if int(round(t * 100)) % 10 == 0:
            run.download(Sol, mpv)
            snaps[round(t, 3)] = (Sol.rhoY / Sol.rho).copy()
    touts = np.arange(0.0, 1.01, 0.01)[10:]
    t, step = run.run_outputs(touts, 10000, t_ref=1000.0, precision=precision, on_output=on_output)
    run.download(Sol, mpv)
    for st in run.stats:
        assert st["status"] == 0 and st["relres"] <= 1e-10, st
    return snaps, Sol, mpv, t, step, run.stats


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_rising_bubble_full_run_theta(precision, capsys):
    o = np.load(golden("fullrun_oracle_kat.npz"))
    snaps, Sol, mpv, t, step, stats = _device_run(o, precision)
    assert t == pytest.approx(1.0, abs=1e-12) and step == int(o["out_step"])
    lines = []
    refs = [("oracle", o)]
    if os.path.exists(golden("fullrun_kat.npz")):
        refs.append(("reference", np.load(golden("fullrun_kat.npz"))))
    for name, d in refs:
        for tk, th in zip(d["theta_t"], d["theta"]):
            mine = snaps[round(float(tk), 3)]
            e, ep = _rel(mine, th), _rel(mine - 1.0, th - 1.0)
            assert e <= BAR, (name, tk, e)
            lines.append("%-9s t = %.1f: theta rel. L2 %.2e (of theta - 1: %.2e)" % (name, tk, e, ep))
    for k in FIELDS:
        if k in ("rhow", "rhoX"):
            continue
        e = _rel(getattr(Sol, k), o["out_" + k])
        lines.append("oracle    t = 1.0: %-5s rel. L2 %.2e" % (k, e))
        assert e <= BAR, (k, e)
    its = [s["iterations"] for s in stats]
    with capsys.disabled():
        print("\nrising bubble to t_end (%s): %d steps, %d solves, %.0f iterations per solve\n  %s"
              % (precision, step, len(its), np.mean(its), "\n  ".join(lines)))
