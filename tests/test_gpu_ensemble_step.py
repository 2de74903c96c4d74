"""The ensemble's time steps with batched solves (pybella_gb300.time_update.
EnsembleStep2D: every member's stages in turn, both projections of a step with
all members' solves in one persistent launch, bella_projection2d_batched)
against the same members stepped one by one (DeviceStep2D), on members of three
grid sizes, and one member against the oracle's time step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _members(specs):
    from pybella_gb300 import workloads
    from pybella_gb300.time_update import DeviceStep2D
    out = []
    for (cx, cy, amp, x0) in specs:
        st = workloads.bubble_2d_state(inx=cx + 1, iny=cy + 1, delth=amp, x0=x0)
        out.append((DeviceStep2D(st["Sol"], st["mpv"], st["elem"], st["node"], st["ud"], st["th"]), st))
    return out


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_ensemble_steps_match_single_members(precision):
    from pybella_gb300.time_update import EnsembleStep2D
    specs = [(32, 16, 2.0, 0.0), (64, 32, 2.2, 0.02), (64, 32, 1.8, -0.01), (128, 64, 2.1, 0.0)]
    ens, alone = _members(specs), _members(specs)
    E = EnsembleStep2D([m for m, _ in ens], precision=precision)
    for step in range(4):
        dts = E.time_steps(step, t_ref=1000.0)
        E.step(step, dts)
        for (m, _), dt in zip(alone, dts):
            m.step(step, dt, precision=precision)
    for stats in E.stats:
        for st in stats:
            assert st["status"] == 0 and st["relres"] <= 1e-10, st
    for (me, se), (ma, sa) in zip(ens, alone):
        me.download(se["Sol"], se["mpv"])
        ma.download(sa["Sol"], sa["mpv"])
        for k in ("rho", "rhoY"):
            assert _rel(getattr(se["Sol"], k), getattr(sa["Sol"], k)) < 1e-10, k
        for k in ("rhou", "rhov"):
            assert _rel(getattr(se["Sol"], k), getattr(sa["Sol"], k)) < 1e-8, (k, _rel(getattr(se["Sol"], k),
                                                                                      getattr(sa["Sol"], k)))


def test_ensemble_member_matches_oracle_step():
    """Member 0 of a three-member ensemble (two fixed 'CFLfixed' steps, FP64
    batched solves) against the oracle's restatement of time_update.do with its
    solves converged to 1e-13: as close as the tol-1e-10 solve allows."""
    from oracle import advection2d as adv, cases, step2d
    from pybella_gb300.time_update import EnsembleStep2D
    specs = [(64, 32, 2.0, 0.0), (32, 16, 2.2, 0.0), (128, 64, 1.9, 0.0)]
    ens = _members(specs)
    E = EnsembleStep2D([m for m, _ in ens], precision="fp64")
    grid, prm, Sol, p2, hn, hc, sf = cases.rising_bubble(inx=65, iny=33)
    st0 = ens[0][1]
    Sc = {k: getattr(st0["Sol"], k).copy() for k in FIELDS}
    pc = st0["mpv"].p2_nodes.copy()
    hn = dict(hn, S0=st0["mpv"].HydroState_n.S0)
    hc = dict(hc, rhoY0=st0["mpv"].HydroState.rhoY0)
    S0c = st0["mpv"].HydroState.get_S0c(None)
    prm_c = cases.n2.Params(Msq=prm.Msq, g=prm.g, gamm=prm.gamm, tol=1e-13, max_iterations=20000)
    flux = adv.new_flux(grid)
    for step in (0, 1):
        dts = [0.02169] * len(specs)
        E.step(step, dts)
        Sc = step2d.time_step(Sc, pc, flux, step, 0.02169, grid, prm_c, hn, hc, S0c, sf)
    m, st = ens[0]
    m.download(st["Sol"], st["mpv"])
    for k in ("rho", "rhoY"):
        assert _rel(getattr(st["Sol"], k), Sc[k]) < 1e-10, k
    for k in ("rhou", "rhov"):
        assert _rel(getattr(st["Sol"], k), Sc[k]) < 1e-6, (k, _rel(getattr(st["Sol"], k), Sc[k]))
