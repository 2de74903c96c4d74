"""The orchestration of the device time steps (pybella_gb300.time_update) on the
CPU: the library's entry points are replaced by stand-ins that run on the same
host memory -- the host builds of the advection and 3D explicit-part arithmetic
(tests/advect_host.cpp, tests/expl3d_host.cpp, the source the kernels run) and
the oracle's projection pieces -- and torch tensors live on the host.  What is
checked is DeviceStep2D / DeviceStep3D themselves: the order of the stages, the
argument blocks they fill, Sol0 and p2 handling, the flux containers.  2D
against two reference steps (step_kat.npz), 3D against oracle/step3d.py."""
import ctypes
import os
import shutil
import subprocess
from types import SimpleNamespace as NS

import numpy as np
import pytest

from conftest import ROOT, golden

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")


def _build(tmp, src):
    out = str(tmp / (src + ".so"))
    subprocess.run([shutil.which("g++"), "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", out,
                    os.path.join(ROOT, "tests", src)], check=True)
    return ctypes.CDLL(out)


def _arr(ptr, shape):
    return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_double)), shape=shape)


def _vp(x):
    return ctypes.c_void_p(x.ctypes.data) if isinstance(x, np.ndarray) else ctypes.c_void_p(x)


class _Stream:
    cuda_stream = 0


class _NoDevice:
    def __init__(self, *a, **k):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


@pytest.fixture
def host_torch(monkeypatch):
    """torch on the host: device keywords dropped, CUDA calls no-ops."""
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    import torch
    for name in ("tensor", "zeros", "empty"):
        orig = getattr(torch, name)
        monkeypatch.setattr(torch, name, (lambda f: lambda *a, **k: f(*a, **{q: v for q, v in k.items()
                                                                           if q != "device"}))(orig))
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a, **k: _Stream())
    monkeypatch.setattr(torch.cuda, "device", _NoDevice)
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    return torch


def _adv_args(a, nd):
    ic = (a.inx + 3, a.iny + 3, a.inz + 3 if nd == 3 else 1)
    walls = (a.x_wall, a.y_wall, a.z_wall if nd == 3 else 0)
    geo = np.array([nd, *ic, *walls], dtype=np.int32)
    dg = np.array([a.dx, a.dy, a.dz if nd == 3 else 1.0, a.g, a.gamm])
    F = (ctypes.c_void_p * 6)(a.rho, a.rhou, a.rhov, a.rhow, a.rhoY, a.rhoX)
    faces = [a.fx[q] for q in range(6)] + [a.fy[q] for q in range(6)] + ([a.fz[q] for q in range(6)] if nd == 3 else [])
    return geo, dg, F, (ctypes.c_void_p * len(faces))(*faces)


class _Stand:
    """The entry points DeviceStep2D/3D call, on host memory."""

    def __init__(self, adv, e3, ctx):
        self.adv, self.e3, self.c = adv, e3, ctx

    def bella_solve_opts_default(self, p):
        return 0

    def _sol(self, s, shape):
        return {k: _arr(getattr(s, k), shape) for k in FIELDS}

    def _boundary(self, p, set_bd):
        Sol = self._sol(p._obj, self.c.grid.elem_sc)
        S = {k: v.copy() for k, v in Sol.items()}
        set_bd(S, self.c.grid, self.c.prm, self.c.hc, self.c.sf)
        for k in FIELDS:
            Sol[k][...] = S[k]
        return 0

    def _mass(self, p, nd):
        geo, dg, F, fc = _adv_args(p._obj, nd)
        self.adv.adv_host_mass(_vp(geo), _vp(dg), F, fc)
        return 0

    def _strang(self, p, dt, odd, nd):
        a = p._obj
        geo, dg, F, fc = _adv_args(a, nd)
        self.adv.adv_host_strang(_vp(geo), _vp(dg), ctypes.c_int(0), F, fc, _vp(a.hydro_rhoY0), _vp(a.strat_inv),
                                 ctypes.c_double(dt), ctypes.c_int(odd))
        return 0

    def _rk(self, p, dt, nd):
        a = p._obj
        geo, dg, F, fc = _adv_args(a, nd)
        self.adv.adv_host_rk(_vp(geo), _vp(dg), ctypes.c_int(0), F, fc, _vp(a.hydro_rhoY0), _vp(a.strat_inv),
                             ctypes.c_double(dt), _vp(a.pwchi))
        return 0

    def _project(self, p, st, impl, extra):
        r = p._obj
        g = self.c.grid
        Sol = self._sol(r, g.elem_sc)
        S = {k: v.copy() for k, v in Sol.items()}
        S0 = None
        if r.rho0:
            Sol0 = {k: _arr(getattr(r, k + "0"), g.elem_sc) for k in FIELDS}
            S0 = {k: v.copy() for k, v in Sol0.items()}
        p2 = _arr(r.p2, g.node_sc)
        q = p2.copy()
        impl(S, q, self.c.hn["S0"], self.c.hc, self.c.sf, g, self.c.prm, r.dt, Sol0=S0, **extra)
        for k in FIELDS:
            Sol[k][...] = S[k]
            if S0 is not None:
                Sol0[k][...] = S0[k]
        p2[...] = q
        st._obj.status, st._obj.relres = 0, 0.0
        return 0

    # 2D
    def bella_boundary2d(self, p, s):
        from oracle import nodal2d as n2
        return self._boundary(p, n2.set_explicit_boundary_data)

    def bella_advective_fluxes2d(self, p, s):
        return self._mass(p, 2)

    def bella_advect2d(self, p, dt, odd, s):
        return self._strang(p, dt, odd, 2)

    def bella_advect_rk2d(self, p, dt, s):
        return self._rk(p, dt, 2)

    def bella_expl_part2d(self, p, s):
        from oracle import nodal2d as n2
        e = p._obj
        Sol = self._sol(e, self.c.grid.elem_sc)
        S = {k: v.copy() for k, v in Sol.items()}
        n2.euler_backward_non_advective_expl_part(S, self.c.hn["S0"], self.c.grid, self.c.prm, e.dt, self.c.hc,
                                                  self.c.sf)
        for k in FIELDS:
            Sol[k][...] = S[k]
        return 0

    def bella_euler_forward2d(self, p, s):
        from oracle import nodal2d as n2
        e = p._obj
        g = self.c.grid
        Sol = self._sol(e, g.elem_sc)
        S = {k: v.copy() for k, v in Sol.items()}
        p2 = _arr(e.p2, g.node_sc)
        q = p2.copy()
        n2.euler_forward_non_advective(S, q, _arr(e.S0c, g.elem_sc), self.c.hn["S0"], g, self.c.prm, e.dt,
                                       self.c.hc, self.c.sf)
        for k in FIELDS:
            Sol[k][...] = S[k]
        p2[...] = q
        return 0

    def bella_projection2d(self, h, p, o, st, s):
        from oracle import nodal2d as n2
        return self._project(p, st, n2.impl_part, {})

    def bella_projection2d_batched(self, W, P, n, o, cfg, st, s):
        from oracle import nodal2d as n2
        from pybella_gb300 import _lib
        for m in range(n):
            self._project(ctypes.byref(_lib.Proj2D.from_address(P[m])), ctypes.byref(st[m]), n2.impl_part, {})
        return 0

    def bella_cfl_maxima(self, rho, rhou, rhov, rhow, rhoY, n, gamm, Msq, scratch, out, s):
        a = {k: _arr(v, (n,)) for k, v in (("rho", rho), ("rhou", rhou), ("rhov", rhov), ("rhow", rhow),
                                            ("rhoY", rhoY))}
        c = np.sqrt(gamm * a["rhoY"] ** gamm / a["rho"]) * (1.0 / np.sqrt(Msq))
        u, v, w = (np.abs(a[k] / a["rho"]) for k in ("rhou", "rhov", "rhow"))
        for k, m in enumerate((u.max(), v.max(), w.max(), (u + c).max(), (v + c).max(), (w + c).max())):
            out[k] = m
        return 0

    # 3D
    def bella_boundary3d(self, p, s):
        from oracle import proj3d as o3
        return self._boundary(p, o3.set_explicit_boundary_data)

    def bella_advective_fluxes3d(self, p, s):
        return self._mass(p, 3)

    def bella_advect3d(self, p, dt, odd, s):
        return self._strang(p, dt, odd, 3)

    def bella_advect_rk3d(self, p, dt, s):
        return self._rk(p, dt, 3)

    def _e3(self, e):
        gi = np.array([e.inx + 3, e.iny + 3, e.inz + 3, e.x_wall, e.y_wall, e.z_wall, e.is_compressible,
                       e.is_ArakawaKonor, e.div_sign_2d], dtype=np.int32)
        gd = np.array([e.dx, e.dy, e.dz, e.dt, e.Msq, e.g, e.gamm, e.nonhydro, e.compressibility, *e.coriolis,
                       *e.wind])
        return gi, gd, (ctypes.c_void_p * 6)(e.rho, e.rhou, e.rhov, e.rhow, e.rhoY, e.rhoX)

    def bella_expl_part3d(self, p, s):
        e = p._obj
        gi, gd, F = self._e3(e)
        self.e3.e3_host_expl_part(_vp(gi), _vp(gd), F, _vp(e.S0n), _vp(e.hydro_rhoY0), _vp(e.strat_inv))
        return 0

    def bella_euler_forward3d(self, p, s):
        e = p._obj
        gi, gd, F = self._e3(e)
        self.e3.e3_host_forward(_vp(gi), _vp(gd), F, _vp(e.p2), _vp(e.rhs_out), _vp(e.scratch), _vp(e.S0c),
                                _vp(e.S0n), _vp(e.hydro_rhoY0), _vp(e.strat_inv))
        return 0

    def bella_projection3d(self, h, p, o, st, s):
        from oracle import proj3d as o3
        from oracle.krylov import bicgstab_legacy
        x_sign = 1.0 if p._obj.div_sign_2d else -1.0
        return self._project(p, st, o3.impl_part,
                             dict(solver=lambda op, b, tol, mi: bicgstab_legacy(op, b, 1e-13, 20000), x_sign=x_sign))


def _install(monkeypatch, tmp_path, ctx):
    from pybella_gb300 import _lib
    stand = _Stand(_build(tmp_path, "advect_host.cpp"), _build(tmp_path, "expl3d_host.cpp"), ctx)

    class _Workspace:
        def __init__(self, device=0):
            self._lib, self.handle = stand, ctypes.c_void_p(0)
    monkeypatch.setattr(_lib, "Workspace", _Workspace)


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_device_step2d_orchestration_vs_reference(host_torch, monkeypatch, tmp_path):
    from oracle import cases
    from pybella_gb300.time_update import DeviceStep2D
    d = np.load(golden("step_kat.npz"))
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble(inx=64, iny=32)
    hn, hc = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"])
    _install(monkeypatch, tmp_path, NS(grid=grid, prm=prm, hn=hn, hc=hc, sf=sf))
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
    dt = float(d["meta"][2])
    for step in (0, 1):
        run.step(step, dt)
        run.download(Sol, mpv)
        t = "s%d_" % (step + 1)
        # the face mass fluxes are direct sums here, FFT convolutions in the reference
        for k in FIELDS:
            assert _rel(getattr(Sol, k), d[t + k]) < 1e-10, (step, k)
        assert _rel(mpv.p2_nodes, d[t + "p2"]) < 1e-10


def test_device_step3d_orchestration_vs_oracle(host_torch, monkeypatch, tmp_path):
    from oracle import advection3d as a3, cases, step3d
    from oracle.krylov import bicgstab_legacy
    from pybella_gb300.time_update import DeviceStep3D
    grid, prm, Sol, p2, hn, hc, sf = cases.bubble_3d(13, 9, 13, seed=3, wind=0.0)
    _install(monkeypatch, tmp_path, NS(grid=grid, prm=prm, hn=hn, hc=hc, sf=sf))
    S0c = np.broadcast_to(hc["S0"][None, :, None], grid.elem_sc).copy()
    S = NS(**{k: Sol[k].copy() for k in FIELDS})
    mpv = NS(p2_nodes=p2.copy(), HydroState=NS(rhoY0=hc["rhoY0"], get_S0c=lambda elem: S0c),
             HydroState_n=NS(S0=hn["S0"]))
    node = NS(iicx=grid.inx, iicy=grid.iny, iicz=grid.inz, dx=grid.dx, dy=grid.dy, dz=grid.dz)
    ud = NS(bdry_type=["wrap", "symmetric", "wrap"], gravity_strength=[0.0, prm.g, 0.0], Msq=prm.Msq,
            nonhydrostasy=1.0, compressibility=0.0, is_compressible=0, coriolis_strength=np.zeros(3),
            u_wind_speed=0.0, v_wind_speed=0.0, w_wind_speed=0.0, stratification=sf, tol=1e-12,
            max_iterations=20000)
    run = DeviceStep3D(S, mpv, NS(ndim=3, y=grid.elem_y), node, ud, NS(gamm=prm.gamm))
    Sc = {k: v.copy() for k, v in Sol.items()}
    pc = p2.copy()
    flux = a3.new_flux(grid)
    solver = lambda op, b, tol, maxiter: bicgstab_legacy(op, b, 1e-13, 20000)
    for step in (0, 1):
        run.step(step, 0.02169)
        run.download(S, mpv)
        Sc = step3d.time_step(Sc, pc, flux, step, 0.02169, grid, prm, hn, hc, S0c, sf, solver=solver)
        for k in FIELDS:
            assert _rel(getattr(S, k), Sc[k]) < 1e-10, (step, k)


def test_device_step2d_run_to_tout_vs_reference(host_torch, monkeypatch, tmp_path):
    """DeviceStep2D.run: the CFL time step from the device state's maxima and the
    loop of time_update.do, to tout = 0.1 (two fixed steps, a third cut to tout),
    against the reference's run (step_kat.npz)."""
    from oracle import cases
    from pybella_gb300.time_update import DeviceStep2D
    d = np.load(golden("step_kat.npz"))
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble(inx=64, iny=32)
    hn, hc = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"])
    _install(monkeypatch, tmp_path, NS(grid=grid, prm=prm, hn=hn, hc=hc, sf=sf))
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
    assert len(dts) == 3 and t == pytest.approx(float(d["meta"][7]), rel=1e-15)
    for k in FIELDS:
        assert _rel(getattr(Sol, k), d["s4_" + k]) < 1e-10, k
    assert _rel(mpv.p2_nodes, d["s4_p2"]) < 1e-10


def test_dynamic_timestep_matches_oracle():
    """The host arithmetic of the CFL time step (pybella_gb300.time_update) from the
    state's maxima equals the oracle's cfl.py restatement, both branches."""
    from oracle import cases, step2d
    from pybella_gb300.time_update import dynamic_timestep
    grid, prm, Sol, p2, hn, hc, sf = cases.rising_bubble(inx=64, iny=32)
    rng = np.random.default_rng(2)
    Sol = dict(Sol, rhou=0.3 * Sol["rho"] * rng.standard_normal(Sol["rho"].shape),
               rhov=0.2 * Sol["rho"] * rng.standard_normal(Sol["rho"].shape))
    c = np.sqrt(prm.gamm * Sol["rhoY"] ** prm.gamm / Sol["rho"]) * (1.0 / np.sqrt(prm.Msq))
    u, v, w = (np.abs(Sol[k] / Sol["rho"]) for k in ("rhou", "rhov", "rhow"))
    maxima = [u.max(), v.max(), w.max(), (u + c).max(), (v + c).max(), (w + c).max()]
    for step, t, tout in ((0, 0.0, 1.0), (3, 0.0, 1.0), (3, 0.99, 1.0)):
        ref, _, _ = step2d.dynamic_timestep(Sol, t, tout, grid, prm, step, dtfixed=0.01)
        assert dynamic_timestep(maxima, t, tout, (grid.dx, grid.dy, 1.0), step, dtfixed=0.01) == ref
        ref_ac = step2d.dynamic_timestep(Sol, t, tout, grid, prm, step, acoustic_timestep=1)
        assert dynamic_timestep(maxima, t, tout, (grid.dx, grid.dy, 1.0), step, acoustic_timestep=1) == ref_ac


def test_device_step2d_run_outputs_carries_the_step(host_torch, monkeypatch, tmp_path):
    """Two output times (0.1, then 0.11) through DeviceStep2D.run_outputs continue one
    run: the step index carries over, so the second window neither repeats the fixed
    first steps ('CFLfixed') nor restarts the Strang order, and t is reset to the
    rounded output time between them -- as the oracle's restatement of the
    reference's output loop (__main__.py:198-393) does."""
    from oracle import cases, step2d
    from pybella_gb300.time_update import DeviceStep2D
    d = np.load(golden("step_kat.npz"))
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble(inx=64, iny=32)
    hn, hc = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"])
    _install(monkeypatch, tmp_path, NS(grid=grid, prm=prm, hn=hn, hc=hc, sf=sf))
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
    touts = [0.1, 0.11]
    seen = []
    t, step = run.run_outputs(touts, 10000, t_ref=1000.0, on_output=lambda t, s: seen.append((t, s)))
    run.download(Sol, mpv)
    rec = []
    Sc = {k: d["in_" + k].copy() for k in FIELDS}
    pc = d["p2_in"].copy()
    Sc, tc, stepc = step2d.run_outputs(Sc, pc, touts, 10000, grid, prm, hn, hc, S0c, sf, 1000.0,
                                       on_output=lambda t, S, p, s: rec.append((t, s)))
    assert seen == rec and step == stepc and t == tc == 0.11
    assert seen[0][1] == 3 and seen[1][1] > 3
    for k in FIELDS:
        assert _rel(getattr(Sol, k), Sc[k]) < 1e-10, k
    assert _rel(mpv.p2_nodes, pc) < 1e-10


def test_dynamic_timestep_propagates_nan():
    """A NaN maximum (a state that is no longer finite) gives a NaN time step, as
    numpy's .max() does in the reference (cfl.py:25-45), instead of a finite dt
    from the other maxima."""
    from pybella_gb300.time_update import dynamic_timestep
    ok = [0.1, 0.2, 0.0, 1.1, 1.2, 1.0]
    assert np.isfinite(dynamic_timestep(ok, 0.0, 1.0, (0.01, 0.01, 1.0), 3))
    for k in range(6):
        bad = list(ok)
        bad[k] = float("nan")
        assert np.isnan(dynamic_timestep(bad, 0.0, 1.0, (0.01, 0.01, 1.0), 3))
        assert np.isnan(dynamic_timestep(bad, 0.0, 1.0, (0.01, 0.01, 1.0), 3, acoustic_timestep=1))


def test_device_run_stops_on_a_non_finite_state(host_torch, monkeypatch, tmp_path):
    """DeviceStep2D.run raises on a NaN in the state before it takes a step."""
    from oracle import cases
    from pybella_gb300.time_update import DeviceStep2D
    d = np.load(golden("step_kat.npz"))
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble(inx=64, iny=32)
    hn, hc = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"])
    _install(monkeypatch, tmp_path, NS(grid=grid, prm=prm, hn=hn, hc=hc, sf=sf))
    S0c = d["S0c"]
    rhou = d["in_rhou"].copy()
    rhou[10, 10] = np.nan
    Sol = NS(**{k: d["in_" + k].copy() for k in FIELDS})
    Sol.rhou = rhou
    mpv = NS(p2_nodes=d["p2_in"].copy(), HydroState=NS(rhoY0=hc["rhoY0"], get_S0c=lambda elem: S0c),
             HydroState_n=NS(S0=hn["S0"]))
    ud = NS(bdry_type=["wrap", "symmetric", "symmetric"], gravity_strength=[0.0, prm.g, 0.0], Msq=prm.Msq,
            nonhydrostasy=1.0, compressibility=0.0, is_compressible=0, coriolis_strength=np.zeros(3),
            u_wind_speed=0.0, v_wind_speed=0.0, w_wind_speed=0.0, stratification=sf, tol=1e-10,
            max_iterations=6000)
    run = DeviceStep2D(Sol, mpv, NS(ndim=2, y=grid.elem_y), NS(iicx=grid.inx, iicy=grid.iny, dx=grid.dx, dy=grid.dy),
                       ud, NS(gamm=prm.gamm))
    with pytest.raises(FloatingPointError):
        run.run(0.0, 0.1, 10, t_ref=1000.0, step=2)


def test_ensemble_step2d_orchestration(host_torch, monkeypatch, tmp_path):
    """EnsembleStep2D: each member's stages in the order of DeviceStep2D.step and
    both projections through the batched entry point (stood in for by the oracle's
    impl_part per member): two members of the 64x32 bubble (different amplitudes)
    after two steps equal the same members stepped one by one."""
    from oracle import cases
    from pybella_gb300.time_update import DeviceStep2D, EnsembleStep2D
    d = np.load(golden("step_kat.npz"))
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble(inx=64, iny=32)
    hn, hc = dict(hn, S0=d["S0n"]), dict(hc, rhoY0=d["rhoY0"])
    _install(monkeypatch, tmp_path, NS(grid=grid, prm=prm, hn=hn, hc=hc, sf=sf))
    S0c = d["S0c"]
    ud = NS(bdry_type=["wrap", "symmetric", "symmetric"], gravity_strength=[0.0, prm.g, 0.0], Msq=prm.Msq,
            nonhydrostasy=1.0, compressibility=0.0, is_compressible=0, coriolis_strength=np.zeros(3),
            u_wind_speed=0.0, v_wind_speed=0.0, w_wind_speed=0.0, stratification=sf, tol=1e-10,
            max_iterations=6000)

    def member(scale):
        Sol = NS(**{k: d["in_" + k].copy() for k in FIELDS})
        Sol.rho = Sol.rhoY / (1.0 + scale * (Sol.rhoY / d["in_rho"] - 1.0))
        mpv = NS(p2_nodes=d["p2_in"].copy(), HydroState=NS(rhoY0=hc["rhoY0"], get_S0c=lambda elem: S0c),
                 HydroState_n=NS(S0=hn["S0"]))
        run = DeviceStep2D(Sol, mpv, NS(ndim=2, y=grid.elem_y),
                           NS(iicx=grid.inx, iicy=grid.iny, dx=grid.dx, dy=grid.dy), ud, NS(gamm=prm.gamm))
        return run, Sol, mpv
    ens = [member(1.0), member(1.2)]
    alone = [member(1.0), member(1.2)]
    E = EnsembleStep2D([m[0] for m in ens], precision="fp64")
    dts = [0.02169, 0.02169]
    for step in (0, 1):
        E.step(step, dts)
        for (run, _, _), dt in zip(alone, dts):
            run.step(step, dt)
    assert len(E.stats) == 4 and all(len(x) == 2 for x in E.stats)
    for (re, Se, me), (ra, Sa, ma) in zip(ens, alone):
        re.download(Se, me)
        ra.download(Sa, ma)
        for k in FIELDS:
            np.testing.assert_array_equal(getattr(Se, k), getattr(Sa, k), err_msg=k)
        np.testing.assert_array_equal(me.p2_nodes, ma.p2_nodes)
