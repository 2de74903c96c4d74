"""Device-resident time steps, 2D and 3D: the reference's ``time_update.do``
(time_update.py:129-489) for the pseudo-incompressible case without blending,
data assimilation or Rayleigh damping, with every array on the GPU between
steps, and its loop with the CFL time step (cfl.py:5-74).

One step, as the reference orders it: boundary data; ``Sol0`` = the state;
face mass fluxes and first-order advection over dt/2 (``bella_advective_fluxes2d``,
``bella_advect_rk2d``); the explicit and implicit projection halves with
``Sol0``'s coefficients (``bella_expl_part2d``, ``bella_projection2d``); face mass
fluxes of that half-step state; the state reset to ``Sol0`` (``p2`` kept); the
forward explicit projection (``bella_euler_forward2d``), Strang-split advection
over dt (``bella_advect2d``) and both projection halves again.  The host only
launches; the state stays in HBM until :meth:`DeviceStep2D.download`.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .second_projection import _is_wall

_FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")
_EPS = np.finfo(float).eps


def dynamic_timestep(maxima, time, time_output, dxyz, step, CFL=0.5, dtfixed0=100.0, dtfixed=100.0,
                     acoustic_timestep=0):
    """The time step of cfl.py:5-74 from the state's maxima (``bella_cfl_maxima``:
    |u|, |v|, |w|, |u|+c, |v|+c, |w|+c); ``dxyz`` = (dx, dy, dz) with dz = 1 in 2D
    (grid.py:110, 171).  Returns dt; NaN when a maximum is NaN (a state that is
    not finite), as the reference's numpy arithmetic gives it (cfl.py:25-45)."""
    if any(m != m for m in maxima):
        return float("nan")
    u_max, v_max, w_max, upc_max, vpc_max, wpc_max = (max(m, _EPS) for m in maxima)
    dx, dy, dz = dxyz
    if acoustic_timestep == 1:
        dt_cfl = min(min(CFL * dx / upc_max, CFL * dy / vpc_max), CFL * dz / wpc_max)
        dt = min(dt_cfl, dtfixed0 + min(step, 1.) * (dtfixed - dtfixed0))
        if dt > (time_output - time):
            dt = (time_output - time) + _EPS
        return dt
    dt_cfl = min(min(CFL * dx / u_max, CFL * dy / v_max), CFL * dz / w_max)
    dt = min(dt_cfl, dtfixed0 + min(step, 1.) * (dtfixed - dtfixed0))
    dt *= min(float(step + 1), 1.0)
    if dt > (time_output - time):
        dt = (time_output - time)
    return dt


class _Loop:
    """The loop of ``do`` (time_update.py:129-140, 686-706) over a device step."""

    def boundary(self):
        fn = self.lib.bella_boundary3d if isinstance(self.adv, _lib.Adv3D) else self.lib.bella_boundary2d
        with torch.cuda.device(self.dev):
            _lib.check(fn(ctypes.byref(self.adv), self._stream()), "set_explicit_boundary_data")

    def cfl_maxima(self):
        out = (ctypes.c_double * 6)()
        f = self.f
        if getattr(self, "_cfl_scratch", None) is None:       # 6 words, allocated once per run
            self._cfl_scratch = torch.zeros(6, dtype=torch.int64, device=self.dev)
        with torch.cuda.device(self.dev):
            _lib.check(self.lib.bella_cfl_maxima(*[ctypes.c_void_p(f[k].data_ptr()) for k in
                                                   ("rho", "rhou", "rhov", "rhow", "rhoY")],
                                                 f["rho"].numel(), self.gamm, self.Msq,
                                                 ctypes.c_void_p(self._cfl_scratch.data_ptr()), out,
                                                 self._stream()),
                       "bella_cfl_maxima")
        return list(out)

    def run(self, t, tout, nsteps, t_ref=None, CFL=0.5, dtfixed0=100.0, dtfixed=100.0, acoustic_timestep=0,
            precision="fp64", step=0):
        """Steps until ``tout`` or until the global step index reaches ``nsteps``
        (the reference's ``stepmax``), dt from the CFL condition of the state at each
        step's start ('CFLfixed': 21.69 / ``t_ref`` while the step index is below 2,
        when ``t_ref`` is given).  ``step`` is the global index to start from: ``do``
        takes it in ``steps`` and returns it (time_update.py:129-135, 706-708), so
        consecutive calls for successive output times continue one run (the Strang
        order, the fixed first steps and the dt ramp follow the global index).
        Returns ``(t, dts, step)``."""
        dts = []
        while t < tout and step < nsteps:
            self.boundary()                                 # :130, before the time step of :135
            dt = dynamic_timestep(self.cfl_maxima(), t, tout, self.dxyz, step, CFL, dtfixed0, dtfixed,
                                  acoustic_timestep)
            if not np.isfinite(dt):
                raise FloatingPointError("non-finite time step at step %d: the state is not finite" % step)
            if t_ref is not None and step < 2:
                dt = 21.69 / t_ref
            self.step(step, dt, precision)
            dts.append(dt)
            t += dt
            step += 1
        return t, dts, step

    def run_outputs(self, touts, stepmax, t=0.0, t_ref=None, precision="fp64", on_output=None, **cfl):
        """The output loop of the reference's driver for one member
        (__main__.py:198-393): :meth:`run` once per output time with the step index
        carried across them, and ``t`` set to the output time rounded to three
        decimals after each (__main__.py:266, 388).  ``on_output(t, step)`` is called
        at every output time (the state is still on the device).  Returns
        ``(t, step)``."""
        step = 0
        for tout in touts:
            t, _, step = self.run(t, float(tout), stepmax, t_ref=t_ref, precision=precision, step=step, **cfl)
            t = float(np.around(tout, 3))
            if on_output is not None:
                on_output(t, step)
        return t, step


class DeviceStep2D(_Loop):
    """The state of a 2D run on one GPU and its time step.

    Built from the reference's objects (``Sol``, ``mpv``, ``elem``, ``node``,
    ``ud``, ``th``); :meth:`step` advances by ``dt`` (``step`` is the step index,
    whose parity picks the Strang order), :meth:`download` writes the state
    back into ``Sol`` and ``mpv.p2_nodes``.
    """

    def __init__(self, Sol, mpv, elem, node, ud, th, device=None):
        if elem.ndim != 2:
            raise NotImplementedError("the device time step is 2D")
        if int(ud.is_compressible) != 0:
            raise NotImplementedError("the pseudo-incompressible step only")
        self.dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        d = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device=self.dev)
        self.f = {k: d(getattr(Sol, k)) for k in _FIELDS}
        self.f0 = {k: torch.empty_like(v) for k, v in self.f.items()}
        self.p2 = d(mpv.p2_nodes)
        icx, icy = self.f["rho"].shape
        self.fx = [torch.zeros((icy, icx + 1), dtype=torch.float64, device=self.dev) for _ in _FIELDS]
        self.fy = [torch.zeros((icx, icy + 1), dtype=torch.float64, device=self.dev) for _ in _FIELDS]
        self.pwchi = torch.zeros((icx, icy), dtype=torch.float64, device=self.dev)
        self.rhs = torch.empty((icx - 1, icy - 1), dtype=torch.float64, device=self.dev)
        self.S0c = d(mpv.HydroState.get_S0c(elem))
        self.S0n = d(mpv.HydroState_n.S0)
        self.rhoY0 = d(mpv.HydroState.rhoY0)
        self.strat_inv = d(np.array([1.0 / ud.stratification(y) for y in elem.y], dtype=np.float64))
        self.ws = _lib.Workspace(self.dev.index)
        self.lib = self.ws._lib
        p = lambda t: ctypes.c_void_p(t.data_ptr())
        inx, iny = int(node.iicx), int(node.iicy)
        xw, yw = int(_is_wall(ud.bdry_type[0])), int(_is_wall(ud.bdry_type[1]))
        g, gamm = float(ud.gravity_strength[1]), float(th.gamm)
        # advection
        a = _lib.Adv2D()
        a.inx, a.iny, a.x_wall, a.y_wall = inx, iny, xw, yw
        a.dx, a.dy, a.g, a.gamm, a.is_compressible = float(node.dx), float(node.dy), g, gamm, 0
        for k in _FIELDS:
            setattr(a, k, p(self.f[k]))
        for q in range(6):
            a.fx[q], a.fy[q] = p(self.fx[q]), p(self.fy[q])
        a.hydro_rhoY0, a.strat_inv, a.pwchi = p(self.rhoY0), p(self.strat_inv), p(self.pwchi)
        self.adv = a
        # explicit projection parts
        e = _lib.Expl2D()
        e.inx, e.iny, e.x_wall, e.y_wall = inx, iny, xw, yw
        e.dx, e.dy = float(node.dx), float(node.dy)
        e.Msq, e.g, e.gamm = float(ud.Msq), g, gamm
        e.nonhydro, e.compressibility = float(ud.nonhydrostasy), float(ud.compressibility)
        for k in range(3):
            e.coriolis[k] = float(ud.coriolis_strength[k])
        e.wind[0], e.wind[1], e.wind[2] = float(ud.u_wind_speed), float(ud.v_wind_speed), float(ud.w_wind_speed)
        e.is_compressible, e.is_ArakawaKonor = 0, int(getattr(ud, "is_ArakawaKonor", 0))
        for k in _FIELDS:
            setattr(e, k, p(self.f[k]))
        e.p2, e.rhs_out = p(self.p2), p(self.rhs)
        e.S0c, e.S0n, e.hydro_rhoY0, e.strat_inv = p(self.S0c), p(self.S0n), p(self.rhoY0), p(self.strat_inv)
        self.expl = e
        # implicit projection (coefficients from Sol0 in the half step)
        r = _lib.Proj2D()
        r.inx, r.iny, r.x_wall, r.y_wall = inx, iny, xw, yw
        r.dx, r.dy = float(node.dx), float(node.dy)
        r.Msq, r.g, r.gamm = float(ud.Msq), g, gamm
        r.nonhydro, r.compressibility = float(ud.nonhydrostasy), float(ud.compressibility)
        for k in range(3):
            r.coriolis[k] = float(ud.coriolis_strength[k])
        r.is_compressible = 0
        for k in _FIELDS:
            setattr(r, k, p(self.f[k]))
        r.p2, r.rhs_out = p(self.p2), p(self.rhs)
        r.hydro_rhoY0, r.S0n, r.strat_inv = p(self.rhoY0), p(self.S0n), p(self.strat_inv)
        self.proj = r
        self.opts = _lib.SolveOpts()
        self.lib.bella_solve_opts_default(ctypes.byref(self.opts))
        self.opts.tol, self.opts.maxiter = float(ud.tol), int(ud.max_iterations)
        self.stats = []
        self.gamm, self.Msq, self.dxyz = gamm, float(ud.Msq), (float(node.dx), float(node.dy), 1.0)

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def _project(self, dt, with_sol0):
        r = self._proj_args(dt, with_sol0)
        st = _lib.SolveStats()
        rc = self.lib.bella_projection2d(self.ws.handle, ctypes.byref(r), ctypes.byref(self.opts), ctypes.byref(st),
                                         self._stream())
        _lib.check(rc, "bella_projection2d")
        self.stats.append(st.as_dict())

    def _expl_part(self, dt):
        self.expl.dt = float(dt)
        _lib.check(self.lib.bella_expl_part2d(ctypes.byref(self.expl), self._stream()), "bella_expl_part2d")

    def _half_step(self, dt):
        """The step up to its first projection: boundary data, Sol0, face mass fluxes,
        advection over dt/2, explicit projection half (time_update.py:130-247)."""
        lib, s, h = self.lib, self._stream(), 0.5 * dt
        with torch.cuda.device(self.dev):
            _lib.check(lib.bella_boundary2d(ctypes.byref(self.adv), s), "bella_boundary2d")   # :130
            for k in _FIELDS:                                                  # Sol0 (:205)
                self.f0[k].copy_(self.f[k])
            _lib.check(lib.bella_advective_fluxes2d(ctypes.byref(self.adv), s), "bella_advective_fluxes2d")
            _lib.check(lib.bella_advect_rk2d(ctypes.byref(self.adv), h, s), "bella_advect_rk2d")    # :224
            self._expl_part(h)                                                 # :247

    def _full_step(self, step, dt):
        """Between the two projections: fluxes of the half-step state, Sol reset to
        Sol0, forward explicit part, Strang-split advection over dt, explicit
        projection half (time_update.py:337-455)."""
        lib, s, h = self.lib, self._stream(), 0.5 * dt
        with torch.cuda.device(self.dev):
            _lib.check(lib.bella_advective_fluxes2d(ctypes.byref(self.adv), s), "bella_advective_fluxes2d")
            for k in _FIELDS:                                                  # Sol = Sol0 (:376)
                self.f[k].copy_(self.f0[k])
            self.expl.dt = float(h)                                            # :419
            _lib.check(lib.bella_euler_forward2d(ctypes.byref(self.expl), s), "bella_euler_forward2d")
            _lib.check(lib.bella_advect2d(ctypes.byref(self.adv), dt, int(step) % 2, s), "bella_advect2d")  # :434
            self._expl_part(h)                                                 # :455

    def _proj_args(self, dt, with_sol0):
        """The projection's argument block for a projection over ``dt`` (with Sol0's
        coefficients in the half step)."""
        r = self.proj
        r.dt = float(dt)
        for k in _FIELDS:
            setattr(r, k + "0", ctypes.c_void_p(self.f0[k].data_ptr()) if with_sol0 else ctypes.c_void_p(0))
        return r

    def step(self, step, dt, precision="fp64"):
        """One time step of length ``dt`` (time_update.py:129-489)."""
        self.opts.precision = {"fp64": 0, "mixed": 1, "df64": 2}[precision]
        with torch.cuda.device(self.dev):
            self._half_step(dt)
            self._project(0.5 * dt, True)                                      # :251
            self._full_step(step, dt)
            self._project(0.5 * dt, False)                                     # :462

    def download(self, Sol, mpv):
        torch.cuda.synchronize(self.dev)
        for k in _FIELDS:
            setattr(Sol, k, self.f[k].cpu().numpy())
        mpv.p2_nodes[...] = self.p2.cpu().numpy()


class EnsembleStep2D:
    """Time steps of an ensemble of 2D members on one GPU, the members' elliptic
    solves batched.

    The reference runs an ensemble's members one after another through
    ``time_update.do`` (__main__.py:223-254).  Here every member is a
    :class:`DeviceStep2D` (its own state and workspace, any grid size); each
    stage of the step runs for all members in turn, and at each of the step's
    two projections (time_update.py:251, 462) all members' solves run in one
    persistent launch (``bella_projection2d_batched``), so a step of the whole
    ensemble is two solver launches whatever the number of members.  Every
    member takes its own time step (its CFL condition; 'CFLfixed' while the step
    index is below 2).
    """

    def __init__(self, members, precision="df64", config=-1):
        if not members:
            raise ValueError("an ensemble needs members")
        self.members = list(members)
        self.dev = self.members[0].dev
        if any(m.dev != self.dev for m in self.members):
            raise ValueError("all members must live on one GPU")
        self.lib = self.members[0].lib
        self.config = int(config)
        self.opts = _lib.SolveOpts()
        self.lib.bella_solve_opts_default(ctypes.byref(self.opts))
        self.opts.tol = float(self.members[0].opts.tol)
        self.opts.maxiter = int(self.members[0].opts.maxiter)
        self.opts.precision = {"fp64": 0, "df64": 2}[precision]
        n = len(self.members)
        self._ws = (ctypes.c_void_p * n)(*[m.ws.handle.value for m in self.members])
        self.stats = []

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def _project_all(self, dts, with_sol0):
        n = len(self.members)
        args = [m._proj_args(0.5 * dt, with_sol0) for m, dt in zip(self.members, dts)]
        ptrs = (ctypes.c_void_p * n)(*[ctypes.addressof(a) for a in args])
        st = (_lib.SolveStats * n)()
        rc = self.lib.bella_projection2d_batched(self._ws, ptrs, n, ctypes.byref(self.opts), self.config, st,
                                                 self._stream())
        _lib.check(rc, "bella_projection2d_batched")
        self.stats.append([s_.as_dict() for s_ in st])

    def step(self, step, dts):
        """One time step of every member, member m by ``dts[m]``."""
        with torch.cuda.device(self.dev):
            for m, dt in zip(self.members, dts):
                m._half_step(dt)
            self._project_all(dts, True)
            for m, dt in zip(self.members, dts):
                m._full_step(step, dt)
            self._project_all(dts, False)

    def time_steps(self, step, t_ref=None, CFL=0.5):
        """Each member's dt from the CFL condition of its state (cfl.py:5-74), no
        output time in reach; 'CFLfixed' (21.69 / t_ref) while ``step`` < 2."""
        dts = []
        for m in self.members:
            m.boundary()
            dt = dynamic_timestep(m.cfl_maxima(), 0.0, float("inf"), m.dxyz, step, CFL)
            if not np.isfinite(dt):
                raise FloatingPointError("non-finite time step in a member at step %d" % step)
            dts.append(21.69 / t_ref if (t_ref is not None and step < 2) else dt)
        return dts

    def run(self, nsteps, t_ref=None, step=0):
        """``nsteps`` steps of every member; returns the final step index."""
        for _ in range(nsteps):
            self.step(step, self.time_steps(step, t_ref))
            step += 1
        return step


class DeviceStep3D(_Loop):
    """The 3D time step with the state resident on the GPU (the reference's
    ``time_update.do`` in 3D, which the reference itself cannot run: its 3D
    projection step and forward explicit part break on unassigned names and
    array shapes).  The same stages as :class:`DeviceStep2D` on the 3D entry
    points (``bella_advect3d``, ``bella_advect_rk3d``, ``bella_expl_part3d``,
    ``bella_euler_forward3d``, ``bella_projection3d``), with the divergence's x
    term in the 2D branch's sign: with the reference's 3D sign the step blows up
    within a few steps.  ``preconditioner='background'`` solves the projections
    with the background solve (y a wall).
    """

    def __init__(self, Sol, mpv, elem, node, ud, th, device=None, preconditioner="none"):
        if elem.ndim != 3:
            raise NotImplementedError("DeviceStep3D is the 3D step")
        if int(ud.is_compressible) != 0:
            raise NotImplementedError("the pseudo-incompressible step only")
        self.dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        d = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device=self.dev)
        self.f = {k: d(getattr(Sol, k)) for k in _FIELDS}
        self.f0 = {k: torch.empty_like(v) for k, v in self.f.items()}
        self.p2 = d(mpv.p2_nodes)
        icx, icy, icz = self.f["rho"].shape
        z = lambda *shape: torch.zeros(shape, dtype=torch.float64, device=self.dev)
        self.fx = [z(icy, icz, icx + 1) for _ in _FIELDS]
        self.fy = [z(icz, icx, icy + 1) for _ in _FIELDS]
        self.fz = [z(icx, icy, icz + 1) for _ in _FIELDS]
        self.pwchi = z(icx, icy, icz)
        self.rhs = z(icx - 1, icy - 1, icz - 1)
        self.scratch = z(icx - 1, icy - 1, icz - 1)
        self.S0c = d(mpv.HydroState.get_S0c(elem))
        self.S0n = d(mpv.HydroState_n.S0)
        self.rhoY0 = d(mpv.HydroState.rhoY0)
        self.strat_inv = d(np.array([1.0 / ud.stratification(y) for y in elem.y], dtype=np.float64))
        self.ws = _lib.Workspace(self.dev.index)
        self.lib = self.ws._lib
        p = lambda t: ctypes.c_void_p(t.data_ptr())
        inx, iny, inz = int(node.iicx), int(node.iicy), int(node.iicz)
        walls = [int(_is_wall(ud.bdry_type[k])) for k in range(3)]
        dx, dy, dz = float(node.dx), float(node.dy), float(node.dz)
        g, gamm = float(ud.gravity_strength[1]), float(th.gamm)
        a = _lib.Adv3D()
        a.inx, a.iny, a.inz = inx, iny, inz
        a.x_wall, a.y_wall, a.z_wall = walls
        a.dx, a.dy, a.dz, a.g, a.gamm, a.is_compressible = dx, dy, dz, g, gamm, 0
        for k in _FIELDS:
            setattr(a, k, p(self.f[k]))
        for q in range(6):
            a.fx[q], a.fy[q], a.fz[q] = p(self.fx[q]), p(self.fy[q]), p(self.fz[q])
        a.hydro_rhoY0, a.strat_inv, a.pwchi = p(self.rhoY0), p(self.strat_inv), p(self.pwchi)
        self.adv = a
        e = _lib.Expl3D()
        e.inx, e.iny, e.inz = inx, iny, inz
        e.x_wall, e.y_wall, e.z_wall = walls
        e.dx, e.dy, e.dz = dx, dy, dz
        e.Msq, e.g, e.gamm = float(ud.Msq), g, gamm
        e.nonhydro, e.compressibility = float(ud.nonhydrostasy), float(ud.compressibility)
        for k in range(3):
            e.coriolis[k] = float(ud.coriolis_strength[k])
        e.wind[0], e.wind[1], e.wind[2] = float(ud.u_wind_speed), float(ud.v_wind_speed), float(ud.w_wind_speed)
        e.is_compressible, e.is_ArakawaKonor = 0, int(getattr(ud, "is_ArakawaKonor", 0))
        for k in _FIELDS:
            setattr(e, k, p(self.f[k]))
        e.p2, e.rhs_out, e.scratch = p(self.p2), p(self.rhs), p(self.scratch)
        e.S0c, e.S0n, e.hydro_rhoY0, e.strat_inv = p(self.S0c), p(self.S0n), p(self.rhoY0), p(self.strat_inv)
        e.div_sign_2d = 1
        self.expl = e
        r = _lib.Proj3D()
        r.inx, r.iny, r.inz = inx, iny, inz
        r.x_wall, r.y_wall, r.z_wall = walls
        r.dx, r.dy, r.dz = dx, dy, dz
        r.Msq, r.g, r.gamm = float(ud.Msq), g, gamm
        r.nonhydro, r.compressibility = float(ud.nonhydrostasy), float(ud.compressibility)
        for k in range(3):
            r.coriolis[k] = float(ud.coriolis_strength[k])
        r.is_compressible = 0
        r.precond = 1 if preconditioner == "background" else 0
        r.div_sign_2d = 1
        for k in _FIELDS:
            setattr(r, k, p(self.f[k]))
        r.p2, r.rhs_out = p(self.p2), p(self.rhs)
        r.hydro_rhoY0, r.S0n, r.strat_inv = p(self.rhoY0), p(self.S0n), p(self.strat_inv)
        self.proj = r
        self.opts = _lib.SolveOpts()
        self.lib.bella_solve_opts_default(ctypes.byref(self.opts))
        self.opts.tol, self.opts.maxiter = float(ud.tol), int(ud.max_iterations)
        self.stats = []
        self.gamm, self.Msq, self.dxyz = gamm, float(ud.Msq), (dx, dy, dz)

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def _project(self, dt, with_sol0):
        r = self.proj
        r.dt = float(dt)
        for k in _FIELDS:
            setattr(r, k + "0", ctypes.c_void_p(self.f0[k].data_ptr()) if with_sol0 else ctypes.c_void_p(0))
        st = _lib.SolveStats()
        rc = self.lib.bella_projection3d(self.ws.handle, ctypes.byref(r), ctypes.byref(self.opts), ctypes.byref(st),
                                         self._stream())
        _lib.check(rc, "bella_projection3d")
        self.stats.append(st.as_dict())

    def _expl_part(self, dt):
        self.expl.dt = float(dt)
        _lib.check(self.lib.bella_expl_part3d(ctypes.byref(self.expl), self._stream()), "bella_expl_part3d")

    def step(self, step, dt, precision="fp64"):
        """One time step of length ``dt``."""
        self.opts.precision = {"fp64": 0, "mixed": 1, "df64": 2}[precision]
        lib, s, h = self.lib, self._stream(), 0.5 * dt
        with torch.cuda.device(self.dev):
            _lib.check(lib.bella_boundary3d(ctypes.byref(self.adv), s), "bella_boundary3d")
            for k in _FIELDS:
                self.f0[k].copy_(self.f[k])
            _lib.check(lib.bella_advective_fluxes3d(ctypes.byref(self.adv), s), "bella_advective_fluxes3d")
            _lib.check(lib.bella_advect_rk3d(ctypes.byref(self.adv), h, s), "bella_advect_rk3d")
            self._expl_part(h)
            self._project(h, True)
            _lib.check(lib.bella_advective_fluxes3d(ctypes.byref(self.adv), s), "bella_advective_fluxes3d")
            for k in _FIELDS:
                self.f[k].copy_(self.f0[k])
            self.expl.dt = float(h)
            _lib.check(lib.bella_euler_forward3d(ctypes.byref(self.expl), s), "bella_euler_forward3d")
            _lib.check(lib.bella_advect3d(ctypes.byref(self.adv), dt, int(step) % 2, s), "bella_advect3d")
            self._expl_part(h)
            self._project(h, False)

    def download(self, Sol, mpv):
        torch.cuda.synchronize(self.dev)
        for k in _FIELDS:
            setattr(Sol, k, self.f[k].cpu().numpy())
        mpv.p2_nodes[...] = self.p2.cpu().numpy()
