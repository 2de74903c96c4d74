"""Drop-in for the reference's implicit projection step on the GPU.

``euler_backward_non_advective_impl_part`` keeps the reference's signature
(second_projection.py:97) and effect: ``Sol`` (momenta, rhoX) and
``mpv.p2_nodes`` are updated in place and ``mpv.rhs`` receives the nodal
divergence right-hand side.  The whole step -- boundary data, coefficients,
Coriolis factors, Jacobi diagonal, divergence, the BiCGStab solve, ghost
nodes, correction -- runs as kernels of libbella_gb300
(``bella_projection2d``, ``bella_projection3d``).  The reference's 3D step
cannot run (second_projection.py:183-203); its 3D pieces can, and the 3D
device step assembles them with the glue of the 2D branch.

``euler_forward_non_advective`` (second_projection.py:22) and
``euler_backward_non_advective_expl_part`` (:77) are the explicit parts of the
step (bella_euler_forward2d, bella_expl_part2d), with the same signatures and
in-place effects.

Not reproduced: the side-effect attributes ``mpv.wplus``, ``mpv.wcenter``,
``mpv.nu_c`` and ``mpv.u/v/w`` that the reference leaves behind; nothing on
the projection path reads them afterwards.
"""
import ctypes
import logging

import numpy as np
import torch

from . import _lib

_FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")
_ws_cache = {}
total_iter = 0
total_calls = 0


def _is_wall(bt):
    v = getattr(bt, "value", bt)
    return v in ("symmetric", "radiation") or str(v).lower() in ("wall", "rayleigh")


def _workspace(dev):
    ws = _ws_cache.get(dev.index)
    if ws is None:
        ws = _lib.Workspace(dev.index)
        _ws_cache[dev.index] = ws
    return ws


def euler_backward_non_advective_impl_part(Sol, mpv, elem, node, ud, th, t, dt, alpha_diff, Sol0=None,
                                           writer=None, label=None, debug=False, precision="df64",
                                           stats=None, device=None, preconditioner="none", div_sign_2d=False):
    """Implicit nodal pressure projection of one (half) time step on the GPU.

    Mirrors second_projection.py:97-277 in 2D (``bella_projection2d``) and in 3D
    (``bella_projection3d``: the reference's 3D pieces with the glue of its 2D
    branch, whose own 3D branch cannot run).  ``precision`` selects the Krylov
    arithmetic ('df64' double-float by default, 'fp64', 'mixed'); the stop test
    is the reference's ``tol=ud.tol`` on the FP64 true residual.
    ``preconditioner='background'`` solves with the background solve as the
    preconditioner of flexible BiCGStab (y must be a wall).  3D: ``div_sign_2d``
    gives the divergence's x term the 2D branch's sign instead of the 3D
    branch's (second_projection.py:563), which a 3D time step needs to stay bounded.
    """
    global total_iter, total_calls
    if elem.ndim not in (2, 3):
        raise NotImplementedError("the device projection is 2D or 3D")
    if hasattr(ud, "LAMB_BDRY"):
        raise NotImplementedError("the LAMB_BDRY variant is not on this path")
    if preconditioner not in ("none", "background"):
        raise ValueError("preconditioner must be 'none' or 'background'")
    three = elem.ndim == 3
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    keep = {}

    def d(a, name):
        t_ = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
        keep[name] = t_
        return ctypes.c_void_p(t_.data_ptr())

    args = _lib.Proj3D() if three else _lib.Proj2D()
    args.inx, args.iny = int(node.iicx), int(node.iicy)
    args.x_wall, args.y_wall = int(_is_wall(ud.bdry_type[0])), int(_is_wall(ud.bdry_type[1]))
    args.dx, args.dy, args.dt = float(node.dx), float(node.dy), float(dt)
    args.precond = 1 if preconditioner == "background" else 0
    if three:
        args.inz, args.z_wall, args.dz = int(node.iicz), int(_is_wall(ud.bdry_type[2])), float(node.dz)
        args.div_sign_2d = int(bool(div_sign_2d))
    args.Msq, args.g, args.gamm = float(ud.Msq), float(ud.gravity_strength[1]), float(th.gamm)
    args.nonhydro, args.compressibility = float(ud.nonhydrostasy), float(ud.compressibility)
    for k in range(3):
        args.coriolis[k] = float(ud.coriolis_strength[k])
    args.is_compressible = int(ud.is_compressible)
    for f in _FIELDS:
        setattr(args, f, d(getattr(Sol, f), f))
        setattr(args, f + "0", d(getattr(Sol0, f), f + "0") if Sol0 is not None else ctypes.c_void_p(0))
    args.p2 = d(mpv.p2_nodes, "p2")
    args.hydro_rhoY0 = d(mpv.HydroState.rhoY0, "hydro_rhoY0")
    args.S0n = d(mpv.HydroState_n.S0, "S0n")
    strat = np.array([1.0 / ud.stratification(y) for y in elem.y], dtype=np.float64)
    args.strat_inv = d(strat, "strat_inv")
    rhs = torch.empty(tuple(node.isc[:elem.ndim]), dtype=torch.float64, device=dev)
    args.rhs_out = ctypes.c_void_p(rhs.data_ptr())
    ws = _workspace(dev)
    o = _lib.SolveOpts()
    ws._lib.bella_solve_opts_default(ctypes.byref(o))
    o.tol = float(ud.tol)
    o.maxiter = int(ud.max_iterations)
    o.precision = {"fp64": 0, "mixed": 1, "df64": 2}[precision]
    st = _lib.SolveStats()
    with torch.cuda.device(dev):
        fn = ws._lib.bella_projection3d if three else ws._lib.bella_projection2d
        rc = fn(ws.handle, ctypes.byref(args), ctypes.byref(o), ctypes.byref(st),
                ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    _lib.check(rc, "bella_projection%dd" % elem.ndim)
    for f in _FIELDS:
        getattr(Sol, f)[...] = keep[f].cpu().numpy()
        if Sol0 is not None:
            getattr(Sol0, f)[...] = keep[f + "0"].cpu().numpy()
    mpv.p2_nodes[...] = keep["p2"].cpu().numpy()
    mpv.rhs[...] = rhs.cpu().numpy()
    total_iter += st.iterations
    total_calls += 1
    logging.info(st.iterations)
    logging.info("Total calls to BiCGStab routine = %i, total iterations = %i" % (total_calls, total_iter))
    if stats is not None:
        stats.update(st.as_dict())
    if rc != _lib.BELLA_OK:
        logging.warning("projection solve status %d (%s), true relative residual %.3e",
                        rc, ws._lib.bella_status_string(rc).decode(), st.relres)
    return None


def _expl_args(Sol, mpv, elem, node, ud, th, dt, keep, dev, with_p2):
    def d(a, name):
        t_ = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
        keep[name] = t_
        return ctypes.c_void_p(t_.data_ptr())

    a = _lib.Expl2D()
    a.inx, a.iny = int(node.iicx), int(node.iicy)
    a.x_wall, a.y_wall = int(_is_wall(ud.bdry_type[0])), int(_is_wall(ud.bdry_type[1]))
    a.dx, a.dy, a.dt = float(node.dx), float(node.dy), float(dt)
    a.Msq, a.g, a.gamm = float(ud.Msq), float(ud.gravity_strength[1]), float(th.gamm)
    a.nonhydro, a.compressibility = float(ud.nonhydrostasy), float(ud.compressibility)
    for k in range(3):
        a.coriolis[k] = float(ud.coriolis_strength[k])
    a.wind[0], a.wind[1], a.wind[2] = float(ud.u_wind_speed), float(ud.v_wind_speed), float(ud.w_wind_speed)
    a.is_compressible = int(ud.is_compressible)
    a.is_ArakawaKonor = int(getattr(ud, "is_ArakawaKonor", 0))
    for f in _FIELDS:
        setattr(a, f, d(getattr(Sol, f), f))
    if with_p2:
        a.p2 = d(mpv.p2_nodes, "p2")
        a.S0c = d(mpv.HydroState.get_S0c(elem), "S0c")
        rhs = torch.empty(tuple(node.isc[:2]), dtype=torch.float64, device=dev)
        keep["rhs"] = rhs
        a.rhs_out = ctypes.c_void_p(rhs.data_ptr())
    a.S0n = d(mpv.HydroState_n.S0, "S0n")
    a.hydro_rhoY0 = d(mpv.HydroState.rhoY0, "hydro_rhoY0")
    a.strat_inv = d(np.array([1.0 / ud.stratification(y) for y in elem.y], dtype=np.float64), "strat_inv")
    return a


def euler_forward_non_advective(Sol, mpv, elem, node, dt, ud, th, writer=None, label=None, debug=False,
                                device=None):
    """Explicit (forward) projection of second_projection.py:22-74 on the GPU (2D).

    Updates ``Sol`` (momenta, rhoX, ghost cells), ``mpv.p2_nodes`` and
    ``mpv.rhs`` in place, as the reference does.
    """
    if elem.ndim != 2:
        raise NotImplementedError("the device explicit projection is 2D")
    if hasattr(ud, "LAMB_BDRY"):
        raise NotImplementedError("the LAMB_BDRY variant is not on this path")
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    keep = {}
    a = _expl_args(Sol, mpv, elem, node, ud, th, dt, keep, dev, True)
    lib = _lib.load()
    with torch.cuda.device(dev):
        _lib.check(lib.bella_euler_forward2d(ctypes.byref(a), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)),
                   "bella_euler_forward2d")
    for f in _FIELDS:
        setattr(Sol, f, keep[f].cpu().numpy())
    mpv.p2_nodes[...] = keep["p2"].cpu().numpy()
    mpv.rhs[...] = keep["rhs"].cpu().numpy()


def euler_backward_non_advective_expl_part(Sol, mpv, elem, dt, ud, th, device=None):
    """Explicit part of the implicit step, second_projection.py:77-92, on the GPU (2D); updates ``Sol``."""
    if elem.ndim != 2:
        raise NotImplementedError("the device explicit projection is 2D")
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    keep = {}
    # elem doubles as the node grid for the sizes this call needs (the reference passes elem, elem
    # to multiply_inverse_coriolis); the node counts come from elem.sc
    node = _NodeSizes(elem)
    a = _expl_args(Sol, mpv, elem, node, ud, th, dt, keep, dev, False)
    lib = _lib.load()
    with torch.cuda.device(dev):
        _lib.check(lib.bella_expl_part2d(ctypes.byref(a), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)),
                   "bella_expl_part2d")
    for f in _FIELDS:
        setattr(Sol, f, keep[f].cpu().numpy())


class _NodeSizes:
    """Node-grid sizes derived from the cell grid (elem.sc = inx - 1 + 4 per axis)."""

    def __init__(self, elem):
        self.iicx, self.iicy = int(elem.sc[0]) - 3, int(elem.sc[1]) - 3
        self.dx, self.dy = float(elem.dx), float(elem.dy)
