"""Drop-in for the reference's implicit projection step on the GPU.

``euler_backward_non_advective_impl_part`` keeps the reference's signature
(second_projection.py:97) and effect: ``Sol`` (momenta, rhoX) and
``mpv.p2_nodes`` are updated in place and ``mpv.rhs`` receives the nodal
divergence right-hand side.  The whole step -- boundary data, coefficients,
Coriolis factors, Jacobi diagonal, divergence, the BiCGStab solve, ghost
nodes, correction -- runs as kernels of libbella_gb300
(``bella_projection2d``).  2D only; the reference's 3D branches cannot run.

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
                                           stats=None, device=None):
    """Implicit nodal pressure projection of one (half) time step on the GPU.

    Mirrors second_projection.py:97-277.  ``precision`` selects the Krylov
    arithmetic ('df64' double-float by default, 'fp64', 'mixed'); the stop
    test is the reference's ``tol=ud.tol`` on the FP64 true residual.
    """
    global total_iter, total_calls
    if elem.ndim != 2:
        raise NotImplementedError("the device projection is 2D (the reference's 3D branches cannot run)")
    if hasattr(ud, "LAMB_BDRY"):
        raise NotImplementedError("the LAMB_BDRY variant is not on this path")
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    keep = {}

    def d(a, name):
        t_ = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
        keep[name] = t_
        return ctypes.c_void_p(t_.data_ptr())

    args = _lib.Proj2D()
    args.inx, args.iny = int(node.iicx), int(node.iicy)
    args.x_wall, args.y_wall = int(_is_wall(ud.bdry_type[0])), int(_is_wall(ud.bdry_type[1]))
    args.dx, args.dy, args.dt = float(node.dx), float(node.dy), float(dt)
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
    rhs = torch.empty(tuple(node.isc[:2]), dtype=torch.float64, device=dev)
    args.rhs_out = ctypes.c_void_p(rhs.data_ptr())
    ws = _workspace(dev)
    o = _lib.SolveOpts()
    ws._lib.bella_solve_opts_default(ctypes.byref(o))
    o.tol = float(ud.tol)
    o.maxiter = int(ud.max_iterations)
    o.precision = {"fp64": 0, "mixed": 1, "df64": 2}[precision]
    st = _lib.SolveStats()
    with torch.cuda.device(dev):
        rc = ws._lib.bella_projection2d(ws.handle, ctypes.byref(args), ctypes.byref(o), ctypes.byref(st),
                                        ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    _lib.check(rc, "bella_projection2d")
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
