"""The 3D projection on the device (bella_projection3d, called through the
reference-facing drop-in ``euler_backward_non_advective_impl_part``) against the
oracle's 3D step, whose pieces reproduce the reference's own 3D outputs bit for
bit (tests/test_oracle_golden.py), and the 257x129x257 projection's fields
across the solver precisions."""
from types import SimpleNamespace as NS

import numpy as np
import pytest

from oracle import cases, proj3d as o3

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")


def _ref_objects(grid, prm, Sol, p2, hn, hc, tol):
    """Reference-shaped Sol / mpv / elem / node / ud / th objects of a 3D state."""
    S = NS(**{f: Sol[f].copy() for f in FIELDS})
    mpv = NS(p2_nodes=p2.copy(), rhs=np.zeros(grid.node_isc), HydroState=NS(rhoY0=hc["rhoY0"]),
             HydroState_n=NS(S0=hn["S0"]))
    elem = NS(ndim=3, y=grid.elem_y)
    node = NS(iicx=grid.inx, iicy=grid.iny, iicz=grid.inz, dx=grid.dx, dy=grid.dy, dz=grid.dz, isc=grid.node_isc)
    ud = NS(bdry_type=["symmetric" if grid.wall(d) else "wrap" for d in range(3)], Msq=prm.Msq,
            gravity_strength=[0.0, prm.g, 0.0], nonhydrostasy=prm.nonhydro, compressibility=prm.compressibility,
            is_compressible=prm.is_compressible, coriolis_strength=np.asarray(prm.coriolis, dtype=np.float64),
            tol=tol, max_iterations=prm.max_iterations, stratification=lambda y: 1.0)
    return S, mpv, elem, node, ud, NS(gamm=prm.gamm)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


CASES = {
    # periodic x / wall y / periodic z, pseudo-incompressible (singular operator)
    "pwp": dict(shape=(13, 9, 13), bdry=(o3.PERIODIC, o3.WALL, o3.PERIODIC), coriolis=(0.0, 0.0, 0.0),
                compressible=False, dt=0.01, sol0=False),
    # wall x / wall y / periodic z, Coriolis, compressible, coefficients from Sol0
    "wwp": dict(shape=(12, 9, 11), bdry=(o3.WALL, o3.WALL, o3.PERIODIC), coriolis=(3.0, 2.0, 1.0),
                compressible=True, dt=0.05, sol0=True),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_projection3d_matches_oracle_step(name):
    """Right-hand side, pressure and corrected momenta of one 3D projection: the
    device step (FP64 BiCGStab) against the oracle's step (scipy-semantics
    BiCGStab), both to tol 1e-12."""
    from pybella_gb300 import second_projection as sp
    c = CASES[name]
    grid, prm, Sol, p2, hn, hc, sf = cases.bubble_3d(*c["shape"], seed=3, bdry=c["bdry"], coriolis=c["coriolis"],
                                                     compressible=c["compressible"], tol=1e-12)
    p2[...] = 0.05 * np.random.default_rng(4).standard_normal(p2.shape)
    Sol0 = None
    if c["sol0"]:
        Sol0 = {k: v.copy() for k, v in Sol.items()}
        Sol0["rho"] = Sol0["rho"] * (1.0 + 0.01 * np.random.default_rng(5).standard_normal(Sol0["rho"].shape))
    # oracle step
    So = {k: v.copy() for k, v in Sol.items()}
    po = p2.copy()
    So0 = None if Sol0 is None else {k: v.copy() for k, v in Sol0.items()}
    out = o3.impl_part(So, po, hn["S0"], hc, sf, grid, prm, c["dt"], Sol0=So0)
    assert out["info"] == 0
    # device step through the drop-in
    S, mpv, elem, node, ud, th = _ref_objects(grid, prm, Sol, p2, hn, hc, 1e-12)
    S0 = None if Sol0 is None else NS(**{f: Sol0[f].copy() for f in FIELDS})
    st = {}
    sp.euler_backward_non_advective_impl_part(S, mpv, elem, node, ud, th, 0.0, c["dt"], 0.0, Sol0=S0,
                                              precision="fp64", stats=st)
    assert st["status"] == 0, st
    assert _rel(mpv.rhs, out["rhs"]) < 1e-12
    assert st["relres"] <= 1e-12
    if c["compressible"]:                # unique pressure
        assert _rel(mpv.p2_nodes, po) < 1e-9
    # corrected momenta: null modes of the operator have zero cell gradients
    for f in ("rhou", "rhov", "rhow", "rhoX"):
        change = np.abs(So[f] - Sol[f]).max()
        assert np.abs(getattr(S, f) - So[f]).max() <= 1e-8 * max(change, 1e-300), f


def _project(grid, prm, Sol, p2, hn, hc, dt, precision, preconditioner="none", tol=1e-10):
    from pybella_gb300 import second_projection as sp
    S, mpv, elem, node, ud, th = _ref_objects(grid, prm, Sol, p2, hn, hc, tol)
    st = {}
    sp.euler_backward_non_advective_impl_part(S, mpv, elem, node, ud, th, 0.0, dt, 0.0, precision=precision,
                                              stats=st, preconditioner=preconditioner)
    return S, mpv, st


def test_projection3d_fields_across_precisions(capsys):
    """One 3D projection at 129x65x129 nodes (warm bubble, seeded momenta), tol
    1e-10: pressure and corrected momenta of the double-float, mixed-precision
    and background-preconditioned solves against the FP64 solve."""
    grid, prm, Sol, p2, hn, hc, sf = cases.bubble_3d(129, 65, 129, seed=7)
    dt = 0.01
    ref_S, ref_mpv, ref_st = _project(grid, prm, Sol, p2, hn, hc, dt, "fp64")
    assert ref_st["status"] == 0, ref_st
    inc = {f: getattr(ref_S, f) - Sol[f] for f in ("rhou", "rhov", "rhow")}
    lines = ["fp64: %d iterations" % ref_st["iterations"]]
    for prec, pc in (("df64", "none"), ("mixed", "none"), ("fp64", "background")):
        S, mpv, st = _project(grid, prm, Sol, p2, hn, hc, dt, prec, pc)
        assert st["status"] == 0, (prec, pc, st)
        # pressure up to the operator's null modes: compare cell gradients via the momenta
        err = {f: np.linalg.norm(getattr(S, f) - getattr(ref_S, f)) / np.linalg.norm(inc[f])
               for f in ("rhou", "rhov", "rhow")}
        for f, e in err.items():
            assert e < 1e-6, (prec, pc, f, e)
        lines.append("%s/%s: %d iterations, fallback %d; rel. L2 error of the momentum increments %s"
                     % (prec, pc, st["iterations"], st["fallback"],
                        ", ".join("%s %.1e" % kv for kv in err.items())))
    with capsys.disabled():
        print("\n3D projection 129x65x129:\n  " + "\n  ".join(lines))


def test_projection3d_background_full_size(capsys):
    """The 3D projection at 257x129x257 nodes with the background-preconditioned
    solve: converged to tol 1e-10 on the FP64 true residual, device time of the
    whole step (coefficients, divergence, background set-up and solve, correction)."""
    import time
    import torch
    grid, prm, Sol, p2, hn, hc, sf = cases.bubble_3d(257, 129, 257, seed=11)
    S, mpv, st = _project(grid, prm, Sol, p2, hn, hc, 0.01, "fp64", "background")
    assert st["status"] == 0 and st["relres"] <= 1e-10, st
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    S, mpv, st = _project(grid, prm, Sol, p2, hn, hc, 0.01, "fp64", "background")
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    assert st["status"] == 0
    dev_ms = _device_projection_ms(grid, prm, Sol, p2, hn, hc, 0.01)
    with capsys.disabled():
        print("\n3D projection 257x129x257, background-preconditioned: %d iterations, relres %.2e, "
              "%.1f ms per call through the drop-in (host arrays), %.1f ms on device-resident arrays"
              % (st["iterations"], st["relres"], t * 1e3, dev_ms))


def _device_projection_ms(grid, prm, Sol, p2, hn, hc, dt, reps=3):
    """CUDA-event time of bella_projection3d (background-preconditioned) on
    device-resident arrays: the state is restored from a device copy between calls."""
    import ctypes
    import torch
    from pybella_gb300 import _lib
    keep = {}

    def dev(name, arr):
        keep[name] = torch.tensor(np.ascontiguousarray(arr, dtype=np.float64), device="cuda")
        return ctypes.c_void_p(keep[name].data_ptr())
    a = _lib.Proj3D()
    a.inx, a.iny, a.inz = grid.inx, grid.iny, grid.inz
    a.x_wall, a.y_wall, a.z_wall = (int(grid.wall(d)) for d in range(3))
    a.dx, a.dy, a.dz, a.dt = grid.dx, grid.dy, grid.dz, dt
    a.Msq, a.g, a.gamm, a.nonhydro, a.compressibility = prm.Msq, prm.g, prm.gamm, prm.nonhydro, prm.compressibility
    a.is_compressible, a.precond = prm.is_compressible, 1
    for f in FIELDS:
        setattr(a, f, dev(f, Sol[f]))
    a.p2 = dev("p2", p2)
    a.hydro_rhoY0 = dev("rhoY0", hc["rhoY0"])
    a.S0n = dev("S0n", hn["S0"])
    a.strat_inv = dev("strat", np.ones(grid.elem_sc[1]))
    saved = {k: keep[k].clone() for k in FIELDS + ("p2",)}
    ws = _lib.Workspace(0)
    o = _lib.SolveOpts()
    ws._lib.bella_solve_opts_default(ctypes.byref(o))
    o.tol, o.maxiter = 1e-10, 1000
    st = _lib.SolveStats()
    times = []
    for _ in range(reps + 1):
        for k, v in saved.items():
            keep[k].copy_(v)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = ws._lib.bella_projection3d(ws.handle, ctypes.byref(a), ctypes.byref(o), ctypes.byref(st),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        e1.record()
        torch.cuda.synchronize()
        assert rc == 0 and st.relres <= 1e-10, (rc, st.as_dict())
        times.append(e0.elapsed_time(e1))
    return float(np.median(times[1:]))
