"""The explicit parts of the projection on the device (bella_euler_forward2d,
bella_expl_part2d) against the reference's outputs (tests/golden/explicit_kat.npz)."""
import ctypes

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")


def _args(d, tag, keep):
    import torch
    from pybella_gb300 import _lib
    sc = d[tag + "_scalars"]
    Msq, g, gamm, nonhydro, compressibility, is_comp, dt = sc[:7]
    a = _lib.Expl2D()
    a.inx, a.iny, a.x_wall, a.y_wall = 64, 32, 0, 1
    a.dx, a.dy, a.dt = 2.0 / 63.0, 1.0 / 31.0, float(dt)
    a.Msq, a.g, a.gamm, a.nonhydro, a.compressibility = Msq, g, gamm, nonhydro, compressibility
    for k in range(3):
        a.coriolis[k] = sc[7 + k]
        a.wind[k] = sc[10 + k]
    a.is_compressible, a.is_ArakawaKonor = int(is_comp), int(sc[13])

    def dev(name, arr):
        t = torch.tensor(np.ascontiguousarray(arr, dtype=np.float64), device="cuda")
        keep[name] = t
        return ctypes.c_void_p(t.data_ptr())
    for f in FIELDS:
        setattr(a, f, dev(f, d["%s_in_%s" % (tag, f)]))
    a.p2 = dev("p2", d[tag + "_p2_in"])
    keep["rhs"] = torch.empty(66, 34, dtype=torch.float64, device="cuda")
    a.rhs_out = ctypes.c_void_p(keep["rhs"].data_ptr())
    a.S0c = dev("S0c", d[tag + "_S0c"])
    a.S0n = dev("S0n", d[tag + "_S0n"])
    a.hydro_rhoY0 = dev("rhoY0", d[tag + "_rhoY0"])
    a.strat_inv = dev("strat_inv", d[tag + "_strat_inv"])
    return a


def _close(got, ref, what):
    scale = max(np.abs(ref).max(), 1e-300)
    assert np.abs(got - ref).max() <= 1e-13 * scale, (what, np.abs(got - ref).max() / scale)


@pytest.mark.parametrize("tag", ["a", "b"])
def test_euler_forward_matches_reference(tag):
    import torch
    from pybella_gb300 import _lib
    d = np.load(golden("explicit_kat.npz"))
    keep = {}
    a = _args(d, tag, keep)
    lib = _lib.load()
    assert lib.bella_euler_forward2d(ctypes.byref(a), None) == 0
    torch.cuda.synchronize()
    for f in FIELDS:
        _close(keep[f].cpu().numpy(), d["%s_fw_%s" % (tag, f)], f)
    _close(keep["p2"].cpu().numpy(), d[tag + "_fw_p2"], "p2")
    _close(keep["rhs"].cpu().numpy(), d[tag + "_fw_rhs"], "rhs")


@pytest.mark.parametrize("tag", ["a", "b"])
def test_expl_part_matches_reference(tag):
    import torch
    from pybella_gb300 import _lib
    d = np.load(golden("explicit_kat.npz"))
    keep = {}
    a = _args(d, tag, keep)
    lib = _lib.load()
    assert lib.bella_expl_part2d(ctypes.byref(a), None) == 0
    torch.cuda.synchronize()
    for f in FIELDS:
        _close(keep[f].cpu().numpy(), d["%s_ex_%s" % (tag, f)], f)


def test_euler_forward_two_walls_vs_oracle():
    """Walls in x and y: the divergence's wall rows are doubled by
    scale_wall_node_values, whose index carries over from the x wall to the y
    wall (pinned in tests/test_oracle_golden.py); device against the oracle."""
    import torch
    from pybella_gb300 import _lib
    from oracle import nodal2d as n2
    d = np.load(golden("explicit_kat.npz"))
    keep = {}
    a = _args(d, "a", keep)
    a.x_wall = 1
    lib = _lib.load()
    assert lib.bella_euler_forward2d(ctypes.byref(a), None) == 0
    torch.cuda.synchronize()
    sc = d["a_scalars"]
    grid = n2.Grid2D(64, 32, -1.0, 1.0, 0.0, 1.0, (n2.WALL, n2.WALL))
    prm = n2.Params(Msq=sc[0], g=sc[1], gamm=sc[2], coriolis=sc[7:10], nonhydro=sc[3],
                    is_compressible=int(sc[5]), compressibility=sc[4])
    Sol = {f: d["a_in_" + f].copy() for f in FIELDS}
    p2 = d["a_p2_in"].copy()
    div = n2.euler_forward_non_advective(Sol, p2, d["a_S0c"], d["a_S0n"], grid, prm, float(sc[6]),
                                         dict(rhoY0=d["a_rhoY0"]), lambda y: 1.0)
    _close(keep["rhs"].cpu().numpy(), div, "rhs")
    for f in FIELDS:
        _close(keep[f].cpu().numpy(), Sol[f], f)
    _close(keep["p2"].cpu().numpy(), p2, "p2")


def test_explicit_parts_time(capsys):
    """Device time of both explicit parts at 640x320 cells (the largest ensemble grid)."""
    import torch
    from pybella_gb300 import _lib
    lib = _lib.load()
    nx, ny = 641, 321
    icx, icy, ncx, ncy = nx + 3, ny + 3, nx + 4, ny + 4
    keep = {}
    a = _lib.Expl2D()
    a.inx, a.iny, a.x_wall, a.y_wall, a.dx, a.dy, a.dt = nx, ny, 0, 1, 2.0 / (nx - 1), 1.0 / (ny - 1), 1e-3
    a.Msq, a.g, a.gamm, a.nonhydro, a.compressibility = 1.16e-3, 1.16, 1.4, 1.0, 0.0
    for f in FIELDS:
        t = torch.ones(icx, icy, dtype=torch.float64, device="cuda")
        keep[f] = t
        setattr(a, f, ctypes.c_void_p(t.data_ptr()))
    for name, shape in (("p2", (ncx, ncy)), ("rhs", (ncx - 2, ncy - 2)), ("S0c", (icx, icy)), ("S0n", (ncy,)),
                        ("rhoY0", (icy,)), ("strat", (icy,))):
        keep[name] = torch.ones(shape, dtype=torch.float64, device="cuda")
    a.p2, a.rhs_out = ctypes.c_void_p(keep["p2"].data_ptr()), ctypes.c_void_p(keep["rhs"].data_ptr())
    a.S0c, a.S0n = ctypes.c_void_p(keep["S0c"].data_ptr()), ctypes.c_void_p(keep["S0n"].data_ptr())
    a.hydro_rhoY0, a.strat_inv = ctypes.c_void_p(keep["rhoY0"].data_ptr()), ctypes.c_void_p(keep["strat"].data_ptr())
    for fn in (lib.bella_euler_forward2d, lib.bella_expl_part2d):
        for _ in range(3):
            assert fn(ctypes.byref(a), None) == 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(20):
            fn(ctypes.byref(a), None)
        e1.record()
        torch.cuda.synchronize()
        with capsys.disabled():
            print("\n%s at 640x320 cells: %.1f us per call" % (fn.__name__, e0.elapsed_time(e1) / 20 * 1e3))


def _ref_objects(d, tag):
    """Reference-shaped Sol / mpv / elem / node / ud / th objects for the drop-ins."""
    from types import SimpleNamespace as NS
    sc = d[tag + "_scalars"]
    Msq, g, gamm, nonhydro, compressibility, is_comp, dt = sc[:7]
    Sol = NS(**{f: d["%s_in_%s" % (tag, f)].copy() for f in FIELDS})
    S0c = d[tag + "_S0c"]
    mpv = NS(p2_nodes=d[tag + "_p2_in"].copy(), rhs=np.zeros((66, 34)),
             HydroState=NS(get_S0c=lambda elem: S0c, rhoY0=d[tag + "_rhoY0"]),
             HydroState_n=NS(S0=d[tag + "_S0n"]))
    dx, dy = 2.0 / 63.0, 1.0 / 31.0
    y = -2 * dy + 0.5 * dy + dy * np.arange(35)
    elem = NS(ndim=2, sc=(67, 35), y=y, dx=dx, dy=dy)
    node = NS(iicx=64, iicy=32, dx=dx, dy=dy, isc=(66, 34))
    ud = NS(bdry_type=["periodic", "wall", "wall"], Msq=Msq, gravity_strength=[0.0, g, 0.0],
            nonhydrostasy=nonhydro, compressibility=compressibility, is_compressible=int(is_comp),
            coriolis_strength=sc[7:10], u_wind_speed=sc[10], v_wind_speed=sc[11], w_wind_speed=sc[12],
            is_ArakawaKonor=int(sc[13]), stratification=lambda yy: 1.0)
    th = NS(gamm=gamm)
    return Sol, mpv, elem, node, ud, th, float(dt)


@pytest.mark.parametrize("tag", ["a", "b"])
def test_python_drop_ins_match_reference(tag):
    """pybella_gb300.second_projection.euler_forward_non_advective and
    euler_backward_non_advective_expl_part with the reference's argument objects."""
    from pybella_gb300 import second_projection as sp
    d = np.load(golden("explicit_kat.npz"))
    Sol, mpv, elem, node, ud, th, dt = _ref_objects(d, tag)
    sp.euler_forward_non_advective(Sol, mpv, elem, node, dt, ud, th)
    for f in FIELDS:
        _close(getattr(Sol, f), d["%s_fw_%s" % (tag, f)], f)
    _close(mpv.p2_nodes, d[tag + "_fw_p2"], "p2")
    _close(mpv.rhs, d[tag + "_fw_rhs"], "rhs")
    Sol, mpv, elem, node, ud, th, dt = _ref_objects(d, tag)
    sp.euler_backward_non_advective_expl_part(Sol, mpv, elem, dt, ud, th)
    for f in FIELDS:
        _close(getattr(Sol, f), d["%s_ex_%s" % (tag, f)], f)
