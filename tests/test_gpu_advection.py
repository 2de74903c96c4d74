"""The 2D advection on the device (bella_advective_fluxes2d, bella_advect2d,
bella_advect_rk2d) against the reference's outputs (tests/golden/advect_kat.npz):
the kernels run the arithmetic that tests/test_advect_host.py checks on the CPU."""
import ctypes

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("tag", ["odd", "even", "rk"])
def test_device_advection_matches_reference(tag):
    import torch
    from oracle import cases
    from pybella_gb300 import _lib
    d = np.load(golden("advect_kat.npz"))
    inx, iny, dt = int(d["meta"][0]), int(d["meta"][1]), float(d["meta"][2])
    grid, prm, _, _, _, _, _ = cases.rising_bubble(inx=inx, iny=iny)
    icx, icy = grid.elem_sc
    keep = {}

    def dev(name, arr):
        keep[name] = torch.tensor(np.ascontiguousarray(arr, dtype=np.float64), device="cuda")
        return ctypes.c_void_p(keep[name].data_ptr())
    a = _lib.Adv2D()
    a.inx, a.iny, a.x_wall, a.y_wall = inx, iny, int(grid.x_wall), int(grid.y_wall)
    a.dx, a.dy, a.g, a.gamm, a.is_compressible = grid.dx, grid.dy, prm.g, prm.gamm, prm.is_compressible
    for k in FIELDS:
        setattr(a, k, dev(k, d["in_" + k]))
    for q in range(6):
        a.fx[q] = dev("fx%d" % q, np.zeros((icy, icx + 1)))
        a.fy[q] = dev("fy%d" % q, np.zeros((icx, icy + 1)))
    a.hydro_rhoY0 = dev("rhoY0", d["rhoY0"])
    a.strat_inv = dev("strat", np.ones(icy))
    a.pwchi = dev("pwchi", np.zeros((icx, icy)))
    lib = _lib.load()
    assert lib.bella_advective_fluxes2d(ctypes.byref(a), None) == 0
    torch.cuda.synchronize()
    assert _rel(keep["fx4"].cpu().numpy(), d["flux0_rhoY"]) < 1e-13
    assert _rel(keep["fy4"].cpu().numpy(), d["flux1_rhoY"]) < 1e-13
    if tag == "rk":
        assert lib.bella_advect_rk2d(ctypes.byref(a), 0.5 * dt, None) == 0
    else:
        assert lib.bella_advect2d(ctypes.byref(a), dt, 1 if tag == "odd" else 0, None) == 0
    torch.cuda.synchronize()
    if tag == "rk":
        assert _rel(keep["pwchi"].cpu().numpy(), d["rk_pwchi"]) < 1e-10
    for k in FIELDS:
        got, ref = keep[k].cpu().numpy(), d["%s_%s" % (tag, k)]
        assert _rel(got, ref) < 1e-12, (k, _rel(got, ref))
        change = np.abs(ref - d["in_" + k]).max()
        assert np.abs(got - ref).max() <= 1e-9 * max(change, 1e-300), (k, np.abs(got - ref).max(), change)


@pytest.mark.parametrize("case", ["pwp", "wwp"])
@pytest.mark.parametrize("tag", ["odd", "even", "rk"])
def test_device_advection3d_matches_reference(case, tag):
    """The 3D advection on the device (bella_advect3d, bella_advect_rk3d) against
    the reference's 3D outputs (tests/golden/advect3d_kat.npz)."""
    import torch
    from oracle import proj3d as o3
    from pybella_gb300 import _lib
    d = np.load(golden("advect3d_kat.npz"))
    m = d[case + "_meta"]
    inx, iny, inz, dt = int(m[0]), int(m[1]), int(m[2]), float(m[6])
    grid = o3.Grid3D(inx, iny, inz, -1.0, 1.0, 0.0, 1.0, -1.0, 1.0)
    icx, icy, icz = grid.elem_sc
    keep = {}

    def dev(name, arr):
        keep[name] = torch.tensor(np.ascontiguousarray(arr, dtype=np.float64), device="cuda")
        return ctypes.c_void_p(keep[name].data_ptr())
    a = _lib.Adv3D()
    a.inx, a.iny, a.inz = inx, iny, inz
    a.x_wall, a.y_wall, a.z_wall = int(m[3]), int(m[4]), int(m[5])
    a.dx, a.dy, a.dz, a.g, a.gamm, a.is_compressible = grid.dx, grid.dy, grid.dz, float(m[8]), float(m[9]), 0
    for k in FIELDS:
        setattr(a, k, dev(k, d["%s_in_%s" % (case, k)]))
    shapes = [(icy, icz, icx + 1), (icz, icx, icy + 1), (icx, icy, icz + 1)]
    for q in range(6):
        a.fx[q] = dev("fx%d" % q, np.zeros(shapes[0]))
        a.fy[q] = dev("fy%d" % q, np.zeros(shapes[1]))
        a.fz[q] = dev("fz%d" % q, np.zeros(shapes[2]))
    a.hydro_rhoY0 = dev("rhoY0", d[case + "_rhoY0"])
    a.strat_inv = dev("strat", np.ones(icy))
    a.pwchi = dev("pwchi", np.zeros((icx, icy, icz)))
    lib = _lib.load()
    assert lib.bella_advective_fluxes3d(ctypes.byref(a), None) == 0
    torch.cuda.synchronize()
    for q, nm in enumerate(("fx4", "fy4", "fz4")):
        assert _rel(keep[nm].cpu().numpy(), d["%s_flux%d_rhoY" % (case, q)]) < 1e-13
    if tag == "rk":
        assert lib.bella_advect_rk3d(ctypes.byref(a), 0.5 * dt, None) == 0
    else:
        assert lib.bella_advect3d(ctypes.byref(a), dt, 1 if tag == "odd" else 0, None) == 0
    torch.cuda.synchronize()
    if tag == "rk":
        assert _rel(keep["pwchi"].cpu().numpy(), d[case + "_rk_pwchi"]) < 1e-10
    for k in FIELDS:
        got, ref = keep[k].cpu().numpy(), d["%s_%s_%s" % (case, tag, k)]
        assert _rel(got, ref) < 1e-12, (k, _rel(got, ref))
        change = np.abs(ref - d["%s_in_%s" % (case, k)]).max()
        assert np.abs(got - ref).max() <= 1e-9 * max(change, 1e-300), (k, np.abs(got - ref).max(), change)
