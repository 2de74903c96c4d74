"""The 3D explicit projection parts' device arithmetic, compiled for the host
(tests/expl3d_host.cpp includes pybella_gb300/csrc/bella_expl3d.cuh and the
advection's boundary lines, as the kernels of bella_expl3d.cu do): the backward
explicit part against the reference's 3D outputs (tests/golden/proj3d_kat.npz),
the forward part against the oracle's (the reference's 3D forward part cannot run)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, proj3d_case

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("expl3d") / "libexpl3d_host.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", out,
                    os.path.join(ROOT, "tests", "expl3d_host.cpp")], check=True)
    return ctypes.CDLL(out)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _geom(grid, prm, dt, wind, ak=0, sign_2d=0):
    gi = np.array([*grid.elem_sc, *[int(grid.wall(d)) for d in range(3)], prm.is_compressible, ak, sign_2d],
                  dtype=np.int32)
    gd = np.array([grid.dx, grid.dy, grid.dz, dt, prm.Msq, prm.g, prm.gamm, prm.nonhydro, prm.compressibility,
                   *prm.coriolis, *wind])
    return gi, gd


@pytest.mark.parametrize("tag", ["a", "b"])
def test_expl_part3d_host_vs_reference(host_lib, tag):
    from oracle import proj3d as o3
    d = np.load(golden("proj3d_kat.npz"))
    grid, prm, dt, S0n, hc, sf = proj3d_case(d, tag)
    Sol = {k: d["%s_in_%s" % (tag, k)].copy() for k in FIELDS}
    o3.set_explicit_boundary_data(Sol, grid, prm, hc, sf)
    F = [np.ascontiguousarray(Sol[k]) for k in FIELDS]
    gi, gd = _geom(grid, prm, dt, d[tag + "_wind"])
    sinv = np.ones(grid.elem_sc[1])
    host_lib.e3_host_expl_part(_ptr(gi), _ptr(gd), (ctypes.c_void_p * 6)(*[a.ctypes.data for a in F]),
                               _ptr(np.ascontiguousarray(S0n)), _ptr(np.ascontiguousarray(hc["rhoY0"])), _ptr(sinv))
    for k, a in zip(FIELDS, F):
        # bit for bit but for the compressible hydrostatic ghost cells of case b, where
        # C's pow and NumPy's ** may differ in the last bit
        np.testing.assert_allclose(a, d["%s_xp_%s" % (tag, k)], rtol=2e-15 if tag == "b" else 0, atol=0,
                                   err_msg=k)


@pytest.mark.parametrize("sign_2d", [0, 1])
@pytest.mark.parametrize("walls,cor,wind", [
    ((False, True, False), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)),
    ((True, True, False), (3.0, 2.0, 1.0), (0.5, 0.0, 0.2)),
])
def test_euler_forward3d_host_vs_oracle(host_lib, walls, cor, wind, sign_2d):
    """Momenta, rhoX, the divergence (mpv.rhs) bit for bit; p2 (compressible, so the
    increment counts) to rounding: the oracle's 2x2x2 mean of rhoY^(gamma-2) is an
    FFT convolution."""
    from oracle import cases, proj3d as o3
    bdry = tuple(o3.WALL if w else o3.PERIODIC for w in walls)
    grid, prm, Sol, p2, hn, hc, sf = cases.bubble_3d(13, 9, 11, seed=5, bdry=bdry, coriolis=cor, compressible=True)
    p2[...] = 0.05 * np.random.default_rng(6).standard_normal(p2.shape)
    S0c = np.broadcast_to(hc["S0"][None, :, None], grid.elem_sc).copy()
    dt = 0.02
    So = {k: v.copy() for k, v in Sol.items()}
    po = p2.copy()
    div = o3.euler_forward_non_advective(So, po, S0c, hn["S0"], grid, prm, dt, hc, sf, wind=wind,
                                         x_sign=1.0 if sign_2d else -1.0)
    F = [np.ascontiguousarray(Sol[k]).copy() for k in FIELDS]
    ph = np.ascontiguousarray(p2).copy()
    rhs = np.zeros(grid.node_isc)
    dp = np.zeros(grid.node_isc)
    gi, gd = _geom(grid, prm, dt, wind, sign_2d=sign_2d)
    sinv = np.ones(grid.elem_sc[1])
    host_lib.e3_host_forward(_ptr(gi), _ptr(gd), (ctypes.c_void_p * 6)(*[a.ctypes.data for a in F]), _ptr(ph),
                             _ptr(rhs), _ptr(dp), _ptr(S0c), _ptr(np.ascontiguousarray(hn["S0"])),
                             _ptr(np.ascontiguousarray(hc["rhoY0"])), _ptr(sinv))
    np.testing.assert_array_equal(rhs, div)
    for k, a in zip(FIELDS, F):
        np.testing.assert_array_equal(a, So[k], err_msg=k)
    assert np.abs(ph - po).max() <= 1e-13 * np.abs(po - p2).max()
