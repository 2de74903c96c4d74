"""The device advection's arithmetic, compiled for the host (tests/adv2d_host.cpp
includes pybella_gb300/csrc/bella_adv2d.cuh, whose functions the kernels of
bella_adv2d.cu run one thread per item), against the reference's advection
outputs (tests/golden/advect_kat.npz).  Same sweep sequences, per-face and
per-cell functions and boundary lines as on the GPU, executed by loops."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden

FIELDS = ("rho", "rhou", "rhov", "rhow", "rhoY", "rhoX")


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("adv2d") / "libadv2d_host.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", out,
                    os.path.join(ROOT, "tests", "adv2d_host.cpp")], check=True)
    return ctypes.CDLL(out)


def _ptrs(arrs):
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


def _state(d):
    return [np.ascontiguousarray(d["in_" + k], dtype=np.float64).copy() for k in FIELDS]


def _faces(icx, icy):
    return [np.zeros((icy, icx + 1)) for _ in FIELDS], [np.zeros((icx, icy + 1)) for _ in FIELDS]


def _geom(d):
    from oracle import cases
    inx, iny = int(d["meta"][0]), int(d["meta"][1])
    grid, prm, _, _, _, hc, _ = cases.rising_bubble(inx=inx, iny=iny)
    return grid, prm, np.ascontiguousarray(d["rhoY0"]), np.ones(grid.elem_sc[1])


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_mass_fluxes_host_vs_reference(host_lib):
    d = np.load(golden("advect_kat.npz"))
    grid, prm, rhoY0, sinv = _geom(d)
    icx, icy = grid.elem_sc
    F = _state(d)
    fx, fy = _faces(icx, icy)
    host_lib.adv_host_mass(icx, icy, _ptrs(F), ctypes.c_void_p(fx[4].ctypes.data), ctypes.c_void_p(fy[4].ctypes.data))
    # direct sums against the reference's FFT convolution: rounding only
    assert _rel(fx[4], d["flux0_rhoY"]) < 1e-13
    assert _rel(fy[4], d["flux1_rhoY"]) < 1e-13


@pytest.mark.parametrize("own_fluxes", [True, False])
@pytest.mark.parametrize("tag", ["odd", "even", "rk"])
def test_advection_host_vs_reference(host_lib, tag, own_fluxes):
    """With the reference's face mass fluxes the sweeps reproduce the reference
    bit for bit; with the library's own (direct 2x3 sums instead of the
    reference's FFT convolution) to rounding."""
    d = np.load(golden("advect_kat.npz"))
    grid, prm, rhoY0, sinv = _geom(d)
    icx, icy = grid.elem_sc
    dt = float(d["meta"][2])
    F = _state(d)
    fx, fy = _faces(icx, icy)
    if own_fluxes:
        host_lib.adv_host_mass(icx, icy, _ptrs(F), ctypes.c_void_p(fx[4].ctypes.data),
                               ctypes.c_void_p(fy[4].ctypes.data))
    else:
        fx[4][...] = d["flux0_rhoY"]
        fy[4][...] = d["flux1_rhoY"]
    geo = (ctypes.c_int(icx), ctypes.c_int(icy), ctypes.c_int(int(grid.x_wall)), ctypes.c_int(int(grid.y_wall)),
           ctypes.c_double(grid.dx), ctypes.c_double(grid.dy), ctypes.c_double(prm.g), ctypes.c_double(prm.gamm),
           ctypes.c_int(prm.is_compressible))
    bufs = (_ptrs(F), _ptrs(fx), _ptrs(fy), ctypes.c_void_p(rhoY0.ctypes.data), ctypes.c_void_p(sinv.ctypes.data))
    if tag == "rk":
        pw = np.zeros((icx, icy))
        host_lib.adv_host_rk(*geo, *bufs, ctypes.c_double(0.5 * dt), ctypes.c_void_p(pw.ctypes.data))
        if own_fluxes:
            assert _rel(pw, d["rk_pwchi"]) < 1e-10
        else:
            np.testing.assert_array_equal(pw, d["rk_pwchi"])
    else:
        host_lib.adv_host_strang(*geo, *bufs, ctypes.c_double(dt), ctypes.c_int(1 if tag == "odd" else 0))
    for k, a in zip(FIELDS, F):
        ref = d["%s_%s" % (tag, k)]
        if not own_fluxes:
            np.testing.assert_array_equal(a, ref, err_msg=k)
            continue
        # the state itself to rounding; the change of the state well inside it
        assert _rel(a, ref) < 1e-12, (k, _rel(a, ref))
        change = np.abs(ref - d["in_" + k]).max()
        assert np.abs(a - ref).max() <= 1e-9 * max(change, 1e-300), (k, np.abs(a - ref).max(), change)
