"""The device advection's arithmetic, compiled for the host (tests/advect_host.cpp
includes pybella_gb300/csrc/bella_advect.cuh, whose functions the kernels of
bella_advect.cu run one thread per item), against the reference's advection
outputs in 2D (tests/golden/advect_kat.npz) and 3D (advect3d_kat.npz).  Same
sweep sequences, per-face and per-cell functions and boundary lines as on the
GPU, executed by loops."""
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
    out = str(tmp_path_factory.mktemp("advect") / "libadvect_host.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", out,
                    os.path.join(ROOT, "tests", "advect_host.cpp")], check=True)
    return ctypes.CDLL(out)


def _ptrs(arrs):
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _case(dim, case):
    """(reference arrays, key prefix, geometry ints, geometry doubles, face shapes, hydro rhoY0, dt)."""
    from oracle import cases
    if dim == 2:
        d = np.load(golden("advect_kat.npz"))
        inx, iny, dt = int(d["meta"][0]), int(d["meta"][1]), float(d["meta"][2])
        grid, prm, _, _, _, _, _ = cases.rising_bubble(inx=inx, iny=iny)
        icx, icy = grid.elem_sc
        geo = np.array([2, icx, icy, 1, int(grid.x_wall), int(grid.y_wall), 0], dtype=np.int32)
        dg = np.array([grid.dx, grid.dy, 1.0, prm.g, prm.gamm])
        shapes = [(icy, icx + 1), (icx, icy + 1)]
        return d, "", geo, dg, shapes, np.ascontiguousarray(d["rhoY0"]), dt, "flux%d_rhoY", "rk_pwchi"
    from oracle import proj3d as o3
    d = np.load(golden("advect3d_kat.npz"))
    m = d[case + "_meta"]
    inx, iny, inz = int(m[0]), int(m[1]), int(m[2])
    grid = o3.Grid3D(inx, iny, inz, -1.0, 1.0, 0.0, 1.0, -1.0, 1.0)
    icx, icy, icz = grid.elem_sc
    geo = np.array([3, icx, icy, icz, int(m[3]), int(m[4]), int(m[5])], dtype=np.int32)
    dg = np.array([grid.dx, grid.dy, grid.dz, float(m[8]), float(m[9])])
    shapes = [(icy, icz, icx + 1), (icz, icx, icy + 1), (icx, icy, icz + 1)]
    return (d, case + "_", geo, dg, shapes, np.ascontiguousarray(d[case + "_rhoY0"]), float(m[6]),
            case + "_flux%d_rhoY", case + "_rk_pwchi")


CASES = [(2, None), (3, "pwp"), (3, "wwp")]


@pytest.mark.parametrize("dim,case", CASES)
def test_mass_fluxes_host_vs_reference(host_lib, dim, case):
    d, pre, geo, dg, shapes, rhoY0, dt, fkey, _ = _case(dim, case)
    F = [np.ascontiguousarray(d[pre + "in_" + k], dtype=np.float64).copy() for k in FIELDS]
    faces = [np.zeros(s) for s in shapes for _ in FIELDS]
    host_lib.adv_host_mass(ctypes.c_void_p(geo.ctypes.data), ctypes.c_void_p(dg.ctypes.data), _ptrs(F), _ptrs(faces))
    for s in range(dim):
        # direct sums against the reference's FFT convolution: rounding only
        assert _rel(faces[6 * s + 4], d[fkey % s]) < 1e-13, s


@pytest.mark.parametrize("own_fluxes", [True, False])
@pytest.mark.parametrize("tag", ["odd", "even", "rk"])
@pytest.mark.parametrize("dim,case", CASES)
def test_advection_host_vs_reference(host_lib, dim, case, tag, own_fluxes):
    """With the reference's face mass fluxes the sweeps reproduce the reference
    bit for bit; with the library's own (direct sums instead of the reference's
    FFT convolution) to rounding."""
    d, pre, geo, dg, shapes, rhoY0, dt, fkey, pkey = _case(dim, case)
    F = [np.ascontiguousarray(d[pre + "in_" + k], dtype=np.float64).copy() for k in FIELDS]
    faces = [np.zeros(s) for s in shapes for _ in FIELDS]
    if own_fluxes:
        host_lib.adv_host_mass(ctypes.c_void_p(geo.ctypes.data), ctypes.c_void_p(dg.ctypes.data), _ptrs(F),
                               _ptrs(faces))
    else:
        for s in range(dim):
            faces[6 * s + 4][...] = d[fkey % s]
    sinv = np.ones(int(geo[2]))
    args = (ctypes.c_void_p(geo.ctypes.data), ctypes.c_void_p(dg.ctypes.data), ctypes.c_int(0), _ptrs(F),
            _ptrs(faces), ctypes.c_void_p(rhoY0.ctypes.data), ctypes.c_void_p(sinv.ctypes.data))
    if tag == "rk":
        pw = np.zeros(F[0].shape)
        host_lib.adv_host_rk(*args, ctypes.c_double(0.5 * dt), ctypes.c_void_p(pw.ctypes.data))
        if own_fluxes:
            assert _rel(pw, d[pkey]) < 1e-10
        else:
            np.testing.assert_array_equal(pw, d[pkey])
    else:
        host_lib.adv_host_strang(*args, ctypes.c_double(dt), ctypes.c_int(1 if tag == "odd" else 0))
    for k, a in zip(FIELDS, F):
        ref = d["%s%s_%s" % (pre, tag, k)]
        if not own_fluxes:
            np.testing.assert_array_equal(a, ref, err_msg=k)
            continue
        # the state itself to rounding; the change of the state well inside it
        assert _rel(a, ref) < 1e-12, (k, _rel(a, ref))
        change = np.abs(ref - d[pre + "in_" + k]).max()
        assert np.abs(a - ref).max() <= 1e-9 * max(change, 1e-300), (k, np.abs(a - ref).max(), change)
