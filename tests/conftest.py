import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libbella_gb300.so")


# Tests of the advection and of whole time steps build on the projection and solver
# entry points the other files test: they run after those (in this order), so that a
# failure in a building block is reported by that block's own test first.
_COMPOSED = ("test_gpu_advection.py", "test_gpu_projection_walls.py", "test_gpu_step.py", "test_gpu_step3d.py",
             "test_gpu_fullrun.py")


def pytest_collection_modifyitems(config, items):
    rank = {name: k + 1 for k, name in enumerate(_COMPOSED)}
    rank["test_zz_no_alloc.py"] = len(_COMPOSED) + 1      # the allocation-free entry point's test runs last
    items.sort(key=lambda it: rank.get(os.path.basename(str(it.fspath)), 0))


def golden(name):
    return os.path.join(ROOT, "tests", "golden", name)


def rb_background(d):
    """Rising-bubble backgrounds exactly as the reference computed them (from the fixture).

    Recomputing them with np.exp on another platform changes the last bit,
    and dS/dy (a difference of nearly equal numbers) turns that into ~1e-11.
    """
    from oracle import cases
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble()
    hn = dict(hn)
    hc = dict(hc)
    hn["S0"] = d["hydro_n_S0"].copy()
    hc["rhoY0"] = d["hydro_c_rhoY0"].copy()
    return grid, prm, hn, hc, sf


def lap3d_case(d, tag, seam_copy=True):
    """Operands of one ``lap3d_kat`` case for the oracle: inner nodes of the
    halo-carrying reference vector, after lap3D's periodic seam overwrite
    (inner node 0 <- inner node n-1, laplacian.py:927-960) when ``seam_copy``."""
    g = lambda k: d["%s_%s" % (tag, k)]
    m = g("meta")
    nx, ny, nz = (int(v) for v in m[:3])
    per = [bool(v) for v in m[3:6]]
    dx, dy, dz, corrf = (float(v) for v in m[6:10])
    p = g("p").copy()
    if seam_copy:
        for axis in range(3):
            if per[axis]:
                src = [slice(None)] * 3
                dst = [slice(None)] * 3
                src[axis], dst[axis] = -2, 1
                p[tuple(dst)] = p[tuple(src)]
    inner = (slice(1, -1),) * 3
    from oracle import nodal3d as n3
    op = n3.pack_27pt(g("hx"), g("hy"), g("hz"), g("hc"), g("dinv")[inner], nx, ny, nz, dx, dy, dz,
                      walls=[not v for v in per], corrf=corrf)
    y = g("y").reshape(nx + 2, ny + 2, nz + 2)
    return op, p[inner].reshape(-1), y


def proj3d_case(d, tag):
    """Grid, parameters and backgrounds of one ``proj3d_kat`` case for the oracle:
    ``(grid, prm, dt, S0n, hydro_c, strat_fn)``.  The state is the reference's
    rising-bubble domain extended to z in [-1, 1] (stratification 1)."""
    import numpy as np
    from oracle import nodal2d as n2, proj3d as o3
    m = d[tag + "_meta"]
    inx, iny, inz = (int(v) for v in m[:3])
    walls = [bool(v) for v in m[3:6]]
    dx, dy, dz, dt, Msq, g, gamm, nonhydro, comp, is_comp = (float(v) for v in m[6:16])
    grid = o3.Grid3D(inx, iny, inz, -1.0, 1.0, 0.0, 1.0, -1.0, 1.0,
                     bdry=[n2.WALL if w else n2.PERIODIC for w in walls])
    assert np.allclose((grid.dx, grid.dy, grid.dz), (dx, dy, dz), rtol=1e-15, atol=0)
    prm = n2.Params(Msq=Msq, g=g, gamm=gamm, coriolis=m[16:19], nonhydro=nonhydro, is_compressible=int(is_comp),
                    compressibility=comp)
    sinv = d[tag + "_strat_inv"]
    assert np.all(sinv == 1.0)
    return grid, prm, dt, d[tag + "_S0n"], dict(rhoY0=d[tag + "_rhoY0"]), (lambda y: 1.0)


def step2d_case(d, tag):
    """Grid, parameters and backgrounds of one ``step2d_kat`` case (33x17 nodes)."""
    from oracle import nodal2d as n2
    m = d[tag + "_meta"]
    inx, iny, xw = int(m[0]), int(m[1]), bool(m[2])
    dt, Msq, g, gamm, is_comp, comp = (float(v) for v in m[3:9])
    grid = n2.Grid2D(inx, iny, -1.0, 1.0, 0.0, 1.0, (n2.WALL if xw else n2.PERIODIC, n2.WALL))
    prm = n2.Params(Msq=Msq, g=g, gamm=gamm, coriolis=m[9:12], nonhydro=1.0, is_compressible=int(is_comp),
                    compressibility=comp, tol=1e-10, max_iterations=6000)
    return grid, prm, dt, dict(S0=d[tag + "_S0n"]), dict(rhoY0=d[tag + "_rhoY0"]), (lambda y: 1.0)
