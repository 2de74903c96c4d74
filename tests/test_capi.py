"""C-ABI checks that need no GPU: the library builds, loads and exports every
function that include/bella.h declares (no compute calls)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "bella.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bella_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_functions():
    names = _declared()
    assert "bella_bicgstab" in names and "bella_op2d_set" in names


def test_library_builds_and_exports_all_declared_symbols():
    from pybella_gb300 import build as B
    path = B.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from pybella_gb300 import _lib
    assert set(_declared()) <= set(_lib.SIGNATURES), set(_declared()) - set(_lib.SIGNATURES)


def test_status_strings_without_gpu():
    from pybella_gb300 import build as B, _lib
    B.build()
    lib = _lib.load()
    assert lib.bella_status_string(0) == b"converged"
    assert lib.bella_version() >= 100


def test_product_path_does_not_import_oracle():
    pkg = os.path.join(ROOT, "pybella_gb300")
    for dp, _, files in os.walk(pkg):
        for f in files:
            if f.endswith(".py"):
                txt = open(os.path.join(dp, f)).read()
                assert "import oracle" not in txt and "from oracle" not in txt, f


def test_projection_and_advection_reject_missing_arguments_without_gpu():
    """Argument checks come before any CUDA call: a NULL argument block, a grid
    below the ghost-layer minimum or a missing array returns BELLA_EINVAL."""
    from pybella_gb300 import build as B, _lib
    B.build()
    lib = _lib.load()
    null = ctypes.c_void_p(0)
    for fn in (lib.bella_advective_fluxes2d, lib.bella_boundary2d, lib.bella_advective_fluxes3d,
               lib.bella_boundary3d):
        assert fn(None, null) == _lib.BELLA_EINVAL
    assert lib.bella_advect2d(None, 0.01, 1, null) == _lib.BELLA_EINVAL
    assert lib.bella_advect_rk3d(None, 0.01, null) == _lib.BELLA_EINVAL
    a = _lib.Adv2D()
    a.inx, a.iny = 64, 32                       # every array missing
    assert lib.bella_advect2d(ctypes.byref(a), 0.01, 0, null) == _lib.BELLA_EINVAL
    small = _lib.Adv3D()
    small.inx, small.iny, small.inz = 4, 9, 9   # below the five-node minimum
    assert lib.bella_advect3d(ctypes.byref(small), 0.01, 0, null) == _lib.BELLA_EINVAL
    assert lib.bella_projection3d(None, None, None, None, null) == _lib.BELLA_EINVAL
    assert lib.bella_projection2d(None, None, None, None, null) == _lib.BELLA_EINVAL
