"""pybella_gb300 -- GB300 (sm_103a) implicit nodal pressure projection of pyBELLA.

The compute path is libbella_gb300.so (hand-written CUDA for sm_103a behind
the C ABI in include/bella.h); this package is the host side that mirrors
the reference's ``laplacian`` / ``scipy.sparse.linalg`` call contract.
"""
from . import _lib  # noqa: F401

__version__ = "0.1.0"


def library_path():
    return _lib.LIB_PATH
