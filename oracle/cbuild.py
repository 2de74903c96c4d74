"""Build and load the oracle's C restatement (``cpu_port.c``) -- test and
measurement infrastructure only (the CPU baseline of ``bench.py`` and the tests
that check it against the NumPy oracle).

    python -m oracle.cbuild

Compiles ``oracle/cpu_port.c`` with gcc (-O3, OpenMP) into
``oracle/_build/libport.so`` (git-ignored); rebuilds when the source is newer.
"""
import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_port.c")
LIB = os.path.join(HERE, "_build", "libport.so")


class PortOp3D(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("x_wall", ctypes.c_int), ("y_wall", ctypes.c_int), ("z_wall", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("corrf", ctypes.c_double),
                ("hplusx", ctypes.c_void_p), ("hplusy", ctypes.c_void_p), ("hplusz", ctypes.c_void_p),
                ("hcenter", ctypes.c_void_p), ("diag_inv", ctypes.c_void_p)]


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle's C restatement")
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + ".tmp"
    subprocess.run([cc, "-O3", "-fopenmp", "-shared", "-fPIC", "-o", tmp, SRC, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        lib.port_threads.restype = ctypes.c_int
        lib.port_lap3d.argtypes = [ctypes.POINTER(PortOp3D), ctypes.c_void_p, ctypes.c_void_p]
        lib.port_lap3d.restype = ctypes.c_int
        lib.port_bicgstab3d.argtypes = [ctypes.POINTER(PortOp3D), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
        lib.port_bicgstab3d.restype = ctypes.c_int
        _lib = lib
    return _lib


def _op3d(op):
    """A :class:`PortOp3D` for a packed oracle operator (``oracle.nodal3d.pack_27pt``);
    returns it with the arrays it points to."""
    import numpy as np
    keep = {k: np.ascontiguousarray(op[k], dtype=np.float64) for k in ("hplusx", "hplusy", "hplusz", "diag_inv")}
    hc = op.get("hcenter")
    if hc is not None and np.any(hc):
        keep["hcenter"] = np.ascontiguousarray(hc, dtype=np.float64)
    s = PortOp3D()
    s.nx, s.ny, s.nz = op["nx"], op["ny"], op["nz"]
    s.x_wall, s.y_wall, s.z_wall = (int(w) for w in op["walls"])
    s.dx, s.dy, s.dz, s.corrf = op["dx"], op["dy"], op["dz"], op.get("corrf", 0.0)
    for k in ("hplusx", "hplusy", "hplusz", "diag_inv"):
        setattr(s, k, keep[k].ctypes.data)
    s.hcenter = keep["hcenter"].ctypes.data if "hcenter" in keep else None
    return s, keep


def lap3d(p, op):
    """``lap3D`` on the host cores (C restatement); same contract as ``oracle.nodal3d.lap3d``."""
    import numpy as np
    s, keep = _op3d(op)
    p = np.ascontiguousarray(p, dtype=np.float64)
    y = np.empty_like(p)
    if load().port_lap3d(ctypes.byref(s), p.ctypes.data, y.ctypes.data) != 0:
        raise MemoryError("port_lap3d: out of host memory")
    return y


def bicgstab3d(op, b, tol, maxiter):
    """Plain FP64 BiCGStab (scipy's control flow) with the C ``lap3D`` on the host
    cores; returns ``(x, info, iterations, relres)``."""
    import numpy as np
    s, keep = _op3d(op)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty_like(b)
    it, rr = ctypes.c_int(0), ctypes.c_double(0.0)
    info = load().port_bicgstab3d(ctypes.byref(s), b.ctypes.data, x.ctypes.data, float(tol), int(maxiter),
                                  ctypes.byref(it), ctypes.byref(rr))
    if info == -100:
        raise MemoryError("port_bicgstab3d: out of host memory")
    return x, info, it.value, rr.value


def threads():
    return int(load().port_threads())


if __name__ == "__main__":
    print(build(force=True))
