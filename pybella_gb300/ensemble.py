"""Ensemble solves: the elliptic solves of many 2D members in one persistent launch.

``solve_ensemble`` is the batched counterpart of calling the reference's
``bicgstab(lap, rhs, tol=ud.tol, maxiter=ud.max_iterations)``
(second_projection.py:230) once per member: every member keeps its own
operator (a :class:`pybella_gb300.linalg.NodalHelmholtz2D` with its own
workspace) and right-hand side, and ``bella_bicgstab_batched`` iterates all of
them in one cooperative kernel.  ``autotune`` picks the launch configuration
(tile shape, CTAs per SM) for a set of member sizes by timing each one.
"""
import ctypes

import numpy as np
import torch

from . import _lib


def _arrays(ops, bs, xs):
    n = len(ops)
    W = (ctypes.c_void_p * n)(*[op.ws.handle.value for op in ops])
    B = (ctypes.c_void_p * n)(*[b.data_ptr() for b in bs])
    X = (ctypes.c_void_p * n)(*[x.data_ptr() for x in xs])
    return W, B, X


def _prep(ops, bs):
    dev = ops[0].dev
    bd = [torch.as_tensor(b, dtype=torch.float64).to(dev).contiguous().reshape(-1) for b in bs]
    for op, b in zip(ops, bd):
        if op.ws.device != ops[0].ws.device:
            raise ValueError("all members must live on one GPU")
        if b.numel() != op.n:
            raise ValueError("rhs has %d entries, operator has %d" % (b.numel(), op.n))
    xs = [torch.zeros_like(b) for b in bd]
    return dev, bd, xs


def configs():
    lib = _lib.load()
    out = []
    for i in range(int(lib.bella_batch_config_count())):
        tx, ty, ps = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(lib.bella_batch_config(i, ctypes.byref(tx), ctypes.byref(ty), ctypes.byref(ps)),
                   "bella_batch_config")
        out.append({"tile": (tx.value, ty.value), "ctas_per_sm": ps.value or "max"})
    return out


PRECISIONS = {"fp64": 0, "df64": 2}


def autotune(ops, bs, probe_iters=20, precision="df64"):
    """Time every launch configuration on this ensemble; returns (choice, ms per config)."""
    lib = _lib.load()
    dev, bd, xs = _prep(ops, bs)
    W, B, X = _arrays(ops, bd, xs)
    n = int(lib.bella_batch_config_count())
    ms = (ctypes.c_double * n)()
    choice = ctypes.c_int()
    with torch.cuda.device(dev):
        _lib.check(lib.bella_batch_autotune(W, len(ops), B, X, PRECISIONS[precision], int(probe_iters),
                                            ctypes.byref(choice), ms,
                                            ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)),
                   "bella_batch_autotune")
    return choice.value, list(ms)


def solve_ensemble(ops, bs, tol=1e-10, atol=0.0, maxiter=6000, config=-1, out=None, precision="df64"):
    """Solve ``ops[m] x_m = bs[m]`` for all members in one launch; returns (xs, stats list).

    ``precision='df64'`` (default) iterates in double-float on the FP32 pipe with
    FP64 refinement of members whose FP64 true residual misses the tolerance
    (``stats[m]['fallback']`` counts those rounds); ``'fp64'`` iterates in FP64."""
    lib = _lib.load()
    dev, bd, xs = _prep(ops, bs)
    if out is not None:
        xs = out
    W, B, X = _arrays(ops, bd, xs)
    o = _lib.SolveOpts()
    lib.bella_solve_opts_default(ctypes.byref(o))
    o.tol, o.atol, o.maxiter = float(tol), float(atol or 0.0), int(maxiter)
    o.precision = PRECISIONS[precision]
    st = (_lib.SolveStats * len(ops))()
    with torch.cuda.device(dev):
        rc = lib.bella_bicgstab_batched(W, len(ops), B, X, ctypes.byref(o), int(config), st,
                                        ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    if rc < 0:
        _lib.check(rc, "bella_bicgstab_batched")
    return xs, [s.as_dict() for s in st]
