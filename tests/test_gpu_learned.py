"""The learned preconditioner end to end on the GPU: pairs harvested from the
solver's own iterations, training by the library's forward/backward/Adam kernels
from a seeded init, and the flexible solve checked by the FP64 true residual
against plain BiCGStab on the same inputs and tolerance.

The network alone (no background solve) is a local map of reach 13 nodes: it
cannot invert the operator's global slow modes and takes more iterations than
plain BiCGStab here (printed, finished by the reported fallback).  The network
as a correction of the background solve, the configuration the bench measures,
is checked in tests/test_gpu_spectral.py."""
import warnings

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_trained_network_lowers_its_training_loss_and_solves_are_checked_by_true_residual(capsys):
    import torch
    from pybella_gb300 import learned, workloads
    pairs = learned.harvest_pairs([1], shape=(97, 49, 97), npairs=256, crop=40, random_fraction=0.25)
    net0 = learned.CNN((40, 40, 40), block=2, nsamples=16, mode="linear", skip=1.0)
    net0.init(0, last_gain=0.01)
    losses = [l for _, l in learned.train(net0, pairs, steps=240, batch=16, lr=5e-4, log_every=1)]
    params = net0.get_params()
    assert np.all(np.isfinite(losses))
    # per-batch losses are noisy: compare the means over the first and last 60 steps
    assert np.mean(losses[-60:]) < np.mean(losses[:60]), (np.mean(losses[:60]), np.mean(losses[-60:]))
    ev = (41, 21, 41)
    w = workloads.stratified_3d(7, *ev)
    A = learned.operator_3d(w)
    net = learned.CNN(ev, block=2, mode="linear", skip=1.0)
    net.set_params(params)
    xp, sp = A.solve(w["b"], tol=1e-8, maxiter=20000, precision="df64")
    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        xl, sl = A.solve(w["b"], tol=1e-8, maxiter=20000, preconditioner=net)
    # the plain method decides: the returned x meets the tolerance on the FP64
    # true residual, and a fallback to it is never silent
    for x, st in ((xp, sp), (xl, sl)):
        assert st["status"] == 0, st
        r = w["b"] - A.matvec(x)
        assert float(torch.linalg.norm(r) / torch.linalg.norm(w["b"])) <= 1e-8
    assert bool(sl["fallback"]) == any("preconditioned solve failed" in str(m.message) for m in rec)
    with capsys.disabled():
        print("\nlearned vs plain (%s): learned %d iterations in %.3f s (fallback %d), plain %d in %.3f s"
              % ("x".join(map(str, ev)), sl["iterations"], sl["seconds"], sl["fallback"], sp["iterations"],
                 sp["seconds"]))
