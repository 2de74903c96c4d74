"""GPU checks of the learned preconditioner's CNN kernels against the NumPy oracle:
forward pass, parameter gradients (the backward kernels), and an Adam training step."""
import numpy as np
import pytest

from oracle import cnn as ocnn

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _params(block, seed):
    rng = np.random.default_rng(seed)
    p = ocnn.init_params(seed, block)
    for l in range(6):
        p["b%d" % l] = rng.uniform(-0.1, 0.1, p["b%d" % l].shape).astype(np.float32)
    return p


@pytest.mark.parametrize("block,shape", [(1, (5, 6, 17)), (1, (9, 4, 33)), (2, (9, 10, 35)), (2, (16, 8, 32))])
def test_cnn_forward_matches_oracle(block, shape):
    import torch
    from pybella_gb300.learned import CNN
    rng = np.random.default_rng(sum(shape))
    params = _params(block, 3)
    r = rng.standard_normal(shape).astype(np.float32)
    ref, _ = ocnn.forward(r, params, block)
    net = CNN(shape, block=block)
    net.set_params(params)
    y = net.forward(torch.tensor(r.ravel(), device="cuda"), shape, scale=1.0).cpu().numpy().reshape(shape)
    # BF16 activations: a rounding boundary crossed by FP32-vs-FP64 accumulation moves an
    # activation by one BF16 ulp (2^-8); the output error stays at the percent level
    assert _rel(y, ref) < 2e-2, _rel(y, ref)
    # scale equivariance of the normalised preconditioner
    y2 = net.forward(torch.tensor(3.0 * r.ravel(), device="cuda"), shape, scale=1.0 / 3.0).cpu().numpy()
    np.testing.assert_allclose(y2.reshape(shape), 3.0 * y, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("block,shape", [(1, (6, 5, 18)), (2, (11, 8, 34))])
def test_cnn_gradients_match_oracle(block, shape):
    """Backward kernels (mirrored tensor-core input gradients, FP32 weight gradients)
    against the oracle's float64 backward on the same BF16 activations."""
    import torch
    from pybella_gb300.learned import CNN
    rng = np.random.default_rng(11 + block)
    params = _params(block, 4)
    r = rng.standard_normal(shape).astype(np.float32)
    gout = rng.standard_normal(shape).astype(np.float32)
    _, acts = ocnn.forward(r, params, block)
    ref = ocnn.backward(acts, params, gout, block)
    net = CNN(shape, block=block)
    net.set_params(params)
    g, _ = net.gradients(torch.tensor(r.ravel(), device="cuda"), torch.tensor(gout.ravel(), device="cuda"), shape)
    got = ocnn.unflatten(g.cpu().numpy(), block)
    for k in ref:
        # input gradients travel between layers in BF16 (as the activations do)
        assert _rel(got[k], ref[k]) < 3e-2, (k, _rel(got[k], ref[k]))


@pytest.mark.parametrize("block", [1, 2])
def test_cnn_train_step_reduces_loss(block):
    """Adam on the GPU fits a fixed smoothing map on a batch of 16^3 samples."""
    import torch
    from pybella_gb300.learned import CNN
    torch.manual_seed(0)
    ns, S = 8, 16
    x = torch.randn(ns, S, S, S, device="cuda")
    # target: a 3-point box smoothing of the input along each axis
    t = x.clone()
    for ax in (1, 2, 3):
        t = (torch.roll(t, 1, ax) + t + torch.roll(t, -1, ax)) / 3.0
    net = CNN((S, S, S), block=block, nsamples=ns)
    net.init(0)
    p0 = net.get_params()
    losses = [net.train_step(x, t, 2e-3) for _ in range(60)]
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.5 * losses[0], (losses[0], losses[-1])
    assert not np.array_equal(net.get_params(), p0)
