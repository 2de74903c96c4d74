"""GPU checks of the learned preconditioner's CNN kernels against the NumPy oracle."""
import numpy as np
import pytest

from oracle import cnn as ocnn

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("shape", [(5, 6, 17), (9, 4, 33)])
def test_cnn_forward_matches_oracle(shape):
    import torch
    from pybella_gb300.learned import CNN
    rng = np.random.default_rng(sum(shape))
    params = ocnn.init_params(3)
    for l in range(6):
        params["b%d" % l] = rng.uniform(-0.1, 0.1, params["b%d" % l].shape).astype(np.float32)
    r = rng.standard_normal(shape).astype(np.float32)
    ref, _ = ocnn.forward(r, params)
    net = CNN(max_voxels=int(np.prod(shape)))
    net.set_params(params)
    y = net.forward(torch.tensor(r.ravel(), device="cuda"), shape, scale=1.0).cpu().numpy().reshape(shape)
    # BF16 activations: a rounding boundary crossed by FP32-vs-FP64 accumulation moves an
    # activation by one BF16 ulp (2^-8); the output error stays at the percent level
    assert _rel(y, ref) < 2e-2, _rel(y, ref)
    # scale equivariance of the normalised preconditioner
    y2 = net.forward(torch.tensor(3.0 * r.ravel(), device="cuda"), shape, scale=1.0 / 3.0).cpu().numpy()
    np.testing.assert_allclose(y2.reshape(shape), 3.0 * y, rtol=1e-5, atol=1e-6)
