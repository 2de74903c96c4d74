"""CPU checks of the CNN oracle: blocking round trip and backward vs finite differences."""
import numpy as np
import pytest

from oracle import cnn as ocnn


@pytest.mark.parametrize("block", [1, 2])
def test_blocking_round_trip(block):
    r = np.random.default_rng(1).standard_normal((5, 6, 7))
    x = ocnn.blocked(r, block)
    assert x.shape == (-(-5 // block), -(-6 // block), -(-7 // block), block ** 3)
    assert np.array_equal(ocnn.unblocked(x, r.shape, block), r)
    if block == 2:
        assert x[0, 0, 0, 1] == r[0, 0, 1] and x[0, 0, 0, 4] == r[1, 0, 0] and x[0, 0, 0, 7] == r[1, 1, 1]
        assert x[2, 2, 3, 7] == 0.0            # beyond the odd edges


@pytest.mark.parametrize("block", [1, 2])
def test_backward_matches_finite_differences(block):
    rng = np.random.default_rng(7 + block)
    shape = (4, 3, 5) if block == 1 else (6, 4, 5)
    p = ocnn.init_params(5, block)
    for l in range(6):
        p["b%d" % l] = rng.uniform(0.05, 0.2, p["b%d" % l].shape)    # keep ReLUs mostly active
        p["W%d" % l] = p["W%d" % l].astype(np.float64)
    r = rng.standard_normal(shape)
    gout = rng.standard_normal(shape)
    _, acts = ocnn.forward(r, p, block, rounding=False)
    grads = ocnn.backward(acts, p, gout, block, rounding=False)

    def f(q):
        y, _ = ocnn.forward(r, q, block, rounding=False)
        return float(np.sum(gout * y))
    h = 1e-6
    for name in ("W0", "b0", "W2", "b3", "W5", "b5"):
        flat = p[name].reshape(-1)
        for idx in rng.choice(flat.size, size=min(4, flat.size), replace=False):
            q = {k: v.copy() for k, v in p.items()}
            q[name].reshape(-1)[idx] += h
            fp = f(q)
            q[name].reshape(-1)[idx] -= 2 * h
            fm = f(q)
            fd = (fp - fm) / (2 * h)
            an = grads[name].reshape(-1)[idx]
            assert abs(fd - an) <= 1e-5 * max(1.0, abs(fd)), (name, idx, fd, an)


def test_flatten_round_trip():
    p = ocnn.init_params(2, 2)
    q = ocnn.unflatten(ocnn.flatten(p), 2)
    for k in p:
        assert np.array_equal(p[k], q[k])
