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


@pytest.mark.parametrize("block,shape", [(1, (6, 5, 18)), (2, (11, 8, 34)), (1, (7, 20, 30)), (2, (20, 38, 62))])
def test_cnn_gradients_match_oracle(block, shape):
    """Backward kernels (tcgen05 input gradients with the mirrored weights, tcgen05
    weight gradients) against the oracle's float64 backward on the same BF16
    activations; the last two shapes span three 256-row blocks of the padded plane."""
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


@pytest.mark.parametrize("block,shape", [(2, (10, 8, 18))])
def test_cnn_linear_mode_gradients_match_oracle(block, shape):
    """Linear mode (no ReLU, no biases): forward and weight gradients against the oracle;
    bias gradients are held at zero."""
    import torch
    from pybella_gb300.learned import CNN
    rng = np.random.default_rng(21)
    params = ocnn.init_params(6, block)
    r = rng.standard_normal(shape).astype(np.float32)
    gout = rng.standard_normal(shape).astype(np.float32)
    yref, acts = ocnn.forward(r, params, block, linear=True)
    ref = ocnn.backward(acts, params, gout, block, linear=True)
    net = CNN(shape, block=block, mode="linear")
    net.set_params(params)
    g, y = net.gradients(torch.tensor(r.ravel(), device="cuda"), torch.tensor(gout.ravel(), device="cuda"), shape)
    assert _rel(y.cpu().numpy().reshape(shape), yref) < 2e-2
    got = ocnn.unflatten(g.cpu().numpy(), block)
    for l in range(6):
        assert _rel(got["W%d" % l], ref["W%d" % l]) < 3e-2, (l, _rel(got["W%d" % l], ref["W%d" % l]))
        assert np.all(got["b%d" % l] == 0.0)
    # linearity of the map: M(a + 2b) = M(a) + 2 M(b) up to BF16 rounding
    a = torch.randn(int(np.prod(shape)), device="cuda")
    b = torch.randn_like(a)
    lhs = net.forward(a + 2 * b, shape, scale=1.0)
    rhs = net.forward(a, shape, scale=1.0) + 2 * net.forward(b, shape, scale=1.0)
    assert float(torch.linalg.norm(lhs - rhs) / torch.linalg.norm(rhs)) < 2e-2


def test_crop_operator_matches_full_operator():
    """The batched crop operator of the training loss equals the device 27-point
    operator on the crop's interior nodes."""
    import ctypes
    import torch
    from pybella_gb300 import _lib, learned, workloads
    shape = (33, 21, 29)
    w = workloads.stratified_3d(3, *shape)
    A = learned.operator_3d(w)
    u = torch.randn(A.n, device="cuda", dtype=torch.float64)
    Au = A.matvec(u).reshape(shape)
    h = learned.wall_zeroed_cells(w)
    S = 16
    offs = [(0, 0, 0), (17, 5, 13)]
    U = torch.stack([u.reshape(shape)[i:i + S, j:j + S, k:k + S] for i, j, k in offs]).float().contiguous()
    H = torch.stack([h[i:i + S + 1, j:j + S + 1, k:k + S + 1] for i, j, k in offs]).float().contiguous()
    D = torch.stack([w["diag_inv"].reshape(shape)[i:i + S, j:j + S, k:k + S] for i, j, k in offs]).float().contiguous()
    flux = torch.empty(len(offs) * (S + 1) ** 3 * 3, device="cuda")
    y = torch.empty_like(U)
    lib = _lib.load()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    _lib.check(lib.bella_crop_apply(len(offs), S, p(U), p(H), p(D), w["dx"], w["dy"], w["dz"], 1, p(flux), p(y),
                                    None), "bella_crop_apply")
    torch.cuda.synchronize()
    for q, (i, j, k) in enumerate(offs):
        got = y[q, 1:-1, 1:-1, 1:-1].double()
        ref = Au[i + 1:i + S - 1, j + 1:j + S - 1, k + 1:k + S - 1]
        assert float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref)) < 1e-6
        assert float(y[q, 0].abs().max()) == 0.0          # face nodes masked


def test_flexible_solver_reaches_tolerance_and_reports():
    """Flexible BiCGStab with an (untrained) network: the FP64 true residual meets the
    tolerance, either by the learned iteration or by the reported plain fallback."""
    import torch
    from pybella_gb300 import learned, workloads
    shape = (33, 17, 33)
    w = workloads.stratified_3d(2, *shape)
    A = learned.operator_3d(w)
    net = learned.CNN(shape, block=2, mode="linear")
    net.init(0)
    with _nullctx():
        x, st = A.solve(w["b"], tol=1e-8, maxiter=20000, preconditioner=net)
    assert st["status"] == 0, st
    r = w["b"] - A.matvec(x)
    assert float(torch.linalg.norm(r) / torch.linalg.norm(w["b"])) <= 1e-8
    assert st["fallback"] in (0, 1)


class _nullctx:
    def __enter__(self):
        import warnings
        self._w = warnings.catch_warnings()
        self._w.__enter__()
        warnings.simplefilter("ignore", RuntimeWarning)

    def __exit__(self, *a):
        self._w.__exit__(*a)


@pytest.mark.parametrize("mode", ["relu", "linear"])
@pytest.mark.parametrize("block,shape", [(2, (16, 8, 32)), (2, (9, 10, 35)), (2, (66, 40, 130)), (1, (9, 7, 21))])
def test_tcgen05_forward_matches_mma_sync_and_oracle(mode, block, shape):
    """All six forward layers on tcgen05 (tensor memory accumulators; the output
    layer's 8 or 1 channels padded to 16): same output as the mma.sync kernels
    and the oracle, no completion wait given up."""
    import torch
    from pybella_gb300.learned import CNN
    rng = np.random.default_rng(sum(shape))
    params = _params(block, 9)
    if mode == "linear":
        for l in range(6):
            params["b%d" % l] = np.zeros_like(params["b%d" % l])
    r = rng.standard_normal(shape).astype(np.float32)
    net = CNN(shape, block=block, mode=mode)
    net.set_params(params)
    x = torch.tensor(r.ravel(), device="cuda")
    net.set_tensor_cores(False)
    y_mma = net.forward(x, shape, scale=1.0).cpu().numpy()
    net.set_tensor_cores(True)
    y_tc = net.forward(x, shape, scale=1.0).cpu().numpy()
    assert not net.tensor_core_error()
    # same BF16 operands, FP32 accumulation in another order
    assert _rel(y_tc, y_mma) < 1e-2, _rel(y_tc, y_mma)
    if shape[0] * shape[1] * shape[2] < 40000:
        ref, _ = ocnn.forward(r, params, block, linear=(mode == "linear"))
        assert _rel(y_tc.reshape(shape), ref) < 2e-2


@pytest.mark.parametrize("mode", ["relu", "linear"])
@pytest.mark.parametrize("block,shape", [(2, (11, 8, 34)), (2, (20, 38, 62)), (1, (7, 20, 30))])
def test_tcgen05_gradients_match_cuda_core_gradients(mode, block, shape):
    """Weight and bias gradients on tcgen05 (GEMM over voxels, MN-major operands from the
    staged planes) against the FP32 CUDA-core loops with mma.sync input gradients: both
    against the oracle's float64 backward, the tensor-core path at least as accurate.
    The two paths sum the same BF16 products in different orders, so BF16 activations
    and, with ReLUs, their masks differ in a few places; without ReLUs the gradients
    agree directly."""
    import torch
    from pybella_gb300.learned import CNN
    rng = np.random.default_rng(31 + sum(shape))
    params = _params(block, 5)
    linear = mode == "linear"
    if linear:
        for l in range(6):
            params["b%d" % l] = np.zeros_like(params["b%d" % l])
    r = rng.standard_normal(shape).astype(np.float32)
    gout = rng.standard_normal(shape).astype(np.float32)
    _, acts = ocnn.forward(r, params, block, linear=linear)
    ref = ocnn.backward(acts, params, gout, block, linear=linear)
    net = CNN(shape, block=block, mode=mode)
    net.set_params(params)
    got = {}
    for tc in (False, True):
        net.set_tensor_cores(tc)
        g = net.gradients(torch.tensor(r.ravel(), device="cuda"), torch.tensor(gout.ravel(), device="cuda"), shape)[0]
        got[tc] = ocnn.unflatten(g.cpu().numpy(), block)
    assert not net.tensor_core_error()
    for k in ref:
        if linear and k.startswith("b"):           # biases are held at zero in linear mode
            assert not np.any(got[True][k]) and not np.any(got[False][k]), k
            continue
        e_tc, e_cc = _rel(got[True][k], ref[k]), _rel(got[False][k], ref[k])
        # the output layer's gradient enters the tensor-core weight gradient in BF16
        assert e_tc <= max(1.5 * e_cc, 1e-2), (k, e_tc, e_cc)
        if linear:
            assert _rel(got[True][k], got[False][k]) < 1e-2, (k, _rel(got[True][k], got[False][k]))


@pytest.mark.parametrize("block", [1, 2])
def test_tcgen05_batched_training_tracks_cuda_cores(block):
    """Adam on a batch of samples stacked along x (one x-segment each): the tensor-core
    backward and the CUDA-core backward give the same loss curve."""
    import torch
    from pybella_gb300.learned import CNN
    torch.manual_seed(1)
    ns, S = 4, 24
    x = torch.randn(ns, S, S, S, device="cuda")
    t = x.clone()
    for ax in (1, 2, 3):
        t = (torch.roll(t, 1, ax) + t + torch.roll(t, -1, ax)) / 3.0
    curves = []
    for tc in (False, True):
        net = CNN((S, S, S), block=block, nsamples=ns)
        net.init(0)
        net.set_tensor_cores(tc)
        curves.append(np.array([net.train_step(x, t, 1e-3) for _ in range(12)]))
        assert not net.tensor_core_error()
    cc, tcv = curves
    assert np.all(np.isfinite(tcv))
    assert tcv[-1] < tcv[0]
    np.testing.assert_allclose(tcv, cc, rtol=2e-2)
