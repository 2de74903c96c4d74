"""Learned preconditioner: the CNN of libbella_gb300 (bella_cnn_*), host side.

A 6-layer 3x3x3 convolutional network with 32 hidden channels (ReLU after the
first five), BF16 weights and activations, FP32 accumulation, run -- forward,
backward and the Adam update -- by the library's own kernels.  With
``block=2`` the convolutions run on the grid of 2x2x2 node blocks (8 channels
in and out), which costs an eighth of the node-grid network and doubles its
reach.  As a preconditioner it maps a residual r to an approximate error
e ~ A^-1 r; inputs are normalised by their RMS so the map is scale-equivariant
(M(c r) = c M(r), c > 0).  No counterpart in the reference (pyBELLA has no
learned component).
"""
import ctypes

import numpy as np
import torch

from . import _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def net_voxels(shape, block, nsamples=1):
    nx, ny, nz = shape
    return nsamples * (-(-nx // block)) * (-(-ny // block)) * (-(-nz // block))


class CNN:
    """Device-resident network.  ``capacity``: largest (shape, nsamples) it must run."""

    MODES = {"relu": 0, "linear": 1, "relu_nobias": 2}

    def __init__(self, shape, block=2, nsamples=1, device=None, mode="relu", skip=0.0):
        self._lib = _lib.load()
        self.dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.block = int(block)
        h = ctypes.c_void_p()
        cap = net_voxels(shape, self.block, nsamples)
        _lib.check(self._lib.bella_cnn_create(ctypes.byref(h), self.dev.index, self.block, int(cap)),
                   "bella_cnn_create")
        self.handle = h
        self.nparams = int(self._lib.bella_cnn_param_count(self.block))
        self.mode = mode
        _lib.check(self._lib.bella_cnn_set_mode(self.handle, self.MODES[mode]), "bella_cnn_set_mode")
        self.skip = float(skip)
        _lib.check(self._lib.bella_cnn_set_skip(self.handle, self.skip), "bella_cnn_set_skip")

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def set_params(self, params):
        """params: dict W0..W5 (27, cin, cout), b0..b5 (cout) as in the oracle layout, or a flat array."""
        if isinstance(params, dict):
            params = np.concatenate([np.concatenate([np.asarray(params["W%d" % l], np.float32).ravel(),
                                                     np.asarray(params["b%d" % l], np.float32).ravel()])
                                     for l in range(6)])
        t = torch.as_tensor(np.ascontiguousarray(params, dtype=np.float32)).to(self.dev)
        if t.numel() != self.nparams:
            raise ValueError("expected %d parameters, got %d" % (self.nparams, t.numel()))
        _lib.check(self._lib.bella_cnn_set_params(self.handle, _ptr(t), self._stream()), "bella_cnn_set_params")
        torch.cuda.synchronize(self.dev)

    def get_params(self):
        t = torch.empty(self.nparams, dtype=torch.float32, device=self.dev)
        _lib.check(self._lib.bella_cnn_get_params(self.handle, _ptr(t), self._stream()), "bella_cnn_get_params")
        return t.cpu().numpy()

    def init(self, seed, last_gain=None):
        """He-normal weights (seeded; variance 1/fan-in for the linear net), zero biases.
        ``last_gain`` scales the output layer (small with an identity path, so that
        training starts from the plain method)."""
        rng = np.random.default_rng(seed)
        b3 = self.block ** 3
        cin, cout = [b3, 32, 32, 32, 32, 32], [32, 32, 32, 32, 32, b3]
        gain = 1.0 if self.mode == "linear" else 2.0
        parts = []
        for l in range(6):
            g = 1.0 if (l < 5 or last_gain is None) else float(last_gain)
            parts.append((g * rng.standard_normal(27 * cin[l] * cout[l]) * np.sqrt(gain / (27 * cin[l])))
                         .astype(np.float32))
            parts.append(np.zeros(cout[l], np.float32))
        self.set_params(np.concatenate(parts))

    def forward(self, x, shape, scale=None, out=None):
        """x: CUDA float32 tensor with prod(shape) entries -> CNN(x * s) / s (s = 1/RMS by default)."""
        nx, ny, nz = shape
        x = x.reshape(-1)
        if scale is None:
            rms = float(torch.sqrt(torch.mean(x.double() ** 2)))
            scale = 1.0 / rms if rms > 0 else 1.0
        y = torch.empty_like(x) if out is None else out
        _lib.check(self._lib.bella_cnn_forward(self.handle, nx, ny, nz, _ptr(x), _ptr(y), float(scale),
                                               self._stream()), "bella_cnn_forward")
        return y

    def gradients(self, x, gout, shape):
        """(d/dparams sum(gout * CNN(x)), CNN(x)) for float32 CUDA tensors on the node grid."""
        nx, ny, nz = shape
        g = torch.empty(self.nparams, dtype=torch.float32, device=self.dev)
        y = torch.empty(nx * ny * nz, dtype=torch.float32, device=self.dev)
        _lib.check(self._lib.bella_cnn_gradients(self.handle, nx, ny, nz, _ptr(x.reshape(-1)), _ptr(gout.reshape(-1)),
                                                 _ptr(g), _ptr(y), self._stream()), "bella_cnn_gradients")
        return g, y

    def train_step(self, inputs, targets, lr, want_loss=True):
        """One Adam step on a batch: inputs/targets float32 CUDA tensors (nsamples, nx, ny, nz)."""
        ns, nx, ny, nz = inputs.shape
        loss = ctypes.c_double(float("nan"))
        _lib.check(self._lib.bella_cnn_train_step(self.handle, ns, nx, ny, nz, _ptr(inputs), _ptr(targets),
                                                  float(lr), ctypes.byref(loss) if want_loss else None,
                                                  self._stream()), "bella_cnn_train_step")
        return loss.value

    def set_tensor_cores(self, on):
        """Forward, input-gradient and weight-gradient passes on tcgen05 (True) or on
        mma.sync and FP32 CUDA-core loops (False)."""
        _lib.check(self._lib.bella_cnn_set_tc(self.handle, int(bool(on))), "bella_cnn_set_tc")

    def tensor_core_error(self):
        """True if a tensor-core completion wait gave up (synchronises)."""
        return bool(_lib.check(self._lib.bella_cnn_tc_error(self.handle), "bella_cnn_tc_error"))

    @property
    def launches(self):
        return int(self._lib.bella_cnn_launches(self.handle))

    def __del__(self):
        try:
            if getattr(self, "handle", None) is not None and self.handle.value:
                self._lib.bella_cnn_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


class LearnedPreconditioner:
    """The background solve corrected by the network, each stage applied to the
    residual the previous ones leave (:class:`pybella_gb300.spectral.BackgroundSolve`):

    * ``order="post"``: ``y = A_bg^+ r``, ``y += net(r - A y)``;
    * ``order="pre"``: ``y = net(r)``, ``y += A_bg^+ (r - A y)``;
    * ``order="sym"``: background, network, background.

    The background solve inverts the horizontally averaged (stratified)
    operator exactly; the network, trained on the residuals and errors the
    background solve leaves (:func:`harvest_pairs` with ``background=True``),
    corrects it where the cell coefficients depart from their horizontal means.
    Pass as ``preconditioner=`` to :meth:`~pybella_gb300.linalg.NodalHelmholtz3D.solve`.
    """

    ORDERS = {"post": 0, "pre": 1, "sym": 2}

    def __init__(self, background, network, order="post"):
        self.background = background
        self.network = network
        self.order = order
        self.compose = self.ORDERS[order]


# ---------------------------------------------------------------------------
# training data and training
# ---------------------------------------------------------------------------
def operator_3d(w, ws=None):
    """Device 27-point operator of a :func:`pybella_gb300.workloads.stratified_3d` workload."""
    from .linalg import NodalHelmholtz3D
    return NodalHelmholtz3D(w["hplusx"], w["hplusy"], w["hplusz"], w["hcenter"], w["diag_inv"], w["nx"], w["ny"],
                            w["nz"], w["dx"], w["dy"], w["dz"], walls=w["walls"], corrf=w["corrf"], ws=ws)


def wall_zeroed_cells(w):
    """The cell coefficient (hplusx = hplusy = hplusz) with the wall cell planes zeroed, as the operator uses it."""
    nx, ny, nz = w["nx"], w["ny"], w["nz"]
    h = w["hplusx"].reshape(nx + 1, ny + 1, nz + 1).clone()
    for ax, wall in enumerate(w["walls"]):
        if wall:
            h.index_fill_(ax, torch.tensor([0, h.shape[ax] - 1], device=h.device), 0.0)
    return h


class PairSet:
    """Training windows on the device: residual R, error E (S^3 nodes), the window's
    cell coefficients H ((S+1)^3) and Jacobi scaling D (S^3), FP32; grid spacing."""

    def __init__(self, n, S, spacing):
        kw = dict(dtype=torch.float32, device="cuda")
        self.R = torch.empty((n, S, S, S), **kw)
        self.E = torch.empty((n, S, S, S), **kw)
        self.H = torch.empty((n, S + 1, S + 1, S + 1), **kw)
        self.D = torch.empty((n, S, S, S), **kw)
        self.S, self.n, self.spacing = S, 0, tuple(float(v) for v in spacing)

    def add(self, r, e, h, dinv, shape, count, gen):
        """Random windows of the node fields r, e (unit-RMS residual per window)."""
        nx, ny, nz = shape
        S = self.S
        R, E, D = r.reshape(nx, ny, nz), e.reshape(nx, ny, nz), dinv.reshape(nx, ny, nz)
        for _ in range(count):
            i0 = int(torch.randint(0, nx - S + 1, (1,), generator=gen))
            j0 = int(torch.randint(0, ny - S + 1, (1,), generator=gen))
            k0 = int(torch.randint(0, nz - S + 1, (1,), generator=gen))
            rc = R[i0:i0 + S, j0:j0 + S, k0:k0 + S]
            sc = 1.0 / torch.sqrt(torch.mean(rc * rc)).clamp_min(1e-300)
            q = self.n
            self.R[q] = (rc * sc).to(torch.float32)
            self.E[q] = (E[i0:i0 + S, j0:j0 + S, k0:k0 + S] * sc).to(torch.float32)
            self.H[q] = h[i0:i0 + S + 1, j0:j0 + S + 1, k0:k0 + S + 1].to(torch.float32)
            self.D[q] = D[i0:i0 + S, j0:j0 + S, k0:k0 + S].to(torch.float32)
            self.n += 1

    def trim(self):
        for k in ("R", "E", "H", "D"):
            setattr(self, k, getattr(self, k)[:self.n])
        return self


def harvest_pairs(seeds, shape=(129, 65, 129), npairs=20000, crop=32, checkpoints=None,
                  random_fraction=0.25, powers=(0.0, 2.0, 4.0), solve_tol=1e-9, solve_maxiter=200000,
                  gen_seed=0, log=None, background=False):
    """(residual, error) training windows on the device (a :class:`PairSet`).

    For every seed a :func:`~pybella_gb300.workloads.stratified_3d` problem of
    ``shape`` is solved to ``solve_tol`` (x*), then plain BiCGStab is run again
    from x = 0 and stopped at each of ``checkpoints`` iterations: each stop
    gives r = b - A x and e = x* - x, cut into random windows of ``crop``^3
    nodes with their operator coefficients.  A further ``random_fraction`` of
    the pairs are (A e, e) for seeded Gaussian fields e with power ~k^-p
    (``powers``), covering error components the solver's own iterates leave
    out.  A seed whose x* solve fails contributes only the latter.

    ``background=True`` harvests for the correction stage of a
    :class:`LearnedPreconditioner`: the iterates come from the
    background-preconditioned solver itself (stopped after 0..4 iterations by
    default) and every pair (r, e) becomes (r - A y, e - y) with y = A_bg^+ r,
    the residual and error the background solve leaves.  ``checkpoints``
    defaults to (2, 8, 32, 128, 512, 2048) plain iterations, or (0, 1, 2, 3, 4)
    preconditioned ones with ``background``.
    """
    if checkpoints is None:
        checkpoints = (0, 1, 2, 3, 4) if background else (2, 8, 32, 128, 512, 2048)
    from . import workloads
    gen = torch.Generator(device="cpu")
    gen.manual_seed(int(gen_seed))
    n_rand = int(round(npairs * random_fraction))
    n_iter = npairs - n_rand
    per_state = max(1, -(-n_iter // (len(seeds) * len(checkpoints))))
    per_rand = max(1, -(-n_rand // (len(seeds) * len(powers)))) if n_rand else 0
    ps = None
    for seed in seeds:
        w = workloads.stratified_3d(seed, *shape)
        if ps is None:
            ps = PairSet(npairs, crop, (w["dx"], w["dy"], w["dz"]))
        A = operator_3d(w)
        h = wall_zeroed_cells(w)
        if background:
            from .spectral import BackgroundSolve
            bg = BackgroundSolve(A)

            def add(r, e, count):
                y = bg.apply(r).to(torch.float64)
                ps.add(r - A.matvec(y), e - y, h, w["diag_inv"], shape, count, gen)
        else:
            def add(r, e, count):
                ps.add(r, e, h, w["diag_inv"], shape, count, gen)
        b = w["b"]
        if background:
            xs, st = A.solve(b, tol=solve_tol, maxiter=solve_maxiter, preconditioner=bg)
        else:
            xs, st = A.solve(b, tol=solve_tol, maxiter=solve_maxiter, precision="df64")
        ok = st["status"] == 0
        if log:
            log("seed %d: x* %s in %d iterations (relres %.2e)" % (seed, "found" if ok else "NOT found",
                                                                   st["iterations"], st["relres"]))
        x, done = None, 0
        for k in (checkpoints if ok else ()):
            if ps.n >= n_iter:
                break
            if background:
                x = torch.zeros_like(b) if k == 0 else A.solve(b, tol=1e-300, maxiter=k, preconditioner=bg)[0]
            else:
                x, _ = A.solve(b, x0=x, tol=1e-300, maxiter=k - done, precision="df64")
                done = k
            r = b - A.matvec(x)
            add(r, xs - x, min(per_state, n_iter - ps.n))
        if n_rand:
            g = torch.Generator(device="cuda")
            g.manual_seed(1000 + int(seed))
            for p in powers:
                if ps.n >= npairs:
                    break
                e = workloads._power_field(shape, p, g, torch.device("cuda")).reshape(-1)
                add(A.matvec(e), e, min(per_rand, npairs - ps.n))
        if background:
            bg.close()
        del A
    return ps.trim()


def reach(block):
    """Nodes the network's output depends on in each direction (six 3x3x3 layers)."""
    return 6 * block + block - 1


def train(net, pairs, steps=3000, batch=32, lr=1e-3, lr_final=1e-5, seed=0, log=None, log_every=250, margin=None):
    """Adam on the device with the net's own kernels and the operator-residual loss
    (``bella_cnn_train_step_op``) on each window's core (``margin``: the network's
    reach plus one by default); cosine learning-rate decay.  Returns [(step, loss)]."""
    if margin is None:
        margin = reach(net.block) + 1
    gen = torch.Generator(device="cuda")
    gen.manual_seed(int(seed))
    losses = []
    lib = net._lib
    dx, dy, dz = pairs.spacing
    for it in range(steps):
        idx = torch.randint(0, pairs.n, (batch,), generator=gen, device="cuda")
        lr_t = lr_final + 0.5 * (lr - lr_final) * (1.0 + np.cos(np.pi * it / max(1, steps - 1)))
        want = (it % log_every == 0) or it == steps - 1
        R, E, H, D = (t[idx].contiguous() for t in (pairs.R, pairs.E, pairs.H, pairs.D))
        loss = ctypes.c_double(float("nan"))
        _lib.check(lib.bella_cnn_train_step_op(net.handle, batch, pairs.S, _ptr(R), _ptr(E), _ptr(H), _ptr(D),
                                               dx, dy, dz, int(margin), float(lr_t),
                                               ctypes.byref(loss) if want else None,
                                               net._stream()), "bella_cnn_train_step_op")
        if want:
            losses.append((it, loss.value))
            if log:
                log("step %d  loss %.4f  lr %.2e" % (it, loss.value, lr_t))
    return losses


def train_preconditioner(shape=(129, 65, 129), seeds=(1, 2, 3, 5), npairs=6000, crop=48, steps=2000, batch=32,
                         block=2, mode="linear", skip=1.0, last_gain=0.01, random_fraction=0.25,
                         powers=(0.0, 2.0, 4.0), lr=5e-4, seed=0, log=None, background=False):
    """Harvest pairs, train from a seeded init on the GPU and return the flat FP32 parameters.

    The defaults are the configuration measured for the 3D stratified problem:
    a linear network on 2x2x2 node blocks with an identity path (training
    starts from the plain method), trained on the operator residual of each
    window's core.  ``background=True`` trains the correction stage of a
    :class:`LearnedPreconditioner` (pairs left by the background solve).
    """
    pairs = harvest_pairs(list(seeds), shape=shape, npairs=npairs, crop=crop, random_fraction=random_fraction,
                          powers=powers, gen_seed=seed, log=log, background=background)
    net = CNN((crop, crop, crop), block=block, nsamples=batch, mode=mode, skip=skip)
    net.init(seed, last_gain=last_gain)
    losses = train(net, pairs, steps=steps, batch=batch, lr=lr, seed=seed, log=log, log_every=max(1, steps // 8))
    return net.get_params(), losses
