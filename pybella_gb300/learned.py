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

    def __init__(self, shape, block=2, nsamples=1, device=None):
        self._lib = _lib.load()
        self.dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.block = int(block)
        h = ctypes.c_void_p()
        cap = net_voxels(shape, self.block, nsamples)
        _lib.check(self._lib.bella_cnn_create(ctypes.byref(h), self.dev.index, self.block, int(cap)),
                   "bella_cnn_create")
        self.handle = h
        self.nparams = int(self._lib.bella_cnn_param_count(self.block))

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

    def init(self, seed):
        """He-normal weights (seeded), zero biases."""
        rng = np.random.default_rng(seed)
        b3 = self.block ** 3
        cin, cout = [b3, 32, 32, 32, 32, 32], [32, 32, 32, 32, 32, b3]
        parts = []
        for l in range(6):
            parts.append((rng.standard_normal(27 * cin[l] * cout[l]) * np.sqrt(2.0 / (27 * cin[l]))).astype(np.float32))
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
