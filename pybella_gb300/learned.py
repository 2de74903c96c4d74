"""Learned preconditioner: the CNN of libbella_gb300 (bella_cnn_*), host side.

A 6-layer 3x3x3 convolutional network with 32 channels (1 -> 32 -> ... -> 32 -> 1,
ReLU), BF16 weights and activations, FP32 accumulation, run by the library's
own tensor-core kernels.  As a preconditioner it maps a residual r to an
approximate error e ~ A^-1 r; inputs are normalised by their RMS so the map is
scale-equivariant (M(c r) = c M(r)).  No counterpart in the reference.
"""
import ctypes

import numpy as np
import torch

from . import _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class CNN:
    def __init__(self, max_voxels, device=None):
        self._lib = _lib.load()
        self.dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        h = ctypes.c_void_p()
        _lib.check(self._lib.bella_cnn_create(ctypes.byref(h), self.dev.index, int(max_voxels)), "bella_cnn_create")
        self.handle = h
        self.nparams = int(self._lib.bella_cnn_param_count())
        self.max_voxels = int(max_voxels)

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def set_params(self, params):
        """params: dict W0..W5 (27, cin, cout), b0..b5 (cout) as in oracle.cnn, or a flat array."""
        flat = params if not isinstance(params, dict) else np.concatenate(
            [np.concatenate([np.asarray(params["W%d" % l], np.float32).ravel(),
                             np.asarray(params["b%d" % l], np.float32).ravel()]) for l in range(6)])
        t = torch.as_tensor(np.ascontiguousarray(flat, dtype=np.float32)).to(self.dev)
        assert t.numel() == self.nparams, (t.numel(), self.nparams)
        _lib.check(self._lib.bella_cnn_set_params(self.handle, _ptr(t), self._stream()), "bella_cnn_set_params")
        torch.cuda.synchronize(self.dev)

    def get_params(self):
        t = torch.empty(self.nparams, dtype=torch.float32, device=self.dev)
        _lib.check(self._lib.bella_cnn_get_params(self.handle, _ptr(t), self._stream()), "bella_cnn_get_params")
        return t.cpu().numpy()

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
