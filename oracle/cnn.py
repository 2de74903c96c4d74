"""NumPy oracle of the learned preconditioner's CNN (test infrastructure only).

Six 3x3x3 convolutions with zero ("same") padding on a (nx, ny, nz) grid:
1 -> 32 -> 32 -> 32 -> 32 -> 32 -> 1 channels, ReLU after the first five.
Weights, the (scaled) input and the hidden activations are rounded to BF16
exactly where the GPU kernels store them in BF16 (all weights, the packed
input, the outputs of layers 1-5); accumulation is FP32-or-better.  Tap order t = (dx+1)*9 +
(dy+1)*3 + (dz+1); the input of tap t at voxel v is in[v + (dx, dy, dz)].

This network has no counterpart in the reference (pyBELLA has no learned
component); the oracle pins the GPU forward pass and its gradients.
"""
import numpy as np

C = 32
TAPS = [(dx, dy, dz) for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)]


def bf16(a):
    """Round-to-nearest-even to bfloat16, returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def _shift(x, d):
    """x[v + d] with zeros outside (x has spatial dims first)."""
    out = np.zeros_like(x)
    src = [slice(max(0, k), x.shape[i] + min(0, k)) for i, k in enumerate(d)]
    dst = [slice(max(0, -k), x.shape[i] + min(0, -k)) for i, k in enumerate(d)]
    out[tuple(dst)] = x[tuple(src)]
    return out


def conv(x, W, b):
    """x: (nx,ny,nz,Cin); W: (27, Cin, Cout); b: (Cout,) -> (nx,ny,nz,Cout), float64 accumulation."""
    x = x.astype(np.float64)
    out = np.zeros(x.shape[:3] + (W.shape[2],))
    for t, d in enumerate(TAPS):
        out += np.tensordot(_shift(x, d), W[t].astype(np.float64), axes=([3], [0]))
    return out + b


def forward(r, params):
    """r: (nx,ny,nz) float -> (output, activations list)."""
    a = bf16(r[..., None].astype(np.float32))
    acts = [a]
    for layer in range(6):
        W, b = params["W%d" % layer], params["b%d" % layer]
        W = bf16(W)
        z = conv(acts[-1], W, b)
        if layer < 5:
            a = bf16(np.maximum(z, 0.0).astype(np.float32))
        else:
            a = z.astype(np.float32)
        acts.append(a)
    return acts[-1][..., 0], acts


def conv_transpose(g, W):
    """Gradient w.r.t. the input of conv: g (nx,ny,nz,Cout), W (27,Cin,Cout) -> (nx,ny,nz,Cin)."""
    out = np.zeros(g.shape[:3] + (W.shape[1],))
    for t, d in enumerate(TAPS):
        out += _shift(np.tensordot(g.astype(np.float64), W[t].T.astype(np.float64), axes=([3], [0])),
                      tuple(-k for k in d))
    return out


def weight_grad(x, g):
    """dL/dW for conv: x (..,Cin), g (..,Cout) -> (27, Cin, Cout)."""
    out = np.zeros((27, x.shape[3], g.shape[3]))
    for t, d in enumerate(TAPS):
        out[t] = np.tensordot(_shift(x.astype(np.float64), d), g.astype(np.float64), axes=([0, 1, 2], [0, 1, 2]))
    return out


def backward(acts, params, gout):
    """Gradients of sum(gout * output) w.r.t. all weights and biases."""
    grads = {}
    g = gout[..., None].astype(np.float64)
    for layer in range(5, -1, -1):
        W = bf16(params["W%d" % layer])
        x = acts[layer]
        grads["W%d" % layer] = weight_grad(x, g)
        grads["b%d" % layer] = g.sum(axis=(0, 1, 2))
        if layer > 0:
            gin = conv_transpose(g, W)
            g = gin * (acts[layer] > 0)
    return grads


def init_params(seed):
    """He-normal initialisation (seeded), zero biases; shapes as on the GPU."""
    rng = np.random.default_rng(seed)
    cin = [1, C, C, C, C, C]
    cout = [C, C, C, C, C, 1]
    p = {}
    for layer in range(6):
        std = np.sqrt(2.0 / (27 * cin[layer]))
        p["W%d" % layer] = (rng.standard_normal((27, cin[layer], cout[layer])) * std).astype(np.float32)
        p["b%d" % layer] = np.zeros(cout[layer], np.float32)
    return p
