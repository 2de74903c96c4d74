"""NumPy oracle of the learned preconditioner's CNN (test infrastructure only).

Six 3x3x3 convolutions with zero ("same") padding, ReLU after the first five,
32 hidden channels.  With ``block`` = 1 the network runs on the (nx, ny, nz)
grid itself with one input and one output channel; with ``block`` = 2 it runs
on the grid of 2x2x2 node blocks, each block's 8 nodes being 8 channels
(sub-node c = (a*2 + b)*2 + d for offsets (a, b, d); nodes beyond an odd edge
are zero on input and dropped on output).
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


def blocked(r, block):
    """(nx,ny,nz) -> (ceil(nx/b), ceil(ny/b), ceil(nz/b), b^3), zero beyond the edges."""
    nx, ny, nz = r.shape
    c = [-(-n // block) for n in (nx, ny, nz)]
    pad = np.zeros([k * block for k in c], r.dtype)
    pad[:nx, :ny, :nz] = r
    x = pad.reshape(c[0], block, c[1], block, c[2], block).transpose(0, 2, 4, 1, 3, 5)
    return np.ascontiguousarray(x.reshape(c[0], c[1], c[2], block ** 3))


def unblocked(y, shape, block):
    """Inverse of ``blocked``, cropped to ``shape``."""
    c = y.shape[:3]
    x = y.reshape(c[0], c[1], c[2], block, block, block).transpose(0, 3, 1, 4, 2, 5)
    x = x.reshape(c[0] * block, c[1] * block, c[2] * block)
    return np.ascontiguousarray(x[:shape[0], :shape[1], :shape[2]])


def forward(r, params, block=1, rounding=True, linear=False):
    """r: (nx,ny,nz) float -> (output on the same grid, activations list on the net grid).

    ``rounding=False`` evaluates the same network in float64 throughout (for
    finite-difference checks of ``backward``).  ``linear=True``: no ReLU and no
    biases (the linear preconditioner mode)."""
    rnd = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    a = rnd(blocked(np.asarray(r, np.float32 if rounding else np.float64), block))
    acts = [a]
    for layer in range(6):
        W, b = params["W%d" % layer], params["b%d" % layer]
        W = rnd(W)
        z = conv(acts[-1], W, 0.0 * b if linear else b)
        if layer < 5:
            a = rnd((z if linear else np.maximum(z, 0.0)).astype(np.float32 if rounding else np.float64))
        else:
            a = z.astype(np.float32 if rounding else np.float64)
        acts.append(a)
    return unblocked(acts[-1], np.shape(r), block), acts


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


def backward(acts, params, gout, block=1, rounding=True, linear=False):
    """Gradients of sum(gout * output) w.r.t. all weights and biases (gout on the node grid)."""
    grads = {}
    g = blocked(np.asarray(gout, np.float64), block)
    for layer in range(5, -1, -1):
        W = bf16(params["W%d" % layer]) if rounding else np.asarray(params["W%d" % layer], np.float64)
        x = acts[layer]
        grads["W%d" % layer] = weight_grad(x, g)
        grads["b%d" % layer] = g.sum(axis=(0, 1, 2))
        if layer > 0:
            gin = conv_transpose(g, W)
            g = gin if linear else gin * (acts[layer] > 0)
    return grads


def init_params(seed, block=1):
    """He-normal initialisation (seeded), zero biases; shapes as on the GPU."""
    rng = np.random.default_rng(seed)
    cin = [block ** 3, C, C, C, C, C]
    cout = [C, C, C, C, C, block ** 3]
    p = {}
    for layer in range(6):
        std = np.sqrt(2.0 / (27 * cin[layer]))
        p["W%d" % layer] = (rng.standard_normal((27, cin[layer], cout[layer])) * std).astype(np.float32)
        p["b%d" % layer] = np.zeros(cout[layer], np.float32)
    return p


def flatten(params):
    """Parameter dict -> the flat FP32 layout of the GPU net: per layer W (27, cin, cout) then b."""
    return np.concatenate([np.concatenate([np.asarray(params["W%d" % l], np.float32).ravel(),
                                           np.asarray(params["b%d" % l], np.float32).ravel()]) for l in range(6)])


def unflatten(flat, block=1):
    cin = [block ** 3, C, C, C, C, C]
    cout = [C, C, C, C, C, block ** 3]
    p, o = {}, 0
    for l in range(6):
        n = 27 * cin[l] * cout[l]
        p["W%d" % l] = np.asarray(flat[o:o + n]).reshape(27, cin[l], cout[l])
        o += n
        p["b%d" % l] = np.asarray(flat[o:o + cout[l]])
        o += cout[l]
    return p
