"""CPU restatement of the surrogate ln g(E) network -- test infrastructure.

Only the tests import this module: it is the checker for the tensor-core
forward/backward kernels, never part of the product.  The network is the
one the library trains: 7 inputs (zero-padded to 64), four hidden layers of
256 SiLU units, one linear output, mean-squared-error loss.  The network has
no counterpart in the reference (its ladder is the multihistogram one,
src/cae_estimator.cc:295-428), so this module is pinned by a finite-
difference check of its own FP64 gradient instead of by reference vectors.

With `emulate_bf16=True` it rounds to bfloat16 (round to nearest even) at the
points where the device kernels store BF16: the padded inputs, the weight
copies, each layer's activations and the pre-activation gradients that feed
the tensor-core GEMMs.  Sums run in FP64.
"""
import numpy as np

IN = 7
K0 = 64
H = 256
LAYERS = 4
KIN = [K0, H, H, H]


def _layout():
    off, o = {}, 0
    for layer in range(LAYERS):
        off[f"W{layer}"] = (o, (H, KIN[layer]))
        o += H * KIN[layer]
        off[f"b{layer}"] = (o, (H,))
        o += H
    off["w5"] = (o, (H,))
    o += H
    off["b5"] = (o, (1,))
    o += 1
    return off, o


OFFSETS, PARAM_COUNT = _layout()


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in OFFSETS.items()}


def pack(d):
    p = np.zeros(PARAM_COUNT)
    for k, (o, s) in OFFSETS.items():
        p[o:o + int(np.prod(s))] = np.asarray(d[k]).reshape(-1)
    return p


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, X, emulate_bf16=True):
    """Returns (y, cache).  X is n x 7."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    P = unpack(p)
    X = np.asarray(X, np.float64)
    h = np.zeros((len(X), K0))
    h[:, :IN] = X
    h = r(h)
    ins, zs = [], []
    for layer in range(LAYERS):
        ins.append(h)
        z = h @ r(P[f"W{layer}"]).T + P[f"b{layer}"]
        if emulate_bf16:
            z = z.astype(np.float32).astype(np.float64)
        zs.append(z)
        h = r(_silu(z))
    y = h @ P["w5"] + P["b5"][0]
    return y, (ins, zs, h)


def loss_and_grad(p, X, t, emulate_bf16=True):
    """Mean squared error over the rows and its gradient (flat vector)."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    P = unpack(p)
    y, (ins, zs, h4) = forward(p, X, emulate_bf16)
    n = len(y)
    e = y - np.asarray(t, np.float64)
    loss = float((e * e).sum() / n)
    dy = 2.0 * e / n
    G = {"w5": h4.T @ dy, "b5": np.array([dy.sum()])}
    dz = dy[:, None] * P["w5"][None, :] * _silu_grad(zs[3])
    for layer in range(LAYERS - 1, -1, -1):
        G[f"W{layer}"] = r(dz).T @ ins[layer]
        G[f"b{layer}"] = dz.sum(axis=0)
        if layer == 0:
            break
        dh = r(dz) @ r(P[f"W{layer}"])
        dz = dh * _silu_grad(zs[layer - 1])
    return loss, pack(G)


def init_like_device(seed):
    """Random parameters with the device's shapes (He scaling); unused input
    columns of W0 zero."""
    rng = np.random.default_rng(seed)
    d = {}
    for layer in range(LAYERS):
        fan = IN if layer == 0 else H
        w = rng.normal(0, np.sqrt(2.0 / fan), (H, KIN[layer]))
        if layer == 0:
            w[:, IN:] = 0
        d[f"W{layer}"] = w
        d[f"b{layer}"] = rng.normal(0, 0.05, H)
    d["w5"] = rng.normal(0, np.sqrt(1.0 / H), H)
    d["b5"] = np.array([0.1])
    return pack(d)
