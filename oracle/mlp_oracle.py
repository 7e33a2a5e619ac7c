"""CPU oracle of the order-parameter surrogate MLP (TEST INFRASTRUCTURE ONLY).

Imported only by ``tests/`` as the checker of libkura's MLP kernels (kura_mlp_* in
include/kura.h).  The network is a plain multilayer perceptron: layers
in -> hidden -> hidden -> hidden -> out, SiLU between layers, mean squared error.  The
reference program has no learned component, so this oracle is pinned by finite
differences (tests/test_mlp_oracle.py), not by reference outputs.

``bf16=True`` rounds at the points where the GPU stores BF16 (the input rows, the weights,
the hidden activations and the backward signals dZ) and keeps everything else in FP64, so
the remaining GPU-vs-oracle difference is FP32 accumulation order alone.
"""
import numpy as np


def bf16_round(a):
    """Round float values to bfloat16 (round to nearest, ties to even), returned as float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def dims_of(in_dim, hidden, out_dim, layers=4):
    return [in_dim] + [hidden] * (layers - 1) + [out_dim]


def split(params, dims):
    """Flat parameters (per layer W [out][in] row-major, then b [out]) -> [(W, b)]."""
    p = np.asarray(params, np.float64)
    out, k = [], 0
    for i, o in zip(dims[:-1], dims[1:]):
        W = p[k:k + o * i].reshape(o, i)
        k += o * i
        b = p[k:k + o]
        k += o
        out.append((W, b))
    assert k == p.size
    return out


def join(layers):
    return np.concatenate([np.concatenate([W.ravel(), b]) for W, b in layers])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def init_params(dims, seed):
    """Glorot-uniform weights from the splitmix64 stream the library uses, zero biases."""
    s = [seed & 0xFFFFFFFFFFFFFFFF]
    M = 0xFFFFFFFFFFFFFFFF

    def nxt():
        s[0] = (s[0] + 0x9E3779B97F4A7C15) & M
        z = s[0]
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    layers = []
    for i, o in zip(dims[:-1], dims[1:]):
        a = np.sqrt(6.0 / (i + o))
        W = np.array([(2.0 * ((nxt() >> 11) * (1.0 / 9007199254740992.0)) - 1.0) * a for _ in range(o * i)])
        layers.append((W.astype(np.float32).astype(np.float64).reshape(o, i), np.zeros(o)))
    return join(layers)


def forward(params, x, dims, bf16=True):
    r = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
    layers = split(params, dims)
    h = r(x)
    cache = []
    for l, (W, b) in enumerate(layers):
        Wq = r(W)
        z = h @ Wq.T + b
        cache.append((h, Wq, z))
        if l < len(layers) - 1:
            h = r(silu(z))
        else:
            h = z
    return h, cache


def loss_and_grads(params, x, t, dims, bf16=True):
    """Mean squared error over all outputs and its gradient (flat parameter order)."""
    r = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
    y, cache = forward(params, x, dims, bf16)
    n, out = y.shape
    e = y - np.asarray(t, np.float64)
    loss = float(np.sum(e * e) / (n * out))
    dz = r(2.0 * e / (n * out))
    grads = [None] * len(cache)
    for l in range(len(cache) - 1, -1, -1):
        h, Wq, z = cache[l]
        gW = dz.T @ h
        gb = dz.sum(axis=0)
        grads[l] = (gW, gb)
        if l > 0:
            zp = cache[l - 1][2]
            dz = r((dz @ Wq) * dsilu(zp))
    return loss, join(grads)


def adam_step(params, grads, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba) at 0-based step `step`; returns new params, m, v."""
    m = b1 * m + (1 - b1) * grads
    v = b2 * v + (1 - b2) * grads * grads
    mh = m / (1 - b1 ** (step + 1))
    vh = v / (1 - b2 ** (step + 1))
    return params - lr * mh / (np.sqrt(vh) + eps), m, v
