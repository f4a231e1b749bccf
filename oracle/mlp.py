"""FP64 NumPy restatement of the selector network's forward and backward
passes — TEST INFRASTRUCTURE ONLY (the checker for the CUDA training kernels
in portblas_gb300/csrc/mlp.cu; portBLAS has no counterpart).

Network: in -> hid -> hid -> hid -> out, GELU (erf form) after the three
hidden layers; parameters packed [W1 b1 W2 b2 W3 b3 W4 b4] with W row-major
(out x in); loss = sum(mask * (y - t)^2) / valid_count.
"""
import math

import numpy as np

_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def unpack(p, din, hid, dout):
    p = np.asarray(p, dtype=np.float64)
    dims = [din, hid, hid, hid, dout]
    out, o = [], 0
    for l in range(4):
        w = p[o:o + dims[l + 1] * dims[l]].reshape(dims[l + 1], dims[l])
        o += dims[l + 1] * dims[l]
        b = p[o:o + dims[l + 1]]
        o += dims[l + 1]
        out.append((w, b))
    return out, o


def forward(p, x, din, hid, dout):
    layers, _ = unpack(p, din, hid, dout)
    a = np.asarray(x, dtype=np.float64)
    zs, acts = [], [a]
    for l, (w, b) in enumerate(layers):
        z = a @ w.T + b
        zs.append(z)
        a = gelu(z) if l < 3 else z
        acts.append(a)
    return a, zs, acts


def loss_grad(p, x, t, mask, din, hid, dout, valid):
    y, zs, acts = forward(p, x, din, hid, dout)
    d = (y - t) * mask
    loss = float((d * d).sum() / valid)
    dz = 2.0 * d / valid
    layers, count = unpack(p, din, hid, dout)
    grads = [None] * 4
    for l in range(3, -1, -1):
        w, _ = layers[l]
        grads[l] = (dz.T @ acts[l], dz.sum(0))
        if l == 0:
            break
        dz = (dz @ w) * gelu_grad(zs[l - 1])
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    assert flat.size == count
    return loss, flat
