"""CPU oracle of the warm-start MLP (test infrastructure only).

Forward and backward of n_in -> width (GELU) x depth -> n_out in float64,
replaying the roundings the GPU kernels apply: weights, layer inputs, the
output gradient and the hidden-layer gradients rounded to BF16 (round to
nearest even), everything else exact.  The GPU accumulates in FP32, so the
two agree to about 1e-3 relative; tests compare at 1e-2.
"""
import math

import numpy as np


def bf16(x):
    a = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32)
    r = (a + np.uint32(0x7FFF) + ((a >> np.uint32(16)) & np.uint32(1))) & np.uint32(0xFFFF0000)
    return r.view(np.float32).astype(np.float64)


def unpack(params, n_in, width, depth, n_out):
    dims_in = [n_in] + [width] * depth
    dims_out = [width] * depth + [n_out]
    out, p = [], 0
    for i, o in zip(dims_in, dims_out):
        W = np.asarray(params[p:p + i * o], np.float64).reshape(o, i)
        p += i * o
        b = np.asarray(params[p:p + o], np.float64)
        p += o
        out.append((W, b))
    return out


_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def loss_grad(params, x, y, n_in, width, depth, n_out):
    layers = unpack(params, n_in, width, depth, n_out)
    n = x.shape[0]
    acts, pres = [bf16(x)], []
    for l, (W, b) in enumerate(layers):
        z = acts[-1] @ bf16(W).T + b
        pres.append(z)
        if l < len(layers) - 1:
            acts.append(bf16(gelu(z)))
    yhat = pres[-1]
    loss = float(((yhat - y) ** 2).mean())
    dz = bf16(2.0 * (yhat - y) / (n * n_out))
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, b = layers[l]
        grads[l] = (dz.T @ acts[l], dz.sum(0))
        if l == 0:
            break
        da = dz @ bf16(W)
        dz = bf16(da * gelu_grad(pres[l - 1]))
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat
