"""CPU oracle of the delayed-acceptance surrogate.  TEST INFRASTRUCTURE ONLY.

The same network as aspartik_gb300/csrc/mlp.cu in float64 numpy: inputs ->
H -> H -> H -> 1, GELU in its tanh form (Hendrycks and Gimpel 2016) on the
hidden layers, flat parameters layer by layer (W [out][in] row-major, then
b [out]), and the pair objective mean_n (f(x_new) - f(x_old) - delta)^2 with
its analytic gradient.
"""

from __future__ import annotations

import numpy as np

C = np.sqrt(2.0 / np.pi)
A = 0.044715


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C * (x + A * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C * (x + A * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * C * (1.0 + 3.0 * A * x * x)


def shapes(inputs: int, hidden: int):
    dims = [inputs, hidden, hidden, hidden, 1]
    return [(dims[i + 1], dims[i]) for i in range(4)]


def unflatten(params, inputs: int, hidden: int):
    out, k = [], 0
    for o, i in shapes(inputs, hidden):
        W = params[k:k + o * i].reshape(o, i)
        k += o * i
        b = params[k:k + o]
        k += o
        out.append((W, b))
    return out


def forward(params, x, inputs: int, hidden: int, keep=False):
    layers = unflatten(np.asarray(params, dtype=np.float64), inputs, hidden)
    a = np.asarray(x, dtype=np.float64).reshape(-1, inputs)
    cache = [a]
    for l, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = gelu(z) if l < 3 else z
        cache.append((z, a))
    y = a[:, 0]
    return (y, cache) if keep else y


def loss_grad(params, x_new, x_old, delta, inputs: int, hidden: int):
    x = np.vstack([np.asarray(x_new).reshape(-1, inputs), np.asarray(x_old).reshape(-1, inputs)])
    n = len(delta)
    y, cache = forward(params, x, inputs, hidden, keep=True)
    r = y[:n] - y[n:] - np.asarray(delta, dtype=np.float64)
    loss = np.mean(r * r)
    dy = np.concatenate([2 * r / n, -2 * r / n])[:, None]
    layers = unflatten(np.asarray(params, dtype=np.float64), inputs, hidden)
    grads = [None] * 4
    dz = dy
    for l in range(3, -1, -1):
        a_prev = cache[0] if l == 0 else cache[l][1]
        W, _ = layers[l]
        grads[l] = (dz.T @ a_prev, dz.sum(axis=0))
        if l == 0:
            break
        z_prev = cache[l][0]
        dz = (dz @ W) * gelu_grad(z_prev)
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat
