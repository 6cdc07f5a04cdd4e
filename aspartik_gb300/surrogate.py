"""Python face of the delayed-acceptance surrogate (``b3g_surrogate_*``).

A fully connected network inputs -> H -> H -> H -> 1 (GELU, FP32) trained and
evaluated by the library's own CUDA kernels; parameters are flat, layer by
layer W [out][in] row-major then b [out].
"""

from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _native as nat
from ._native import check, lib


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


class Surrogate:
    def __init__(self, inputs: int, hidden: int = 256, seed: int = 4, device: int = 0):
        h = ct.c_void_p()
        check(lib.b3g_surrogate_create(inputs, hidden, seed, device, ct.byref(h)))
        self._h = h
        self.inputs = inputs
        self.hidden = hidden

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.b3g_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return int(lib.b3g_surrogate_num_params(self._h))

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        check(lib.b3g_surrogate_get_params(self._h, nat.as_ptr(out, ct.c_float)))
        return out

    def set_params(self, p) -> None:
        p = _f32(p)
        assert p.size == self.num_params
        check(lib.b3g_surrogate_set_params(self._h, nat.as_ptr(p, ct.c_float)))

    def forward(self, x) -> np.ndarray:
        x = _f32(x).reshape(-1, self.inputs)
        out = np.empty(x.shape[0], dtype=np.float32)
        check(lib.b3g_surrogate_forward(self._h, nat.as_ptr(x, ct.c_float), x.shape[0],
                                        nat.as_ptr(out, ct.c_float)))
        return out

    def loss_grad(self, x_new, x_old, delta):
        xn = _f32(x_new).reshape(-1, self.inputs)
        xo = _f32(x_old).reshape(-1, self.inputs)
        d = _f32(delta)
        loss = ct.c_float()
        grad = np.empty(self.num_params, dtype=np.float32)
        check(lib.b3g_surrogate_loss_grad(self._h, nat.as_ptr(xn, ct.c_float),
                                          nat.as_ptr(xo, ct.c_float), nat.as_ptr(d, ct.c_float),
                                          d.size, ct.byref(loss), nat.as_ptr(grad, ct.c_float)))
        return loss.value, grad

    def train(self, x_new, x_old, delta, epochs=20, batch=512, lr=1e-3, seed=7) -> float:
        xn = _f32(x_new).reshape(-1, self.inputs)
        xo = _f32(x_old).reshape(-1, self.inputs)
        d = _f32(delta)
        loss = ct.c_float()
        check(lib.b3g_surrogate_train(self._h, nat.as_ptr(xn, ct.c_float),
                                      nat.as_ptr(xo, ct.c_float), nat.as_ptr(d, ct.c_float),
                                      d.size, epochs, batch, lr, seed, ct.byref(loss)))
        return loss.value

    def delta(self, x_new, x_old) -> float:
        xn, xo = _f32(x_new), _f32(x_old)
        out = ct.c_float()
        check(lib.b3g_surrogate_delta(self._h, nat.as_ptr(xn, ct.c_float),
                                      nat.as_ptr(xo, ct.c_float), ct.byref(out)))
        return out.value

    def deltas(self, x_new, x_old) -> np.ndarray:
        """f(x_new[k]) - f(x_old[k]) for every row, one launch."""
        xn, xo = _f32(x_new), _f32(x_old)
        out = np.empty(xn.shape[0], np.float32)
        check(lib.b3g_surrogate_deltas(self._h, nat.as_ptr(xn, ct.c_float),
                                       nat.as_ptr(xo, ct.c_float), xn.shape[0],
                                       nat.as_ptr(out, ct.c_float)))
        return out
