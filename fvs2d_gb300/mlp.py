"""The warm-start network through the C-ABI (fvs_mlp_*): training and
inference run on the GPU with the library's own BF16 tensor-core kernels."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .solver import FvsError


class MLP:
    def __init__(self, n_in: int, width: int, depth: int, n_out: int, seed: int = 0):
        self._lib = capi.load()
        h = C.c_void_p()
        rc = self._lib.fvs_mlp_create(n_in, width, depth, n_out, C.c_uint64(seed), C.byref(h))
        if rc != capi.FVS_OK:
            raise FvsError(rc, self._lib.fvs_mlp_last_error(None).decode())
        self._h = h
        self.n_in, self.width, self.depth, self.n_out = n_in, width, depth, n_out

    def _check(self, rc):
        if rc != capi.FVS_OK:
            raise FvsError(rc, self._lib.fvs_mlp_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fvs_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_engine(self, engine: str) -> None:
        """GEMM engine: "tcgen05" (default; tensor-core MMA, accumulator in
        tensor memory) or "mma.sync" (warp-level MMA)."""
        self._check(self._lib.fvs_mlp_set_engine(self._h, {"tcgen05": 0, "mma.sync": 1}[engine]))

    def num_params(self) -> int:
        n = C.c_int64(0)
        self._check(self._lib.fvs_mlp_num_params(self._h, C.byref(n)))
        return n.value

    def get_params(self) -> np.ndarray:
        p = np.empty(self.num_params(), np.float32)
        self._check(self._lib.fvs_mlp_get_params(self._h, capi.ptr(p), p.size))
        return p

    def set_params(self, p) -> None:
        a = np.ascontiguousarray(p, np.float32)
        self._check(self._lib.fvs_mlp_set_params(self._h, capi.ptr(a), a.size))

    def loss_grad(self, x, y):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.empty(self.num_params(), np.float32)
        loss = C.c_float(0)
        self._check(self._lib.fvs_mlp_loss_grad(self._h, capi.ptr(x), capi.ptr(y), x.shape[0], C.byref(loss), capi.ptr(g)))
        return loss.value, g

    def train(self, x, y, batch=4096, epochs=10, lr=1e-3, seed=0) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        losses = np.empty(epochs, np.float32)
        self._check(self._lib.fvs_mlp_train(self._h, capi.ptr(x), capi.ptr(y), x.shape[0], batch, epochs, C.c_float(lr),
                                            C.c_uint64(seed), capi.ptr(losses)))
        return losses

    def predict(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty((x.shape[0], self.n_out), np.float32)
        self._check(self._lib.fvs_mlp_predict(self._h, capi.ptr(x), x.shape[0], capi.ptr(y)))
        return y
