"""Python binding of the learned candidate filter (include/rvgpu_mlp.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import api

N_FEATURES = 40
N_PARAMS = 41473
# offsets of the parameter vector (W[out][in], W1 input padded to 64 columns)
H, KIN = 128, 64
OFFSETS = {"W1": (0, (H, KIN)), "b1": (H * KIN, (H,)), "W2": (H * KIN + H, (H, H)),
           "b2": (H * KIN + H + H * H, (H,)), "W3": (H * KIN + 2 * H + H * H, (H, H)),
           "b3": (H * KIN + 2 * H + 2 * H * H, (H,)), "w4": (H * KIN + 3 * H + 2 * H * H, (H,)),
           "b4": (H * KIN + 4 * H + 2 * H * H, (1,))}

_bound = False


def _lib():
    global _bound
    L = api.lib()
    if not _bound:
        vp, i64, f32p = C.c_void_p, C.c_int64, C.POINTER(C.c_float)
        L.rv_mlp_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_uint64]
        L.rv_mlp_destroy.argtypes = [vp]
        L.rv_mlp_last_error.argtypes = [vp]
        L.rv_mlp_last_error.restype = C.c_char_p
        L.rv_mlp_set_params.argtypes = [vp, vp]
        L.rv_mlp_get_params.argtypes = [vp, vp]
        L.rv_mlp_train.argtypes = [vp, vp, vp, i64, C.c_int, C.c_float, C.c_float, C.c_uint64, vp]
        L.rv_mlp_gradients.argtypes = [vp, vp, vp, i64, C.c_float, vp, f32p]
        L.rv_mlp_predict.argtypes = [vp, vp, i64, vp]
        L.rv_mlp_step_ms.argtypes = [vp, C.POINTER(C.c_double)]
        _bound = True
    return L


def unpack(vec: np.ndarray) -> dict:
    return {k: vec[o:o + int(np.prod(s))].reshape(s).copy() for k, (o, s) in OFFSETS.items()}


def pack(p: dict) -> np.ndarray:
    v = np.zeros(N_PARAMS, np.float32)
    for k, (o, s) in OFFSETS.items():
        v[o:o + int(np.prod(s))] = np.asarray(p[k], np.float32).reshape(-1)
    return v


class Mlp:
    def __init__(self, device: int = 0, batch: int = 4096, seed: int = 0):
        self.L = _lib()
        self.h = C.c_void_p()
        self.batch = batch
        self._check(self.L.rv_mlp_create(C.byref(self.h), device, batch, seed))

    def _check(self, st):
        if st != 0:
            msg = self.L.rv_mlp_last_error(self.h).decode() if self.h else ""
            raise api.RvError(st, msg)

    def close(self):
        if self.h:
            self.L.rv_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        v = np.zeros(N_PARAMS, np.float32)
        self._check(self.L.rv_mlp_get_params(self.h, v.ctypes.data))
        return v

    def set_params(self, v: np.ndarray):
        v = np.ascontiguousarray(v, np.float32)
        assert v.shape == (N_PARAMS,)
        self._check(self.L.rv_mlp_set_params(self.h, v.ctypes.data))

    def gradients(self, x: np.ndarray, y: np.ndarray, pos_weight: float = 1.0):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.zeros(N_PARAMS, np.float32)
        loss = C.c_float()
        self._check(self.L.rv_mlp_gradients(self.h, x.ctypes.data, y.ctypes.data, x.shape[0], pos_weight,
                                            g.ctypes.data, C.byref(loss)))
        return g, loss.value

    def train(self, x: np.ndarray, y: np.ndarray, epochs: int = 5, lr: float = 1e-3, pos_weight: float = 1.0,
              seed: int = 1) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        losses = np.zeros(epochs, np.float32)
        self._check(self.L.rv_mlp_train(self.h, x.ctypes.data, y.ctypes.data, x.shape[0], epochs, lr, pos_weight,
                                        seed, losses.ctypes.data))
        return losses

    def step_ms(self) -> float:
        v = C.c_double()
        self._check(self.L.rv_mlp_step_ms(self.h, C.byref(v)))
        return v.value

    def predict(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        out = np.zeros(x.shape[0], np.float32)
        self._check(self.L.rv_mlp_predict(self.h, x.ctypes.data, x.shape[0], out.ctypes.data))
        return out
