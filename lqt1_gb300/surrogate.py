"""The learned surrogate's network on the GPU (lqt_mlp_*).

48 -> 128 -> 128 -> 48 MLP with SiLU, BF16 weights, FP32 accumulation.
Inference runs on the tcgen05 tensor cores (TMEM accumulators); training uses
hand-written BF16 mma.sync GEMMs and Adam.  Device buffers are torch tensors
owned by the caller.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

IN, HID, OUT = 48, 128, 48
N_STATE, N_PARAM = 38, 6


def _bind():
    L = N.lib()
    P = C.c_void_p
    sig = {
        "lqt_mlp_create": ([C.c_uint64, P, C.POINTER(P)], C.c_int),
        "lqt_mlp_destroy": ([P], None),
        "lqt_mlp_num_params": ([], C.c_int64),
        "lqt_mlp_set_params": ([P, P], C.c_int),
        "lqt_mlp_get_params": ([P, P, P], C.c_int),
        "lqt_mlp_set_norm": ([P, P, P, P, C.c_int32], C.c_int),
        "lqt_mlp_set_layout": ([P, C.c_int32], C.c_int),
        "lqt_mlp_infer": ([P, P, P, C.c_int64], C.c_int),
        "lqt_mlp_gradients": ([P, P, P, C.c_int64, C.POINTER(C.c_double)], C.c_int),
        "lqt_mlp_train_step": ([P, P, P, C.c_int64, C.c_float, C.POINTER(C.c_double)], C.c_int),
    }
    for k, (a, r) in sig.items():
        f = getattr(L, k)
        f.argtypes, f.restype = a, r
    return L


class Mlp:
    def __init__(self, seed: int = 0, stream: int | None = None):
        self.L = _bind()
        h = C.c_void_p()
        N.check(self.L.lqt_mlp_create(seed, C.c_void_p(stream or 0), C.byref(h)), "lqt_mlp_create")
        self._h = h
        self.nparam = int(self.L.lqt_mlp_num_params())

    def close(self):
        if getattr(self, "_h", None):
            self.L.lqt_mlp_destroy(self._h)
            self._h = None

    __del__ = close

    def params(self):
        p = np.zeros(self.nparam, np.float32)
        N.check(self.L.lqt_mlp_get_params(self._h, p.ctypes.data, None), "lqt_mlp_get_params")
        return p

    def grads(self):
        g = np.zeros(self.nparam, np.float32)
        N.check(self.L.lqt_mlp_get_params(self._h, None, g.ctypes.data), "lqt_mlp_get_params")
        return g

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        N.check(self.L.lqt_mlp_set_params(self._h, p.ctypes.data), "lqt_mlp_set_params")

    def set_norm(self, in_mean, in_scale, out_scale, nvalid=N_STATE):
        a = [np.ascontiguousarray(x, np.float32) for x in (in_mean, in_scale, out_scale)]
        N.check(self.L.lqt_mlp_set_norm(self._h, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data, nvalid),
                "lqt_mlp_set_norm")

    def set_layout(self, layout: int):
        N.check(self.L.lqt_mlp_set_layout(self._h, layout), "lqt_mlp_set_layout")

    def infer(self, x_bf16, y_f32):
        """x_bf16: torch bfloat16 [n, 48] cuda; y_f32: torch float32 [n, 48] cuda."""
        N.check(self.L.lqt_mlp_infer(self._h, x_bf16.data_ptr(), y_f32.data_ptr(), x_bf16.shape[0]), "lqt_mlp_infer")

    def gradients(self, x_bf16, t_f32):
        loss = C.c_double()
        N.check(self.L.lqt_mlp_gradients(self._h, x_bf16.data_ptr(), t_f32.data_ptr(), x_bf16.shape[0],
                                         C.byref(loss)), "lqt_mlp_gradients")
        return loss.value

    def train_step(self, x_bf16, t_f32, lr=1e-3):
        loss = C.c_double()
        N.check(self.L.lqt_mlp_train_step(self._h, x_bf16.data_ptr(), t_f32.data_ptr(), x_bf16.shape[0], lr,
                                          C.byref(loss)), "lqt_mlp_train_step")
        return loss.value
