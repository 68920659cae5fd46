"""Learned initial guess of the multigrid solve (binding of pgb_net_* in
libpamr_gb300): a 4-level convolutional encoder-decoder from the source rho
to a guess of u, trained on (rho, u) pairs the plain multigrid generates.
The kernels (BF16 tensor-core convolutions, training step) are in
pamr_amrd_gb300/csrc/pgb_net.cu; this module only sequences calls."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .solver import _check, lib

_vp, _dp = C.c_void_p, C.POINTER(C.c_double)
_bound = False


def _bind():
    global _bound
    L = lib()
    if _bound:
        return L
    L.pgb_net_create.argtypes = [C.c_int, C.c_ulonglong, C.POINTER(_vp)]
    L.pgb_net_destroy.argtypes = [_vp]
    L.pgb_net_destroy.restype = None
    L.pgb_net_set_scales.argtypes = [_vp, C.c_double, C.c_double]
    L.pgb_net_num_params.argtypes = [_vp]
    L.pgb_net_num_params.restype = C.c_long
    L.pgb_net_params.argtypes = [_vp, C.c_int, C.POINTER(C.c_float), C.c_int]
    L.pgb_net_predict.argtypes = [_vp, _vp, _vp, _vp]
    L.pgb_net_loss_grad.argtypes = [_vp, _vp, _vp, _dp, _vp]
    L.pgb_net_train_step.argtypes = [_vp, _vp, _vp, C.c_float, _dp, _vp]
    L.pgb_conv3d_geometry.argtypes = [C.c_int] * 3 + [_vp, _vp]
    L.pgb_conv3d_pack_weights.argtypes = [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp]
    L.pgb_conv3d_bf16.argtypes = [_vp] * 4 + [C.c_int] * 6 + [_vp, _vp]
    _bound = True
    return L


def conv_lib():
    """the library with the tensor-core convolution entry points bound"""
    return _bind()


class Net:
    """n: grid points per side of the solve (n-1 a multiple of 8, n >= 65)"""

    # layer table in parameter order: (name, cin, cout)
    LAYERS = [("in", 1, 16)] + [(f"tc{i}", a, b) for i, (a, b) in enumerate(
        [(16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 64), (64, 64), (64, 32), (32, 16),
         (16, 16)])] + [("out", 16, 1)]

    def __init__(self, n: int, seed: int = 1):
        L = _bind()
        h = _vp()
        _check(L.pgb_net_create(n, seed, C.byref(h)))
        self.h, self.n = h, n
        self.s_in = self.s_out = 1.0

    def close(self):
        if self.h:
            lib().pgb_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_scales(self, s_in: float, s_out: float):
        self.s_in, self.s_out = s_in, s_out
        _check(lib().pgb_net_set_scales(self.h, s_in, s_out))

    def num_params(self) -> int:
        return int(lib().pgb_net_num_params(self.h))

    def params(self, which: int = 0) -> np.ndarray:
        out = np.zeros(self.num_params(), dtype=np.float32)
        _check(lib().pgb_net_params(self.h, which, out.ctypes.data_as(C.POINTER(C.c_float)), 0))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().pgb_net_params(self.h, 0, p.ctypes.data_as(C.POINTER(C.c_float)), 1))

    def split(self, flat: np.ndarray) -> dict:
        """parameter vector -> {name: (w[27][cin][cout], b[cout])}"""
        out, o = {}, 0
        for name, ci, co in self.LAYERS:
            w = flat[o:o + 27 * ci * co].reshape(27, ci, co)
            o += 27 * ci * co
            out[name] = (w, flat[o:o + co])
            o += co
        return out

    def predict(self, rho_ptr: int, u_ptr: int, stream=None):
        _check(lib().pgb_net_predict(self.h, rho_ptr, u_ptr, stream))

    def loss_grad(self, rho_ptr: int, ut_ptr: int, stream=None) -> float:
        loss = C.c_double()
        _check(lib().pgb_net_loss_grad(self.h, rho_ptr, ut_ptr, C.byref(loss), stream))
        return loss.value

    def train_step(self, rho_ptr: int, ut_ptr: int, lr: float, stream=None, want_loss: bool = True):
        loss = C.c_double()
        _check(lib().pgb_net_train_step(self.h, rho_ptr, ut_ptr, lr, C.byref(loss) if want_loss else None,
                                        stream))
        return loss.value if want_loss else None
