"""Learned KT corrector: host side of the CUDA network (asg_net_* in the C ABI).

The network maps one coarse KT step of a t-column (scaled by the column's peak)
to the correction that brings it to the fully sub-cycled KT step:

    out = coarse + s * net(coarse / s),   s = max|u| of the column entering the step

Forward and backward run in the library's own kernels (BF16 tensor-core GEMMs
for the 64x64 layers, FP32 accumulation, FP32 master weights, Adam); this
module only orchestrates: parameter initialisation, the training loop over
device batches and the data generation from the plain KT kernel.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

NCH, KT5 = 64, 5
SHAPES = [("W1", (NCH, 1, KT5)), ("b1", (NCH,)), ("W2", (NCH, NCH, KT5)), ("b2", (NCH,)),
          ("W3", (NCH, NCH, KT5)), ("b3", (NCH,)), ("W4", (1, NCH, KT5)), ("b4", (1,))]


def param_count() -> int:
    return int(sum(np.prod(s) for _, s in SHAPES))


def to_dict(theta):
    """Flat parameter vector -> {name: array} with W[out][in][tap] shapes."""
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(theta[o:o + n], dtype=np.float32).reshape(shp)
        o += n
    return out


def from_dict(d):
    return np.concatenate([np.asarray(d[name], np.float32).reshape(-1) for name, _ in SHAPES])


def init_params(seed: int = 0, last_scale: float = 1e-2):
    """He-style initialisation; the last layer starts small so that the
    untrained correction is close to zero."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shp in SHAPES:
        if name.startswith("b"):
            d[name] = np.zeros(shp, np.float32)
        else:
            fan_in = shp[1] * shp[2]
            d[name] = (rng.standard_normal(shp) * np.sqrt(2.0 / fan_in)).astype(np.float32)
    d["W4"] *= last_scale
    return from_dict(d)


class Corrector:
    """The network on the current CUDA device."""

    def __init__(self, theta=None, seed: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self.lib.asg_net_create(C.byref(h)))
        self.h = h
        assert self.lib.asg_net_param_count() == param_count()
        self.set_params(init_params(seed) if theta is None else theta)

    def close(self):
        if getattr(self, "h", None):
            self.lib.asg_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, theta):
        t = np.ascontiguousarray(theta, dtype=np.float32)
        _lib.check(self.lib.asg_net_set_params(self.h, _lib.fptr(t), t.size))

    def get_params(self):
        t = np.empty(param_count(), np.float32)
        _lib.check(self.lib.asg_net_get_params(self.h, _lib.fptr(t), t.size))
        return t

    def forward(self, x, y=None, stream=None):
        """x: CUDA float32 tensor (ncols, nT) -> y (same shape)."""
        import torch
        assert x.is_cuda and x.dtype == torch.float32 and x.dim() == 2 and x.is_contiguous()
        if y is None:
            y = torch.empty_like(x)
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _lib.check(self.lib.asg_net_forward(self.h, C.c_void_p(x.data_ptr()),
                                            C.c_void_p(y.data_ptr()), x.shape[0], x.shape[1],
                                            C.c_void_p(s)))
        return y

    def train_step(self, x, target, mask, lr: float, want_grad: bool = False):
        """One Adam step (lr > 0) or a gradient evaluation (lr = 0) on a device
        batch; returns the masked MSE loss (and the gradient vector)."""
        import torch
        torch.cuda.synchronize()
        loss = C.c_double(0.0)
        g = np.empty(param_count(), np.float32) if want_grad else None
        _lib.check(self.lib.asg_net_train_step(
            self.h, C.c_void_p(x.data_ptr()), C.c_void_p(target.data_ptr()),
            C.c_void_p(mask.data_ptr()), x.shape[0], x.shape[1], float(lr), C.byref(loss),
            _lib.fptr(g)))
        return (loss.value, g) if want_grad else loss.value
