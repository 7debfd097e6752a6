"""Drop-in replacement of the reference's JIT module ``total_variation_cuda``.

lib/cuda/total_variation.cpp:29-32: ``total_variation_add_grad(param, grad,
wx, wy, wz, dense_mode)`` and ``total_variation_add_grad_new(param, grad,
mask, wx, wy, wz, dense_mode)``, in place on ``grad``.  ``param`` is the
reference's channel-first [1, C, X, Y, Z] float32 grid.
"""
from __future__ import annotations

import torch

from ._torch import call, check_input, ptr, stream_ptr


def _dims(param):
    if param.dim() != 5:
        raise RuntimeError("param must be [1, C, X, Y, Z]")
    X, Y, Z = param.size(2), param.size(3), param.size(4)
    return param.numel() // max(X * Y * Z, 1), X, Y, Z


def total_variation_add_grad(param, grad, wx: float, wy: float, wz: float, dense_mode: bool) -> None:
    check_input(param, "param", torch.float32)
    check_input(grad, "grad", torch.float32)
    C, X, Y, Z = _dims(param)
    call("vx_total_variation_add_grad", ptr(param), ptr(grad), float(wx), float(wy), float(wz), int(bool(dense_mode)),
         C, X, Y, Z, 0, stream_ptr())


def total_variation_add_grad_new(param, grad, mask, wx: float, wy: float, wz: float, dense_mode: bool) -> None:
    check_input(param, "param", torch.float32)
    check_input(grad, "grad", torch.float32)
    check_input(mask, "mask", torch.float32)
    C, X, Y, Z = _dims(param)
    call("vx_total_variation_add_grad_new", ptr(param), ptr(grad), ptr(mask), float(wx), float(wy), float(wz),
         int(bool(dense_mode)), C, X, Y, Z, 0, stream_ptr())
