"""Drop-in replacement of the reference's ``adam_upd_cuda`` module.

lib/cuda/adam_upd.cpp:79-86 (built by the reference but never loaded by its
models): ``adam_upd``, ``masked_adam_upd`` and ``adam_upd_with_perlr``, all
in place.  The step size is derived on the host in float exactly as
adam_upd_kernel.cu:72 does.
"""
from __future__ import annotations

import torch

from ._torch import call, check_input, ptr, stream_ptr


def _check(*named):
    for n, t in named:
        check_input(t, n, torch.float32)


def adam_upd(param, grad, exp_avg, exp_avg_sq, step: int, beta1: float, beta2: float, lr: float, eps: float) -> None:
    _check(("param", param), ("grad", grad), ("exp_avg", exp_avg), ("exp_avg_sq", exp_avg_sq))
    call("vx_adam_upd", ptr(param), ptr(grad), ptr(exp_avg), ptr(exp_avg_sq), param.numel(), int(step), float(beta1),
         float(beta2), float(lr), float(eps), stream_ptr())


def masked_adam_upd(param, grad, exp_avg, exp_avg_sq, step: int, beta1: float, beta2: float, lr: float,
                    eps: float) -> None:
    _check(("param", param), ("grad", grad), ("exp_avg", exp_avg), ("exp_avg_sq", exp_avg_sq))
    call("vx_masked_adam_upd", ptr(param), ptr(grad), ptr(exp_avg), ptr(exp_avg_sq), param.numel(), int(step),
         float(beta1), float(beta2), float(lr), float(eps), stream_ptr())


def adam_upd_with_perlr(param, grad, exp_avg, exp_avg_sq, perlr, step: int, beta1: float, beta2: float, lr: float,
                        eps: float) -> None:
    _check(("param", param), ("grad", grad), ("exp_avg", exp_avg), ("exp_avg_sq", exp_avg_sq), ("perlr", perlr))
    call("vx_adam_upd_with_perlr", ptr(param), ptr(grad), ptr(exp_avg), ptr(exp_avg_sq), ptr(perlr), param.numel(),
         int(step), float(beta1), float(beta2), float(lr), float(eps), stream_ptr())
