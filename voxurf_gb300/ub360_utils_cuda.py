"""Drop-in replacement of the reference's JIT module ``ub360_utils_cuda``.

lib/cuda/ub360_utils.cpp: ``cumdist_thres(dist, thres) -> mask``, dist a
[n_rays, n_pts] float32 CUDA tensor, mask bool of the same shape
(kernel at ub360_utils_kernel.cu:13-31).  The reference dispatches on every
floating type and accumulates in float32; this module takes float32.
"""
from __future__ import annotations

import torch

from ._torch import call, check_input, ptr, stream_ptr


def cumdist_thres(dist, thres: float):
    check_input(dist, "dist", torch.float32)
    if dist.dim() != 2:
        raise RuntimeError("dist must be [n_rays, n_pts]")
    n_rays, n_pts = dist.size(0), dist.size(1)
    mask = torch.zeros((n_rays, n_pts), dtype=torch.bool, device=dist.device)
    if dist.numel() == 0:
        return mask
    call("vx_cumdist_thres", ptr(dist), n_rays, n_pts, float(thres), ptr(mask), stream_ptr())
    return mask
