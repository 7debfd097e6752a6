"""ORACLE — test infrastructure only (never imported by the product).

Torch-facing restatement of the reference's JIT CUDA modules
(``render_utils_cuda``, ``total_variation_cuda``; lib/cuda/render_utils.cpp:
170-184, total_variation.cpp:29-32) on the CPU, backed by oracle/cref.c.
Tensors go in and out on the CPU; float32 inputs follow the reference
kernels' float arithmetic exactly, float64 inputs (the FP64 oracle) run the
same algorithms in double.  Also used as the stand-in for the reference's
`load()` when the reference's own Python model is executed to make golden
vectors (tests/golden/make_golden.py).
"""
from __future__ import annotations

import numpy as np
import torch

from . import cref

# When set to a list, the branch taken by every non-smooth operation of the
# oracle's step (thresholds, the transmittance stop, relu of the cosine, the
# alpha clip, output clamps) is appended to it: gradient checks use it to
# skip finite differences that straddle a kink.
TRACE = None


def trace(name, value):
    if TRACE is not None:
        TRACE.append((name, value.detach().clone()))


def _np(t):
    return t.detach().cpu().numpy()


class RenderUtilsOracle:
    """Mirror of render_utils_cuda's functions."""

    @staticmethod
    def infer_t_minmax(rays_o, rays_d, xyz_min, xyz_max, near, far):
        a, b = cref.infer_t_minmax(_np(rays_o), _np(rays_d), _np(xyz_min), _np(xyz_max), float(near), float(far))
        dt = rays_o.dtype
        return [torch.from_numpy(a).to(dt), torch.from_numpy(b).to(dt)]

    @staticmethod
    def infer_n_samples(rays_d, t_min, t_max, stepdist):
        return torch.from_numpy(cref.infer_n_samples(_np(rays_d), _np(t_min), _np(t_max), float(stepdist)))

    @staticmethod
    def sample_pts_on_rays(rays_o, rays_d, xyz_min, xyz_max, near, far, stepdist):
        """Sampling is always computed in float32 with the kernel's operation
        order (integer outputs bit-exact); point coordinates are returned in
        the input dtype."""
        out = cref.sample_pts_on_rays(_np(rays_o), _np(rays_d), _np(xyz_min), _np(xyz_max), float(near),
                                      float(far), float(stepdist))
        pts, mask, ray_id, step_id, n_steps, t_min, t_max = out
        dt = rays_o.dtype
        return [torch.from_numpy(pts).to(dt), torch.from_numpy(mask), torch.from_numpy(ray_id),
                torch.from_numpy(step_id), torch.from_numpy(n_steps), torch.from_numpy(t_min).to(dt),
                torch.from_numpy(t_max).to(dt)]

    @staticmethod
    def maskcache_lookup(world, xyz, xyz2ijk_scale, xyz2ijk_shift):
        xyz32 = _np(xyz).astype(np.float32)
        return torch.from_numpy(cref.maskcache_lookup(_np(world), xyz32, _np(xyz2ijk_scale).astype(np.float32),
                                                      _np(xyz2ijk_shift).astype(np.float32)))

    @staticmethod
    def alpha2weight(alpha, ray_id, n_rays):
        w, T, last, i_s, i_e = cref.alpha2weight(_np(alpha), _np(ray_id), int(n_rays))
        return [torch.from_numpy(w), torch.from_numpy(T), torch.from_numpy(last), torch.from_numpy(i_s),
                torch.from_numpy(i_e)]

    @staticmethod
    def alpha2weight_backward(alpha, weight, T, alphainv_last, i_start, i_end, n_rays, grad_weights, grad_last):
        g = cref.alpha2weight_backward(_np(alpha), _np(weight), _np(T), _np(alphainv_last), _np(i_start),
                                       _np(i_end), int(n_rays), _np(grad_weights), _np(grad_last))
        return torch.from_numpy(g)


class TotalVariationOracle:
    """Mirror of total_variation_cuda (total_variation_kernel.cu:14-134)."""

    @staticmethod
    def total_variation_add_grad(param, grad, wx, wy, wz, dense_mode):
        _tv(param, grad, None, wx, wy, wz, dense_mode)

    @staticmethod
    def total_variation_add_grad_new(param, grad, mask, wx, wy, wz, dense_mode):
        _tv(param, grad, mask, wx, wy, wz, dense_mode)


def tv_add_grad_torch(param, grad, wx, wy, wz, dense_mode, mask=None):
    """Vectorised restatement for any float dtype (same semantics as the C
    oracle, including the reference's axis weighting quirk)."""
    wx, wy, wz = wx / 6, wy / 6, wz / 6
    p = param.detach()
    g = grad
    add = torch.zeros_like(p)
    m = None if mask is None else mask.to(p.dtype)
    w_axes = {4: (wz if m is None else wx), 3: wy, 2: wz}
    for dim in (4, 3, 2):
        w = w_axes[dim]
        n = p.size(dim)
        if n < 2:
            continue
        lo = p.narrow(dim, 0, n - 1)
        hi = p.narrow(dim, 1, n - 1)
        d_lo = (lo - hi).clamp(-1, 1) * w  # term for the lower index (its +1 neighbour)
        d_hi = (hi - lo).clamp(-1, 1) * w  # term for the upper index (its -1 neighbour)
        if m is not None:
            mlo = m.narrow(dim, 0, n - 1)
            mhi = m.narrow(dim, 1, n - 1)
            d_lo = d_lo * mlo * mhi
            d_hi = d_hi * mhi * mlo
        add.narrow(dim, 0, n - 1).add_(d_lo)
        add.narrow(dim, 1, n - 1).add_(d_hi)
    sel = torch.ones_like(p, dtype=torch.bool) if dense_mode else (g != 0)
    g += torch.where(sel, add, torch.zeros_like(add))


def _tv(param, grad, mask, wx, wy, wz, dense_mode):
    if param.dtype == torch.float32:
        g = _np(grad).copy()
        cref.tv_add_grad(_np(param[0]) if param.dim() == 5 else _np(param), g.reshape(param.shape[-4:]),
                         float(wx), float(wy), float(wz), dense_mode,
                         mask=None if mask is None else _np(mask).reshape(param.shape[-4:]))
        grad.copy_(torch.from_numpy(g).reshape(grad.shape))
    else:
        tv_add_grad_torch(param, grad, wx, wy, wz, dense_mode, mask)


class Alphas2WeightsOracle(torch.autograd.Function):
    """lib/voxurf_fine.py:981-997 over the oracle ops."""

    @staticmethod
    def forward(ctx, alpha, ray_id, N):
        w, T, last, i_s, i_e = RenderUtilsOracle.alpha2weight(alpha, ray_id, N)
        trace("alpha2weight stop", i_e)
        ctx.save_for_backward(alpha, w, T, last, i_s, i_e)
        ctx.n_rays = N
        return w, last

    @staticmethod
    def backward(ctx, grad_w, grad_last):
        alpha, w, T, last, i_s, i_e = ctx.saved_tensors
        g = RenderUtilsOracle.alpha2weight_backward(alpha, w, T, last, i_s, i_e, ctx.n_rays, grad_w.contiguous(),
                                                    grad_last.contiguous())
        return g, None, None
