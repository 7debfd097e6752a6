"""Drop-in replacement of the reference's JIT module ``render_utils_cuda``.

Same function names, argument meaning, return tuples and error behaviour as
the pybind11 table at lib/cuda/render_utils.cpp:170-184, computed by the
sm_103a kernels of ``libvoxurf_gb300.so`` on the current CUDA stream (the
reference launches on the legacy default stream).  Inputs must be CUDA,
contiguous float32 tensors (the reference dispatches float32/float64 but
every Voxurf model feeds float32).

The three ops the Voxurf models never call (sample_ndc_pts_on_rays,
sample_bg_pts_on_rays and the raw2alpha family) are outside this build's
scope and raise NotImplementedError.
"""
from __future__ import annotations

import torch

from ._torch import call, check_input, ptr, scratch, stream_ptr
from . import _native

__all__ = [
    "infer_t_minmax", "infer_n_samples", "infer_ray_start_dir", "sample_pts_on_rays", "maskcache_lookup",
    "alpha2weight", "alpha2weight_backward",
]

_F32 = torch.float32
_I64 = torch.int64


def infer_t_minmax(rays_o, rays_d, xyz_min, xyz_max, near: float, far: float):
    """render_utils.cpp:50-58 -> [t_min, t_max]."""
    for n, t in (("rays_o", rays_o), ("rays_d", rays_d), ("xyz_min", xyz_min), ("xyz_max", xyz_max)):
        check_input(t, n, _F32)
    n = rays_o.size(0)
    t_min = torch.empty(n, dtype=_F32, device=rays_o.device)
    t_max = torch.empty(n, dtype=_F32, device=rays_o.device)
    call("vx_infer_t_minmax", ptr(rays_o), ptr(rays_d), ptr(xyz_min), ptr(xyz_max), float(near), float(far), n,
         ptr(t_min), ptr(t_max), stream_ptr())
    return [t_min, t_max]


def infer_n_samples(rays_d, t_min, t_max, stepdist: float):
    """render_utils.cpp:60-65 -> N_steps (int64)."""
    for n, t in (("rays_d", rays_d), ("t_min", t_min), ("t_max", t_max)):
        check_input(t, n, _F32)
    n = t_min.size(0)
    out = torch.empty(n, dtype=_I64, device=t_min.device)
    call("vx_infer_n_samples", ptr(rays_d), ptr(t_min), ptr(t_max), float(stepdist), n, ptr(out), stream_ptr())
    return out


def infer_ray_start_dir(rays_o, rays_d, t_min):
    """render_utils.cpp:67-72 -> [rays_start, rays_dir]."""
    for n, t in (("rays_o", rays_o), ("rays_d", rays_d), ("t_min", t_min)):
        check_input(t, n, _F32)
    n = rays_o.size(0)
    start = torch.empty_like(rays_o)
    direc = torch.empty_like(rays_o)
    call("vx_infer_ray_start_dir", ptr(rays_o), ptr(rays_d), ptr(t_min), n, ptr(start), ptr(direc), stream_ptr())
    return [start, direc]


def sample_pts_count(rays_o, rays_d, xyz_min, xyz_max, near: float, far: float, stepdist: float):
    """Phase 1 of sample_pts_on_rays, fully on the device (no sync).

    Returns (t_min, t_max, N_steps, offsets) with offsets[-1] = total samples.
    """
    for n, t in (("rays_o", rays_o), ("rays_d", rays_d), ("xyz_min", xyz_min), ("xyz_max", xyz_max)):
        check_input(t, n, _F32)
    if rays_o.dim() != 2 or rays_o.size(1) != 3:
        raise RuntimeError("rays_o must be [N, 3]")
    dev = rays_o.device
    n = rays_o.size(0)
    t_min = torch.empty(n, dtype=_F32, device=dev)
    t_max = torch.empty(n, dtype=_F32, device=dev)
    n_steps = torch.empty(n, dtype=_I64, device=dev)
    offsets = torch.empty(n + 1, dtype=_I64, device=dev)
    nb = _native.load().vx_scan_scratch_bytes(n)
    tmp = scratch(nb, dev)
    call("vx_sample_pts_count", ptr(rays_o), ptr(rays_d), ptr(xyz_min), ptr(xyz_max), float(near), float(far),
         float(stepdist), n, ptr(t_min), ptr(t_max), ptr(n_steps), ptr(offsets), ptr(tmp), nb, stream_ptr())
    return t_min, t_max, n_steps, offsets


def sample_pts_on_rays(rays_o, rays_d, xyz_min, xyz_max, near: float, far: float, stepdist: float):
    """render_utils.cpp:74-85 ->
    [ray_pts, mask_outbbox, ray_id, step_id, N_steps, t_min, t_max].

    Like the reference (render_utils_kernel.cu:212), exact-size outputs need
    the total sample count on the host: one 8-byte device->host read.
    """
    t_min, t_max, n_steps, offsets = sample_pts_count(rays_o, rays_d, xyz_min, xyz_max, near, far, stepdist)
    total = int(offsets[-1].item())
    dev = rays_o.device
    n = rays_o.size(0)
    ray_pts = torch.empty((total, 3), dtype=_F32, device=dev)
    mask_outbbox = torch.empty(total, dtype=torch.bool, device=dev)
    ray_id = torch.empty(total, dtype=_I64, device=dev)
    step_id = torch.empty(total, dtype=_I64, device=dev)
    call("vx_sample_pts_fill", ptr(rays_o), ptr(rays_d), ptr(xyz_min), ptr(xyz_max), ptr(t_min), ptr(offsets),
         float(stepdist), n, total, ptr(ray_pts), ptr(mask_outbbox), ptr(ray_id), ptr(step_id), stream_ptr())
    return [ray_pts, mask_outbbox, ray_id, step_id, n_steps, t_min, t_max]


def maskcache_lookup(world, xyz, xyz2ijk_scale, xyz2ijk_shift):
    """render_utils.cpp:109-118 -> bool[M]; False outside the grid."""
    check_input(world, "world", torch.bool)
    check_input(xyz, "xyz", _F32)
    check_input(xyz2ijk_scale, "xyz2ijk_scale", _F32)
    check_input(xyz2ijk_shift, "xyz2ijk_shift", _F32)
    if world.dim() != 3 or xyz.dim() != 2 or xyz.size(1) != 3:
        raise RuntimeError("world must be [X,Y,Z] and xyz [M,3]")
    n = xyz.size(0)
    out = torch.zeros(n, dtype=torch.bool, device=xyz.device)
    if n == 0:
        return out
    call("vx_maskcache_lookup", ptr(world), world.size(0), world.size(1), world.size(2), ptr(xyz), n,
         ptr(xyz2ijk_scale), ptr(xyz2ijk_shift), ptr(out), stream_ptr())
    return out


def alpha2weight(alpha, ray_id, n_rays: int):
    """render_utils.cpp:142-149 -> [weight, T, alphainv_last, i_start, i_end]."""
    check_input(alpha, "alpha", _F32)
    check_input(ray_id, "ray_id", _I64)
    if alpha.dim() != 1 or ray_id.dim() != 1 or alpha.shape != ray_id.shape:
        raise RuntimeError("alpha and ray_id must be 1-D of equal length")
    dev = alpha.device
    n_pts = alpha.size(0)
    n_rays = int(n_rays)
    weight = torch.empty_like(alpha)
    T = torch.empty_like(alpha)
    alphainv_last = torch.empty(n_rays, dtype=_F32, device=dev)
    i_start = torch.empty(n_rays, dtype=_I64, device=dev)
    i_end = torch.empty(n_rays, dtype=_I64, device=dev)
    call("vx_alpha2weight", ptr(alpha), ptr(ray_id), n_pts, n_rays, ptr(weight), ptr(T), ptr(alphainv_last),
         ptr(i_start), ptr(i_end), stream_ptr())
    return [weight, T, alphainv_last, i_start, i_end]


def alpha2weight_backward(alpha, weight, T, alphainv_last, i_start, i_end, n_rays: int, grad_weights, grad_last):
    """render_utils.cpp:151-167 -> grad[S]."""
    for n, t in (("alpha", alpha), ("weight", weight), ("T", T), ("alphainv_last", alphainv_last),
                 ("grad_weights", grad_weights), ("grad_last", grad_last)):
        check_input(t, n, _F32)
    check_input(i_start, "i_start", _I64)
    check_input(i_end, "i_end", _I64)
    grad = torch.empty_like(alpha)
    call("vx_alpha2weight_backward", ptr(alpha), ptr(weight), ptr(T), ptr(alphainv_last), ptr(i_start), ptr(i_end),
         alpha.numel(), int(n_rays), ptr(grad_weights), ptr(grad_last), ptr(grad), stream_ptr())
    return grad


def _out_of_scope(name):
    def fn(*args, **kwargs):
        raise NotImplementedError(f"render_utils_cuda.{name} is not used by the Voxurf models and is not built")
    fn.__name__ = name
    return fn


sample_ndc_pts_on_rays = _out_of_scope("sample_ndc_pts_on_rays")
sample_bg_pts_on_rays = _out_of_scope("sample_bg_pts_on_rays")
raw2alpha = _out_of_scope("raw2alpha")
raw2alpha_backward = _out_of_scope("raw2alpha_backward")
raw2alpha_nonuni = _out_of_scope("raw2alpha_nonuni")
raw2alpha_nonuni_backward = _out_of_scope("raw2alpha_nonuni_backward")
