"""Host-side mirror of the Voxurf fine model (lib/voxurf_fine.py:25-802).

``Voxurf`` keeps the reference's constructor arguments, parameter names
(``sdf.grid``, ``k0.grid``, ``rgbnet.*``, ``k_rgbnet.*``, ``density``),
buffers and the ``forward(rays_o, rays_d, viewdirs, global_step=None,
**render_kwargs) -> dict`` contract (keys of voxurf_fine.py:781-801), so it
drops into run.py's training and render loops.  The forward is computed by
the fused sm_103a kernels of libvoxurf_gb300.so:

  _FineGeometry (autograd.Function): Gaussian smoothing of the SDF grid,
      ray march (sampling, mask, SDF + FD normals, NeuS alpha, both
      fast_color_thres compactions, transmittance scan), compaction of the
      shaded samples, hierarchical features + k0 + positional encodings.
      backward: recomputes interpolated values, reverse transmittance scan,
      NeuS alpha adjoint, trilinear scatter into the smoothed-grid gradient
      and k0, then the smoothing adjoint.
  rgbnet / k_rgbnet: nn.Linear stacks run by the library's own MLP
      engines (mlp.apply_mlp): tcgen05 BF16 kernels in the mixed-precision
      mode, CUDA-core FP32 kernels in the plain mode.
  _FineComposite (autograd.Function): per-ray compositing and its backward.

precision='fp32' is the plain FP32 path; precision='bf16' samples k0 from a
BF16 shadow copy and runs both MLPs in BF16 with FP32 accumulation, while
the SDF grid, alpha, normals and the transmittance stay FP32 (an FP64
carry for rays of more than 512 samples).
"""
from __future__ import annotations

import ctypes
import math
from copy import deepcopy

import numpy as np
import torch
import torch.nn as nn
import torch.nn.functional as F

from . import _abi, _native
from . import grid as grid_mod
from ._torch import ptr, stream_ptr
from .mlp import apply_mlp, row_stride


def gaussian_taps(ksize: int, sigma: float) -> np.ndarray:
    """1-D factor of Voxurf._gaussian_3dconv (voxurf_fine.py:246-258):
    exp(-(x^2+y^2+z^2)/(2 s^2)) / sum == g(x) g(y) g(z) with g normalised."""
    x = np.arange(-(ksize // 2), ksize // 2 + 1, 1, dtype=np.float64)
    g = np.exp(-(x ** 2) / (2 * sigma ** 2))
    return (g / g.sum()).astype(np.float32)


def smooth_grid(src: torch.Tensor, taps: np.ndarray) -> torch.Tensor:
    """[X,Y,Z]-shaped smoothing through vx_smooth3d (returns a new tensor)."""
    X, Y, Z = src.shape[-3:]
    out = torch.empty((X, Y, Z), dtype=torch.float32, device=src.device)
    th = np.ascontiguousarray(taps, np.float32)
    _abi.call("vx_smooth3d", ptr(src), ptr(out), None, None, X, Y, Z, th.ctypes.data, len(th), stream_ptr())
    return out


def smooth_grid_adjoint(grad_out: torch.Tensor, taps: np.ndarray, out: torch.Tensor | None = None,
                        accumulate: bool = False) -> torch.Tensor:
    X, Y, Z = grad_out.shape[-3:]
    if out is None:
        out = torch.empty((X, Y, Z), dtype=torch.float32, device=grad_out.device)
    th = np.ascontiguousarray(taps, np.float32)
    _abi.call("vx_smooth3d_adjoint", ptr(grad_out), ptr(out), None, None, X, Y, Z, th.ctypes.data, len(th),
              int(accumulate), stream_ptr())
    return out


@torch.no_grad()
def extract_fields(sdf_grid: torch.Tensor, xyz_min, xyz_max, bound_min, bound_max, resolution: int,
                   sign: float = -1.0) -> torch.Tensor:
    """extract_fields (lib/dvgo_ori.py:679-693) with query_func =
    grid_sampler(pts, sign * sdf_grid): the [R, R, R] field over the lattice
    linspace(bound_min, bound_max, R)^3 in one launch (vx_sdf_field), left
    on the device."""
    X, Y, Z = sdf_grid.shape[-3:]
    src = sdf_grid.reshape(X, Y, Z).float().contiguous()
    geom = grid_mod.grid_geom((X, Y, Z), grid_mod.host_values(xyz_min), grid_mod.host_values(xyz_max))
    R = int(resolution)
    out = torch.empty((R, R, R), dtype=torch.float32, device=src.device)
    bmin = np.ascontiguousarray([float(v) for v in bound_min], np.float32)
    bmax = np.ascontiguousarray([float(v) for v in bound_max], np.float32)
    _abi.call("vx_sdf_field", ptr(src), ctypes.byref(geom), bmin.ctypes.data, bmax.ctypes.data, R, float(sign),
              ptr(out), stream_ptr(src.device))
    return out


def marching_cubes(u: np.ndarray, threshold: float, bound_min, bound_max, resolution: int):
    """extract_geometry (lib/dvgo_ori.py:695-703): marching cubes of the host
    copy of the field (PyMCubes, as the reference), vertices mapped back to
    [bound_min, bound_max]."""
    try:
        import mcubes
    except ImportError as e:  # the field itself comes from extract_fields
        raise RuntimeError("marching cubes needs PyMCubes (mcubes), which is not installed; "
                           "extract_fields returns the [R,R,R] field for any host-side mesher") from e
    vertices, triangles = mcubes.marching_cubes(u, threshold)
    b_max = np.asarray([float(v) for v in bound_max], np.float64)
    b_min = np.asarray([float(v) for v in bound_min], np.float64)
    vertices = vertices / (resolution - 1.0) * (b_max - b_min)[None, :] + b_min[None, :]
    return vertices, triangles


@torch.no_grad()
def get_training_rays_in_maskcache_sampling(rgb_tr_ori, train_poses, HW, Ks, ndc, inverse_y, flip_x, flip_y, model,
                                            render_kwargs, rgbnet_sup_reduce=1):
    """voxurf_fine.py:1127-1164: the training rays of every view that hit
    the mask cache (model.hit_coarse_geo), with their colours, packed in view
    order.  Rays per view come from vx_camera_rays (pinhole, pixel centres
    +0.5); returns (rgb_tr, rays_o_tr, rays_d_tr, viewdirs_tr, imsz)."""
    if ndc or flip_x or flip_y:
        raise NotImplementedError("ndc / flipped cameras are not used by the Voxurf configs")
    dev = model.sdf.grid.device
    out = [[], [], [], []]
    imsz = []
    for c2w, img, (H, W), K in zip(train_poses, rgb_tr_ori, HW, Ks):
        H, W = int(H), int(W)
        K = np.asarray(K.cpu() if torch.is_tensor(K) else K, np.float32)
        o = torch.empty((H * W, 3), dtype=torch.float32, device=dev)
        d = torch.empty_like(o)
        v = torch.empty_like(o)
        m = (ctypes.c_float * 12)(*np.asarray(c2w.cpu() if torch.is_tensor(c2w) else c2w, np.float32)[:3, :4].reshape(-1))
        _abi.call("vx_camera_rays", m, float(K[0, 0]), float(K[1, 1]), float(K[0, 2]), float(K[1, 2]), H, W,
                  int(inverse_y), ptr(o), ptr(d), ptr(v), stream_ptr(dev))
        hit = model.hit_coarse_geo(o, d, **render_kwargs)
        out[0].append(img.reshape(H * W, -1).to(dev)[hit])
        out[1].append(o[hit])
        out[2].append(d[hit])
        out[3].append(v[hit])
        imsz.append(int(hit.sum()))
    rgb_tr, rays_o_tr, rays_d_tr, viewdirs_tr = (torch.cat(x, 0) for x in out)
    return rgb_tr, rays_o_tr, rays_d_tr, viewdirs_tr, imsz


@torch.no_grad()
def query_mask(mask_cache, pts: torch.Tensor) -> torch.Tensor:
    """Point query of a MaskGrid / MaskCache on the GPU (a device copy of a
    module that still sits on the host, as during model construction)."""
    buf = mask_cache.mask if isinstance(mask_cache, grid_mod.MaskGrid) else mask_cache.density
    mc = mask_cache if buf.is_cuda else deepcopy(mask_cache).to("cuda")
    dev = (mc.mask if isinstance(mc, grid_mod.MaskGrid) else mc.density).device
    return mc(pts.to(dev))


def max_steps_bound(xyz_min, xyz_max, stepdist: float) -> int:
    """Upper bound of N_steps for any ray: the bbox diagonal in steps, +2."""
    diag = math.sqrt(sum((float(b) - float(a)) ** 2 for a, b in zip(xyz_min, xyz_max)))
    return int(math.ceil(diag / float(stepdist))) + 2


class FineFrame:
    """Per-forward device state shared by the two autograd Functions."""
    pass


def _feature_cfg(model) -> _abi.FineFeatureCfg:
    c = _abi.FineFeatureCfg()
    ks = model.hier_disps
    c.K = len(ks)
    for i, d in enumerate(ks):
        c.disp[i] = float(d)
    c.posbase_pe = model.posbase_pe
    c.viewbase_pe = model.viewbase_pe
    c.k_posbase_pe = model.k_posbase_pe
    c.k_viewbase_pe = model.k_viewbase_pe
    c.center_sdf = int(bool(model.center_sdf))
    c.use_rgbnet_k0 = int(bool(model.use_rgbnet_k0))
    c.k_center_sdf = int(bool(model.k_center_sdf))
    c.k0_channels = model.k0_dim
    return c


class _FineGeometry(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sdf_grid, k0_grid, fr: FineFrame):
        dev = sdf_grid.device
        st = stream_ptr()
        X, Y, Z = fr.geom.X, fr.geom.Y, fr.geom.Z
        fr.sdf_s = smooth_grid(sdf_grid, fr.taps) if fr.taps is not None else sdf_grid.reshape(X, Y, Z)
        N = fr.n_rays
        ms = fr.max_steps
        rec = torch.empty((N * ms, 4), dtype=torch.float32, device=dev)
        dw_slot = torch.empty(N * ms, dtype=torch.float32, device=dev)
        n1 = torch.empty(N, dtype=torch.int32, device=dev)
        n2 = torch.empty(N, dtype=torch.int32, device=dev)
        alphainv_last = torch.empty(N, dtype=torch.float32, device=dev)
        a = _abi.FineMarchArgs()
        a.rays_o, a.rays_d, a.viewdirs = ptr(fr.rays_o), ptr(fr.rays_d), ptr(fr.viewdirs)
        a.n_rays, a.near, a.stepdist = N, fr.near, fr.stepdist
        a.grid = fr.geom
        a.sdf_smooth = ptr(fr.sdf_s)
        a.voxel_size = fr.voxel_size
        if fr.mask_cache is not None:
            fr.mask_cache.fill_march(a)
        a.inv_s, a.dist, a.fast_color_thres = fr.inv_s, fr.dist, fr.thres
        a.max_steps = ms
        a.rec, a.dw_slot, a.n1, a.n2, a.alphainv_last = ptr(rec), ptr(dw_slot), ptr(n1), ptr(n2), ptr(alphainv_last)
        _abi.call_struct("vx_fine_march", a, st)

        s2_off = torch.empty(N + 1, dtype=torch.int64, device=dev)
        nb = _native.load().vx_scan_scratch_bytes(N)
        scratch = torch.empty(max(nb, 16), dtype=torch.uint8, device=dev)
        _native.call("vx_exclusive_scan_i32", ptr(n2), N, ptr(s2_off), ptr(scratch), nb, st)
        S2 = int(s2_off[-1].item())  # host needs the row count to size the GEMMs
        fr.S2 = S2
        ray2 = torch.empty(S2, dtype=torch.int32, device=dev)
        step2 = torch.empty(S2, dtype=torch.int32, device=dev)
        slot2 = torch.empty(S2, dtype=torch.int32, device=dev)
        w2 = torch.empty(S2, dtype=torch.float32, device=dev)
        alpha2 = torch.empty(S2, dtype=torch.float32, device=dev)
        pts2 = torch.empty((S2, 3), dtype=torch.float32, device=dev)
        c = _abi.FineCompactArgs()
        c.rays_o, c.rays_d, c.n_rays, c.near, c.stepdist = ptr(fr.rays_o), ptr(fr.rays_d), N, fr.near, fr.stepdist
        for i in range(3):
            c.xyz_min[i] = fr.geom.xyz_min[i]
            c.xyz_max[i] = fr.geom.xyz_max[i]
        c.max_steps, c.rec, c.n1, c.s2_off = ms, ptr(rec), ptr(n1), ptr(s2_off)
        c.ray2, c.step2, c.slot2, c.w2, c.alpha2, c.pts2 = ptr(ray2), ptr(step2), ptr(slot2), ptr(w2), ptr(alpha2), \
            ptr(pts2)
        _abi.call_struct("vx_fine_compact", c, st)

        xdt = torch.bfloat16 if fr.bf16 else torch.float32
        X1 = torch.empty((S2, fr.ld1), dtype=xdt, device=dev)
        X2 = torch.empty((S2, fr.ld2), dtype=xdt, device=dev)
        normal2 = torch.empty((S2, 3), dtype=torch.float32, device=dev)
        f = _abi.FineFeaturesArgs()
        f.n_rows, f.ray2, f.pts2, f.viewdirs = S2, ptr(ray2), ptr(pts2), ptr(fr.viewdirs)
        f.grid, f.sdf_smooth, f.voxel_size = fr.geom, ptr(fr.sdf_s), fr.voxel_size
        if fr.k0_bf16 is not None:
            f.k0_bf16 = ptr(fr.k0_bf16)
        else:
            f.k0_f32 = ptr(k0_grid)
        f.cfg = fr.cfg
        f.ld1, f.ld2 = fr.ld1, fr.ld2
        f.X1, f.X2, f.out_bf16, f.normal_out = ptr(X1), ptr(X2), int(fr.bf16), ptr(normal2)
        _abi.call_struct("vx_fine_features", f, st)

        fr.rec, fr.dw_slot, fr.n1, fr.alphainv_last = rec, dw_slot, n1, alphainv_last
        fr.s2_off, fr.ray2, fr.step2, fr.slot2, fr.w2, fr.alpha2, fr.pts2 = s2_off, ray2, step2, slot2, w2, alpha2, pts2
        ctx.fr = fr
        ctx.k0_like = k0_grid
        ctx.sdf_shape = sdf_grid.shape
        ctx.mark_non_differentiable(normal2, alpha2)
        return X1, X2, w2, alphainv_last, normal2, alpha2

    @staticmethod
    def backward(ctx, dX1, dX2, dw2, dlast, _dn, _da):
        fr = ctx.fr
        dev = dX1.device if dX1 is not None else fr.w2.device
        st = stream_ptr()
        X, Y, Z = fr.geom.X, fr.geom.Y, fr.geom.Z
        xdt = torch.bfloat16 if fr.bf16 else torch.float32
        S2, N = fr.S2, fr.n_rays
        dX1 = torch.zeros((S2, fr.ld1), dtype=xdt, device=dev) if dX1 is None else dX1.contiguous()
        dX2 = torch.zeros((S2, fr.ld2), dtype=xdt, device=dev) if dX2 is None else dX2.contiguous()
        dw2 = torch.zeros(S2, dtype=torch.float32, device=dev) if dw2 is None else dw2.contiguous().float()
        dlast = torch.zeros(N, dtype=torch.float32, device=dev) if dlast is None else dlast.contiguous().float()
        d_sdf_s = torch.zeros((X, Y, Z), dtype=torch.float32, device=dev)
        d_k0 = torch.zeros_like(ctx.k0_like)  # channels_last_3d: [X,Y,Z,12] storage
        b = _abi.FineBackwardArgs()
        b.n_rays, b.n_rows = N, S2
        b.rays_o, b.rays_d, b.viewdirs = ptr(fr.rays_o), ptr(fr.rays_d), ptr(fr.viewdirs)
        b.near, b.stepdist, b.grid = fr.near, fr.stepdist, fr.geom
        b.sdf_smooth, b.voxel_size, b.inv_s, b.dist = ptr(fr.sdf_s), fr.voxel_size, fr.inv_s, fr.dist
        b.max_steps, b.rec, b.dw_slot, b.n1 = fr.max_steps, ptr(fr.rec), ptr(fr.dw_slot), ptr(fr.n1)
        b.alphainv_last, b.d_last = ptr(fr.alphainv_last), ptr(dlast)
        b.pts2, b.slot2, b.dw2 = ptr(fr.pts2), ptr(fr.slot2), ptr(dw2)
        b.cfg, b.ld1, b.ld2 = fr.cfg, fr.ld1, fr.ld2
        b.dX1, b.dX2, b.in_bf16 = ptr(dX1), ptr(dX2), int(fr.bf16)
        b.d_sdf_smooth, b.d_k0 = ptr(d_sdf_s), ptr(d_k0)
        _abi.call_struct("vx_fine_backward", b, st)
        if fr.taps is not None:
            d_sdf = smooth_grid_adjoint(d_sdf_s, fr.taps)
        else:
            d_sdf = d_sdf_s
        return d_sdf.reshape(ctx.sdf_shape), d_k0, None


class _FineComposite(torch.autograd.Function):
    @staticmethod
    def forward(ctx, w2, alphainv_last, logit, klogit, fr: FineFrame, bg: float):
        N = fr.n_rays
        dev = w2.device
        logit = logit.float().contiguous()
        klogit = None if klogit is None else klogit.float().contiguous()
        rgb0 = torch.empty((N, 3), dtype=torch.float32, device=dev)
        rgbk = torch.empty((N, 3), dtype=torch.float32, device=dev)
        rgbk_raw = torch.empty((N, 3), dtype=torch.float32, device=dev)
        a = _abi.FineCompositeArgs()
        a.n_rays, a.s2_off, a.w2 = N, ptr(fr.s2_off), ptr(w2)
        a.logit, a.klogit, a.alphainv_last, a.bg = ptr(logit), ptr(klogit), ptr(alphainv_last), float(bg)
        a.rgb0, a.rgbk, a.rgbk_raw = ptr(rgb0), ptr(rgbk), ptr(rgbk_raw)
        a.has_k = int(klogit is not None)
        if fr.render_extras:
            fr.normal_marched = torch.empty((N, 3), dtype=torch.float32, device=dev)
            fr.depth = torch.empty(N, dtype=torch.float32, device=dev)
            a.normal2, a.normal_out = ptr(fr.normal2), ptr(fr.normal_marched)
            a.step2, a.depth_out, a.dist = ptr(fr.step2), ptr(fr.depth), fr.dist
        _abi.call_struct("vx_fine_composite", a, stream_ptr())
        ctx.save_for_backward(w2, logit, klogit, rgbk_raw)
        ctx.fr, ctx.bg, ctx.has_k = fr, float(bg), klogit is not None
        return rgbk, rgb0

    @staticmethod
    def backward(ctx, g_rgbk, g_rgb0):
        w2, logit, klogit, rgbk_raw = ctx.saved_tensors
        fr = ctx.fr
        S2, N = fr.S2, fr.n_rays
        dev = w2.device
        d_logit = torch.empty((S2, 3), dtype=torch.float32, device=dev)
        d_klogit = torch.empty((S2, 3), dtype=torch.float32, device=dev) if ctx.has_k else None
        d_w2 = torch.empty(S2, dtype=torch.float32, device=dev)
        d_last = torch.empty(N, dtype=torch.float32, device=dev)
        a = _abi.FineCompositeBwdArgs()
        a.n_rays, a.s2_off, a.w2, a.logit = N, ptr(fr.s2_off), ptr(w2), ptr(logit)
        a.klogit, a.rgbk_raw = ptr(klogit), ptr(rgbk_raw)
        g_rgb0 = None if g_rgb0 is None else g_rgb0.contiguous()
        g_rgbk = None if (g_rgbk is None or not ctx.has_k) else g_rgbk.contiguous()
        a.g_rgb0, a.g_rgbk, a.bg = ptr(g_rgb0), ptr(g_rgbk), ctx.bg
        a.d_logit, a.d_klogit, a.d_w2, a.d_last = ptr(d_logit), ptr(d_klogit), ptr(d_w2), ptr(d_last)
        a.has_k = int(ctx.has_k)
        _abi.call_struct("vx_fine_composite_backward", a, stream_ptr())
        return d_w2, d_last, d_logit, d_klogit, None, None


class _SmoothGradTV(torch.autograd.Function):
    """smooth_grad_tv term of Voxurf.density_total_variation
    (voxurf_fine.py:417-420): mean over the non-empty voxels and the 3
    channels of (tv_smooth_conv(G).detach() - G)^2, G the central-difference
    gradient grid of the raw SDF (neus_sdf_gradient, 'interpolate')."""

    @staticmethod
    def forward(ctx, sdf_grid, mask_u8, voxel_size: float, n_voxels: int):
        X, Y, Z = sdf_grid.shape[-3:]
        dev = sdf_grid.device
        st = stream_ptr()
        G = torch.empty((X, Y, Z, 4), dtype=torch.float32, device=dev)
        _abi.call("vx_sdf_gradient_grid", ptr(sdf_grid), ptr(G), X, Y, Z, float(voxel_size), 1, st)
        count = 3 * n_voxels
        partial = torch.empty(_abi_scratch_bytes(X, Y, Z) // 8, dtype=torch.float64, device=dev)
        dG = torch.empty_like(G)
        scale = 2.0 / max(count, 1)
        _abi.call("vx_smooth_grad_tv", ptr(G), ptr(mask_u8), X, Y, Z, float(scale), ptr(dG), ptr(partial), st)
        ctx.dG, ctx.shape, ctx.voxel_size = dG, sdf_grid.shape, float(voxel_size)
        return (partial.sum() / max(count, 1)).float()

    @staticmethod
    def backward(ctx, g):
        X, Y, Z = ctx.shape[-3:]
        d_sdf = torch.zeros(ctx.shape, dtype=torch.float32, device=g.device)
        dG = ctx.dG * g.float()
        _abi.call("vx_sdf_gradient_grid_adjoint", ptr(dG), ptr(d_sdf), X, Y, Z, ctx.voxel_size, 1, 0, stream_ptr())
        return d_sdf, None, None, None


def tv_mask(owner, mask, grid):
    """(uint8 [X, Y, Z] copy of a bool voxel mask on the grid's device, or
    None; its voxel count), cached on ``owner`` while the mask tensor is
    unchanged (one host read of the count per new mask)."""
    X, Y, Z = (int(v) for v in grid.shape[-3:])
    if mask is None:
        return None, X * Y * Z
    key = (mask.data_ptr(), mask.numel(), mask._version, str(grid.device))
    cache = owner.__dict__.setdefault("_tv_mask_cache", {})
    hit = cache.get(key)
    if hit is None:
        cache.clear()
        u8 = grid_mod.voxel_mask_u8(mask, (X, Y, Z)).to(grid.device)
        hit = cache[key] = (u8, int(u8.sum().item()))
    return hit


def _abi_scratch_bytes(X, Y, Z) -> int:
    _abi._declare()
    return int(_native.load().vx_smooth_grad_tv_scratch_bytes(X, Y, Z))


def _mlp(d_in: int, width: int, depth: int, use_layer_norm: bool = False) -> nn.Sequential:
    """rgbnet / k_rgbnet layout of voxurf_fine.py:131-148, 167-184."""
    if use_layer_norm:
        raise NotImplementedError("use_layer_norm is not used by the Voxurf configs and is not built")
    return nn.Sequential(
        nn.Linear(d_in, width), nn.ReLU(inplace=True),
        *[nn.Sequential(nn.Linear(width, width), nn.ReLU(inplace=True)) for _ in range(depth - 2)],
        nn.Linear(width, 3),
    )


class Voxurf(nn.Module):
    """lib/voxurf_fine.py:25-203 (constructor) and :620-802 (forward)."""

    def __init__(self, xyz_min, xyz_max, num_voxels=0, num_voxels_base=0, alpha_init=None, nearest=False,
                 mask_cache_path=None, mask_cache_thres=1e-3, fast_color_thres=0, rgbnet_dim=0, rgbnet_direct=False,
                 rgbnet_full_implicit=False, rgbnet_depth=3, rgbnet_width=128, posbase_pe=5, viewbase_pe=4,
                 center_sdf=False, grad_feat=(1.0,), sdf_feat=(), use_layer_norm=False, grad_mode="interpolate",
                 s_ratio=2000, s_start=0.2, s_learn=False, step_start=0, smooth_sdf=False, smooth_ksize=0,
                 smooth_sigma=1, k_rgbnet_depth=3, k_res=False, k_posbase_pe=5, k_viewbase_pe=4,
                 k_center_sdf=False, k_grad_feat=(1.0,), k_sdf_feat=(), smooth_scale=True, use_grad_norm=True,
                 use_rgb_k=True, k_detach_1=True, k_detach_2=True, use_rgbnet_k0=False, precision="fp32",
                 mask_grid=None, **kwargs):
        super().__init__()
        self.register_buffer("xyz_min", torch.as_tensor(np.asarray(xyz_min, np.float32)).clone())
        self.register_buffer("xyz_max", torch.as_tensor(np.asarray(xyz_max, np.float32)).clone())
        self.fast_color_thres = fast_color_thres
        self.nearest = nearest
        if nearest:
            raise NotImplementedError("nearest interpolation is not used by the Voxurf configs and is not built")
        self.smooth_scale = smooth_scale
        self.s_ratio, self.s_start, self.s_learn, self.step_start = s_ratio, s_start, s_learn, step_start
        self.s_val = torch.ones(1) * s_start
        self.sdf_init_mode = "ball_init"
        self.num_voxels_base = num_voxels_base
        self.voxel_size_base = ((self.xyz_max - self.xyz_min).prod() / self.num_voxels_base).pow(1 / 3)
        self.alpha_init = alpha_init
        self.act_shift = np.log(1 / (1 - alpha_init) - 1)
        self._set_grid_resolution(num_voxels)
        self.density = nn.Parameter(torch.zeros([1, 1, *self.world_size]))
        self.sdf = grid_mod.create_grid("DenseGrid", channels=1, world_size=self.world_size, xyz_min=self.xyz_min,
                                        xyz_max=self.xyz_max)
        ws = [int(s) for s in self.world_size]
        x, y, z = np.mgrid[-1.0:1.0:ws[0] * 1j, -1.0:1.0:ws[1] * 1j, -1.0:1.0:ws[2] * 1j]
        self.sdf.grid.data = torch.from_numpy((x ** 2 + y ** 2 + z ** 2) ** 0.5 - 1).float()[None, None, ...]
        self.init_smooth_conv(smooth_ksize, smooth_sigma)
        self.rgbnet_kwargs = {"rgbnet_dim": rgbnet_dim, "rgbnet_direct": rgbnet_direct,
                              "rgbnet_full_implicit": rgbnet_full_implicit, "rgbnet_depth": rgbnet_depth,
                              "rgbnet_width": rgbnet_width, "posbase_pe": posbase_pe, "viewbase_pe": viewbase_pe}
        if rgbnet_dim <= 0:
            raise NotImplementedError("the fine Voxurf model needs a feature grid (rgbnet_dim > 0)")
        self.k0_dim = rgbnet_dim
        self.k0 = grid_mod.create_grid("DenseGrid", channels=self.k0_dim, world_size=self.world_size,
                                       xyz_min=self.xyz_min, xyz_max=self.xyz_max)
        self.rgbnet_direct = rgbnet_direct
        self.posbase_pe, self.viewbase_pe = posbase_pe, viewbase_pe
        self.register_buffer("posfreq", torch.FloatTensor([(2 ** i) for i in range(posbase_pe)]))
        self.register_buffer("viewfreq", torch.FloatTensor([(2 ** i) for i in range(viewbase_pe)]))
        dim0 = (3 + 3 * posbase_pe * 2) + (3 + 3 * viewbase_pe * 2)
        self.use_grad_norm, self.center_sdf = use_grad_norm, center_sdf
        self.grad_feat, self.sdf_feat = tuple(grad_feat), tuple(sdf_feat)
        self.use_rgb_k, self.k_detach_1, self.k_detach_2 = use_rgb_k, k_detach_1, k_detach_2
        self.use_rgbnet_k0, self.use_layer_norm = use_rgbnet_k0, use_layer_norm
        dim0 += len(self.grad_feat) * 3 + len(self.sdf_feat) * 6
        if use_rgbnet_k0:
            dim0 += self.k0_dim
        if center_sdf:
            dim0 += 1
        self.rgbnet = _mlp(dim0, rgbnet_width, rgbnet_depth, use_layer_norm)
        nn.init.constant_(self.rgbnet[-1].bias, 0)
        self.k_res, self.k_center_sdf = k_res, k_center_sdf
        self.k_grad_feat, self.k_sdf_feat = tuple(k_grad_feat), tuple(k_sdf_feat)
        self.k_posbase_pe, self.k_viewbase_pe = k_posbase_pe, k_viewbase_pe
        self.register_buffer("k_posfreq", torch.FloatTensor([(2 ** i) for i in range(k_posbase_pe)]))
        self.register_buffer("k_viewfreq", torch.FloatTensor([(2 ** i) for i in range(k_viewbase_pe)]))
        k_dim0 = (3 + 3 * k_posbase_pe * 2) + (3 + 3 * k_viewbase_pe * 2) + self.k0_dim
        if k_res:
            k_dim0 += 3
        if k_center_sdf:
            k_dim0 += 1
        k_dim0 += len(self.k_grad_feat) * 3 + len(self.k_sdf_feat) * 6
        self.k_rgbnet = _mlp(k_dim0, rgbnet_width, k_rgbnet_depth, use_layer_norm)
        # voxurf_fine.py:185 zeroes rgbnet's last bias a second time (not k_rgbnet's)
        nn.init.constant_(self.rgbnet[-1].bias, 0)
        self.dim0, self.k_dim0 = dim0, k_dim0
        self._grad_col = self.k0_dim + (3 + 6 * k_posbase_pe) + (3 + 6 * k_viewbase_pe)
        # hierarchical displacement set (voxurf_fine.py:680-688)
        all_grad = sorted(set(self.grad_feat + self.k_grad_feat))
        all_sdf = sorted(set(self.sdf_feat + self.k_sdf_feat))
        if all_grad != all_sdf and len(self.sdf_feat) > 0:
            raise ValueError("grad_feat and sdf_feat must name the same displacements (voxurf_fine.py:683)")
        self.hier_disps = all_grad
        if len(self.grad_feat) * 3 + len(self.sdf_feat) * 6 != 9 * len(all_grad) or len(all_grad) > 4:
            # the forward feeds 9 values per displacement of the union set
            # (voxurf_fine.py:680-716); rgbnet's input width must agree
            raise ValueError("grad_feat/sdf_feat must both list every displacement (including 1.0), at most 4")
        if tuple(self.k_grad_feat) != (1.0,) or len(self.k_sdf_feat) != 0:
            raise ValueError("k_grad_feat must be (1.0,) and k_sdf_feat empty (voxurf_fine.py:731-732)")
        if not use_grad_norm:
            raise NotImplementedError("use_grad_norm=False is not used by the Voxurf configs")
        self.mask_cache_path, self.mask_cache_thres = mask_cache_path, mask_cache_thres
        if mask_cache_path:
            # the coarse checkpoint's density (voxurf_fine.py:189-195)
            self.mask_cache = grid_mod.MaskCache(path=mask_cache_path, mask_cache_thres=mask_cache_thres)
        else:
            self.mask_cache = mask_grid
        self.nonempty_mask = None
        if self.mask_cache is not None:
            self._set_nonempty_mask()
        self.grad_mode = grad_mode
        if precision not in ("fp32", "bf16"):
            raise ValueError(precision)
        self.precision = precision
        self._k0_shadow = None

    # -- reference helpers --------------------------------------------------
    def _set_grid_resolution(self, num_voxels):
        self.num_voxels = num_voxels
        self.voxel_size = ((self.xyz_max - self.xyz_min).prod() / num_voxels).pow(1 / 3)
        self.world_size = ((self.xyz_max - self.xyz_min) / self.voxel_size).long()
        self.voxel_size_ratio = self.voxel_size / self.voxel_size_base

    def init_smooth_conv(self, ksize=3, sigma=1):
        self.smooth_sdf = ksize > 0
        self.smooth_ksize, self.smooth_sigma = ksize, sigma
        self.smooth_taps = gaussian_taps(ksize, sigma) if self.smooth_sdf else None

    def get_MaskCache_kwargs(self):
        return {"xyz_min": self.xyz_min.cpu().numpy(), "xyz_max": self.xyz_max.cpu().numpy(),
                "act_shift": self.act_shift, "voxel_size_ratio": self.voxel_size_ratio, "nearest": self.nearest}

    @torch.no_grad()
    def hit_coarse_geo(self, rays_o, rays_d, near, far, stepsize, **render_kwargs):
        """voxurf_fine.py:579-591: whether each ray has an in-bbox sample
        (sample_pts_on_rays, far = 1e9) inside the mask cache; one warp per
        ray stops at the first such sample (vx_hit_coarse_geo)."""
        if self.mask_cache is None:
            raise RuntimeError("hit_coarse_geo needs a mask cache")
        shape = rays_o.shape[:-1]
        dev = self.sdf.grid.device
        o = rays_o.reshape(-1, 3).to(dev, torch.float32).contiguous()
        d = rays_d.reshape(-1, 3).to(dev, torch.float32).contiguous()
        a = _abi.FineMarchArgs()
        a.rays_o, a.rays_d, a.n_rays, a.near = ptr(o), ptr(d), o.shape[0], float(near)
        a.stepdist = float(stepsize * self.voxel_size.float())
        a.grid = grid_mod.grid_geom(self.sdf.grid.shape[2:], grid_mod.host_values(self.xyz_min),
                                    grid_mod.host_values(self.xyz_max))
        self.mask_cache.fill_march(a)
        hit = torch.empty(o.shape[0], dtype=torch.uint8, device=dev)
        _abi.call("vx_hit_coarse_geo", ctypes.byref(a), ptr(hit), stream_ptr(dev))
        return hit.bool().reshape(shape)

    def get_kwargs(self):
        return {"xyz_min": self.xyz_min.cpu().numpy(), "xyz_max": self.xyz_max.cpu().numpy(),
                "num_voxels": self.num_voxels, "num_voxels_base": self.num_voxels_base,
                "alpha_init": self.alpha_init, "nearest": self.nearest, "mask_cache_path": self.mask_cache_path,
                "mask_cache_thres": self.mask_cache_thres, "fast_color_thres": self.fast_color_thres,
                "grad_feat": self.grad_feat, "sdf_feat": self.sdf_feat, "k_grad_feat": self.k_grad_feat,
                "k_sdf_feat": self.k_sdf_feat, **self.rgbnet_kwargs}

    @torch.no_grad()
    def _set_nonempty_mask(self):
        # grid points inside known non-empty space (voxurf_fine.py:353-367)
        ws = self.density.shape[2:]
        pts = torch.stack(torch.meshgrid(
            torch.linspace(float(self.xyz_min[0]), float(self.xyz_max[0]), ws[0]),
            torch.linspace(float(self.xyz_min[1]), float(self.xyz_max[1]), ws[1]),
            torch.linspace(float(self.xyz_min[2]), float(self.xyz_max[2]), ws[2]), indexing="ij"), -1)
        nonempty = query_mask(self.mask_cache, pts)[None, None].contiguous()
        self.nonempty_mask = nonempty
        self.density.data[~nonempty.to(self.density.device)] = -100
        self.sdf.grid.data[~nonempty.to(self.sdf.grid.device)] = 1

    def sdf_total_variation_add_grad(self, weight, dense_mode):
        w = weight * self.world_size.max() / 128
        self.sdf.total_variation_add_grad(w, w, w, dense_mode)

    # -- mesh extraction (voxurf_fine.py:894-910) ----------------------------
    @torch.no_grad()
    def mesh_sdf_grid(self, smooth: bool = True, sigma: float = 0.5) -> torch.Tensor:
        """The grid extract_geometry queries: smooth_conv(sdf) when the model
        smooths, else the 3^3 Gaussian test kernel (init_smooth_conv_test_k3)
        when `smooth`, else the raw grid."""
        g = self.sdf.grid.detach()
        if self.smooth_sdf:
            return smooth_grid(g, self.smooth_taps)
        if smooth:
            return smooth_grid(g, gaussian_taps(3, sigma))
        return g.reshape(g.shape[-3:]).float().contiguous()

    @torch.no_grad()
    def extract_fields(self, bound_min, bound_max, resolution=128, smooth=True, sigma=0.5) -> torch.Tensor:
        """[R, R, R] field -sdf on the lattice (device tensor)."""
        if resolution is None:
            resolution = int(self.world_size[0])
        return extract_fields(self.mesh_sdf_grid(smooth, sigma), self.xyz_min, self.xyz_max, bound_min, bound_max,
                              resolution)

    def extract_geometry(self, bound_min, bound_max, resolution=128, threshold=0.0, smooth=True, sigma=0.5,
                         **kwargs):
        if resolution is None:
            resolution = int(self.world_size[0])
        u = self.extract_fields(bound_min, bound_max, resolution, smooth, sigma).cpu().numpy()
        return marching_cubes(u, threshold, bound_min, bound_max, resolution)

    def density_total_variation(self, sdf_tv=0, smooth_grad_tv=0, grad_tv=0, smooth_sdf_tv=0):
        """voxurf_fine.py:412-421: sdf_tv = total_variation(sdf.grid,
        nonempty_mask) / 2 / voxel_size (the per-axis mean form) and
        smooth_grad_tv on the raw SDF's gradient grid, both on the sm_103a
        kernels.  Without a mask cache the reference's smooth_grad_tv fails
        (nonempty_mask is None); here every voxel counts."""
        if grad_tv > 0 or smooth_sdf_tv > 0:
            raise NotImplementedError("grad_tv / smooth_sdf_tv are accepted but unused by the reference")
        tv = 0
        if sdf_tv > 0:
            tv = tv + grid_mod.total_variation(self.sdf.grid, self.nonempty_mask, mode=1,
                                               weight=float(sdf_tv / 2 / self.voxel_size.float()))
        if smooth_grad_tv > 0:
            u8, count = tv_mask(self, self.nonempty_mask, self.sdf.grid)
            tv = tv + _SmoothGradTV.apply(self.sdf.grid, u8, float(self.voxel_size), count) * smooth_grad_tv
        return tv

    def k0_total_variation(self, k0_tv=1., k0_grad_tv=0.):
        """voxurf_fine.py:423-432 (which passes the DenseGrid module itself to
        total_variation; the grid is meant): the per-axis mean form over the
        non-empty mask."""
        if k0_grad_tv > 0:
            raise NotImplementedError
        tv = 0
        if k0_tv > 0:
            tv = tv + grid_mod.total_variation(self.k0.grid, self.nonempty_mask, mode=1)
        return tv

    def k0_total_variation_add_grad(self, weight, dense_mode):
        w = weight * self.world_size.max() / 128
        self.k0.total_variation_add_grad(w, w, w, dense_mode)

    def neus_s_val(self, global_step):
        """voxurf_fine.py:466-476: returns (s_val reported, inv_s used)."""
        is_train = global_step is not None
        if is_train:
            if not self.s_learn:
                s_val = 1.0 / (global_step + self.s_ratio / self.s_start - self.step_start) * self.s_ratio
                self.s_val = torch.ones(1) * s_val
            else:
                s_val = float(self.s_val.item())
        else:
            s_val = 0
        inv_s = float((torch.ones(1) / self.s_val.float().cpu()).item())
        return s_val, inv_s

    def refresh_k0_shadow(self):
        """BF16 copy of k0 for the mixed-precision path (kept in sync by the
        fused optimizer; call after loading or editing k0 by hand)."""
        g = self.k0.grid
        self._k0_shadow = g.detach().to(torch.bfloat16).contiguous(memory_format=torch.channels_last_3d)
        return self._k0_shadow

    # -- forward ------------------------------------------------------------
    def forward(self, rays_o, rays_d, viewdirs, global_step=None, **render_kwargs):
        N = len(rays_o)
        s_val, inv_s = self.neus_s_val(global_step)
        fr = FineFrame()
        fr.n_rays = N
        fr.rays_o = rays_o.contiguous().float()
        fr.rays_d = rays_d.contiguous().float()
        fr.viewdirs = viewdirs.contiguous().float()
        fr.near = float(render_kwargs["near"])
        vs = self.voxel_size.float()
        stepdist_t = render_kwargs["stepsize"] * vs
        fr.stepdist = float(stepdist_t)
        fr.dist = float(stepdist_t)
        fr.voxel_size = float(vs)
        fr.inv_s = inv_s
        fr.thres = float(self.fast_color_thres)
        fr.geom = grid_mod.grid_geom(self.sdf.grid.shape[2:], grid_mod.host_values(self.xyz_min), grid_mod.host_values(self.xyz_max))
        fr.max_steps = max_steps_bound(grid_mod.host_values(self.xyz_min), grid_mod.host_values(self.xyz_max), fr.stepdist)
        fr.taps = self.smooth_taps if self.smooth_sdf else None
        fr.mask_cache = self.mask_cache  # MaskGrid (bool) or MaskCache (density), or None
        fr.cfg = _feature_cfg(self)
        fr.bf16 = self.precision == "bf16"
        fr.k0_bf16 = None
        if fr.bf16:
            if self._k0_shadow is None or self._k0_shadow.shape != self.k0.grid.shape:
                self.refresh_k0_shadow()
            fr.k0_bf16 = self._k0_shadow
        fr.d1 = self.dim0
        fr.d2a = self.k_dim0 - (3 if self.k_res else 0)
        # MLP input rows, zero-padded to the stride of the MLP engine; the
        # k-branch rows keep 3 columns after the features for the rgbnet
        # logits (k_res), which the rgbnet forward writes there directly
        xdt = torch.bfloat16 if fr.bf16 else torch.float32
        fr.ld1 = row_stride(fr.d1, xdt)
        fr.ld2 = row_stride(self.k_dim0 if self.use_rgb_k else fr.d2a, xdt)
        fr.render_extras = bool(render_kwargs.get("render_depth", False) or render_kwargs.get("render_grad", False))
        X1, X2a, w2, alphainv_last, normal2, alpha2 = _FineGeometry.apply(self.sdf.grid, self.k0.grid, fr)
        fr.normal2 = normal2

        direct_k = self.use_rgb_k and (not self.k_res or self.k_detach_1)
        logit_cols = X2a[:, fr.d2a:fr.d2a + 3] if (direct_k and self.k_res) else None
        rgb_logit = self._run_mlp(self.rgbnet, X1, cols=logit_cols)
        rgb = torch.sigmoid(rgb_logit)
        k_rgb_logit = None
        if self.use_rgb_k:
            if direct_k:
                k_in = X2a          # features, then (k_res) the detached logits written by the rgbnet forward
            else:
                k_in = torch.cat([X2a[:, :fr.d2a], rgb_logit.to(X2a.dtype)], -1)
            k_out = self._run_mlp(self.k_rgbnet, k_in)
            k_rgb_logit = (rgb_logit.detach() if self.k_detach_2 else rgb_logit) + k_out
        bg = render_kwargs["bg"]
        rgbk, rgb0 = _FineComposite.apply(w2, alphainv_last, rgb_logit, k_rgb_logit, fr, float(bg))
        normal_marched = depth = None
        disp = 0
        if fr.render_extras:
            if render_kwargs.get("render_grad", False):
                normal_marched = fr.normal_marched
            if render_kwargs.get("render_depth", False):
                depth = fr.depth
                disp = 1 / depth
        ret = {
            "alphainv_cum": alphainv_last,
            "weights": w2,
            "rgb_marched": rgbk if self.use_rgb_k else rgb0,
            "normal_marched": normal_marched,
            "raw_alpha": alpha2,
            "raw_rgb": rgb,
            "depth": depth,
            "disp": disp,
            "mask": None,          # per-sample masks are never materialised
            "mask_outbbox": None,
            # differentiable FD gradient (xyz) of the shaded samples: the
            # k_rgbnet input columns (voxurf_fine.py:733-739)
            "gradient": X2a[:, self._grad_col:self._grad_col + 3].float(),
            "gradient_error": None,
            "s_val": s_val,
            "ray_id": fr.ray2,
        }
        if self.use_rgb_k:
            ret["rgb_marched0"] = rgb0
        self._last_frame = fr
        return ret

    def _run_mlp(self, net: nn.Sequential, x: torch.Tensor, cols: torch.Tensor | None = None) -> torch.Tensor:
        # x is FP32 or BF16 (the compute dtype); logits come back in FP32
        return apply_mlp(net, x, cols)
