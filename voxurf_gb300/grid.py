"""Host-side mirror of lib/grid.py: DenseGrid and MaskGrid, and the
MaskCache of lib/voxurf_fine.py / lib/voxurf_coarse.py.

Same constructor arguments, attribute names (``grid``, ``xyz_min``,
``xyz_max``, ``mask``, ``xyz2ijk_scale``, ``xyz2ijk_shift``), methods and
state_dict keys/shapes as the reference, so checkpoints move between the two.
Differences by design:
  * multi-channel grids are kept in ``torch.channels_last_3d`` memory format:
    the logical shape stays [1, C, X, Y, Z] but the storage is [X, Y, Z, C],
    so one trilinear corner is one contiguous C-vector;
  * ``forward`` runs the sm_103a trilinear kernel (F.grid_sample semantics,
    align_corners=True, zero padding) with a hand-written backward;
  * ``total_variation_add_grad`` runs the TV kernel directly on either layout.
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np
import torch
import torch.nn as nn
import torch.nn.functional as F

from . import _abi, _native, render_utils_cuda
from ._torch import call, ptr, stream_ptr


def create_grid(type, **kwargs):
    if type == "DenseGrid":
        return DenseGrid(**kwargs)
    raise NotImplementedError(f"{type} is not part of this build (the Voxurf models only create DenseGrid)")


_HOST_CACHE: dict = {}


def host_values(t: torch.Tensor) -> list:
    """Host copy of a small device tensor (bbox, mask scale/shift), cached
    per tensor storage and version: a per-step .tolist() would make the host
    wait for all queued GPU work of the previous step."""
    key = (t.data_ptr(), t._version, tuple(t.shape), str(t.device))
    hit = _HOST_CACHE.get(id(t))
    if hit is not None and hit[0] == key:
        return hit[1]
    vals = t.detach().cpu().tolist()
    if id(t) not in _HOST_CACHE:
        weakref.finalize(t, _HOST_CACHE.pop, id(t), None)
    _HOST_CACHE[id(t)] = (key, vals)
    return vals


def grid_geom(world_size, xyz_min, xyz_max) -> _abi.GridGeom:
    g = _abi.GridGeom()
    g.X, g.Y, g.Z = (int(s) for s in world_size)
    for a in range(3):
        g.xyz_min[a] = float(xyz_min[a])
        g.xyz_max[a] = float(xyz_max[a])
    return g


class _GridSample(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid, xyz, geom, channel_last):
        C = grid.size(1)
        n = xyz.size(0)
        out = torch.empty((n, C), dtype=torch.float32, device=xyz.device)
        _abi.grid_sample("vx_grid_sample", ptr(grid), C, channel_last, geom, ptr(xyz), n, ptr(out), stream_ptr())
        ctx.save_for_backward(xyz)
        ctx.geom, ctx.channel_last, ctx.grid_like = geom, channel_last, grid
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (xyz,) = ctx.saved_tensors
        grid = ctx.grid_like
        g = torch.zeros_like(grid)  # preserves the channels_last_3d layout
        grad_out = grad_out.contiguous()
        _abi.grid_sample("vx_grid_sample_backward", ptr(grad_out), grid.size(1), ctx.channel_last, ctx.geom, ptr(xyz),
                         xyz.size(0), ptr(g), stream_ptr())
        return g, None, None, None


def _is_channel_last(t: torch.Tensor) -> bool:
    return t.size(1) > 1 and t.is_contiguous(memory_format=torch.channels_last_3d) and not t.is_contiguous()


class _TVLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v, mask_u8, mode: int, weight: float):
        X, Y, Z = v.shape[-3:]
        dev = v.device
        cl = _is_channel_last(v)
        if not (cl or v.is_contiguous()):
            v = v.contiguous()
        a = _abi.TvLossArgs()
        a.v, a.C, a.X, a.Y, a.Z, a.channel_last, a.mode = ptr(v), v.size(1), X, Y, Z, int(cl), int(mode)
        a.mask, a.weight = ptr(mask_u8), float(weight)
        loss = torch.empty(1, dtype=torch.float32, device=dev)
        scale = torch.empty(3, dtype=torch.float32, device=dev)
        _abi._declare()
        nb = int(_native.load().vx_tv_loss_scratch_bytes(X, Y, Z))
        sc = torch.empty(nb, dtype=torch.uint8, device=dev)
        a.loss, a.axis_scale, a.scratch, a.scratch_bytes = ptr(loss), ptr(scale), ptr(sc), nb
        _abi.call_struct("vx_tv_loss", a, stream_ptr())
        ctx.save_for_backward(v, mask_u8, scale)
        ctx.mode, ctx.cl = int(mode), cl
        return loss[0]

    @staticmethod
    def backward(ctx, g):
        v, mask_u8, scale = ctx.saved_tensors
        X, Y, Z = v.shape[-3:]
        d = torch.zeros_like(v, memory_format=torch.channels_last_3d if ctx.cl else torch.contiguous_format)
        a = _abi.TvLossArgs()
        a.v, a.C, a.X, a.Y, a.Z, a.channel_last, a.mode = ptr(v), v.size(1), X, Y, Z, int(ctx.cl), ctx.mode
        a.mask, a.axis_scale = ptr(mask_u8), ptr(scale)
        g = g.reshape(1).float().contiguous()
        _abi._declare()
        _native.check(_native.load().vx_tv_loss_backward(ctypes.byref(a), ptr(g), ptr(d), stream_ptr()),
                      "vx_tv_loss_backward")
        return d, None, None, None


def voxel_mask_u8(mask, shape) -> torch.Tensor | None:
    """[X, Y, Z] uint8 copy of a [1, 1, X, Y, Z] (or [X, Y, Z]) bool mask; None
    stays None (every voxel)."""
    if mask is None:
        return None
    m = mask.detach().reshape(mask.shape[-3:])
    if tuple(m.shape) != tuple(shape):
        raise ValueError(f"mask of shape {tuple(m.shape)} on a grid of shape {tuple(shape)}")
    return m.to(torch.uint8).contiguous()


def total_variation(v: torch.Tensor, mask=None, mode: int = 1, weight: float = 1.0) -> torch.Tensor:
    """weight x total_variation(v, mask) of the model files, on the library's
    kernels (vx_tv_loss): v [1, C, X, Y, Z] (either memory layout), mask the
    [1, 1, X, Y, Z] voxel mask (the reference's ``mask.repeat(1, C, ...)``
    is implied) or None.  mode 1: the mean of each axis's selected |diff|,
    averaged over the axes (lib/voxurf_fine.py:956-969 and the maskless
    models); mode 0: their sum over 3 x the mask's entries
    (lib/voxurf_coarse.py:702-715).  Differentiable in v."""
    if v.dim() != 5 or v.size(0) != 1:
        raise ValueError("v must be [1, C, X, Y, Z]")
    m = voxel_mask_u8(mask, v.shape[-3:]).to(v.device) if mask is not None else None
    return _TVLoss.apply(v, m, int(mode), float(weight))


class DenseGrid(nn.Module):
    """lib/grid.py:38-89."""

    def __init__(self, channels, world_size, xyz_min, xyz_max, channel_last: bool = True, **kwargs):
        super().__init__()
        self.channels = channels
        self.world_size = world_size
        self.channel_last = bool(channel_last) and channels > 1
        self.register_buffer("xyz_min", torch.as_tensor(xyz_min, dtype=torch.float32).clone())
        self.register_buffer("xyz_max", torch.as_tensor(xyz_max, dtype=torch.float32).clone())
        self.grid = nn.Parameter(self._layout(torch.zeros([1, channels, *[int(s) for s in world_size]])))

    def _layout(self, t: torch.Tensor) -> torch.Tensor:
        if self.channel_last:
            return t.contiguous(memory_format=torch.channels_last_3d)
        return t.contiguous()

    def _load_from_state_dict(self, state_dict, prefix, *args, **kwargs):
        # checkpoints store [1,C,X,Y,Z] in either layout; keep ours
        key = prefix + "grid"
        if key in state_dict:
            state_dict[key] = self._layout(state_dict[key])
        super()._load_from_state_dict(state_dict, prefix, *args, **kwargs)

    def geom(self) -> _abi.GridGeom:
        return grid_geom(self.grid.shape[2:], host_values(self.xyz_min), host_values(self.xyz_max))

    def forward(self, xyz):
        shape = xyz.shape[:-1]
        pts = xyz.reshape(-1, 3).contiguous().float()
        out = _GridSample.apply(self.grid, pts, self.geom(), _is_channel_last(self.grid))
        out = out.reshape(*shape, self.channels)
        if self.channels == 1:
            out = out.squeeze(-1)
        return out

    def scale_volume_grid(self, new_world_size):
        if self.channels == 0:
            self.grid = nn.Parameter(torch.zeros([1, self.channels, *new_world_size]))
        else:
            self.grid = nn.Parameter(self._layout(
                F.interpolate(self.grid.data.contiguous(), size=tuple(int(s) for s in new_world_size),
                              mode="trilinear", align_corners=True)))

    def total_variation_add_grad(self, wx, wy, wz, dense_mode, mask=None):
        """In place on grid.grad (lib/grid.py:67-78)."""
        g = self.grid
        if g.grad is None:
            g.grad = torch.zeros_like(g)
        cl = _is_channel_last(g)
        C, X, Y, Z = g.size(1), g.size(2), g.size(3), g.size(4)
        if mask is None:
            call("vx_total_variation_add_grad", ptr(g), ptr(g.grad), float(wx), float(wy), float(wz),
                 int(bool(dense_mode)), C, X, Y, Z, int(cl), stream_ptr())
        else:
            mask = mask.detach()
            if C > 1 and mask.size() != g.size():
                mask = mask.repeat(1, C, 1, 1, 1)
            assert mask.size() == g.size()
            mask = mask.float().contiguous(memory_format=torch.channels_last_3d if cl else torch.contiguous_format)
            call("vx_total_variation_add_grad_new", ptr(g), ptr(g.grad), ptr(mask), float(wx), float(wy), float(wz),
                 int(bool(dense_mode)), C, X, Y, Z, int(cl), stream_ptr())

    def get_dense_grid(self):
        return self.grid

    @torch.no_grad()
    def __isub__(self, val):
        self.grid.data -= val
        return self

    def extra_repr(self):
        ws = self.world_size.tolist() if hasattr(self.world_size, "tolist") else list(self.world_size)
        return f"channels={self.channels}, world_size={ws}"


class MaskGrid(nn.Module):
    """lib/grid.py:212-245: nearest-voxel lookup of known free space."""

    def __init__(self, path=None, mask_cache_thres=None, mask=None, xyz_min=None, xyz_max=None):
        super().__init__()
        if path is not None:
            st = torch.load(path, map_location="cpu")
            self.mask_cache_thres = mask_cache_thres
            density = F.max_pool3d(st["model_state_dict"]["density.grid"], kernel_size=3, padding=1, stride=1)
            alpha = 1 - torch.exp(-F.softplus(density + st["model_state_dict"]["act_shift"]) *
                                  st["model_kwargs"]["voxel_size_ratio"])
            mask = (alpha >= self.mask_cache_thres).squeeze(0).squeeze(0)
            xyz_min = torch.Tensor(st["model_kwargs"]["xyz_min"])
            xyz_max = torch.Tensor(st["model_kwargs"]["xyz_max"])
        else:
            mask = mask.bool()
            xyz_min = torch.as_tensor(xyz_min, dtype=torch.float32)
            xyz_max = torch.as_tensor(xyz_max, dtype=torch.float32)
        self.register_buffer("mask", mask.contiguous())
        xyz_len = xyz_max - xyz_min
        self.register_buffer("xyz2ijk_scale", (torch.Tensor(list(mask.shape)) - 1) / xyz_len)
        self.register_buffer("xyz2ijk_shift", -xyz_min * self.xyz2ijk_scale)

    @torch.no_grad()
    def forward(self, xyz):
        shape = xyz.shape[:-1]
        xyz = xyz.reshape(-1, 3).contiguous()
        mask = render_utils_cuda.maskcache_lookup(self.mask, xyz, self.xyz2ijk_scale, self.xyz2ijk_shift)
        return mask.reshape(shape)

    def fill_march(self, a) -> None:
        """Mask fields of a vx_fine_march_args / vx_scene_desc mirror."""
        sc, sh = host_values(self.xyz2ijk_scale), host_values(self.xyz2ijk_shift)
        a.mask = self.mask.data_ptr()
        a.mask_X, a.mask_Y, a.mask_Z = (int(s) for s in self.mask.shape)
        for i in range(3):
            a.mask_scale[i] = float(sc[i])
            a.mask_shift[i] = float(sh[i])

    def extra_repr(self):
        return f"mask.shape={list(self.mask.shape)}"


class MaskCache(nn.Module):
    """The searched coarse geometry of the fine stage (voxurf_fine.py:913-942,
    voxurf_coarse.py:668-696): a coarse checkpoint's density, max-pooled
    ks^3 (stride 1) at load time; a point is inside when
    1 - exp(-softplus(trilinear(density) + act_shift) * voxel_size_ratio)
    >= mask_cache_thres.  The march kernels evaluate the test per sample
    (vx_fine_march_args.mask_density); forward() answers point queries
    (vx_density_mask) and needs the CUDA library.

    `path` is a checkpoint saved by run.py (model_state_dict['density'] and
    MaskCache_kwargs); `state` the same dict already in memory."""

    def __init__(self, path=None, mask_cache_thres=1e-3, ks=3, state=None):
        super().__init__()
        st = torch.load(path, map_location="cpu", weights_only=False) if path is not None else state
        if st is None:
            raise ValueError("MaskCache needs a checkpoint path or its state dict")
        kw = st["MaskCache_kwargs"]
        self.mask_cache_thres = float(mask_cache_thres)
        self.register_buffer("xyz_min", torch.as_tensor(np.asarray(kw["xyz_min"], np.float32)).clone())
        self.register_buffer("xyz_max", torch.as_tensor(np.asarray(kw["xyz_max"], np.float32)).clone())
        dens = st["model_state_dict"]["density"].detach().float()
        self.register_buffer("density", F.max_pool3d(dens, kernel_size=ks, padding=ks // 2, stride=1).contiguous())
        self.act_shift = float(kw["act_shift"])
        self.voxel_size_ratio = float(torch.as_tensor(kw["voxel_size_ratio"]))
        self.nearest = bool(kw.get("nearest", False))
        if self.nearest:
            raise NotImplementedError("nearest MaskCache sampling is not used by the Voxurf configs and is not built")

    def _geom(self):
        return grid_geom(self.density.shape[2:], host_values(self.xyz_min), host_values(self.xyz_max))

    @torch.no_grad()
    def forward(self, xyz):
        """Boolean [...] for points xyz [..., 3] (computed on the mask's device)."""
        if not self.density.is_cuda:
            raise RuntimeError("MaskCache queries run on the GPU: move the module to a CUDA device first")
        shape = xyz.shape[:-1]
        pts = xyz.reshape(-1, 3).to(self.density.device, torch.float32).contiguous()
        out = torch.empty(pts.shape[0], dtype=torch.uint8, device=pts.device)
        import ctypes

        _abi.call("vx_density_mask", self.density.data_ptr(), ctypes.byref(self._geom()), self.act_shift,
                  self.voxel_size_ratio, self.mask_cache_thres, pts.data_ptr(), pts.shape[0], out.data_ptr(),
                  stream_ptr(pts.device))
        return out.bool().reshape(shape).to(xyz.device)

    def fill_march(self, a) -> None:
        """Density-mask fields of a vx_fine_march_args / vx_scene_desc mirror."""
        a.mask_density = self.density.data_ptr()
        a.mask_dgrid = self._geom()
        a.mask_act_shift = self.act_shift
        a.mask_voxel_size_ratio = self.voxel_size_ratio
        a.mask_thres = self.mask_cache_thres

    def extra_repr(self):
        return f"density.shape={list(self.density.shape)}, thres={self.mask_cache_thres}"
