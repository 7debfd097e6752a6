"""Background samples of the scenes without an object mask
(lib/voxurf_womask_fine.py:857-870, the coarse variant at
lib/voxurf_womask_coarse.py:633-650).

The reference builds them with torch ops over dense [N, S] tensors:
``sample_ray_ori`` (voxurf_womask_fine.py:789-818) places S uniform samples
from each ray's bbox entry, ``outside_sphere_trans(..., filtered=True)``
(:820-825) inverts every point (x / |x|^2), the distances between
consecutive inverted points go through ``cumdist_thres`` (:867) and the
samples outside the unit sphere that pass it are compacted with boolean
indexing (:868-870).  The coarse model steps by the background grid's voxel
size, also requires the sample to lie outside the bbox and uses 0.95 instead
of 0.5 in the threshold (voxurf_womask_coarse.py:634, 641-642).  Here the same samples come out of two launches of the
library (a count pass with a device scan, then a fill pass), one thread per
ray, with only the kept samples written.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _abi, _native
from ._torch import check_input, ptr, scratch, stream_ptr


def n_samples_for(grid_shape, stepsize: float) -> int:
    """sample_ray_ori's S (voxurf_womask_fine.py:792-795): int(|shape+1| /
    stepsize) + 1 for the SDF grid's [X, Y, Z]."""
    return int(np.linalg.norm(np.array(grid_shape) + 1) / stepsize) + 1


def background_samples(rays_o, rays_d, xyz_min, xyz_max, near: float, far: float, stepsize: float, voxel_size,
                       n_samples: int, jitter=None, *, step_voxel_size=None, dist_thres_factor: float = 0.5,
                       outbbox_only: bool = False, inner: bool = False):
    """-> (outer_pts [M,3], outer_pts_org [M,3], outer_ray_id [M], outer_step_id [M]).

    ``inner=True`` gives the maskless fine model's foreground samples instead
    (voxurf_womask_fine.py:843-849): the same sample placement, the points
    with |p| < 1, not inverted and without the distance test; the return is
    then (pts [M,3], None, ray_id [M], step_id [M]).

    ``voxel_size`` is the model's float32 voxel size; the step distance
    (``stepsize * step_voxel_size``, :810-812, with step_voxel_size =
    voxel_size for the fine model and voxel_size_bg for the coarse one) and
    the cumdist threshold (``voxel_size * stepsize * dist_thres_factor``,
    :865) are formed in float32 as the reference's tensor arithmetic does.
    ``jitter`` [N] is the per-ray uniform offset of a training batch
    (``torch.rand_like(rng[:, [0]])`` at :808) or None.  One 8-byte
    device->host read gives the output size.
    """
    check_input(rays_o, "rays_o", torch.float32)
    check_input(rays_d, "rays_d", torch.float32)
    if jitter is not None:
        check_input(jitter, "jitter", torch.float32)
    n = rays_o.size(0)
    dev = rays_o.device
    vs = np.float32(float(voxel_size))
    svs = vs if step_voxel_size is None else np.float32(float(step_voxel_size))
    args = _abi.BgSampleArgs()
    args.rays_o, args.rays_d = ptr(rays_o), ptr(rays_d)
    args.jitter = ptr(jitter) if jitter is not None else None
    for i in range(3):
        args.xyz_min[i] = float(xyz_min[i])
        args.xyz_max[i] = float(xyz_max[i])
    args.near, args.far = float(near), float(far)
    args.stepdist = float(np.float32(np.float32(stepsize) * svs))
    args.dist_thres = float(np.float32(np.float32(vs * np.float32(stepsize)) * np.float32(dist_thres_factor)))
    args.n_samples = int(n_samples)
    args.outbbox_only = int(bool(outbbox_only))
    args.inner = int(bool(inner))
    args.n_rays = n
    counts = torch.empty(n, dtype=torch.int64, device=dev)
    offsets = torch.empty(n + 1, dtype=torch.int64, device=dev)
    lib = _native.load()
    _abi._declare()
    nb = int(lib.vx_scan_scratch_bytes(n))
    sc = scratch(nb, dev)
    st = stream_ptr()
    _native.check(lib.vx_bg_samples_count(C.byref(args), ptr(counts), ptr(offsets), ptr(sc), nb, st),
                  "vx_bg_samples_count")
    total = int(offsets[-1].item())
    outer = torch.empty((total, 3), dtype=torch.float32, device=dev)
    org = None if inner else torch.empty((total, 3), dtype=torch.float32, device=dev)
    ray_id = torch.empty(total, dtype=torch.int64, device=dev)
    step_id = torch.empty(total, dtype=torch.int64, device=dev)
    _native.check(lib.vx_bg_samples_fill(C.byref(args), ptr(offsets), total, ptr(outer), ptr(org), ptr(ray_id),
                                         ptr(step_id), st), "vx_bg_samples_fill")
    return outer, org, ray_id, step_id
