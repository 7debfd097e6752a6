"""The allocation-free sampling entry point, vx_sample_pts_count_noalloc.

Some callers of this library cannot allocate device memory: hosts that only
receive device pointers for inputs and outputs from another runtime, and
render loops that reserve all device memory up front.  For them the count
phase of sample_pts_on_rays has a variant whose scan scratch is a fixed
static array inside the library.  This test calls it through the C ABI and
checks it against the allocating entry point, vx_sample_pts_count, on two
calls in a row of different sizes (the shared array keeps the first call's
contents when the second runs).  The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest
import torch

from voxurf_gb300 import _native, synthetic
from voxurf_gb300._torch import ptr, stream_ptr

pytestmark = pytest.mark.gpu

VX_NOALLOC_MAX_RAYS = 4194304
VX_ERR_TOO_LARGE = 7


def _count(lib, name, rays_o, rays_d, bmin, bmax, stepdist, dev):
    n = rays_o.size(0)
    t_min = torch.empty(n, dtype=torch.float32, device=dev)
    t_max = torch.empty(n, dtype=torch.float32, device=dev)
    n_steps = torch.empty(n, dtype=torch.int64, device=dev)
    offsets = torch.full((n + 1,), -1, dtype=torch.int64, device=dev)
    common = (ptr(rays_o), ptr(rays_d), ptr(bmin), ptr(bmax), 0.1, 1e9, stepdist, n, ptr(t_min), ptr(t_max),
              ptr(n_steps), ptr(offsets))
    if name == "vx_sample_pts_count":
        nb = lib.vx_scan_scratch_bytes(n)
        scratch = torch.empty(max(nb, 16), dtype=torch.uint8, device=dev)
        status = lib.vx_sample_pts_count(*common, ptr(scratch), nb, stream_ptr())
    else:
        status = lib.vx_sample_pts_count_noalloc(*common, stream_ptr())
    assert status == 0, lib.vx_status_string(status)
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in (t_min, t_max, n_steps, offsets)]


def test_noalloc_count_matches_allocating_entry_point(cuda):
    lib = _native.load()
    bmin = torch.tensor([-1.0, -1.0, -1.0], device=cuda)
    bmax = torch.tensor([1.0, 1.0, 1.0], device=cuda)
    # two calls in a row: a large batch (many scan tiles), then a smaller one
    for n, seed, R in ((150000, 1, 256), (5000, 2, 96)):
        o, d, _ = synthetic.random_rays(n, seed=seed)
        rays_o = torch.from_numpy(o).to(cuda)
        rays_d = torch.from_numpy(d).to(cuda)
        stepdist = float(np.float32(0.5 * 2.0 / R))
        ref = _count(lib, "vx_sample_pts_count", rays_o, rays_d, bmin, bmax, stepdist, cuda)
        got = _count(lib, "vx_sample_pts_count_noalloc", rays_o, rays_d, bmin, bmax, stepdist, cuda)
        for a, b in zip(got, ref):
            np.testing.assert_array_equal(a, b)
        assert got[3][-1] == got[2].sum()


def test_noalloc_count_empty_and_largest(cuda):
    """n_rays = 0 (only offsets[0] = 0 is written) and n_rays exactly at the
    maximum, the call that uses every entry of the static scratch."""
    lib = _native.load()
    bmin = torch.tensor([-1.0, -1.0, -1.0], device=cuda)
    bmax = torch.tensor([1.0, 1.0, 1.0], device=cuda)
    offsets = torch.full((1,), -1, dtype=torch.int64, device=cuda)
    null = ctypes.c_void_p(0)
    status = lib.vx_sample_pts_count_noalloc(null, null, null, null, 0.1, 1e9, 0.01, 0, null, null, null,
                                             ptr(offsets), stream_ptr())
    assert status == 0, lib.vx_status_string(status)
    torch.cuda.synchronize()
    assert int(offsets.item()) == 0
    n = VX_NOALLOC_MAX_RAYS
    g = torch.Generator(cuda).manual_seed(3)
    rays_o = (torch.rand((n, 3), device=cuda, generator=g) * 2 - 1) * 3
    rays_d = -rays_o + (torch.rand((n, 3), device=cuda, generator=g) - 0.5)
    stepdist = float(np.float32(0.5 * 2.0 / 128))
    ref = _count(lib, "vx_sample_pts_count", rays_o, rays_d, bmin, bmax, stepdist, cuda)
    got = _count(lib, "vx_sample_pts_count_noalloc", rays_o, rays_d, bmin, bmax, stepdist, cuda)
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)
    assert got[3][-1] == got[2].sum()


def test_noalloc_rejects_sizes_above_the_maximum(cuda):
    lib = _native.load()
    # rejected on the host before any pointer is used or any kernel launched
    null = ctypes.c_void_p(0)
    status = lib.vx_sample_pts_count_noalloc(null, null, null, null, 0.1, 1e9, 0.01, VX_NOALLOC_MAX_RAYS + 1, null,
                                             null, null, ctypes.c_void_p(1), stream_ptr())
    assert status == VX_ERR_TOO_LARGE
    assert b"maximum" in lib.vx_status_string(status)
