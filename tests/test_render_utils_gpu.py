"""Parity of the drop-in render_utils_cuda ops with the CPU oracle.

Integer and index outputs (N_steps, ray_id, step_id, mask_outbbox, the mask
lookup, i_start, i_end) must match bit for bit; so must t_min/t_max and the
sample points, whose float pipeline rounds the same operations on both
sides (the reference kernels' fused multiply-adds included).  Transmittance/weights use a warp-parallel FP64 scan on the GPU and
the serial float loop in the oracle: tolerance 2e-6 relative.
"""
import numpy as np
import pytest
import torch

from oracle import cref
from voxurf_gb300 import render_utils_cuda as ru
from voxurf_gb300 import synthetic

pytestmark = pytest.mark.gpu

BMIN = np.array([-1.0, -1.0, -1.0], np.float32)
BMAX = np.array([1.0, 1.0, 1.0], np.float32)


def _edge_rays(n, seed):
    """Camera rays plus adversarial ones: axis-aligned (zero components),
    rays that miss the box, rays starting inside it, tiny/huge directions."""
    o, d, _ = synthetic.random_rays(n, seed=seed)
    rng = np.random.default_rng(seed + 100)
    extra_o = rng.uniform(-3, 3, size=(64, 3)).astype(np.float32)
    extra_d = rng.normal(size=(64, 3)).astype(np.float32)
    extra_d[:8, 1:] = 0  # along x only
    extra_d[8:16, 0] = 0
    extra_d[16:24, 2] = 0
    extra_o[24:32] = rng.uniform(-0.5, 0.5, size=(8, 3))  # inside
    extra_d[32:40] *= 1e-3
    extra_d[40:48] *= 1e3
    extra_o[48:56] = np.array([5.0, 5.0, 5.0], np.float32)  # pointing away
    extra_d[48:56] = np.abs(extra_d[48:56])
    return np.concatenate([o, extra_o]), np.concatenate([d, extra_d])


@pytest.mark.parametrize("R,stepsize,n", [(32, 0.5, 256), (96, 0.5, 2048), (256, 0.5, 1024), (384, 0.25, 512)])
def test_sample_pts_on_rays_bit_exact(cuda, R, stepsize, n):
    o, d = _edge_rays(n, seed=R)
    voxel = 2.0 / R
    stepdist = np.float32(stepsize * voxel)
    near, far = 0.1, 1e9
    ref = cref.sample_pts_on_rays(o, d, BMIN, BMAX, near, far, stepdist)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    out = ru.sample_pts_on_rays(to(o), to(d), to(BMIN), to(BMAX), near, far, float(stepdist))
    names = ["ray_pts", "mask_outbbox", "ray_id", "step_id", "N_steps", "t_min", "t_max"]
    for name, a, b in zip(names, out, ref):
        a = a.cpu().numpy()
        assert a.shape == b.shape, name
        assert np.array_equal(a, b), f"{name}: {np.argwhere(a != b)[:5]}"


def test_infer_ops_bit_exact(cuda):
    o, d = _edge_rays(300, seed=7)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    t_min, t_max = ru.infer_t_minmax(to(o), to(d), to(BMIN), to(BMAX), 0.1, 1e9)
    rt_min, rt_max = cref.infer_t_minmax(o, d, BMIN, BMAX, 0.1, 1e9)
    assert np.array_equal(t_min.cpu().numpy(), rt_min) and np.array_equal(t_max.cpu().numpy(), rt_max)
    ns = ru.infer_n_samples(to(d), t_min, t_max, 0.01)
    assert np.array_equal(ns.cpu().numpy(), cref.infer_n_samples(d, rt_min, rt_max, 0.01))
    st, di = ru.infer_ray_start_dir(to(o), to(d), t_min)
    rst, rdi = cref.infer_ray_start_dir(o, d, rt_min)
    assert np.array_equal(st.cpu().numpy(), rst) and np.array_equal(di.cpu().numpy(), rdi)


def test_sample_empty_batch(cuda):
    z = torch.zeros((0, 3), device=cuda)
    out = ru.sample_pts_on_rays(z, z, torch.tensor(BMIN, device=cuda), torch.tensor(BMAX, device=cuda), 0.1, 1e9,
                                0.01)
    assert out[0].shape == (0, 3) and out[4].shape == (0,)


@pytest.mark.parametrize("shape", [(32, 32, 32), (17, 40, 9), (96, 96, 96)])
def test_maskcache_lookup_bit_exact(cuda, shape):
    rng = np.random.default_rng(sum(shape))
    world = rng.uniform(size=shape) < 0.3
    xyz = rng.uniform(-1.2, 1.2, size=(50000, 3)).astype(np.float32)
    # exact half-way points exercise round-half-away-from-zero
    scale = ((np.array(shape, np.float32) - 1) / (BMAX - BMIN)).astype(np.float32)
    shift = (-BMIN * scale).astype(np.float32)
    half = (np.floor(rng.uniform(0, 1, size=(1000, 3)) * (np.array(shape) - 1)) + 0.5)
    xyz[:1000] = ((half - shift) / scale).astype(np.float32)
    xyz[1000:1010] = np.nan
    ref = cref.maskcache_lookup(world, xyz, scale, shift)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    got = ru.maskcache_lookup(to(world), to(xyz), to(scale), to(shift)).cpu().numpy()
    assert np.array_equal(got, ref)


def _segments(n_rays, seed, max_len=700, empty_frac=0.1, alpha_hi=0.05):
    rng = np.random.default_rng(seed)
    lens = rng.integers(1, max_len, size=n_rays)
    lens[rng.uniform(size=n_rays) < empty_frac] = 0
    ray_id = np.repeat(np.arange(n_rays), lens).astype(np.int64)
    alpha = rng.uniform(0, alpha_hi, size=ray_id.size).astype(np.float32)
    # a few opaque spikes to trigger early termination
    spikes = rng.uniform(size=ray_id.size) < 0.01
    alpha[spikes] = rng.uniform(0.5, 1.0, size=spikes.sum()).astype(np.float32)
    return alpha, ray_id


def _near_tie_rays(alpha, ray_id, n_rays, i_start, i_end_full, rel=1e-4):
    """Rays whose running float transmittance passes within `rel` of the 1e-3
    stop threshold: the stop index is a threshold decision and may differ
    between the serial float loop and the FP64 scan there."""
    bad = set()
    for r in range(n_rays):
        s, e = i_start[r], i_end_full[r]
        if e <= s:
            continue
        Tc = np.cumprod(1.0 - alpha[s:e].astype(np.float64))
        if np.any(np.abs(Tc / 1e-3 - 1.0) < rel):
            bad.add(r)
    return bad


@pytest.mark.parametrize("n_rays,max_len,alpha_hi", [(256, 64, 0.05), (4096, 700, 0.05), (1024, 2200, 0.004)])
def test_alpha2weight_fwd_bwd(cuda, n_rays, max_len, alpha_hi):
    alpha, ray_id = _segments(n_rays, seed=n_rays + max_len, max_len=max_len, alpha_hi=alpha_hi)
    w, T, last, i_s, i_e = cref.alpha2weight(alpha, ray_id, n_rays)
    full_end = np.searchsorted(ray_id, np.arange(n_rays), side="right")
    ties = _near_tie_rays(alpha, ray_id, n_rays, np.searchsorted(ray_id, np.arange(n_rays)), full_end)
    ta, tr = torch.from_numpy(alpha).to(cuda), torch.from_numpy(ray_id).to(cuda)
    gw, gT, glast, gis, gie = [x.cpu().numpy() for x in ru.alpha2weight(ta, tr, n_rays)]
    keep = np.array([r not in ties for r in range(n_rays)])
    assert np.array_equal(gis[keep], i_s[keep])
    assert np.array_equal(gie[keep], i_e[keep])
    samp_keep = keep[ray_id]
    # against the FP64 scan: segments of more than 512 samples carry T in FP64
    # and round once (3e-7); shorter ones carry it in FP32 through the warp
    # prefix products and the chunk carries (3e-6; measured 1.6e-6)
    w64, T64, last64, _, _ = cref.alpha2weight(alpha.astype(np.float64), ray_id, n_rays)
    seg_len = full_end - np.searchsorted(ray_id, np.arange(n_rays))
    long_ray = seg_len > 512
    for sel_r, rtol in ((keep & long_ray, 3e-7), (keep & ~long_ray, 3e-6)):
        sel_s = sel_r[ray_id]
        errs = [float(np.max(np.abs(a[sel_s] - b[sel_s]) / (np.abs(b[sel_s]) + 1e-30), initial=0.0))
                for a, b in ((gw, w64), (gT, T64))]
        print("alpha2weight vs FP64", "long" if rtol < 1e-6 else "short", errs)
        np.testing.assert_allclose(gw[sel_s], w64[sel_s], rtol=rtol, atol=1e-12)
        np.testing.assert_allclose(gT[sel_s], T64[sel_s], rtol=rtol, atol=1e-12)
        np.testing.assert_allclose(glast[sel_r], last64[sel_r], rtol=rtol, atol=1e-12)
    # against the reference's serial float loop: its own rounding grows with
    # the ray length (about sqrt(n) ulps)
    rt = 4e-6 if max_len <= 700 else 2e-5
    np.testing.assert_allclose(gw[samp_keep], w[samp_keep], rtol=rt, atol=1e-9)
    np.testing.assert_allclose(gT[samp_keep], T[samp_keep], rtol=rt, atol=1e-9)
    np.testing.assert_allclose(glast[keep], last[keep], rtol=rt, atol=1e-9)

    rng = np.random.default_rng(3)
    grad_w = rng.normal(size=alpha.size).astype(np.float32)
    grad_last = rng.normal(size=n_rays).astype(np.float32)
    # feed the oracle's forward state to both backwards
    ref = cref.alpha2weight_backward(alpha, w, T, last, i_s, i_e, n_rays, grad_w, grad_last)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    got = ru.alpha2weight_backward(to(alpha), to(w), to(T), to(last), to(i_s), to(i_e), n_rays, to(grad_w),
                                   to(grad_last)).cpu().numpy()
    scale = np.abs(ref).max() + 1e-12
    print("alpha2weight backward vs serial float loop", np.abs(got - ref).max() / scale)
    assert np.abs(got - ref).max() / scale < 2e-5


def test_alpha2weight_empty(cuda):
    a = torch.zeros(0, device=cuda)
    r = torch.zeros(0, dtype=torch.int64, device=cuda)
    w, T, last, i_s, i_e = ru.alpha2weight(a, r, 5)
    assert w.numel() == 0 and torch.all(last == 1) and torch.all(i_s == 0) and torch.all(i_e == 0)


def test_inputs_must_be_cuda(cuda):
    with pytest.raises(RuntimeError):
        ru.alpha2weight(torch.zeros(3), torch.zeros(3, dtype=torch.int64), 1)


@pytest.mark.parametrize("H,W,pose", [(120, 160, 3), (7, 5, 40), (1, 1, 0)])
def test_camera_rays_match_get_rays(cuda, H, W, pose):
    """vx_camera_rays == get_rays + viewdirs (OpenCV axes, pixel centres +0.5)."""
    import ctypes
    from voxurf_gb300 import _native
    from voxurf_gb300._torch import ptr, stream_ptr

    c2w = synthetic.fibonacci_poses()[pose]
    K = synthetic.intrinsics(1200, 1600)
    py, px = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    o, d, v = synthetic.rays_for_pixels(c2w, K, px.reshape(-1), py.reshape(-1))
    out = [torch.empty(H * W, 3, device=cuda) for _ in range(3)]
    m = (ctypes.c_float * 16)(*c2w.astype(np.float32).reshape(-1))
    _native.call("vx_camera_rays", m, float(K[0, 0]), float(K[1, 1]), float(K[0, 2]), float(K[1, 2]), H, W, 1,
                 *[ptr(t) for t in out], stream_ptr())
    for got, want in zip(out, (o, d, v)):
        np.testing.assert_allclose(got.cpu().numpy(), want, rtol=0, atol=2e-6)
