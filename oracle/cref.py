"""ORACLE — test infrastructure only (never imported by the product).

numpy/ctypes front-end of ``oracle/cref.c``, the serial CPU restatement of
the reference's CUDA ops (Voxurf lib/cuda/render_utils_kernel.cu,
total_variation_kernel.cu, adam_upd_kernel.cu).  ``build()`` compiles it with
gcc into ``oracle/_build/libvxoracle.so`` (-ffp-contract=off: one rounding
per operation, except the multiply-adds that the reference's compiled
kernels fuse, written as fmaf in the source).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cref.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libvxoracle.so")

_lib = None


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fno-fast-math", SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.vxo_sample_count.restype = C.c_int64
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def infer_t_minmax(rays_o, rays_d, xyz_min, xyz_max, near, far):
    rays_o, rays_d, mn, mx = _f32(rays_o), _f32(rays_d), _f32(xyz_min), _f32(xyz_max)
    n = rays_o.shape[0]
    t_min = np.empty(n, np.float32)
    t_max = np.empty(n, np.float32)
    lib().vxo_infer_t_minmax(_p(rays_o), _p(rays_d), _p(mn), _p(mx), C.c_float(near), C.c_float(far),
                             C.c_int64(n), _p(t_min), _p(t_max))
    return t_min, t_max


def infer_n_samples(rays_d, t_min, t_max, stepdist):
    rays_d, t_min, t_max = _f32(rays_d), _f32(t_min), _f32(t_max)
    n = t_min.shape[0]
    out = np.empty(n, np.int64)
    lib().vxo_infer_n_samples(_p(rays_d), _p(t_min), _p(t_max), C.c_float(stepdist), C.c_int64(n), _p(out))
    return out


def infer_ray_start_dir(rays_o, rays_d, t_min):
    rays_o, rays_d, t_min = _f32(rays_o), _f32(rays_d), _f32(t_min)
    n = rays_o.shape[0]
    start = np.empty((n, 3), np.float32)
    direc = np.empty((n, 3), np.float32)
    lib().vxo_infer_ray_start_dir(_p(rays_o), _p(rays_d), _p(t_min), C.c_int64(n), _p(start), _p(direc))
    return start, direc


def sample_pts_on_rays(rays_o, rays_d, xyz_min, xyz_max, near, far, stepdist):
    """Returns (ray_pts, mask_outbbox, ray_id, step_id, N_steps, t_min, t_max)."""
    rays_o, rays_d, mn, mx = _f32(rays_o), _f32(rays_d), _f32(xyz_min), _f32(xyz_max)
    n = rays_o.shape[0]
    t_min = np.empty(n, np.float32)
    t_max = np.empty(n, np.float32)
    n_steps = np.empty(n, np.int64)
    total = lib().vxo_sample_count(_p(rays_o), _p(rays_d), _p(mn), _p(mx), C.c_float(near), C.c_float(far),
                                   C.c_float(stepdist), C.c_int64(n), _p(t_min), _p(t_max), _p(n_steps))
    pts = np.empty((total, 3), np.float32)
    mask = np.empty(total, np.uint8)
    ray_id = np.empty(total, np.int64)
    step_id = np.empty(total, np.int64)
    lib().vxo_sample_fill(_p(rays_o), _p(rays_d), _p(mn), _p(mx), _p(t_min), _p(n_steps), C.c_float(stepdist),
                          C.c_int64(n), _p(pts), _p(mask), _p(ray_id), _p(step_id))
    return pts, mask.astype(bool), ray_id, step_id, n_steps, t_min, t_max


def maskcache_lookup(world, xyz, scale, shift):
    world = np.ascontiguousarray(world, dtype=np.uint8)
    xyz, scale, shift = _f32(xyz), _f32(scale), _f32(shift)
    n = xyz.shape[0]
    out = np.empty(n, np.uint8)
    lib().vxo_maskcache_lookup(_p(world), C.c_int64(world.shape[0]), C.c_int64(world.shape[1]),
                               C.c_int64(world.shape[2]), _p(xyz), C.c_int64(n), _p(scale), _p(shift), _p(out))
    return out.astype(bool)


def alpha2weight(alpha, ray_id, n_rays):
    """float32 (reference-exact) or float64 depending on alpha's dtype."""
    f64 = np.asarray(alpha).dtype == np.float64
    dt = np.float64 if f64 else np.float32
    alpha = np.ascontiguousarray(alpha, dtype=dt)
    ray_id = _i64(ray_id)
    n = alpha.shape[0]
    w = np.empty(n, dt)
    T = np.empty(n, dt)
    last = np.empty(n_rays, dt)
    i_s = np.empty(n_rays, np.int64)
    i_e = np.empty(n_rays, np.int64)
    fn = lib().vxo_alpha2weight_f64 if f64 else lib().vxo_alpha2weight
    fn(_p(alpha), _p(ray_id), C.c_int64(n), C.c_int64(n_rays), _p(w), _p(T), _p(last), _p(i_s), _p(i_e))
    return w, T, last, i_s, i_e


def alpha2weight_backward(alpha, weight, T, alphainv_last, i_start, i_end, n_rays, grad_weights, grad_last):
    f64 = np.asarray(alpha).dtype == np.float64
    dt = np.float64 if f64 else np.float32
    arrs = [np.ascontiguousarray(a, dtype=dt) for a in (alpha, weight, T, alphainv_last, grad_weights, grad_last)]
    alpha, weight, T, alphainv_last, grad_weights, grad_last = arrs
    i_start, i_end = _i64(i_start), _i64(i_end)
    n = alpha.shape[0]
    grad = np.empty(n, dt)
    fn = lib().vxo_alpha2weight_backward_f64 if f64 else lib().vxo_alpha2weight_backward
    fn(_p(alpha), _p(weight), _p(T), _p(alphainv_last), _p(i_start), _p(i_end), C.c_int64(n), C.c_int64(n_rays),
       _p(grad_weights), _p(grad_last), _p(grad))
    return grad


def tv_add_grad(param, grad, wx, wy, wz, dense_mode, mask=None, channel_last=False):
    """In place on `grad` (float32).  param/grad/mask shaped [1,C,X,Y,Z]
    (channel_last=False) or [X,Y,Z,C] (channel_last=True)."""
    param = _f32(param)
    assert grad.dtype == np.float32 and grad.flags.c_contiguous
    if channel_last:
        X, Y, Z, Cc = param.shape
    else:
        Cc, X, Y, Z = param.shape[-4:]
    m = None if mask is None else _f32(mask)
    lib().vxo_tv_add_grad(_p(param), _p(grad), None if m is None else _p(m), C.c_float(wx), C.c_float(wy),
                          C.c_float(wz), C.c_int(int(bool(dense_mode))), C.c_int64(Cc), C.c_int64(X), C.c_int64(Y),
                          C.c_int64(Z), C.c_int(int(channel_last)))
    return grad


def adam_upd(mode, param, grad, exp_avg, exp_avg_sq, step, beta1, beta2, lr, eps, perlr=None):
    """In place (float32).  mode 0 plain, 1 masked, 2 per-lr."""
    for a in (param, exp_avg, exp_avg_sq):
        assert a.dtype == np.float32 and a.flags.c_contiguous
    grad = _f32(grad)
    pl = None if perlr is None else _f32(perlr)
    lib().vxo_adam_upd(C.c_int(mode), _p(param), _p(grad), _p(exp_avg), _p(exp_avg_sq),
                       None if pl is None else _p(pl), C.c_int64(param.size), C.c_int(step), C.c_float(beta1),
                       C.c_float(beta2), C.c_float(lr), C.c_float(eps))


def cumdist_thres(dist, thres):
    """ub360_utils_kernel.cu:13-31 -> bool [n_rays, n_pts]."""
    dist = _f32(dist)
    n_rays, n_pts = dist.shape
    mask = np.zeros((n_rays, n_pts), np.uint8)
    lib().vxo_cumdist_thres(_p(dist), C.c_int64(n_rays), C.c_int64(n_pts), C.c_float(thres), _p(mask))
    return mask.astype(bool)


def bg_samples_dense(rays_o, rays_d, xyz_min, xyz_max, near, far, stepdist, dist_thres, n_samples, jitter=None,
                     outbbox_only=False):
    """Background candidates of voxurf_womask_fine.py:857-868 (coarse variant
    with outbbox_only) over all [N, S] samples -> (pts, inverted pts, keep)."""
    rays_o, rays_d, mn, mx = _f32(rays_o), _f32(rays_d), _f32(xyz_min), _f32(xyz_max)
    n = rays_o.shape[0]
    jit = None if jitter is None else _f32(jitter)
    pts = np.zeros((n, n_samples, 3), np.float32)
    inv = np.zeros((n, n_samples, 3), np.float32)
    keep = np.zeros((n, n_samples), np.uint8)
    lib().vxo_bg_samples(_p(rays_o), _p(rays_d), None if jit is None else _p(jit), _p(mn), _p(mx), C.c_float(near),
                         C.c_float(far), C.c_float(stepdist), C.c_float(dist_thres), C.c_int(n_samples),
                         C.c_int(int(bool(outbbox_only))), C.c_int64(n), _p(pts), _p(inv), _p(keep))
    return pts, inv, keep.astype(bool)


def bg_samples(rays_o, rays_d, xyz_min, xyz_max, near, far, stepdist, dist_thres, n_samples, jitter=None,
               outbbox_only=False):
    """Compacted like :868-870 -> (outer_pts, outer_pts_org, ray_id, step_id)."""
    pts, inv, keep = bg_samples_dense(rays_o, rays_d, xyz_min, xyz_max, near, far, stepdist, dist_thres, n_samples,
                                      jitter, outbbox_only)
    ray_id, step_id = np.nonzero(keep)
    return inv[keep], pts[keep], ray_id.astype(np.int64), step_id.astype(np.int64)


def fmaf(a, b, c):
    """Elementwise correctly rounded float32 a*b+c (C99 fmaf), broadcasting."""
    a, b, c = np.broadcast_arrays(np.asarray(a, np.float32), np.asarray(b, np.float32), np.asarray(c, np.float32))
    a, b, c = _f32(a), _f32(b), _f32(c)
    out = np.empty(a.shape, np.float32)
    lib().vxo_fmaf(_p(a), _p(b), _p(c), _p(out), C.c_int64(a.size))
    return out
