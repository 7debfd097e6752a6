"""ORACLE — test infrastructure only (never imported by the product).

Runs the reference's own CUDA kernels on the GPU: the PTX that
``oracle/ref_build.py`` compiled from the reference's lib/cuda/*_kernel.cu is
loaded through the CUDA driver API (ctypes on libcuda, no extra package) and
its ``__global__`` kernels are launched on torch tensors with the launch
shapes and the host-side steps of the reference's launcher functions
(render_utils_kernel.cu:84-242, 396-428, 624-707; total_variation_kernel.cu:
68-134; adam_upd_kernel.cu:60-133; ub360_utils_kernel.cu:33-48).  Those
launchers themselves are host code tied to the reference's torch build; the
steps they take between kernels (cumsum, zero/one fills, the /6 of the TV
weights, the float Adam step size) are restated here with torch on the GPU.

Used only by GPU tests, as a same-GPU pin of the C restatement
(``oracle/cref.c``) and of the product kernels.  ``available()`` is False
(and the tests skip) when the PTX was not built, i.e. when the reference
checkout was absent on the machine that ran the build.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import ref_build

THREADS = 256  # every reference launcher uses 256 threads per block

_drv = None
_modules: dict[str, "_Module"] = {}


def available() -> bool:
    return all(os.path.exists(ref_build.ptx_path(u)) for u in ref_build.UNITS)


def _driver():
    global _drv
    if _drv is None:
        d = C.CDLL("libcuda.so.1")
        d.cuGetErrorString.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        d.cuCtxGetCurrent.argtypes = [C.POINTER(C.c_void_p)]
        d.cuModuleLoadData.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        d.cuModuleGetFunctionCount.argtypes = [C.POINTER(C.c_uint), C.c_void_p]
        d.cuModuleEnumerateFunctions.argtypes = [C.POINTER(C.c_void_p), C.c_uint, C.c_void_p]
        d.cuFuncGetName.argtypes = [C.POINTER(C.c_char_p), C.c_void_p]
        d.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                     C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        _drv = d
    return _drv


def _check(res: int, what: str) -> None:
    if res != 0:
        s = C.c_char_p()
        _driver().cuGetErrorString(res, C.byref(s))
        raise RuntimeError(f"{what}: CUDA driver error {res} ({s.value.decode() if s.value else '?'})")


class _Module:
    """One reference kernel file's PTX, loaded into torch's current context."""

    def __init__(self, unit: str):
        import torch

        torch.cuda.init()
        torch.zeros(1, device="cuda")  # makes torch's primary context current on this thread
        d = _driver()
        ctx = C.c_void_p()
        _check(d.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        with open(ref_build.ptx_path(unit), "rb") as f:
            image = f.read() + b"\0"
        self.mod = C.c_void_p()
        _check(d.cuModuleLoadData(C.byref(self.mod), image), f"cuModuleLoadData({unit})")
        n = C.c_uint()
        _check(d.cuModuleGetFunctionCount(C.byref(n), self.mod), "cuModuleGetFunctionCount")
        funcs = (C.c_void_p * n.value)()
        _check(d.cuModuleEnumerateFunctions(funcs, n.value, self.mod), "cuModuleEnumerateFunctions")
        self.funcs = {}
        for f in funcs:
            name = C.c_char_p()
            _check(d.cuFuncGetName(C.byref(name), f), "cuFuncGetName")
            self.funcs[name.value.decode()] = f

    def kernel(self, name: str, targs: str | None) -> C.c_void_p:
        """The kernel `name` (Itanium-mangled): `targs` is its mangled
        template-argument list ("IfE" for <float>, "IfLb1EE" for
        <float, true>), or None for a plain function."""
        prefix = f"_Z{len(name)}{name}"
        hits = [n for n, _ in self.funcs.items() if n.startswith(prefix)
                and (n[len(prefix):].startswith(targs) if targs else not n[len(prefix):].startswith("I"))]
        if len(hits) != 1:
            near = [n for n in self.funcs if name in n]
            raise RuntimeError(f"kernel {name} {targs}: {len(hits)} matches among {near}")
        return self.funcs[hits[0]]


def _module(unit: str) -> _Module:
    if unit not in _modules:
        _modules[unit] = _Module(unit)
    return _modules[unit]


# argument kinds of the reference kernels' parameters
P, F, I, Z = "ptr", "f32", "i32", "size_t"


def _launch(unit: str, name: str, targs: str | None, n_threads: int, sig: tuple, *args) -> None:
    """Launches `name` over ceil(n_threads / 256) blocks of 256 threads on
    torch's current stream.  `sig` lists each parameter's kind; pointers are
    passed as torch tensors (their data_ptr)."""
    import torch

    if n_threads <= 0:
        return
    if len(sig) != len(args):
        raise ValueError(f"{name}: {len(args)} arguments for {len(sig)} parameters")
    vals = []
    for kind, a in zip(sig, args):
        if kind == P:
            if not (isinstance(a, torch.Tensor) and a.is_cuda and a.is_contiguous()):
                raise ValueError(f"{name}: pointer arguments must be contiguous CUDA tensors")
            vals.append(C.c_void_p(a.data_ptr()))
        elif kind == F:
            vals.append(C.c_float(float(a)))
        elif kind == I:
            if not -2**31 <= int(a) < 2**31:
                raise ValueError(f"{name}: int argument {a} out of range")
            vals.append(C.c_int(int(a)))
        elif kind == Z:
            vals.append(C.c_size_t(int(a)))
        else:
            raise ValueError(kind)
    params = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
    f = _module(unit).kernel(name, targs)
    blocks = (n_threads + THREADS - 1) // THREADS
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _check(_driver().cuLaunchKernel(f, blocks, 1, 1, THREADS, 1, 1, 0, stream, params, None), f"launch {name}")


def _f32(t):
    import torch

    return t.to(torch.float32).contiguous()


# ---- render_utils_kernel.cu ------------------------------------------------------

def infer_t_minmax(rays_o, rays_d, xyz_min, xyz_max, near: float, far: float):
    """render_utils_kernel.cu:84-105."""
    import torch

    n = rays_o.shape[0]
    t_min = torch.empty(n, dtype=torch.float32, device=rays_o.device)
    t_max = torch.empty_like(t_min)
    _launch("render_utils", "infer_t_minmax_cuda_kernel", "IfE", n, (P, P, P, P, F, F, I, P, P),
            rays_o, rays_d, xyz_min, xyz_max, near, far, n, t_min, t_max)
    return t_min, t_max


def infer_n_samples(rays_d, t_min, t_max, stepdist: float):
    """render_utils_kernel.cu:107-122."""
    import torch

    n = t_min.shape[0]
    n_samples = torch.empty(n, dtype=torch.int64, device=rays_d.device)
    _launch("render_utils", "infer_n_samples_cuda_kernel", "IfE", n, (P, P, P, F, I, P),
            rays_d, t_min, t_max, stepdist, n, n_samples)
    return n_samples


def infer_ray_start_dir(rays_o, rays_d, t_min):
    """render_utils_kernel.cu:124-140."""
    import torch

    n = rays_o.shape[0]
    rays_start = torch.empty_like(rays_o)
    rays_dir = torch.empty_like(rays_o)
    _launch("render_utils", "infer_ray_start_dir_cuda_kernel", "IfE", n, (P, P, P, I, P, P),
            rays_o, rays_d, t_min, n, rays_start, rays_dir)
    return rays_start, rays_dir


def sample_pts_on_rays(rays_o, rays_d, xyz_min, xyz_max, near: float, far: float, stepdist: float):
    """render_utils_kernel.cu:196-242: returns [rays_pts, mask_outbbox,
    ray_id, step_id, N_steps, t_min, t_max]."""
    import torch

    rays_o, rays_d, xyz_min, xyz_max = (_f32(t) for t in (rays_o, rays_d, xyz_min, xyz_max))
    dev = rays_o.device
    n = rays_o.shape[0]
    t_min, t_max = infer_t_minmax(rays_o, rays_d, xyz_min, xyz_max, near, far)
    n_steps = infer_n_samples(rays_d, t_min, t_max, stepdist)
    cum = n_steps.cumsum(0)
    total = int(n_steps.sum().item())
    ray_id = torch.zeros(total, dtype=torch.int64, device=dev)
    _launch("render_utils", "__set_1_at_ray_seg_start", None, n, (P, P, I), ray_id, cum, n)
    ray_id.cumsum_(0)
    step_id = torch.empty(total, dtype=torch.int64, device=dev)
    _launch("render_utils", "__set_step_id", None, total, (P, P, P, I), step_id, ray_id, cum, total)
    rays_start, rays_dir = infer_ray_start_dir(rays_o, rays_d, t_min)
    rays_pts = torch.empty((total, 3), dtype=torch.float32, device=dev)
    mask_outbbox = torch.empty(total, dtype=torch.bool, device=dev)
    _launch("render_utils", "sample_pts_on_rays_cuda_kernel", "IfE", total, (P, P, P, P, P, P, F, I, P, P),
            rays_start, rays_dir, xyz_min, xyz_max, ray_id, step_id, stepdist, total, rays_pts, mask_outbbox)
    return [rays_pts, mask_outbbox, ray_id, step_id, n_steps, t_min, t_max]


def maskcache_lookup(world, xyz, xyz2ijk_scale, xyz2ijk_shift):
    """render_utils_kernel.cu:396-428 (world a bool [X, Y, Z] grid)."""
    import torch

    world = world.contiguous()
    xyz, scale, shift = _f32(xyz), _f32(xyz2ijk_scale), _f32(xyz2ijk_shift)
    n = xyz.shape[0]
    out = torch.zeros(n, dtype=torch.bool, device=xyz.device)
    if n == 0:
        return out
    sx, sy, sz = world.shape
    _launch("render_utils", "maskcache_lookup_cuda_kernel", "IfE", n, (P, P, P, P, P, I, I, I, I),
            world, xyz, out, scale, shift, sx, sy, sz, n)
    return out


def alpha2weight(alpha, ray_id, n_rays: int):
    """render_utils_kernel.cu:624-666: [weight, T, alphainv_last, i_start, i_end]."""
    import torch

    alpha = _f32(alpha)
    ray_id = ray_id.to(torch.int64).contiguous()
    n_pts = alpha.shape[0]
    dev = alpha.device
    weight = torch.zeros_like(alpha)
    T = torch.ones_like(alpha)
    last = torch.ones(n_rays, dtype=torch.float32, device=dev)
    i_start = torch.zeros(n_rays, dtype=torch.int64, device=dev)
    i_end = torch.zeros(n_rays, dtype=torch.int64, device=dev)
    if n_pts == 0:
        return [weight, T, last, i_start, i_end]
    _launch("render_utils", "__set_i_for_segment_start_end", None, n_pts, (P, I, P, P), ray_id, n_pts, i_start, i_end)
    i_end[ray_id[n_pts - 1]] = n_pts
    _launch("render_utils", "alpha2weight_cuda_kernel", "IfE", n_rays, (P, I, P, P, P, P, P),
            alpha, n_rays, weight, T, last, i_start, i_end)
    return [weight, T, last, i_start, i_end]


def alpha2weight_backward(alpha, weight, T, alphainv_last, i_start, i_end, n_rays: int, grad_weights, grad_last):
    """render_utils_kernel.cu:668-707."""
    import torch

    alpha, weight, T, last, gw, gl = (_f32(t) for t in (alpha, weight, T, alphainv_last, grad_weights, grad_last))
    i_start, i_end = i_start.to(torch.int64).contiguous(), i_end.to(torch.int64).contiguous()
    grad = torch.zeros_like(alpha)
    if n_rays == 0:
        return grad
    _launch("render_utils", "alpha2weight_backward_cuda_kernel", "IfE", n_rays, (P, P, P, P, P, P, I, P, P, P),
            alpha, weight, T, last, i_start, i_end, n_rays, gw, gl, grad)
    return grad


# ---- total_variation_kernel.cu ------------------------------------------------

def _tv_weights(wx, wy, wz):
    # the launchers divide the float weights by 6 on the host
    # (total_variation_kernel.cu:75-77, 107-109)
    return [np.float32(w) / np.float32(6) for w in (wx, wy, wz)]


def total_variation_add_grad(param, grad, wx: float, wy: float, wz: float, dense_mode: bool) -> None:
    """total_variation_kernel.cu:68-98, in place on grad ([1, C, X, Y, Z])."""
    N = param.numel()
    sx, sy, sz = param.shape[2], param.shape[3], param.shape[4]
    targs = "IfLb1EE" if dense_mode else "IfLb0EE"
    _launch("total_variation", "total_variation_add_grad_cuda_kernel", targs, N, (P, P, F, F, F, Z, Z, Z, Z),
            param, grad, *_tv_weights(wx, wy, wz), sx, sy, sz, N)


def total_variation_add_grad_new(param, grad, mask, wx: float, wy: float, wz: float, dense_mode: bool) -> None:
    """total_variation_kernel.cu:100-134, in place on grad."""
    N = param.numel()
    sx, sy, sz = param.shape[2], param.shape[3], param.shape[4]
    targs = "IfLb1EE" if dense_mode else "IfLb0EE"
    _launch("total_variation", "total_variation_add_grad_cuda_kernel_new", targs, N,
            (P, P, P, F, F, F, Z, Z, Z, Z), param, grad, mask, *_tv_weights(wx, wy, wz), sx, sy, sz, N)


# ---- adam_upd_kernel.cu -----------------------------------------------------------

def adam_step_size(step: int, beta1: float, beta2: float, lr: float) -> np.float32:
    """The launchers' float step size (adam_upd_kernel.cu:72):
    lr * sqrtf(1 - powf(beta2, step)) / (1 - powf(beta1, step))."""
    libm = C.CDLL("libm.so.6")
    libm.powf.restype = C.c_float
    libm.powf.argtypes = [C.c_float, C.c_float]
    f = np.float32
    b2 = f(libm.powf(f(beta2), f(step)))
    b1 = f(libm.powf(f(beta1), f(step)))
    return f(f(lr) * np.sqrt(f(1) - b2)) / (f(1) - b1)


def _adam(name, param, grad, exp_avg, exp_avg_sq, perlr, step, beta1, beta2, lr, eps):
    N = param.numel()
    ss = adam_step_size(step, beta1, beta2, lr)
    if perlr is None:
        _launch("adam_upd", name, "IfE", N, (P, P, P, P, Z, F, F, F, F),
                param, grad, exp_avg, exp_avg_sq, N, ss, beta1, beta2, eps)
    else:
        _launch("adam_upd", name, "IfE", N, (P, P, P, P, P, Z, F, F, F, F),
                param, grad, exp_avg, exp_avg_sq, perlr, N, ss, beta1, beta2, eps)


def adam_upd(param, grad, exp_avg, exp_avg_sq, step, beta1, beta2, lr, eps) -> None:
    """adam_upd_kernel.cu:60-82, in place."""
    _adam("adam_upd_cuda_kernel", param, grad, exp_avg, exp_avg_sq, None, step, beta1, beta2, lr, eps)


def masked_adam_upd(param, grad, exp_avg, exp_avg_sq, step, beta1, beta2, lr, eps) -> None:
    """adam_upd_kernel.cu:84-106, in place."""
    _adam("masked_adam_upd_cuda_kernel", param, grad, exp_avg, exp_avg_sq, None, step, beta1, beta2, lr, eps)


def adam_upd_with_perlr(param, grad, exp_avg, exp_avg_sq, perlr, step, beta1, beta2, lr, eps) -> None:
    """adam_upd_kernel.cu:108-133, in place."""
    _adam("adam_upd_with_perlr_cuda_kernel", param, grad, exp_avg, exp_avg_sq, perlr, step, beta1, beta2, lr, eps)


# ---- ub360_utils_kernel.cu ---------------------------------------------------------

def cumdist_thres(dist, thres: float):
    """ub360_utils_kernel.cu:33-48: bool [n_rays, n_pts]."""
    import torch

    dist = _f32(dist)
    n_rays, n_pts = dist.shape
    mask = torch.zeros((n_rays, n_pts), dtype=torch.bool, device=dist.device)
    _launch("ub360_utils", "cumdist_thres_cuda_kernel", "IfE", n_rays, (P, F, I, I, P), dist, thres, n_rays, n_pts,
            mask)
    return mask
