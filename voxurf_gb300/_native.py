"""ctypes binding of the C ABI in ``include/voxurf_gb300.h``.

The library must exist: there is no CPU or eager-torch fallback anywhere in
this package.  ``load()`` raises ImportError with the build command when the
shared library is missing, and every call converts a non-zero status into a
RuntimeError (the reference's ops raise through TORCH_CHECK,
render_utils.cpp:46-48).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lib = None
_lock = threading.Lock()

c_int = C.c_int
c_i64 = C.c_int64
c_f32 = C.c_float
c_f64 = C.c_double
c_ptr = C.c_void_p
c_size = C.c_size_t

# name -> argtypes (restype is int unless listed in _RESTYPES)
_SIGNATURES = {
    "vx_version": [],
    "vx_status_string": [c_int],
    "vx_last_cuda_error": [],
    "vx_launch_count": [],
    "vx_cuda_error_string": [c_int],
    "vx_device_error": [c_ptr, c_ptr],
    "vx_scan_scratch_bytes": [c_i64],
    "vx_exclusive_scan_i64": [c_ptr, c_i64, c_ptr, c_ptr, c_size, c_ptr],
    "vx_exclusive_scan_i32": [c_ptr, c_i64, c_ptr, c_ptr, c_size, c_ptr],
    "vx_infer_t_minmax": [c_ptr, c_ptr, c_ptr, c_ptr, c_f32, c_f32, c_i64, c_ptr, c_ptr, c_ptr],
    "vx_infer_n_samples": [c_ptr, c_ptr, c_ptr, c_f32, c_i64, c_ptr, c_ptr],
    "vx_infer_ray_start_dir": [c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_ptr],
    "vx_sample_pts_count": [c_ptr, c_ptr, c_ptr, c_ptr, c_f32, c_f32, c_f32, c_i64, c_ptr, c_ptr, c_ptr, c_ptr,
                            c_ptr, c_size, c_ptr],
    "vx_sample_pts_fill": [c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_f32, c_i64, c_i64, c_ptr, c_ptr, c_ptr,
                           c_ptr, c_ptr],
    "vx_sample_pts_count_noalloc": [c_ptr, c_ptr, c_ptr, c_ptr, c_f32, c_f32, c_f32, c_i64, c_ptr, c_ptr, c_ptr,
                                    c_ptr, c_ptr],
    "vx_maskcache_lookup": [c_ptr, c_i64, c_i64, c_i64, c_ptr, c_i64, c_ptr, c_ptr, c_ptr, c_ptr],
    "vx_camera_rays": [c_ptr, c_f32, c_f32, c_f32, c_f32, c_i64, c_i64, c_int, c_ptr, c_ptr, c_ptr, c_ptr],
    "vx_alpha2weight": [c_ptr, c_ptr, c_i64, c_i64, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr],
    "vx_alpha2weight_backward": [c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_i64, c_ptr, c_ptr, c_ptr,
                                 c_ptr],
    "vx_total_variation_add_grad": [c_ptr, c_ptr, c_f32, c_f32, c_f32, c_int, c_i64, c_i64, c_i64, c_i64, c_int,
                                    c_ptr],
    "vx_total_variation_add_grad_new": [c_ptr, c_ptr, c_ptr, c_f32, c_f32, c_f32, c_int, c_i64, c_i64, c_i64,
                                        c_i64, c_int, c_ptr],
    "vx_adam_upd": [c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_int, c_f32, c_f32, c_f32, c_f32, c_ptr],
    "vx_masked_adam_upd": [c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_int, c_f32, c_f32, c_f32, c_f32, c_ptr],
    "vx_adam_upd_with_perlr": [c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_int, c_f32, c_f32, c_f32, c_f32,
                               c_ptr],
    "vx_adam_step": [c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_f64, c_f64, c_f64, c_f64, c_i64, c_int, c_ptr],
    "vx_relu_bwd_colsum": [c_ptr, c_ptr, c_i64, c_i64, c_int, c_ptr, c_ptr, c_ptr],
    "vx_mlp_tc_pack": [c_ptr, c_i64, c_i64, c_i64, c_ptr, c_ptr],
    "vx_mlp_head_backward": [c_ptr, c_ptr, c_ptr, c_i64, c_i64, c_int, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr],
    "vx_mlp_head": [c_ptr, c_i64, c_i64, c_i64, c_int, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_int, c_ptr],
    "vx_adam_step_multi": [c_int, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_f64, c_f64, c_f64, c_ptr],
    "vx_grid_tv_adam_step": [c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_i64, c_i64, c_i64, c_int,
                             c_int, c_f32, c_int, c_f64, c_f64, c_f64, c_f64, c_i64, c_int, c_ptr],
    "vx_grid_tv_adam_step_touched": [c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_i64, c_i64, c_i64,
                                     c_int, c_int, c_f32, c_int, c_f64, c_f64, c_f64, c_f64, c_i64, c_int, c_ptr,
                                     c_ptr],
    "vx_grid_clear_touched": [c_ptr, c_ptr, c_i64, c_i64, c_ptr],
    "vx_cumdist_thres": [c_ptr, c_i64, c_i64, c_f32, c_ptr, c_ptr],
}

_RESTYPES = {
    "vx_status_string": C.c_char_p,
    "vx_cuda_error_string": C.c_char_p,
    "vx_scan_scratch_bytes": c_size,
    "vx_launch_count": C.c_ulonglong,
}


def library_path() -> str:
    return _build.LIB_PATH


def load():
    """Loads the shared library (once) and declares every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise ImportError(
                f"voxurf_gb300 native library not found at {path}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)")
        lib = C.CDLL(path)
        for name, argtypes in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = _RESTYPES.get(name, c_int)
        _lib = lib
    return _lib


def exported_names() -> list[str]:
    return list(_SIGNATURES)


class VxError(RuntimeError):
    pass


def check(status: int, what: str) -> None:
    if status != 0:
        lib = load()
        msg = lib.vx_status_string(status).decode()
        extra = ""
        if status in (4, 5):
            code = lib.vx_last_cuda_error()
            extra = f" (cuda error {code}: {lib.vx_cuda_error_string(code).decode()})"
        raise VxError(f"{what} failed: {msg}{extra}")


def call(name: str, *args) -> None:
    """Calls entry point `name` and raises on a non-zero status.  An entry
    point without declared argument types is never called (ctypes would pass
    Python ints as 32-bit C ints and truncate pointers)."""
    fn = getattr(load(), name)
    if fn.argtypes is None:
        from . import _abi  # declares the struct-based entry points

        _abi._declare()
        if fn.argtypes is None:
            raise VxError(f"{name}: entry point has no declared signature")
    check(fn(*args), name)


def launch_count() -> int:
    """Kernels launched by libvoxurf_gb300 in this process so far."""
    return int(load().vx_launch_count())


def device_error(stream_ptr: int) -> int:
    code = C.c_int(0)
    check(load().vx_device_error(stream_ptr, C.byref(code)), "vx_device_error")
    return code.value
