"""ctypes mirrors of the parameter structs in include/voxurf_gb300.h (fused
renderer, smoothing) and thin callers.  Field order and types must match
the header exactly."""
from __future__ import annotations

import ctypes as C

from . import _native

P = C.c_void_p
F = C.c_float
I64 = C.c_int64
I32 = C.c_int32


class GridGeom(C.Structure):
    _fields_ = [("X", I64), ("Y", I64), ("Z", I64), ("xyz_min", F * 3), ("xyz_max", F * 3)]


class FineMarchArgs(C.Structure):
    _fields_ = [
        ("rays_o", P), ("rays_d", P), ("viewdirs", P), ("n_rays", I64), ("near", F), ("stepdist", F),
        ("grid", GridGeom), ("sdf_smooth", P), ("voxel_size", F),
        ("mask", P), ("mask_X", I64), ("mask_Y", I64), ("mask_Z", I64), ("mask_scale", F * 3), ("mask_shift", F * 3),
        ("inv_s", F), ("dist", F), ("fast_color_thres", F), ("max_steps", I64),
        ("rec", P), ("dw_slot", P), ("n1", P), ("n2", P), ("alphainv_last", P),
        ("mask_density", P), ("mask_dgrid", GridGeom), ("mask_act_shift", F), ("mask_voxel_size_ratio", F),
        ("mask_thres", F), ("unit_sphere", I32), ("reserved0", I32),
    ]


class FineCompactArgs(C.Structure):
    _fields_ = [
        ("rays_o", P), ("rays_d", P), ("n_rays", I64), ("near", F), ("stepdist", F), ("xyz_min", F * 3),
        ("xyz_max", F * 3), ("max_steps", I64), ("rec", P), ("n1", P), ("s2_off", P),
        ("ray2", P), ("step2", P), ("slot2", P), ("w2", P), ("alpha2", P), ("pts2", P),
    ]


class FineFeatureCfg(C.Structure):
    _fields_ = [
        ("K", I64), ("disp", F * 4), ("posbase_pe", I64), ("viewbase_pe", I64), ("k_posbase_pe", I64),
        ("k_viewbase_pe", I64), ("center_sdf", I32), ("use_rgbnet_k0", I32), ("k_center_sdf", I32),
        ("k0_channels", I32),
    ]


class FineFeaturesArgs(C.Structure):
    _fields_ = [
        ("n_rows", I64), ("ray2", P), ("pts2", P), ("viewdirs", P), ("grid", GridGeom), ("sdf_smooth", P),
        ("voxel_size", F), ("k0_f32", P), ("k0_bf16", P), ("cfg", FineFeatureCfg), ("ld1", I64), ("ld2", I64),
        ("X1", P), ("X2", P), ("out_bf16", I32), ("normal_out", P), ("n_rows_dev", P),
    ]


class FineCompositeArgs(C.Structure):
    _fields_ = [
        ("n_rays", I64), ("s2_off", P), ("w2", P), ("logit", P), ("klogit", P), ("alphainv_last", P), ("bg", F),
        ("rgb0", P), ("rgbk", P), ("rgbk_raw", P), ("normal2", P), ("step2", P), ("dist", F),
        ("normal_out", P), ("depth_out", P), ("wsum_out", P), ("has_k", I32),
    ]


class FineCompositeBwdArgs(C.Structure):
    _fields_ = [
        ("n_rays", I64), ("s2_off", P), ("w2", P), ("logit", P), ("klogit", P), ("rgbk_raw", P), ("g_rgb0", P),
        ("g_rgbk", P), ("bg", F), ("g_last_in", P), ("d_logit", P), ("d_klogit", P), ("d_w2", P), ("d_last", P),
        ("has_k", I32),
    ]


class FineCompositeLossArgs(C.Structure):
    _fields_ = [
        ("n_rays", I64), ("s2_off", P), ("w2", P), ("logit", P), ("kout", P), ("alphainv_last", P), ("target", P),
        ("bg", F), ("w_main", F), ("w_rgb0", F), ("w_entropy_last", F), ("rgb0", P), ("rgbk", P), ("d_logit", P),
        ("d_kout", P), ("d_w2", P), ("d_last", P), ("loss", P), ("scratch", P), ("scratch_bytes", C.c_size_t),
        ("k_into_logit", I32),
    ]


class FineBackwardArgs(C.Structure):
    _fields_ = [
        ("n_rays", I64), ("n_rows", I64), ("rays_o", P), ("rays_d", P), ("viewdirs", P), ("near", F),
        ("stepdist", F), ("grid", GridGeom), ("sdf_smooth", P), ("voxel_size", F), ("inv_s", F), ("dist", F),
        ("max_steps", I64), ("rec", P), ("dw_slot", P), ("n1", P), ("alphainv_last", P), ("d_last", P),
        ("pts2", P), ("slot2", P), ("dw2", P), ("cfg", FineFeatureCfg), ("ld1", I64), ("ld2", I64), ("dX1", P),
        ("dX2", P), ("in_bf16", I32), ("d_sdf_smooth", P), ("d_k0", P), ("n_rows_dev", P), ("inv_s_dev", P),
        ("k0_touched", P),
    ]


class CoarseMarchArgs(C.Structure):
    _fields_ = [("march", FineMarchArgs), ("grad4", P), ("n2b", P)]


class BgSampleArgs(C.Structure):
    _fields_ = [
        ("rays_o", P), ("rays_d", P), ("jitter", P), ("xyz_min", F * 3), ("xyz_max", F * 3), ("near", F),
        ("far", F), ("stepdist", F), ("dist_thres", F), ("n_samples", I32), ("outbbox_only", I32),
        ("n_rays", I64), ("inner", I32), ("reserved", I32),
    ]


class TvLossArgs(C.Structure):
    _fields_ = [
        ("v", P), ("C", I64), ("X", I64), ("Y", I64), ("Z", I64), ("channel_last", I32), ("mode", I32),
        ("mask", P), ("weight", F), ("loss", P), ("axis_scale", P), ("scratch", P), ("scratch_bytes", C.c_size_t),
    ]


class WomaskFgAlphaArgs(C.Structure):
    _fields_ = [
        ("n", I64), ("pts", P), ("ray_id", P), ("viewdirs", P), ("grid", GridGeom), ("sdf_smooth", P),
        ("voxel_size", F), ("inv_s", F), ("dist", F), ("alpha", P), ("d_alpha", P), ("d_sdf_smooth", P),
    ]


class WomaskBgAlphaArgs(C.Structure):
    _fields_ = [
        ("n", I64), ("pts", P), ("grid", GridGeom), ("density", P), ("act_shift", F), ("interval", F),
        ("alpha", P), ("d_alpha", P), ("d_density", P),
    ]


class WomaskBgFeaturesArgs(C.Structure):
    _fields_ = [
        ("n", I64), ("outer_pts", P), ("pts_org", P), ("ray_id", P), ("viewdirs", P), ("grid", GridGeom),
        ("bg_k0", P), ("posbase_pe", I64), ("viewbase_pe", I64), ("ld", I64), ("X", P), ("bf16", I32),
        ("reserved", I32), ("dX", P), ("d_bg_k0", P),
    ]


class WomaskCompositeArgs(C.Structure):
    _fields_ = [
        ("n_rays", I64), ("fg_off", P), ("w", P), ("logit", P), ("kout", P), ("bg_off", P), ("bw", P),
        ("blogit", P), ("stats", P), ("rgb0", P), ("rgbk", P), ("ainv", P), ("in_marched", P),
        ("bg_marched", P), ("g_rgb0", P), ("g_rgbk", P), ("g_ainv", P), ("d_logit", P), ("d_kout", P),
        ("d_w", P), ("d_blogit", P), ("d_bw", P), ("k_into_logit", I32), ("unclamped_parts", I32),
    ]


class CastJob(C.Structure):
    _fields_ = [("src", P), ("dst", P), ("rows", I32), ("cols", I32), ("src_ld", I32), ("dst_ld", I32)]


class CoarseFeatureCfg(C.Structure):
    _fields_ = [("use_k0", I32), ("geo_rgb_dim", I32), ("posbase_pe", I64), ("viewbase_pe", I64)]


class CoarseFeaturesArgs(C.Structure):
    _fields_ = [
        ("n_rows", I64), ("ray2", P), ("pts2", P), ("viewdirs", P), ("grid", GridGeom), ("grad4", P),
        ("k0_f32", P), ("k0_bf16", P), ("cfg", CoarseFeatureCfg), ("ld", I64), ("X", P), ("out_bf16", I32),
        ("normal_out", P),
    ]


class CoarseCompositeArgs(C.Structure):
    _fields_ = [
        ("n_rays", I64), ("s2_off", P), ("w2", P), ("logit", P), ("bg", F), ("rgb", P), ("rgb_raw", P),
        ("normal2", P), ("step2", P), ("dist", F), ("normal_out", P), ("depth_out", P), ("wsum_out", P),
    ]


class CoarseCompositeBwdArgs(C.Structure):
    _fields_ = [
        ("n_rays", I64), ("s2_off", P), ("w2", P), ("logit", P), ("rgb_raw", P), ("g_rgb", P), ("bg", F),
        ("d_logit", P), ("d_w2", P),
    ]


class CoarseBackwardArgs(C.Structure):
    _fields_ = [
        ("n_rays", I64), ("n_rows", I64), ("rays_o", P), ("rays_d", P), ("viewdirs", P), ("near", F),
        ("stepdist", F), ("grid", GridGeom), ("sdf_smooth", P), ("grad4", P), ("voxel_size", F), ("inv_s", F),
        ("dist", F), ("max_steps", I64), ("rec", P), ("dw_slot", P), ("n2b", P), ("alphainv_last", P),
        ("d_last", P), ("pts2", P), ("slot2", P), ("dw2", P), ("cfg", CoarseFeatureCfg), ("ld", I64), ("dX", P),
        ("in_bf16", I32), ("d_sdf_smooth", P), ("d_grad4", P), ("d_k0", P), ("d_grad2", P),
    ]


class MlpTcArgs(C.Structure):
    _fields_ = [
        ("X", P), ("ldx", I64), ("K0", I64), ("n_rows", I64), ("width", I64), ("W0p", P), ("W1p", P), ("W2p", P),
        ("b0", P), ("b1", P), ("b2", P), ("Whp", P), ("bh", P), ("add", P), ("out", P), ("cols", P),
        ("ld_cols", I64), ("pipeline", I32), ("reserved0", I32),
    ]


class MlpPackJob(C.Structure):
    _fields_ = [("src", P), ("ld", I64), ("N", I64), ("K", I64), ("Np", I64), ("Kp", I64), ("transpose", I32),
                ("mode", I32), ("dst", P)]


class MlpTrainFwdArgs(C.Structure):
    _fields_ = [
        ("n_rows", I64), ("n_rows_dev", P), ("rows_cap", I64), ("width", I64), ("n_hidden", I64), ("K0", I64),
        ("X", P), ("ldx", I64), ("W0p", P), ("Wp", P), ("bias", P), ("Whp", P), ("bh", P), ("out", P),
        ("cols", P), ("ld_cols", I64), ("H", P), ("relu", P),
    ]


class MlpTrainBwdArgs(C.Structure):
    _fields_ = [
        ("n_rows", I64), ("n_rows_dev", P), ("rows_cap", I64), ("width", I64), ("n_hidden", I64), ("K0", I64),
        ("dY", P), ("Wh", P), ("relu", P), ("WTp", P), ("W0Tp", P), ("dZ", P), ("dYT", P), ("dX", P),
        ("ld_dx", I64), ("dx_bf16", I32), ("dbh_part", P), ("dbh_part_cap", I64),
    ]


class MlpWgradArgs(C.Structure):
    _fields_ = [
        ("n_rows", I64), ("n_rows_dev", P), ("A", P), ("WA", I64), ("B", P), ("WB", I64), ("ldb", I64),
        ("b_rows", I32), ("ones", I32), ("part", P), ("part_cap", I64),
    ]


class MlpReduceJob(C.Structure):
    _fields_ = [
        ("part", P), ("n_part", I64), ("WA", I64), ("NC", I64), ("kind", I32), ("reserved", I32), ("WB", I64),
        ("n_out", I64), ("w", P), ("b", P), ("bh_part", P), ("n_bh", I64),
    ]


class MlpF32RowGemmArgs(C.Structure):
    _fields_ = [
        ("M", I64), ("m_dev", P), ("K", I64), ("A", P), ("lda", I64), ("Bt", P), ("Np", I64), ("mode", I32),
        ("reserved", I32), ("bias", P), ("H", P), ("ldh", I64), ("C", P), ("ldc", I64), ("n_store", I64),
        ("colsum", P), ("colsum_cap", I64),
    ]


class MlpF32WgradArgs(C.Structure):
    _fields_ = [
        ("rows", I64), ("rows_dev", P), ("A", P), ("lda", I64), ("B", P), ("ldb", I64), ("M", I64), ("N", I64),
        ("part", P), ("part_cap", I64),
    ]


class MlpSumJob(C.Structure):
    _fields_ = [("part", P), ("n_part", I64), ("part_stride", I64), ("part_ld", I64), ("rows", I64), ("cols", I64),
                ("out", P), ("out_ld", I64)]


class SceneDesc(C.Structure):
    _fields_ = [
        ("grid", GridGeom), ("sdf_smooth", P), ("k0", P), ("k0_bf16", I32), ("voxel_size", F), ("mask", P),
        ("mask_X", I64), ("mask_Y", I64), ("mask_Z", I64), ("mask_scale", F * 3), ("mask_shift", F * 3),
        ("inv_s", F), ("stepdist", F), ("near", F), ("bg", F), ("fast_color_thres", F), ("occ", P),
        ("occ_X", I64), ("occ_Y", I64), ("occ_Z", I64), ("occ_block", I32),
        ("mask_density", P), ("mask_dgrid", GridGeom), ("mask_act_shift", F), ("mask_voxel_size_ratio", F),
        ("mask_thres", F),
    ]


class ViewChunk(C.Structure):
    _fields_ = [
        ("c2w", F * 12), ("fx", F), ("fy", F), ("cx", F), ("cy", F), ("W", I32), ("inverse_y", I32),
        ("scene", I32), ("reserved", I32), ("pix0", I64), ("ray0", I64), ("out0", I64),
    ]


_STRUCT_FNS = {
    "vx_coarse_march": CoarseMarchArgs,
    "vx_coarse_features": CoarseFeaturesArgs,
    "vx_coarse_composite": CoarseCompositeArgs,
    "vx_coarse_composite_backward": CoarseCompositeBwdArgs,
    "vx_coarse_backward": CoarseBackwardArgs,
    "vx_fine_march": FineMarchArgs,
    "vx_fine_compact": FineCompactArgs,
    "vx_fine_features": FineFeaturesArgs,
    "vx_fine_composite": FineCompositeArgs,
    "vx_fine_composite_backward": FineCompositeBwdArgs,
    "vx_fine_composite_loss": FineCompositeLossArgs,
    "vx_fine_backward": FineBackwardArgs,
    "vx_mlp_tc_forward": MlpTcArgs,
    "vx_mlp_train_forward": MlpTrainFwdArgs,
    "vx_mlp_train_backward": MlpTrainBwdArgs,
    "vx_mlp_train_wgrad": MlpWgradArgs,
    "vx_mlp_f32_rowgemm": MlpF32RowGemmArgs,
    "vx_mlp_f32_wgrad": MlpF32WgradArgs,
    "vx_womask_fg_alpha": WomaskFgAlphaArgs,
    "vx_womask_bg_alpha": WomaskBgAlphaArgs,
    "vx_womask_bg_features": WomaskBgFeaturesArgs,
    "vx_womask_composite": WomaskCompositeArgs,
}

_SERVE_SIGNATURES = {
    "vx_serve_rays": [P, I32, I64, P, P, P, P, P, P],
    "vx_serve_march": ["scenes", I32, P, P, P, P, I64, I64, P, P, P, P],
    "vx_serve_rows": [P, I64, P, I64, P],
    "vx_mask_occupancy": [P, I64, I64, I64, I32, P, P],
    "vx_serve_features": ["scenes", I32, C.POINTER(FineFeatureCfg), P, P, P, P, I64, P, P, P, I64, P, I64, I64, P,
                          P, I32, I32, P],
    "vx_serve_composite": ["scenes", I32, P, I64, I64, P, P, P, P, P, P, P, P, P],
}

_declared = False


def _declare():
    global _declared
    if _declared:
        return
    lib = _native.load()
    for name, st in _STRUCT_FNS.items():
        fn = getattr(lib, name)
        fn.argtypes = [C.POINTER(st), C.c_void_p]
        fn.restype = C.c_int
    lib.vx_smooth3d.argtypes = [P, P, P, P, I64, I64, I64, P, C.c_int, P]
    lib.vx_smooth3d.restype = C.c_int
    lib.vx_smooth3d_adjoint.argtypes = [P, P, P, P, I64, I64, I64, P, C.c_int, C.c_int, P]
    lib.vx_smooth3d_adjoint.restype = C.c_int
    for name in ("vx_grid_sample", "vx_grid_sample_backward"):
        fn = getattr(lib, name)
        fn.argtypes = [P, I64, C.c_int, C.POINTER(GridGeom), P, I64, P, P]
        fn.restype = C.c_int
    lib.vx_sdf_field.argtypes = [P, C.POINTER(GridGeom), P, P, I64, F, P, P]
    lib.vx_sdf_field.restype = C.c_int
    lib.vx_density_mask.argtypes = [P, C.POINTER(GridGeom), F, F, F, P, I64, P, P]
    lib.vx_density_mask.restype = C.c_int
    lib.vx_hit_coarse_geo.argtypes = [C.POINTER(FineMarchArgs), P, P]
    lib.vx_hit_coarse_geo.restype = C.c_int
    lib.vx_cast_rows_bf16.argtypes = [C.POINTER(CastJob), I32, P]
    lib.vx_cast_rows_bf16.restype = C.c_int
    lib.vx_mlp_train_pack.argtypes = [C.POINTER(MlpPackJob), C.c_int, P]
    lib.vx_mlp_train_pack.restype = C.c_int
    lib.vx_mlp_train_reduce.argtypes = [C.POINTER(MlpReduceJob), C.c_int, P]
    lib.vx_mlp_train_reduce.restype = C.c_int
    lib.vx_mlp_train_wgrad_multi.argtypes = [C.POINTER(MlpWgradArgs), P, C.c_int, P]
    lib.vx_mlp_train_wgrad_multi.restype = C.c_int
    lib.vx_mlp_wgrad_split.argtypes = [C.POINTER(MlpWgradArgs), C.c_int, P]
    lib.vx_mlp_wgrad_split.restype = C.c_int
    lib.vx_mlp_wgrad_grid.argtypes = [I64]
    lib.vx_mlp_wgrad_grid.restype = C.c_size_t
    lib.vx_mlp_f32_rowgemm_grid.argtypes = [I64]
    lib.vx_mlp_f32_rowgemm_grid.restype = C.c_size_t
    lib.vx_mlp_f32_wgrad_grid.argtypes = [I64]
    lib.vx_mlp_f32_wgrad_grid.restype = C.c_size_t
    lib.vx_mlp_f32_reduce.argtypes = [C.POINTER(MlpSumJob), C.c_int, P]
    lib.vx_mlp_f32_reduce.restype = C.c_int
    lib.vx_bg_samples_count.argtypes = [C.POINTER(BgSampleArgs), P, P, P, C.c_size_t, P]
    lib.vx_bg_samples_count.restype = C.c_int
    lib.vx_bg_samples_fill.argtypes = [C.POINTER(BgSampleArgs), P, I64, P, P, P, P, P]
    lib.vx_bg_samples_fill.restype = C.c_int
    lib.vx_sdf_gradient_grid.argtypes = [P, P, I64, I64, I64, F, C.c_int, P]
    lib.vx_sdf_gradient_grid.restype = C.c_int
    lib.vx_sdf_gradient_grid_adjoint.argtypes = [P, P, I64, I64, I64, F, C.c_int, C.c_int, P]
    lib.vx_sdf_gradient_grid_adjoint.restype = C.c_int
    lib.vx_fine_composite_loss_scratch_bytes.argtypes = [I64]
    lib.vx_fine_composite_loss_scratch_bytes.restype = C.c_size_t
    lib.vx_smooth_grad_tv_scratch_bytes.argtypes = [I64, I64, I64]
    lib.vx_smooth_grad_tv_scratch_bytes.restype = C.c_size_t
    lib.vx_smooth_grad_tv.argtypes = [P, P, I64, I64, I64, F, P, P, P]
    lib.vx_smooth_grad_tv.restype = C.c_int
    lib.vx_tv_loss_scratch_bytes.argtypes = [I64, I64, I64]
    lib.vx_tv_loss_scratch_bytes.restype = C.c_size_t
    lib.vx_tv_loss.argtypes = [C.POINTER(TvLossArgs), P]
    lib.vx_tv_loss.restype = C.c_int
    lib.vx_tv_loss_backward.argtypes = [C.POINTER(TvLossArgs), P, P, P]
    lib.vx_tv_loss_backward.restype = C.c_int
    SP = C.POINTER(SceneDesc)
    for name, args in _SERVE_SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = [SP if a == "scenes" else a for a in args]
        fn.restype = C.c_int
    _declared = True


def grid_sample(name: str, grid_ptr, C_: int, channel_last: bool, geom: GridGeom, xyz_ptr, n: int, out_ptr,
                stream: int) -> None:
    _declare()
    fn = getattr(_native.load(), name)
    _native.check(fn(grid_ptr, C_, int(channel_last), C.byref(geom), xyz_ptr, n, out_ptr, stream), name)


def call_struct(name: str, args: C.Structure, stream: int) -> None:
    _declare()
    fn = getattr(_native.load(), name)
    _native.check(fn(C.byref(args), stream), name)


def call(name: str, *args) -> None:
    _declare()
    _native.call(name, *args)


def struct_names() -> list[str]:
    return list(_STRUCT_FNS) + ["vx_smooth3d", "vx_smooth3d_adjoint", "vx_grid_sample", "vx_grid_sample_backward",
                                "vx_sdf_gradient_grid", "vx_sdf_gradient_grid_adjoint",
                                "vx_smooth_grad_tv_scratch_bytes", "vx_smooth_grad_tv",
                                "vx_sdf_field", "vx_density_mask", "vx_hit_coarse_geo", "vx_bg_samples_count",
                                "vx_bg_samples_fill", "vx_cast_rows_bf16", "vx_mlp_train_pack",
                                "vx_mlp_train_reduce", "vx_mlp_wgrad_grid", "vx_mlp_train_wgrad_multi", "vx_mlp_wgrad_split", "vx_mlp_f32_rowgemm_grid",
                                "vx_mlp_f32_wgrad_grid", "vx_mlp_f32_reduce",
                                "vx_fine_composite_loss_scratch_bytes", "vx_tv_loss_scratch_bytes", "vx_tv_loss",
                                "vx_tv_loss_backward"] + list(_SERVE_SIGNATURES)
