/*
 * voxurf_gb300 — C ABI of the GB300-native (sm_103a) Voxurf volume-rendering
 * step.
 *
 * Conventions (all entry points):
 *   - every pointer is a DEVICE pointer unless the comment says "host";
 *   - sizes are int64_t element counts; grids are addressed as (C, X, Y, Z)
 *     plus a layout flag: channel_last = 0 for the reference's [1,C,X,Y,Z]
 *     tensors (Z fastest), 1 for [X,Y,Z,C];
 *   - `stream` is a cudaStream_t (passed as void*); work is enqueued on it and
 *     the call returns without synchronising unless stated;
 *   - the library never allocates device memory; callers pass outputs and
 *     any scratch (sized by the *_scratch_bytes helpers);
 *   - the return value is a status code (VX_OK = 0).  Kernels that detect an
 *     out-of-range index or capacity overflow skip the access and record the
 *     error in a device word read back by vx_device_error().
 *
 * Each entry point names the reference interface it replaces as
 * file:line within the Voxurf project (lib/cuda/... and lib/...).
 */
#ifndef VOXURF_GB300_H
#define VOXURF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VX_ABI_VERSION 1

#define VX_OK 0
#define VX_ERR_ARG 1         /* invalid argument (null pointer, bad size)   */
#define VX_ERR_CAPACITY 2    /* output capacity too small                   */
#define VX_ERR_BOUNDS 3      /* index out of bounds detected on the device  */
#define VX_ERR_LAUNCH 4      /* kernel launch failed                        */
#define VX_ERR_CUDA 5        /* other CUDA runtime error                    */
#define VX_ERR_UNSUPPORTED 6 /* configuration not supported by this build   */

/* ---- library ------------------------------------------------------------ */
int vx_version(void);
const char* vx_status_string(int status);
int vx_last_cuda_error(void);
const char* vx_cuda_error_string(int code);
/* Reads and clears the device error word (synchronises `stream`). */
int vx_device_error(void* stream, int* out_code);

/* ---- prefix sums (replaces N_steps.cumsum + .item(),
 *      lib/cuda/render_utils_kernel.cu:211-212) ----------------------------- */
size_t vx_scan_scratch_bytes(int64_t n);
/* out[0..n]: exclusive prefix sum, out[n] = total. */
int vx_exclusive_scan_i64(const int64_t* in, int64_t n, int64_t* out, void* scratch, size_t scratch_bytes,
                          void* stream);
int vx_exclusive_scan_i32(const int32_t* in, int64_t n, int64_t* out, void* scratch, size_t scratch_bytes,
                          void* stream);

/* ---- render_utils_cuda (lib/cuda/render_utils.cpp:170-184) --------------- */

/* render_utils.cpp:50-58 / render_utils_kernel.cu:12-35,82-104 */
int vx_infer_t_minmax(const float* rays_o, const float* rays_d, const float* xyz_min, const float* xyz_max,
                      float near, float far, int64_t n_rays, float* t_min, float* t_max, void* stream);

/* render_utils.cpp:60-65 / render_utils_kernel.cu:38-55,106-121 */
int vx_infer_n_samples(const float* rays_d, const float* t_min, const float* t_max, float stepdist, int64_t n_rays,
                       int64_t* n_samples, void* stream);

/* render_utils.cpp:67-72 / render_utils_kernel.cu:58-79,123-139 */
int vx_infer_ray_start_dir(const float* rays_o, const float* rays_d, const float* t_min, int64_t n_rays,
                           float* rays_start, float* rays_dir, void* stream);

/* render_utils.cpp:74-85 / render_utils_kernel.cu:196-242, phase 1 of 2:
 * t_min, t_max, N_steps [n_rays] and offsets [n_rays+1] (offsets[n_rays] = M,
 * the total sample count), all on the device; no host synchronisation.
 * scratch: vx_scan_scratch_bytes(n_rays) bytes. */
int vx_sample_pts_count(const float* rays_o, const float* rays_d, const float* xyz_min, const float* xyz_max,
                        float near, float far, float stepdist, int64_t n_rays, float* t_min, float* t_max,
                        int64_t* n_steps, int64_t* offsets, void* scratch, size_t scratch_bytes, void* stream);

/* Phase 2: writes ray_pts [M,3], mask_outbbox [M] (0/1 bytes), ray_id [M],
 * step_id [M] for the offsets of phase 1.  Writes at or beyond `capacity` are
 * skipped and reported as VX_ERR_CAPACITY through vx_device_error(). */
int vx_sample_pts_fill(const float* rays_o, const float* rays_d, const float* xyz_min, const float* xyz_max,
                       const float* t_min, const int64_t* offsets, float stepdist, int64_t n_rays, int64_t capacity,
                       float* ray_pts, uint8_t* mask_outbbox, int64_t* ray_id, int64_t* step_id, void* stream);

/* render_utils.cpp:109-118 / render_utils_kernel.cu:374-424 (grid.MaskGrid,
 * lib/grid.py:233-242).  world: [sz_i, sz_j, sz_k] bytes (0/1). */
int vx_maskcache_lookup(const uint8_t* world, int64_t sz_i, int64_t sz_j, int64_t sz_k, const float* xyz,
                        int64_t n_pts, const float* xyz2ijk_scale, const float* xyz2ijk_shift, uint8_t* out,
                        void* stream);

/* render_utils.cpp:142-149 / render_utils_kernel.cu:577-651.  ray_id sorted
 * ascending with values in [0, n_rays).  Writes weight, T for every sample. */
int vx_alpha2weight(const float* alpha, const int64_t* ray_id, int64_t n_pts, int64_t n_rays, float* weight,
                    float* T, float* alphainv_last, int64_t* i_start, int64_t* i_end, void* stream);

/* render_utils.cpp:151-167 / render_utils_kernel.cu:653-707.  grad [n_pts] is
 * fully written (zero outside [i_start, i_end)). */
int vx_alpha2weight_backward(const float* alpha, const float* weight, const float* T, const float* alphainv_last,
                             const int64_t* i_start, const int64_t* i_end, int64_t n_pts, int64_t n_rays,
                             const float* grad_weights, const float* grad_last, float* grad, void* stream);

/* ---- total_variation_cuda (lib/cuda/total_variation.cpp:29-32) ----------- */

/* total_variation.cpp:15-19 / total_variation_kernel.cu:14-36,68-100.
 * In place on grad.  Keeps the reference's axis weighting (wz on the k and i
 * axes, wy on j, wx unused). */
int vx_total_variation_add_grad(const float* param, float* grad, float wx, float wy, float wz, int dense_mode,
                                int64_t C, int64_t X, int64_t Y, int64_t Z, int channel_last, void* stream);

/* total_variation.cpp:21-26 / total_variation_kernel.cu:39-66,102-134. */
int vx_total_variation_add_grad_new(const float* param, float* grad, const float* mask, float wx, float wy, float wz,
                                    int dense_mode, int64_t C, int64_t X, int64_t Y, int64_t Z, int channel_last,
                                    void* stream);

/* ---- adam_upd_cuda (lib/cuda/adam_upd.cpp:79-86) --------------------------- */

/* adam_upd.cpp:48-58 / adam_upd_kernel.cu:9-22,59-82 (in place). */
int vx_adam_upd(float* param, const float* grad, float* exp_avg, float* exp_avg_sq, int64_t n, int step,
                float beta1, float beta2, float lr, float eps, void* stream);
/* adam_upd.cpp:60-68 / adam_upd_kernel.cu:24-39,84-106. */
int vx_masked_adam_upd(float* param, const float* grad, float* exp_avg, float* exp_avg_sq, int64_t n, int step,
                       float beta1, float beta2, float lr, float eps, void* stream);
/* adam_upd.cpp:70-77 / adam_upd_kernel.cu:41-57,108-133. */
int vx_adam_upd_with_perlr(float* param, const float* grad, float* exp_avg, float* exp_avg_sq, const float* perlr,
                           int64_t n, int step, float beta1, float beta2, float lr, float eps, void* stream);

/* ---- optimizer (lib/utils.py:54-199, Adam with per-voxel lr) -------------- */

/* One utils.Adam update of one parameter (utils.py:169-199), `step` = the
 * parameter's state['step'] after the increment; per_lr may be NULL;
 * zero_grad != 0 also resets grad to 0 (replaces zero_grad, run.py:603). */
int vx_adam_step(float* param, float* grad, float* exp_avg, float* exp_avg_sq, const float* per_lr, int64_t n,
                 double lr, double beta1, double beta2, double eps, int64_t step, int zero_grad, void* stream);

/* Fused dense grid sweep: DenseGrid.total_variation_add_grad(w, w, w, dense)
 * (lib/grid.py:67-78; voxurf_fine.py:403-409; total_variation_kernel.cu:14-36)
 * followed by the utils.Adam update and the gradient reset, in one pass.
 * Reads param_in, writes param_out (must differ when tv_enabled); optional
 * BF16 shadow copy of the new parameter (NULL to skip).  All float pointers
 * 16-byte aligned. */
int vx_grid_tv_adam_step(const float* param_in, float* param_out, float* grad, float* exp_avg, float* exp_avg_sq,
                         const float* per_lr, void* shadow_bf16, int64_t C, int64_t X, int64_t Y, int64_t Z,
                         int channel_last, int tv_enabled, float tv_weight, int tv_dense_mode, double lr,
                         double beta1, double beta2, double eps, int64_t step, int zero_grad, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VOXURF_GB300_H */
