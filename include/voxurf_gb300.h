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
#define VX_ERR_TOO_LARGE 7   /* size above the fixed maximum of a no-allocation entry point */
#define VX_ERR_TIMEOUT 8     /* a bounded on-device wait expired (reported via vx_device_error) */

/* Largest ray count vx_sample_pts_count_noalloc accepts. */
#define VX_NOALLOC_MAX_RAYS 4194304

/* ---- library ------------------------------------------------------------ */
int vx_version(void);
const char* vx_status_string(int status);
int vx_last_cuda_error(void);
const char* vx_cuda_error_string(int code);
/* Number of kernels this library has launched in the process so far. */
unsigned long long vx_launch_count(void);
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

/* No counterpart in the reference.  Phase 1 for callers that cannot
 * allocate device memory: hosts that only receive device pointers for their
 * inputs and outputs from another runtime (an FFI binding without access to
 * a CUDA allocator) and render loops that reserve all device memory up
 * front and must not allocate per frame.  Same outputs as
 * vx_sample_pts_count; the scan scratch is a static array inside the library
 * (16 KB per device, held until the process exits), so n_rays is limited to
 * VX_NOALLOC_MAX_RAYS (larger sizes return VX_ERR_TOO_LARGE without touching
 * the GPU).  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  The address is kept for the life of the
 * process: a caller that destroys and recreates the device's primary
 * context (cudaDeviceReset) must not call this entry point afterwards.  All
 * calls on a device share the array: calls that overlap on the GPU race.  No
 * cudaMalloc/cudaFree or other allocating call is made. */
int vx_sample_pts_count_noalloc(const float* rays_o, const float* rays_d, const float* xyz_min,
                                const float* xyz_max, float near, float far, float stepdist, int64_t n_rays,
                                float* t_min, float* t_max, int64_t* n_steps, int64_t* offsets, void* stream);

/* Phase 2: writes ray_pts [M,3], mask_outbbox [M] (0/1 bytes), ray_id [M],
 * step_id [M] for the offsets of phase 1.  Writes at or beyond `capacity` are
 * skipped and reported as VX_ERR_CAPACITY through vx_device_error(). */
int vx_sample_pts_fill(const float* rays_o, const float* rays_d, const float* xyz_min, const float* xyz_max,
                       const float* t_min, const int64_t* offsets, float stepdist, int64_t n_rays, int64_t capacity,
                       float* ray_pts, uint8_t* mask_outbbox, int64_t* ray_id, int64_t* step_id, void* stream);

/* Rays of one pinhole view (get_rays + viewdirs, lib/voxurf_fine.py:1001-1029,
 * 1062-1067): c2w_host is a HOST row-major 3x4 (or 4x4) camera-to-world
 * matrix; pixel centres +0.5; inverse_y = 1 for OpenCV axes.  Outputs
 * [H*W,3] each, row-major over (row j, column i). */
int vx_camera_rays(const float* c2w_host, float fx, float fy, float cx, float cy, int64_t H, int64_t W,
                   int inverse_y, float* rays_o, float* rays_d, float* viewdirs, void* stream);

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

/* utils.Adam (utils.py:169-199) over up to 48 tensors in one launch (the
 * MLP weights and biases).  params/grads/exp_avgs/exp_avg_sqs are HOST arrays
 * of device pointers; sizes, lrs, steps (state['step'] after the increment)
 * HOST arrays of n_tensors entries. */
int vx_adam_step_multi(int n_tensors, float* const* params, float* const* grads, float* const* exp_avgs,
                       float* const* exp_avg_sqs, const int64_t* sizes, const double* lrs, const int64_t* steps,
                       double beta1, double beta2, double eps, void* stream);

/* Colour-MLP backward helper (rgbnet/k_rgbnet ReLU stacks,
 * lib/voxurf_fine.py:132-187): dz = dh * (h > 0) and colsum += sum over rows
 * of dz (the bias gradient), one pass; h == NULL skips the ReLU (bias
 * gradient of the last layer).  dtype 0: float32, 1: bfloat16 for dh/h/dz;
 * colsum [N] FP32, accumulated. */
int vx_relu_bwd_colsum(const void* dh, const void* h, int64_t M, int64_t N, int dtype, void* dz, float* colsum,
                       void* stream);

/* Backward of a colour MLP's 3-output layer (out = W h + b over [M,N] rows
 * h of the last ReLU layer) fused with that ReLU's backward: dW [3,N] +=
 * dout^T h, db [3] += column sums of dout, dz = (h > 0) * (dout W) [M,N]
 * and db_prev [N] += column sums of dz.  dout FP32 [M,3]; h, dz in dtype
 * (0 FP32, 1 BF16), N a multiple of 16 bytes / element size, <= 256. */
int vx_mlp_head_backward(const float* dout, const void* h, const float* W, int64_t M, int64_t N, int dtype, void* dz,
                         float* dW, float* db, float* db_prev, void* stream);

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
/* The same sweep for a gradient that is zero outside the voxels marked in
 * touched [X*Y*Z] (uint8, 4-byte aligned; channel-last 12-channel grids
 * and 1-channel grids with Z % 4 == 0): unmarked voxels take gradient 0
 * without reading it, and zero_grad resets only the marked ones (the marks
 * stay set: clearing them is a memset).  The result equals
 * vx_grid_tv_adam_step on the same (dense) gradient. */
int vx_grid_tv_adam_step_touched(const float* param_in, float* param_out, float* grad, float* exp_avg,
                                 float* exp_avg_sq, const float* per_lr, void* shadow_bf16, int64_t C, int64_t X,
                                 int64_t Y, int64_t Z, int channel_last, int tv_enabled, float tv_weight,
                                 int tv_dense_mode, double lr, double beta1, double beta2, double eps, int64_t step,
                                 int zero_grad, const uint8_t* touched, void* stream);
/* Zeroes the C gradient values of every voxel marked in touched [n_vox]
 * (16-byte aligned) and clears the marks: the reset of a gradient that is
 * nonzero only at marked voxels, at the cost of one read of the marks. */
int vx_grid_clear_touched(float* grad, uint8_t* touched, int64_t n_vox, int64_t C, void* stream);

/* ---- Gaussian smoothing (Voxurf._gaussian_3dconv, lib/voxurf_fine.py:246-258,
 *      used at voxurf_fine.py:638 / voxurf_coarse.py:531) ------------------- */

/* out = G * in on an [X,Y,Z] grid with replicate padding; taps_host: the
 * normalised 1-D kernel (ksize odd, <= 9; the 3-D kernel is its cube).
 * tmp1/tmp2: unused (the three passes run in one sweep); may be NULL. */
int vx_smooth3d(const float* in, float* out, float* tmp1, float* tmp2, int64_t X, int64_t Y, int64_t Z,
                const float* taps_host, int ksize, void* stream);
/* grad_in (+)= G^T grad_out (exact adjoint of the clamped convolution). */
int vx_smooth3d_adjoint(const float* grad_out, float* grad_in, float* tmp1, float* tmp2, int64_t X, int64_t Y,
                        int64_t Z, const float* taps_host, int ksize, int accumulate, void* stream);

/* ---- fused fine-model rendering (Voxurf.forward, lib/voxurf_fine.py:620-802) */

typedef struct {
  int64_t X, Y, Z;     /* grid size (world_size)                   */
  float xyz_min[3];    /* model xyz_min (host copy of the buffer)  */
  float xyz_max[3];
} vx_grid_geom;

/* DenseGrid.forward (lib/grid.py:47-58): trilinear lookup with
 * F.grid_sample(align_corners=True, padding zeros) semantics.  grid: C
 * channels, channel-first ([C,X,Y,Z]) or channel-last ([X,Y,Z,C]);
 * xyz [n,3] world coordinates; out [n,C]. */
int vx_grid_sample(const float* grid, int64_t C, int channel_last, const vx_grid_geom* geom, const float* xyz,
                   int64_t n_pts, float* out, void* stream);
/* Adjoint: grad_grid += scatter of grad_out [n,C] (atomic adds). */
int vx_grid_sample_backward(const float* grad_out, int64_t C, int channel_last, const vx_grid_geom* geom,
                            const float* xyz, int64_t n_pts, float* grad_grid, void* stream);

/* Dense field for mesh extraction: extract_fields (lib/dvgo_ori.py:679-693)
 * with query_func = grid_sampler(pts, sign * sdf) (voxurf_fine.py:894-910,
 * voxurf_coarse.py:652-665).  out [R,R,R] (z fastest) = sign x trilinear
 * lookup of the 1-channel [X,Y,Z] grid at the lattice point
 * (linspace(bound_min[a], bound_max[a], R) per axis, as torch.linspace
 * forms it).  R <= 2048. */
int vx_sdf_field(const float* sdf, const vx_grid_geom* grid, const float* bound_min, const float* bound_max,
                 int64_t R, float sign, float* out, void* stream);

/* Ray march: sample_ray (voxurf_fine.py:593-617) + mask (:631-636) +
 * grid_sampler with FD gradient (:640, 502-534) + neus alpha (:643, 463-500)
 * + alpha/weight compaction (:647-676) + Alphas2Weights (:667, 981-988). */
typedef struct {
  const float* rays_o;      /* [N,3] */
  const float* rays_d;      /* [N,3] */
  const float* viewdirs;    /* [N,3] */
  int64_t n_rays;
  float near;
  float stepdist;           /* stepsize * voxel_size                           */
  vx_grid_geom grid;
  const float* sdf_smooth;  /* [X,Y,Z] smoothed SDF                            */
  float voxel_size;
  const uint8_t* mask;      /* optional MaskGrid bool grid (NULL: none)        */
  int64_t mask_X, mask_Y, mask_Z;
  float mask_scale[3], mask_shift[3];
  float inv_s;              /* 1 / s_val                                       */
  float dist;               /* stepsize * voxel_size                           */
  float fast_color_thres;
  int64_t max_steps;        /* slot capacity per ray (>= every ray's N_steps)  */
  void* rec;                /* out [N*max_steps] 16-byte records               */
  float* dw_slot;           /* out [N*max_steps] (zeroed at written slots)     */
  int32_t* n1;              /* out [N] kept samples (alpha > thres, to stop)   */
  int32_t* n2;              /* out [N] shaded samples (weight > thres)         */
  float* alphainv_last;     /* out [N]                                         */
  /* optional MaskCache density mask (voxurf_fine.py:917-942; exclusive with
     `mask`): a sample is kept when 1 - exp(-softplus(trilinear(
     mask_density) + mask_act_shift) * mask_voxel_size_ratio) >= mask_thres */
  const float* mask_density; /* [X,Y,Z] max-pooled density (NULL: none)       */
  vx_grid_geom mask_dgrid;
  float mask_act_shift, mask_voxel_size_ratio, mask_thres;
  /* 1: keep only the samples with |p| < 1 (torch.linalg.norm in float32), the
     foreground of the maskless coarse model (voxurf_womask_coarse.py:625-628) */
  int32_t unit_sphere;
  int32_t reserved0;
} vx_fine_march_args;
int vx_fine_march(const vx_fine_march_args* args, void* stream);

/* MaskCache.forward (voxurf_fine.py:930-942): out[i] = 1 when
 * 1 - exp(-softplus(trilinear(density, xyz[i]) + act_shift) *
 * voxel_size_ratio) >= thres.  density [X,Y,Z] (already max-pooled). */
int vx_density_mask(const float* density, const vx_grid_geom* dgrid, float act_shift, float voxel_size_ratio,
                    float thres, const float* xyz, int64_t n, uint8_t* out, void* stream);
/* Voxurf.hit_coarse_geo (voxurf_fine.py:579-591): hit[r] = 1 when any
 * in-bbox sample of ray r (sample_pts_on_rays with far = 1e9) lies in the
 * mask of `args` (bool `mask` or `mask_density`; one of them is required).
 * Reads rays_o, rays_d, n_rays, near, stepdist, grid and the mask fields. */
int vx_hit_coarse_geo(const vx_fine_march_args* args, uint8_t* hit, void* stream);

/* Dense rows of the shaded samples, ray-major (s2_off = exclusive scan of n2,
 * [N+1], e.g. from vx_exclusive_scan_i32). */
typedef struct {
  const float* rays_o;
  const float* rays_d;
  int64_t n_rays;
  float near, stepdist;
  float xyz_min[3], xyz_max[3];
  int64_t max_steps;
  const void* rec;
  const int32_t* n1;
  const int64_t* s2_off;
  int32_t* ray2;    /* out [S2] */
  int32_t* step2;   /* out [S2] */
  int32_t* slot2;   /* out [S2] */
  float* w2;        /* out [S2] */
  float* alpha2;    /* out [S2] */
  float* pts2;      /* out [S2,3] */
} vx_fine_compact_args;
int vx_fine_compact(const vx_fine_compact_args* args, void* stream);

/* Feature layout of the two color MLPs (voxurf_fine.py:694-739). */
typedef struct {
  int64_t K;              /* number of displacements in sorted(set(grad_feat+k_grad_feat)) */
  float disp[4];          /* the displacements; 1.0 must be present           */
  int64_t posbase_pe, viewbase_pe, k_posbase_pe, k_viewbase_pe;
  int32_t center_sdf, use_rgbnet_k0, k_center_sdf;
  int32_t k0_channels;    /* 12 */
} vx_fine_feature_cfg;

typedef struct {
  int64_t n_rows;
  const int32_t* ray2;
  const float* pts2;
  const float* viewdirs;
  vx_grid_geom grid;
  const float* sdf_smooth;
  float voxel_size;
  const float* k0_f32;      /* [X,Y,Z,12] FP32, or NULL                        */
  const void* k0_bf16;      /* [X,Y,Z,12] BF16, or NULL                        */
  vx_fine_feature_cfg cfg;
  int64_t ld1, ld2;         /* row strides (elements) of X1 and X2, >= their
                               column counts; columns beyond them are zeroed */
  void* X1;                 /* out rgbnet input [S2, ld1]                      */
  void* X2;                 /* out k_rgbnet input [S2, ld2] without the rgbnet logits */
  int32_t out_bf16;         /* X1/X2 element type: 0 FP32, 1 BF16              */
  float* normal_out;        /* optional [S2,3] FD gradient (render_grad)       */
  const int64_t* n_rows_dev; /* optional DEVICE row count: rows at or beyond
                               it are skipped (n_rows is then a capacity)    */
} vx_fine_features_args;
int vx_fine_features(const vx_fine_features_args* args, void* stream);

/* segment_coo compositing (voxurf_fine.py:753-777). */
typedef struct {
  int64_t n_rays;
  const int64_t* s2_off;
  const float* w2;
  const float* logit;       /* [S2,3] rgbnet logits                            */
  const float* klogit;      /* [S2,3] k-branch logits, or NULL                 */
  const float* alphainv_last;
  float bg;
  float* rgb0;              /* out [N,3] rgb_marched0                          */
  float* rgbk;              /* out [N,3] rgb_marched (clamped), if klogit      */
  float* rgbk_raw;          /* out [N,3] before the clamp, if klogit           */
  const float* normal2;     /* optional [S2,3]                                 */
  const int32_t* step2;     /* optional, for depth                             */
  float dist;
  float* normal_out;        /* optional [N,3]                                  */
  float* depth_out;         /* optional [N]                                    */
  float* wsum_out;          /* optional [N]                                    */
  int32_t has_k;            /* 1: the k-branch is used (klogit/rgbk/rgbk_raw)  */
} vx_fine_composite_args;
int vx_fine_composite(const vx_fine_composite_args* args, void* stream);

typedef struct {
  int64_t n_rays;
  const int64_t* s2_off;
  const float* w2;
  const float* logit;
  const float* klogit;
  const float* rgbk_raw;
  const float* g_rgb0;      /* [N,3] or NULL */
  const float* g_rgbk;      /* [N,3] or NULL */
  float bg;
  const float* g_last_in;   /* [N] extra gradient of alphainv_last, or NULL    */
  float* d_logit;           /* out [S2,3] */
  float* d_klogit;          /* out [S2,3] */
  float* d_w2;              /* out [S2]   */
  float* d_last;            /* out [N]    */
  int32_t has_k;            /* 1: the k-branch is used                         */
} vx_fine_composite_bwd_args;
int vx_fine_composite_backward(const vx_fine_composite_bwd_args* args, void* stream);

/* Training-step compositing, photometric loss and compositing backward in
 * one pass (replaces vx_fine_composite + the torch loss of run.py:604-610,
 * 627 + vx_fine_composite_backward for the fine model with its k-branch).
 * loss = w_main * mse(rgb_marched, target) + w_rgb0 * mse(rgb_marched0,
 * target) + w_entropy_last * entropy(clamp(alphainv_last[N-1], 1e-6,
 * 1-1e-6)); the k-branch logit is logit + kout.  Outputs: rgb0 / rgbk (the
 * clamped rgb_marched), the gradients of logit (plus that of the k-branch
 * logit when k_into_logit), of kout, of the shaded weights and of
 * alphainv_last, and the loss (one float, sums in a fixed order).
 * scratch >= vx_fine_composite_loss_scratch_bytes(n_rays) device bytes.
 * The per-row pointers may be NULL when s2_off[n_rays] is 0. */
typedef struct {
  int64_t n_rays;           /* > 0                                              */
  const int64_t* s2_off;
  const float* w2;
  const float* logit;       /* [S2,3] rgbnet logits                            */
  const float* kout;        /* [S2,3] k_rgbnet output                          */
  const float* alphainv_last;
  const float* target;      /* [N,3]                                           */
  float bg;
  float w_main, w_rgb0, w_entropy_last;
  float* rgb0;              /* out [N,3]                                       */
  float* rgbk;              /* out [N,3]                                       */
  float* d_logit;           /* out [S2,3]                                      */
  float* d_kout;            /* out [S2,3]                                      */
  float* d_w2;              /* out [S2]                                        */
  float* d_last;            /* out [N]                                         */
  float* loss;              /* out [1]                                         */
  void* scratch;
  size_t scratch_bytes;
  int32_t k_into_logit;     /* 1: d_logit also receives the k-branch gradient  */
} vx_fine_composite_loss_args;
size_t vx_fine_composite_loss_scratch_bytes(int64_t n_rays);
int vx_fine_composite_loss(const vx_fine_composite_loss_args* args, void* stream);

/* Backward of the march + features: gradients of the smoothed SDF grid
 * (accumulated into d_sdf_smooth) and of k0 (accumulated, channel-last). */
typedef struct {
  int64_t n_rays;
  int64_t n_rows;
  const float* rays_o;
  const float* rays_d;
  const float* viewdirs;
  float near, stepdist;
  vx_grid_geom grid;
  const float* sdf_smooth;
  float voxel_size;
  float inv_s, dist;
  int64_t max_steps;
  const void* rec;
  float* dw_slot;
  const int32_t* n1;
  const float* alphainv_last;
  const float* d_last;      /* [N] gradient of alphainv_last                    */
  const float* pts2;
  const int32_t* slot2;
  const float* dw2;         /* [S2] gradient of the shaded weights              */
  vx_fine_feature_cfg cfg;
  int64_t ld1, ld2;
  const void* dX1;
  const void* dX2;
  int32_t in_bf16;
  float* d_sdf_smooth;      /* [X,Y,Z] accumulated                              */
  float* d_k0;              /* [X,Y,Z,12] accumulated                           */
  const int64_t* n_rows_dev; /* optional DEVICE row count (as vx_fine_features) */
  const float* inv_s_dev;   /* optional DEVICE inv_s (overrides inv_s)          */
  uint8_t* k0_touched;      /* optional [X*Y*Z]: set to 1 at every k0 voxel the
                               scatter adds to (vx_grid_tv_adam_step_touched) */
} vx_fine_backward_args;
int vx_fine_backward(const vx_fine_backward_args* args, void* stream);

/* ---- dense SDF gradient grid (Voxurf.neus_sdf_gradient 'interpolate',
 *      lib/voxurf_fine.py:440-450, lib/voxurf_coarse.py:323-332) ----------- */

/* G = central differences / (2 voxel_size) on interior points, 0 on the
 * boundary slab of each axis.  layout 0: [3,X,Y,Z]; layout 1: [X,Y,Z,4]. */
int vx_sdf_gradient_grid(const float* sdf, float* G, int64_t X, int64_t Y, int64_t Z, float voxel_size, int layout,
                         void* stream);
/* d_sdf (+)= adjoint of vx_sdf_gradient_grid applied to dG. */
int vx_sdf_gradient_grid_adjoint(const float* dG, float* d_sdf, int64_t X, int64_t Y, int64_t Z, float voxel_size,
                                 int layout, int accumulate, void* stream);
/* smooth_grad_tv (voxurf_fine.py:417-420, run.py:621-622) on a [X,Y,Z,4]
 * gradient grid: dG = -grad_scale * (S(G) - G) on the non-empty voxels
 * (mask bytes, NULL = all), S the normalised [1,2,1]^3 kernel with
 * replicate padding; partial[b] = per-block sums of (S(G)-G)^2. */
size_t vx_smooth_grad_tv_scratch_bytes(int64_t X, int64_t Y, int64_t Z);
int vx_smooth_grad_tv(const float* G, const uint8_t* mask, int64_t X, int64_t Y, int64_t Z, float grad_scale,
                      float* dG, double* partial, void* stream);

/* ---- loss-form total variation over a voxel mask ----------------------------
 * total_variation(v, mask) of the model files and its gradient, for
 * density_total_variation(sdf_tv, bg_density_tv) / k0_total_variation /
 * bg_k0_total_variation (voxurf_coarse.py:300-320, voxurf_fine.py:412-432,
 * voxurf_womask_fine.py:500-548, voxurf_womask_coarse.py:398-440).
 * Selected pairs along axis a: (p, p + e_a) with both voxels inside the grid
 * and in the mask; every channel uses the voxel mask.  S_a = sum of |v[p +
 * e_a] - v[p]| over them, P_a = C x their number, M = C x the mask's voxels.
 *   mode 0 (voxurf_coarse.py:702-715): (S_0 + S_1 + S_2) / 3 / M
 *   mode 1 (voxurf_fine.py:956-969 and the maskless models):
 *          (S_0/P_0 + S_1/P_1 + S_2/P_2) / 3
 * loss = weight x that; axis_scale[a] = d loss / d |diff| of one selected
 * pair of axis a.  Sums in FP64 in a fixed order (deterministic). */
typedef struct {
  const float* v;           /* [C,X,Y,Z] (channel_last 0) or [X,Y,Z,C]           */
  int64_t C, X, Y, Z;
  int32_t channel_last;
  int32_t mode;             /* 0 or 1, above                                    */
  const uint8_t* mask;      /* [X,Y,Z] voxel mask, or NULL (every voxel)        */
  float weight;
  float* loss;              /* out [1] (device)                                 */
  float* axis_scale;        /* out [3] (device), read by the backward           */
  void* scratch;            /* vx_tv_loss_scratch_bytes(X, Y, Z) bytes          */
  size_t scratch_bytes;
} vx_tv_loss_args;
size_t vx_tv_loss_scratch_bytes(int64_t X, int64_t Y, int64_t Z);
int vx_tv_loss(const vx_tv_loss_args* args, void* stream);
/* grad (v's layout) += g_loss[0] (device scalar) x d loss / d v, from the
 * axis_scale the forward wrote; sign(0) = 0 as torch's abs. */
int vx_tv_loss_backward(const vx_tv_loss_args* args, const float* g_loss, float* grad, void* stream);

/* ---- fused coarse-model rendering (lib/voxurf_coarse.py:513-619) ---------- */

/* March with the coarse semantics: gradient from the [X,Y,Z,4] grid of the
 * raw SDF, weights from a second Alphas2Weights over the weight > thres set
 * (:540-550).  Records of that set go to the per-ray slots (all flagged);
 * n1 = n2 = their count, n2b = the count up to the second scan's stop.  The
 * maskless coarse model (voxurf_womask_coarse.py:620-674) marches the same
 * way with march.unit_sphere = 1, no mask, and grad4 built from the smoothed
 * SDF (:657); the backward's d_grad4 then belongs to the smoothed grid. */
typedef struct {
  vx_fine_march_args march;
  const float* grad4;       /* [X,Y,Z,4] vx_sdf_gradient_grid(layout 1) of the SDF */
  int32_t* n2b;             /* out [N]                                          */
} vx_coarse_march_args;
int vx_coarse_march(const vx_coarse_march_args* args, void* stream);

typedef struct {
  int32_t use_k0;           /* k0 columns first (rgbnet_full_implicit = False)  */
  int32_t geo_rgb_dim;      /* 3: normalised gradient columns last, 0: none     */
  int64_t posbase_pe, viewbase_pe;
} vx_coarse_feature_cfg;

/* rgbnet input [k0, PE(xyz), PE(viewdir), normal] (voxurf_coarse.py:552-569). */
typedef struct {
  int64_t n_rows;
  const int32_t* ray2;
  const float* pts2;
  const float* viewdirs;
  vx_grid_geom grid;
  const float* grad4;
  const float* k0_f32;
  const void* k0_bf16;
  vx_coarse_feature_cfg cfg;
  int64_t ld;               /* row stride of X, >= the feature count; columns
                               beyond the features are written as zero       */
  void* X;
  int32_t out_bf16;
  float* normal_out;        /* optional [S2,3] interpolated gradient            */
} vx_coarse_features_args;
int vx_coarse_features(const vx_coarse_features_args* args, void* stream);

/* rgb = clamp(sum w*sigmoid(logit) + (1 - sum w)*bg, 0, 1) (:575-584). */
typedef struct {
  int64_t n_rays;
  const int64_t* s2_off;
  const float* w2;
  const float* logit;
  float bg;
  float* rgb;
  float* rgb_raw;
  const float* normal2;
  const int32_t* step2;
  float dist;
  float* normal_out;
  float* depth_out;
  float* wsum_out;
} vx_coarse_composite_args;
int vx_coarse_composite(const vx_coarse_composite_args* args, void* stream);

typedef struct {
  int64_t n_rays;
  const int64_t* s2_off;
  const float* w2;
  const float* logit;
  const float* rgb_raw;
  const float* g_rgb;
  float bg;
  float* d_logit;
  float* d_w2;
} vx_coarse_composite_bwd_args;
int vx_coarse_composite_backward(const vx_coarse_composite_bwd_args* args, void* stream);

typedef struct {
  int64_t n_rays;
  int64_t n_rows;
  const float* rays_o;
  const float* rays_d;
  const float* viewdirs;
  float near, stepdist;
  vx_grid_geom grid;
  const float* sdf_smooth;
  const float* grad4;
  float voxel_size;
  float inv_s, dist;
  int64_t max_steps;
  const void* rec;
  float* dw_slot;
  const int32_t* n2b;
  const float* alphainv_last;
  const float* d_last;
  const float* pts2;
  const int32_t* slot2;
  const float* dw2;
  vx_coarse_feature_cfg cfg;
  int64_t ld;
  const void* dX;
  int32_t in_bf16;
  float* d_sdf_smooth;      /* [X,Y,Z] accumulated                              */
  float* d_grad4;           /* [X,Y,Z,4] accumulated                            */
  float* d_k0;              /* [X,Y,Z,12] accumulated                           */
  const float* d_grad2;     /* optional [S2,3] gradient w.r.t. the shaded samples'
                               raw interpolated SDF gradient (eikonal term)    */
} vx_coarse_backward_args;
int vx_coarse_backward(const vx_coarse_backward_args* args, void* stream);

/* ---- fused colour-MLP forward on the tcgen05 tensor cores (the rgbnet /
 *      k_rgbnet stacks of lib/voxurf_fine.py:132-187, three 192-wide hidden
 *      layers with ReLU and a 3-output layer) --------------------------------- */

/* Packs W [N,K] (row-major FP32, nn.Linear.weight) into the BF16 operand
 * layout of vx_mlp_tc_forward: [Kp/8][N][8], K zero-padded to Kp (multiple
 * of 8). */
int vx_mlp_tc_pack(const float* W, int64_t N, int64_t K, int64_t Kp, void* out, void* stream);

typedef struct {
  const void* X;            /* [n_rows, ldx] BF16 input rows, 16-byte aligned, ldx % 8 == 0 */
  int64_t ldx;
  int64_t K0;               /* first-layer inputs (multiple of 16, <= 80); X columns [K0_real, K0) must
                               be zero or meet zero weight columns                   */
  int64_t n_rows;
  int64_t width;            /* hidden width: 192                                    */
  const void* W0p;          /* vx_mlp_tc_pack(W0, 192, K, K0)                        */
  const void* W1p;          /* vx_mlp_tc_pack(W1, 192, 192, 192)                     */
  const void* W2p;
  const float* b0;          /* [192] hidden biases (FP32)                           */
  const float* b1;
  const float* b2;
  const void* Whp;          /* output layer as vx_mlp_tc_pack(Wsplit, 16, 192, 192) of
                               Wsplit [16,192] FP32: rows 0-2 = BF16(Wh), rows 3-5 =
                               BF16(Wh - BF16(Wh)), rows 6-15 = 0 (Wh [3,192])     */
  const float* bh;          /* [3]                                                  */
  const float* add;         /* optional [n_rows,3] added to the output (k_rgbnet's residual logits) */
  float* out;               /* [n_rows,3] logits                                    */
  void* cols;               /* optional: the logits also stored as BF16 at cols[row*ld_cols + 0..2] */
  int64_t ld_cols;
  int32_t pipeline;         /* 0: one 128-row tile in flight per CTA; 1: two (the MMAs of one tile
                               run while the other's accumulator is converted; same results) */
  int32_t reserved0;
} vx_mlp_tc_args;

/* out = Wh relu(W2 relu(W1 relu(W0 x + b0) + b1) + b2) + bh (+ add) for every
 * row: BF16 operands, FP32 accumulation in tensor memory, hidden activations
 * rounded to BF16 between layers; the output layer also on the tensor cores,
 * its FP32 weights split into two BF16 parts (hi + lo, relative error below
 * 2^-16).  One persistent CTA per SM holds all weights in shared memory. */
int vx_mlp_tc_forward(const vx_mlp_tc_args* args, void* stream);

/* ---- colour-MLP training on the tensor cores (tcgen05, BF16 operands, FP32
 *      accumulation): forward + backward of the rgbnet / k_rgbnet stacks
 *      (lib/voxurf_fine.py:132-187, applied at :718-752) and of the coarse
 *      rgbnet (lib/voxurf_coarse.py:116-123, applied at :571-573), i.e. what
 *      torch autograd runs for nn.Linear/ReLU in the reference.  Hidden width
 *      32, 64, 128 or 192; 2 or 3 hidden layers; first-layer K0 a multiple of
 *      16 up to 80; a 3-wide output layer.  Intermediate tensors are "T-tiles"
 *      (128-row tiles of a [rows, C] BF16 matrix as 8x8 core matrices,
 *      element (r, c) of tile t at t*128*C + ((r/8)*(C/8) + c/8)*64 + (r%8)*8
 *      + c%8); rows_cap (a multiple of 128 >= n_rows) sizes them. ---- */

/* One operand-preparation job of vx_mlp_train_pack.  mode 0: BF16 [Kp/8][Np][8]
 * of B[n][k] = src[n*ld + k] (transpose 0) or src[k*ld + n] (transpose 1),
 * zero beyond N x K; mode 1: the 3-row output layer as BF16 hi rows 0-2 and
 * lo rows 3-5 (hi + lo = the FP32 weight to 2^-16), [Kp/8][Np][8]; mode 2:
 * FP32 copy of the [N, K] matrix into dst contiguous; mode 3: FP32 [Kp][Np]
 * of Bt[k][n] = src[n*ld + k] (transpose 1) or src[k*ld + n] (transpose 0),
 * zero beyond N x K. */
typedef struct {
  const float* src;
  int64_t ld, N, K, Np, Kp;
  int32_t transpose, mode;
  void* dst;
} vx_mlp_pack_job;

/* Up to 32 jobs in one launch (the per-step operand refresh of both MLPs). */
int vx_mlp_train_pack(const vx_mlp_pack_job* jobs, int n_jobs, void* stream);

typedef struct {
  int64_t n_rows;            /* rows of X                                          */
  const int64_t* n_rows_dev; /* optional device row count <= n_rows (graph replay) */
  int64_t rows_cap;          /* row capacity of H / relu (multiple of 128)         */
  int64_t width, n_hidden, K0;
  const void* X;             /* BF16 [n_rows, ldx], 16-byte aligned rows            */
  int64_t ldx;
  const void* W0p;           /* pack mode 0 of W_0 [width, K]: N = width, Kp = K0   */
  const void* Wp;            /* hidden W_1..W_{L-1}: pack mode 0, N = Kp = width    */
  const float* bias;         /* [n_hidden][width] FP32 (pack mode 2)                */
  const void* Whp;           /* output layer: pack mode 1, Np = 16, Kp = width      */
  const float* bh;           /* [3]                                                 */
  float* out;                /* [n_rows, 3] logits                                  */
  void* cols;                /* optional BF16 copy of the logits: cols[row*ld_cols]  */
  int64_t ld_cols;
  void* H;                   /* T-tiles of h_1..h_L, each rows_cap*width BF16; null
                                for inference                                       */
  void* relu;                /* ReLU bits [L][rows_cap][width/16] uint16; null with H */
} vx_mlp_train_fwd_args;

/* Forward: logits = MLP(X); with H/relu set, keeps what the backward needs. */
int vx_mlp_train_forward(const vx_mlp_train_fwd_args* args, void* stream);

typedef struct {
  int64_t n_rows;
  const int64_t* n_rows_dev;
  int64_t rows_cap, width, n_hidden, K0;
  const float* dY;           /* [n_rows, 3] gradient of the logits                  */
  const float* Wh;           /* [3, width] output-layer weights (FP32)              */
  const void* relu;          /* from the forward                                    */
  const void* WTp;           /* hidden W_1..W_{L-1} transposed: pack mode 0 with
                                transpose 1, N = Kp = width                          */
  const void* W0Tp;          /* W_0 [width, K] transposed: pack mode 0, transpose 1,
                                N = Np = K0 (zero beyond K), K = Kp = width          */
  void* dZ;                  /* out: T-tiles of dz_1..dz_L, each rows_cap*width     */
  void* dYT;                 /* out: T-tiles (width 16) of dy as BF16 hi, lo        */
  void* dX;                  /* out: [n_rows, ld_dx] input gradient, columns < K0   */
  int64_t ld_dx;
  int32_t dx_bf16;
  float* dbh_part;           /* out: [grid][4] per-CTA column sums of dy            */
  int64_t dbh_part_cap;      /* rows of dbh_part (>= vx_mlp_wgrad_grid(n_rows))     */
} vx_mlp_train_bwd_args;

/* Backward, input-gradient chain (dz of every hidden layer, dX). */
int vx_mlp_train_backward(const vx_mlp_train_bwd_args* args, void* stream);

/* CTAs (= partials) of vx_mlp_train_wgrad and vx_mlp_train_backward for n_rows. */
size_t vx_mlp_wgrad_grid(int64_t n_rows);

typedef struct {
  int64_t n_rows;
  const int64_t* n_rows_dev;
  const void* A;             /* T-tiles of width WA (the M side)                     */
  int64_t WA;                /* multiple of 16, <= 256                               */
  const void* B;             /* T-tiles of width WB, or BF16 rows [n_rows, ldb]      */
  int64_t WB, ldb;           /* WB multiple of 16, <= 240                            */
  int32_t b_rows;            /* 1: B is rows                                         */
  int32_t ones;              /* 1: 16 more partial columns, column WB = sum_rows A   */
  float* part;               /* out: [grid][WA][WB + 16 ones] FP32 partials          */
  int64_t part_cap;          /* floats available at part                            */
} vx_mlp_wgrad_args;

/* part[cta][m][n] = sum over the CTA's rows of A[row][m] * B[row][n]. */
int vx_mlp_train_wgrad(const vx_mlp_wgrad_args* args, void* stream);

/* Up to 8 weight-gradient passes in one launch (e.g. every pass of two MLPs
 * after their input-gradient chains): pass p runs on ctas[p] >= 1 CTAs,
 * CTA c of the pass taking tiles c, c + ctas[p], ..., and writes ctas[p]
 * partials (part_cap >= ctas[p] * WA * (WB + 16 ones)). */
int vx_mlp_train_wgrad_multi(const vx_mlp_wgrad_args* passes, const int32_t* ctas, int n_passes, void* stream);

/* A split of the GPU's SMs over n_passes passes in proportion to the bytes
 * each streams per tile (WA + WB), at least 1 and at most
 * vx_mlp_wgrad_grid(n_rows) CTAs per pass, into ctas[n_passes]. */
int vx_mlp_wgrad_split(const vx_mlp_wgrad_args* passes, int n_passes, int32_t* ctas);

/* One ordered sum of vx_mlp_train_wgrad partials.  kind 0: w[m][n] = sum
 * part[.][m][n] for n < n_out (ld n_out), b[m] = sum part[.][m][WB]; kind 1
 * (output layer, A = h_L, B = dYT): w[c][m] = sum part[.][m][c] +
 * part[.][m][c + 3] for c < 3, b[c] = sum bh_part[.][c]. */
typedef struct {
  const float* part;
  int64_t n_part, WA, NC;
  int32_t kind, reserved;
  int64_t WB, n_out;
  float* w;
  float* b;
  const float* bh_part;
  int64_t n_bh;
} vx_mlp_reduce_job;

/* Up to 8 jobs in one launch. */
int vx_mlp_train_reduce(const vx_mlp_reduce_job* jobs, int n_jobs, void* stream);

/* ---- colour-MLP training in plain FP32 on the CUDA cores (the same layers
 *      as above with FP32 operands and FP32 fused multiply-adds; the output
 *      layer runs in vx_mlp_head / vx_mlp_head_backward).  Weights enter as
 *      Bt [Kp][Np] FP32 (vx_mlp_train_pack mode 3), Np in {32, 64, 80, 128,
 *      192}. ---- */
typedef struct {
  int64_t M;                 /* rows                                                */
  const int64_t* m_dev;      /* optional device row count <= M                      */
  int64_t K;                 /* inner dimension (columns of A used)                 */
  const float* A;            /* [M, lda]                                            */
  int64_t lda;
  const float* Bt;           /* [round_up(K,16)][Np], zero rows beyond K            */
  int64_t Np;
  int32_t mode;              /* 0: C = relu(A Bt + bias)   (hidden layer, forward)
                                1: C = (A Bt) * [H > 0], colsum[cta][n] = column sums
                                   of C over the CTA's rows (hidden layer, backward)
                                2: C = A Bt               (input gradient)          */
  int32_t reserved;
  const float* bias;         /* mode 0: [Np]                                        */
  const float* H;            /* mode 1: [M, ldh] the layer's post-ReLU activation   */
  int64_t ldh;
  float* C;                  /* [M, ldc], columns < n_store                         */
  int64_t ldc, n_store;
  float* colsum;             /* mode 1: [vx_mlp_f32_rowgemm_grid(M)][Np]            */
  int64_t colsum_cap;        /* floats available at colsum                          */
} vx_mlp_f32_rowgemm_args;

size_t vx_mlp_f32_rowgemm_grid(int64_t M);
/* C = A Bt with the epilogue of `mode` (lib/voxurf_fine.py:132-151 forward,
 * and its autograd backward). */
int vx_mlp_f32_rowgemm(const vx_mlp_f32_rowgemm_args* args, void* stream);

typedef struct {
  int64_t rows;
  const int64_t* rows_dev;
  const float* A;            /* [rows, lda], columns < M (dz of the layer's output) */
  int64_t lda;
  const float* B;            /* [rows, ldb], columns < N (the layer's input)        */
  int64_t ldb;
  int64_t M, N;              /* each <= 192                                         */
  float* part;               /* out: [grid][MP][NP] (MP, NP = M, N padded up to 32, 64,
                                80, 128 or 192)                                      */
  int64_t part_cap;
} vx_mlp_f32_wgrad_args;

size_t vx_mlp_f32_wgrad_grid(int64_t rows);
/* part[cta][m][n] = sum over the CTA's rows of A[r][m] B[r][n] (dW = dz^T h). */
int vx_mlp_f32_wgrad(const vx_mlp_f32_wgrad_args* args, void* stream);

/* out[m*out_ld + n] = sum_k part[k*part_stride + m*part_ld + n], k in order. */
typedef struct {
  const float* part;
  int64_t n_part, part_stride, part_ld, rows, cols;
  float* out;
  int64_t out_ld;
} vx_mlp_sum_job;

/* Up to 16 jobs in one launch. */
int vx_mlp_f32_reduce(const vx_mlp_sum_job* jobs, int n_jobs, void* stream);

/* ---- render server: the inference form of Voxurf.forward (global_step =
 *      None, lib/voxurf_fine.py:620-802) for rays of several resident scenes
 *      in one launch per stage.  The reference renders one scene per process,
 *      chunk by chunk (run.py:81-126 render_viewpoints, 8192 rays per call);
 *      these entry points have no one-to-one counterpart there. ------------ */

#define VX_SERVE_MAX_SCENES 8

/* One resident scene.  sdf_smooth is the SDF grid after the fine model's
 * Gaussian smoothing (voxurf_fine.py:638), applied once at load time. */
typedef struct {
  vx_grid_geom grid;
  const float* sdf_smooth;  /* [X,Y,Z] FP32                                      */
  const void* k0;           /* [X,Y,Z,12] channel-last                           */
  int32_t k0_bf16;          /* 1: k0 is BF16, 0: FP32                            */
  float voxel_size;
  const uint8_t* mask;      /* optional MaskGrid bool grid (NULL: none)          */
  int64_t mask_X, mask_Y, mask_Z;
  float mask_scale[3], mask_shift[3];
  float inv_s;              /* 1 / s_val (s_val is per scene: not in checkpoints) */
  float stepdist;           /* stepsize * voxel_size (also the NeuS dist)        */
  float near;
  float bg;
  float fast_color_thres;
  const uint8_t* occ;       /* optional occupancy of the mask (vx_mask_occupancy):
                               the march skips runs of samples in empty cells */
  int64_t occ_X, occ_Y, occ_Z;
  int32_t occ_block;
  /* optional MaskCache density mask (as in vx_fine_march_args; exclusive
     with `mask` and `occ`) */
  const float* mask_density;
  vx_grid_geom mask_dgrid;
  float mask_act_shift, mask_voxel_size_ratio, mask_thres;
} vx_scene_desc;

/* Block occupancy of a mask grid for empty-space skipping: cell (I,J,K) of
 * an [occ_X, occ_Y, occ_Z] = [ceil(mX/block)+2, ...] grid (one border cell
 * on each side) is 1 iff a mask voxel lies in its block of voxels
 * [block*(I-1), block*I) (per axis) widened by one voxel on both sides.
 * The widening makes a skip decision taken on a float model of the sample
 * positions safe: a sample the model places in an empty cell has its exact
 * voxel within one voxel of that cell, where the mask is 0. */
int vx_mask_occupancy(const uint8_t* mask, int64_t mX, int64_t mY, int64_t mZ, int32_t block, uint8_t* occ,
                      void* stream);

/* A run of consecutive pixels of one view: rays [ray0, ray0 + n) of a tick
 * come from pixels [pix0, pix0 + n) of an image W pixels wide (row-major)
 * and their results go to pixels [out0, out0 + n) of the output arena. */
typedef struct {
  float c2w[12];            /* row-major 3x4 camera-to-world                     */
  float fx, fy, cx, cy;
  int32_t W;
  int32_t inverse_y;        /* 1: OpenCV axes                                    */
  int32_t scene;            /* index into the scene table                        */
  int32_t reserved;
  int64_t pix0, ray0, out0;
} vx_view_chunk;

/* Rays of a tick (get_rays + viewdirs, voxurf_fine.py:1001-1029, 1064) with
 * their scene index and output pixel.  chunks: DEVICE array sorted by ray0,
 * chunks[0].ray0 = 0. */
int vx_serve_rays(const vx_view_chunk* chunks, int32_t n_chunks, int64_t n_rays, float* rays_o, float* rays_d,
                  float* viewdirs, int32_t* ray_scene, int64_t* ray_out, void* stream);

/* Per ray: exact samples (sample_pts_on_rays), mask lookup, SDF + FD normal,
 * NeuS alpha, alpha > thres compaction, transmittance with the T < 1e-3
 * stop, weight > thres test.  The shaded samples' (step, weight) go to
 * rec[ray * max_steps + j] (8-byte records), their count to n2[ray].
 * scenes_host: HOST array of n_scenes descriptors. */
int vx_serve_march(const vx_scene_desc* scenes_host, int32_t n_scenes, const float* rays_o, const float* rays_d,
                   const float* viewdirs, const int32_t* ray_scene, int64_t n_rays, int64_t max_steps, void* rec,
                   int32_t* n2, float* alphainv_last, void* stream);

/* ray2[s2_off[r] + j] = r for j < s2_off[r+1] - s2_off[r]; rows at or
 * beyond `capacity` are skipped (the caller compares s2_off[n_rays] with its
 * capacity). */
int vx_serve_rows(const int64_t* s2_off, int64_t n_rays, int32_t* ray2, int64_t capacity, void* stream);

/* MLP input rows of the shaded samples (the column layout of
 * vx_fine_features; every scene of one call shares cfg).  Row strides:
 * ld1 >= the rgbnet columns, ld2 >= the k_rgbnet columns + 3, the last 3
 * being the rgbnet logits that vx_mlp_head writes.  n_rows is the row
 * count, or with n_rows_dev != NULL the capacity of X1 / X2 / ray2: the
 * rows then are min(*n_rows_dev, n_rows) (a device count, so the launch
 * needs no host read; rows beyond the capacity are skipped and the caller
 * compares).  staging: 1 assembles each CTA's rows in shared memory and
 * writes them out coalesced (38 KB per CTA at the fine layout), 0 stores
 * from each row's thread (no dynamic shared memory, so CTAs fit beside a
 * kernel that holds most of an SM's shared memory), -1 chooses 1 where it
 * fits the default 48 KB. */
int vx_serve_features(const vx_scene_desc* scenes_host, int32_t n_scenes, const vx_fine_feature_cfg* cfg,
                      const float* rays_o, const float* rays_d, const float* viewdirs, const int32_t* ray_scene,
                      int64_t max_steps, const void* rec, const int64_t* s2_off, const int32_t* ray2, int64_t n_rows,
                      const int64_t* n_rows_dev, int64_t ld1, int64_t ld2, void* X1, void* X2, int32_t out_bf16,
                      int32_t staging, void* stream);

/* Output layer of a colour MLP (voxurf_fine.py:141-151): out[i,:] =
 * H[i,:width] W^T + b (+ add[i,:]) with FP32 accumulation; when cols is
 * given the result is also stored (BF16 when cols_bf16) at cols[i*ld_cols
 * + 0..2].  H: [n_rows, ldh] BF16 (in_bf16) or FP32; W: [3,width] FP32. */
int vx_mlp_head(const void* H, int64_t n_rows, int64_t width, int64_t ldh, int32_t in_bf16, const float* W,
                const float* b, const float* add, float* out, void* cols, int64_t ld_cols, int32_t cols_bf16,
                void* stream);

/* Compositing (voxurf_fine.py:753-777) straight into the output images:
 * rgb = sum w*sigmoid(logit) + alphainv_last*bg, or with klogit (the
 * k-branch) the same sum clamped to [0,1]; depth = sum w*step*stepdist.
 * Written to out_rgb[3*ray_out[r] + c] and out_depth[ray_out[r]] (optional). */
int vx_serve_composite(const vx_scene_desc* scenes_host, int32_t n_scenes, const int32_t* ray_scene, int64_t n_rays,
                       int64_t max_steps, const void* rec, const int64_t* s2_off, const float* logit,
                       const float* klogit, const float* alphainv_last, const int64_t* ray_out, float* out_rgb,
                       float* out_depth, void* stream);

/* Per-step FP32 -> BF16 casts of the colour-MLP weights and biases of the
 * mixed-precision step (the reference keeps FP32 parameters; the BF16
 * copies feed the GEMMs), all in one launch: job j copies rows x cols
 * elements from src (row stride src_ld floats) to dst (row stride dst_ld
 * BF16 elements). */
#define VX_CAST_MAX_JOBS 16
typedef struct {
  const float* src;
  void* dst;
  int32_t rows;
  int32_t cols;
  int32_t src_ld;
  int32_t dst_ld;
} vx_cast_job;
int vx_cast_rows_bf16(const vx_cast_job* jobs_host, int32_t n_jobs, void* stream);

/* ------------------------------------------------------------------------
 * Background branch of the scenes without an object mask
 * (lib/voxurf_womask_fine.py, lib/voxurf_womask_coarse.py).
 * ------------------------------------------------------------------------ */

/* ub360_utils.cpp / ub360_utils_kernel.cu:13-31 (ub360_utils_cuda.
 * cumdist_thres, called at voxurf_womask_fine.py:867 and
 * voxurf_womask_coarse.py:645): mask[r, i] = 1 where the running sum of
 * dist[r, :i+1] since the last mark exceeds thres; the sum restarts from 0
 * after a mark.  dist and mask: [n_rays, n_pts] row-major, float32 / bytes. */
int vx_cumdist_thres(const float* dist, int64_t n_rays, int64_t n_pts, float thres, uint8_t* mask, void* stream);

/* Background samples of voxurf_womask_fine.py:857-870 (sample_ray_ori at
 * :789-818 with use_bg=False, outside_sphere_trans(filtered=True) at
 * :820-825, the inverted-sample distances and cumdist_thres, then the
 * compaction by bg_mask) and of voxurf_womask_coarse.py:633-650.  Sample k
 * of ray r (k < n_samples) is p = o + d*(t_min + stepdist*(k + jitter[r])/|d|)
 * with t_min the slab entry clamped to [near, far]; it is kept when |p| >= 1,
 * when (outbbox_only) it lies outside the bbox or its ray misses the bbox
 * (the coarse model's bg_mask & mask_outbbox), and when k = 0 or the running
 * distance between consecutive inverted points p/|p|^2 exceeds dist_thres.
 * jitter: [n_rays] device floats (the training-time torch.rand of :808) or
 * NULL. */
typedef struct {
  const float* rays_o;      /* [n_rays,3] */
  const float* rays_d;      /* [n_rays,3] */
  const float* jitter;      /* [n_rays] or NULL */
  float xyz_min[3];
  float xyz_max[3];
  float near;
  float far;
  float stepdist;           /* stepsize * voxel size (float32, as the reference's tensor) */
  float dist_thres;         /* voxel_size * stepsize * 0.5 (fine) or * 0.95 (coarse), float32 */
  int32_t n_samples;        /* int(|grid shape + 1| / stepsize) + 1 */
  int32_t outbbox_only;     /* 1: the coarse model's additional mask_outbbox test */
  int64_t n_rays;
  int32_t inner;            /* 1: the foreground samples instead (:846-849): the
                               points with |p| < 1, not inverted, no distance
                               test; outer_pts receives p, pts_org may be NULL */
  int32_t reserved;
} vx_bg_sample_args;

/* Phase 1: counts [n_rays] kept samples per ray and offsets [n_rays+1]
 * (offsets[n_rays] = M); scratch: vx_scan_scratch_bytes(n_rays) bytes. */
int vx_bg_samples_count(const vx_bg_sample_args* args, int64_t* counts, int64_t* offsets, void* scratch,
                        size_t scratch_bytes, void* stream);

/* Phase 2: the kept samples in ray order: outer_pts [M,3] (inverted),
 * pts_org [M,3], ray_id [M], step_id [M] (k).  Writes at or beyond
 * `capacity` are skipped and reported as VX_ERR_CAPACITY through
 * vx_device_error(). */
int vx_bg_samples_fill(const vx_bg_sample_args* args, const int64_t* offsets, int64_t capacity, float* outer_pts,
                       float* pts_org, int64_t* ray_id, int64_t* step_id, void* stream);

/* ---- the maskless fine model (lib/voxurf_womask_fine.py:833-1071) ----
 * Foreground samples: vx_bg_samples_* with inner = 1; their feature rows:
 * vx_fine_features / vx_fine_backward (n_rays = 0); weights:
 * vx_alpha2weight. */

/* Foreground alpha (forward, d_alpha == NULL): the SDF and its +-1-voxel
 * finite-difference gradient on the smoothed grid at each sample
 * (grid_sampler(..., sample_grad=True, displace=1.0), :876) and the NeuS
 * alpha of neus_alpha_from_sdf_scatter(use_mid) (:879-880, :606-634).
 * Backward (d_alpha != NULL): the alpha adjoint accumulated into
 * d_sdf_smooth. */
typedef struct {
  int64_t n;                /* samples                                          */
  const float* pts;         /* [n,3]                                            */
  const int64_t* ray_id;    /* [n]                                              */
  const float* viewdirs;    /* [N,3]                                            */
  vx_grid_geom grid;
  const float* sdf_smooth;  /* [X,Y,Z]                                          */
  float voxel_size, inv_s, dist;
  float* alpha;             /* forward out [n]                                  */
  const float* d_alpha;     /* backward in [n], or NULL for the forward         */
  float* d_sdf_smooth;      /* backward: accumulated [X,Y,Z]                    */
} vx_womask_fg_alpha_args;
int vx_womask_fg_alpha(const vx_womask_fg_alpha_args* args, void* stream);

/* Background alpha: bg_density (trilinear, zero padding) at the inverted
 * points and activate_density, alpha = 1 - exp(-softplus(d + act_shift) *
 * interval) (:898-900, :542-544); backward (d_alpha != NULL) accumulates
 * into d_density. */
typedef struct {
  int64_t n;
  const float* pts;         /* [n,3] inverted points                            */
  vx_grid_geom grid;        /* the background grid                              */
  const float* density;     /* [X,Y,Z]                                          */
  float act_shift, interval;
  float* alpha;             /* forward out [n]                                  */
  const float* d_alpha;     /* backward in [n] or NULL                          */
  float* d_density;         /* backward: accumulated [X,Y,Z]                    */
} vx_womask_bg_alpha_args;
int vx_womask_bg_alpha(const vx_womask_bg_alpha_args* args, void* stream);

/* Background MLP rows (:955-970): [bg_k0 at the inverted point (12, when
 * bg_k0 != NULL), PE((p_org - xyz_min) / (xyz_max - xyz_min), posbase_pe),
 * PE(viewdir, viewbase_pe)], zero to ld; a negative PE count leaves that
 * block out.  Backward (dX != NULL): columns 0-11 of dX accumulated into
 * d_bg_k0 [X,Y,Z,12]. */
typedef struct {
  int64_t n;
  const float* outer_pts;   /* [n,3] inverted                                   */
  const float* pts_org;     /* [n,3]                                            */
  const int64_t* ray_id;    /* [n]                                              */
  const float* viewdirs;    /* [N,3]                                            */
  vx_grid_geom grid;        /* the background grid (xyz_min/max also normalise) */
  const float* bg_k0;       /* [X,Y,Z,12] or NULL                               */
  int64_t posbase_pe, viewbase_pe;
  int64_t ld;
  void* X;                  /* forward out [n, ld] (BF16 when bf16)              */
  int32_t bf16, reserved;
  const void* dX;           /* backward in [n, ld] or NULL                      */
  float* d_bg_k0;           /* backward: accumulated                            */
} vx_womask_bg_features_args;
int vx_womask_bg_features(const vx_womask_bg_features_args* args, void* stream);

/* Foreground/background compositing (:972-1012).  Per ray r: s0 = sum w
 * sigmoid(logit), sk = sum w sigmoid(logit + kout), cum = sum w over rows
 * [fg_off[r], fg_off[r+1]); sb = sum w_bg sigmoid(bg_logit) over
 * [bg_off[r], bg_off[r+1]); bg = clamp(sb, 0, 1); rgb0 = clamp(clamp(s0) +
 * (1 - cum) bg), rgbk = clamp(clamp(sk) + (1 - cum) bg), ainv = 1 - cum,
 * in_marched = clamp(sk) (clamp(s0) without k-branch), bg_marched = bg; the
 * per-ray sums go to stats [N,10] for the backward.  With unclamped_parts =
 * 1 the sums s0, sk and sb enter unclamped (the coarse model,
 * voxurf_womask_coarse.py:731-742: rgb = clamp(s0 + (1 - cum) sb)).
 * Backward (d_w != NULL): gradients of logit (plus the k-branch's when
 * k_into_logit), kout, w, bg_logit and w_bg from g_rgb0, g_rgbk, g_ainv
 * (each may be NULL). */
typedef struct {
  int64_t n_rays;
  const int64_t* fg_off;    /* [N+1]                                            */
  const float* w;           /* [S]                                              */
  const float* logit;       /* [S,3]                                            */
  const float* kout;        /* [S,3] or NULL (no k-branch)                      */
  const int64_t* bg_off;    /* [N+1]                                            */
  const float* bw;          /* [B]                                              */
  const float* blogit;      /* [B,3]                                            */
  float* stats;             /* [N,10]: forward out, backward in                 */
  float* rgb0;
  float* rgbk;
  float* ainv;
  float* in_marched;
  float* bg_marched;
  const float* g_rgb0;
  const float* g_rgbk;
  const float* g_ainv;
  float* d_logit;
  float* d_kout;
  float* d_w;
  float* d_blogit;
  float* d_bw;
  int32_t k_into_logit, unclamped_parts;
} vx_womask_composite_args;
int vx_womask_composite(const vx_womask_composite_args* args, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VOXURF_GB300_H */
