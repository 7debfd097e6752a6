/*
 * ORACLE — test infrastructure only.  A plain-C restatement of the
 * reference's CUDA ops (Voxurf lib/cuda/*.cu), executed serially on the CPU.
 * It is the checker for the sm_103a kernels of voxurf_gb300; nothing in the
 * product links or calls it.
 *
 * Floating-point semantics follow the reference's compiled kernels: one
 * rounding per operation (this file must be compiled with -ffp-contract=off
 * so that the compiler fuses nothing on its own), except for the a*b+c that
 * the reference's nvcc build (default --fmad=true) computes as one fused
 * multiply-add, written here as C99 fmaf: the ray norm
 * sqrt(fma(z,z, fma(x,x, y*y))), the ray start fma(d, t_min, o), the sample
 * point fma(dir, dist, start), the mask index fma(xyz, scale, shift), the
 * suffix sum of alpha2weight's backward and the two Adam moments.  Which
 * expressions are fused was measured by running the reference's own kernels
 * on the GPU against every candidate form (tests/test_zy_reference_kernels_gpu.py).
 * Float arithmetic where the source uses float, and the implicit double
 * promotions of the source where it mixes in double literals
 * (e.g. `T_cum *= (1. - alpha[i])`).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

/* ---- render_utils_kernel.cu:12-35 ---------------------------------------- */
static void clip_one(const float* o, const float* d, const float* mn, const float* mx, float near, float far,
                     float* tmin, float* tmax) {
  float vx = (d[0] == 0) ? 1e-6f : d[0];
  float vy = (d[1] == 0) ? 1e-6f : d[1];
  float vz = (d[2] == 0) ? 1e-6f : d[2];
  float ax = (mx[0] - o[0]) / vx;
  float ay = (mx[1] - o[1]) / vy;
  float az = (mx[2] - o[2]) / vz;
  float bx = (mn[0] - o[0]) / vx;
  float by = (mn[1] - o[1]) / vy;
  float bz = (mn[2] - o[2]) / vz;
  *tmin = fmaxf(fminf(fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz)), far), near);
  *tmax = fmaxf(fminf(fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz)), far), near);
}

/* render_utils_kernel.cu:48-51: the compiled kernel fuses x*x and z*z into
 * the sum, fma(z, z, fma(x, x, y*y)) */
static float rnorm_of(const float* d) {
  return sqrtf(fmaf(d[2], d[2], fmaf(d[0], d[0], d[1] * d[1])));
}

/* render_utils_kernel.cu:53 */
static int64_t nsamples_of(float tmin, float tmax, float rn, float stepdist) {
  float c = ceilf(((tmax - tmin) * rn) / stepdist);
  double m = fmax((double)c, 1.0);
  return (int64_t)m;
}

void vxo_infer_t_minmax(const float* rays_o, const float* rays_d, const float* xyz_min, const float* xyz_max,
                        float near, float far, int64_t n, float* t_min, float* t_max) {
  for (int64_t r = 0; r < n; ++r) clip_one(rays_o + 3 * r, rays_d + 3 * r, xyz_min, xyz_max, near, far, t_min + r, t_max + r);
}

void vxo_infer_n_samples(const float* rays_d, const float* t_min, const float* t_max, float stepdist, int64_t n,
                         int64_t* out) {
  for (int64_t r = 0; r < n; ++r) out[r] = nsamples_of(t_min[r], t_max[r], rnorm_of(rays_d + 3 * r), stepdist);
}

/* render_utils_kernel.cu:58-79 */
void vxo_infer_ray_start_dir(const float* rays_o, const float* rays_d, const float* t_min, int64_t n, float* start,
                             float* dir) {
  for (int64_t r = 0; r < n; ++r) {
    const float* o = rays_o + 3 * r;
    const float* d = rays_d + 3 * r;
    float rn = rnorm_of(d);
    for (int a = 0; a < 3; ++a) {
      start[3 * r + a] = fmaf(d[a], t_min[r], o[a]);
      dir[3 * r + a] = d[a] / rn;
    }
  }
}

/* Phase 1 of render_utils_kernel.cu:196-242: t_min/t_max, N_steps and the
 * total sample count. */
int64_t vxo_sample_count(const float* rays_o, const float* rays_d, const float* xyz_min, const float* xyz_max,
                         float near, float far, float stepdist, int64_t n, float* t_min, float* t_max,
                         int64_t* n_steps) {
  int64_t total = 0;
  for (int64_t r = 0; r < n; ++r) {
    clip_one(rays_o + 3 * r, rays_d + 3 * r, xyz_min, xyz_max, near, far, t_min + r, t_max + r);
    n_steps[r] = nsamples_of(t_min[r], t_max[r], rnorm_of(rays_d + 3 * r), stepdist);
    total += n_steps[r];
  }
  return total;
}

/* Phase 2: render_utils_kernel.cu:144-194 (ray_id/step_id from the cumsum,
 * points start + dir*(stepdist*step), bbox test). */
void vxo_sample_fill(const float* rays_o, const float* rays_d, const float* xyz_min, const float* xyz_max,
                     const float* t_min, const int64_t* n_steps, float stepdist, int64_t n, float* ray_pts,
                     uint8_t* mask_outbbox, int64_t* ray_id, int64_t* step_id) {
  int64_t idx = 0;
  for (int64_t r = 0; r < n; ++r) {
    const float* o = rays_o + 3 * r;
    const float* d = rays_d + 3 * r;
    float rn = rnorm_of(d);
    float st[3], dr[3];
    for (int a = 0; a < 3; ++a) {
      st[a] = fmaf(d[a], t_min[r], o[a]);
      dr[a] = d[a] / rn;
    }
    for (int64_t k = 0; k < n_steps[r]; ++k, ++idx) {
      float dist = stepdist * (float)k;
      float px = fmaf(dr[0], dist, st[0]);
      float py = fmaf(dr[1], dist, st[1]);
      float pz = fmaf(dr[2], dist, st[2]);
      ray_pts[3 * idx + 0] = px;
      ray_pts[3 * idx + 1] = py;
      ray_pts[3 * idx + 2] = pz;
      mask_outbbox[idx] = (xyz_min[0] > px) | (xyz_min[1] > py) | (xyz_min[2] > pz) | (xyz_max[0] < px) |
                          (xyz_max[1] < py) | (xyz_max[2] < pz);
      ray_id[idx] = r;
      step_id[idx] = k;
    }
  }
}

/* C round() then int conversion with the saturation/NaN behaviour of the
 * GPU's float->int conversion (NaN -> 0, out of range -> INT_MIN/INT_MAX). */
static int round_to_int(float v) {
  float r = roundf(v);
  if (r != r) return 0;
  if (r >= 2147483647.f) return 2147483647;
  if (r <= -2147483648.f) return (-2147483647 - 1);
  return (int)r;
}

/* render_utils_kernel.cu:374-392 */
void vxo_maskcache_lookup(const uint8_t* world, int64_t si, int64_t sj, int64_t sk, const float* xyz, int64_t n,
                          const float* scale, const float* shift, uint8_t* out) {
  for (int64_t p = 0; p < n; ++p) {
    int i = round_to_int(fmaf(xyz[3 * p + 0], scale[0], shift[0]));
    int j = round_to_int(fmaf(xyz[3 * p + 1], scale[1], shift[1]));
    int k = round_to_int(fmaf(xyz[3 * p + 2], scale[2], shift[2]));
    uint8_t v = 0;
    if (0 <= i && i < si && 0 <= j && j < sj && 0 <= k && k < sk) v = world[((int64_t)i * sj + j) * sk + k] ? 1 : 0;
    out[p] = v;
  }
}

/* render_utils_kernel.cu:607-635: segment bounds from sorted ray_id. */
static void segment_bounds(const int64_t* ray_id, int64_t n_pts, int64_t n_rays, int64_t* i_start, int64_t* i_end) {
  for (int64_t r = 0; r < n_rays; ++r) i_start[r] = i_end[r] = 0;
  if (n_pts == 0) return;
  for (int64_t idx = 1; idx < n_pts; ++idx) {
    if (ray_id[idx] != ray_id[idx - 1]) {
      i_start[ray_id[idx]] = idx;
      i_end[ray_id[idx - 1]] = idx;
    }
  }
  i_end[ray_id[n_pts - 1]] = n_pts;
}

/* render_utils_kernel.cu:577-605, 619-651 (float, as the reference). */
void vxo_alpha2weight(const float* alpha, const int64_t* ray_id, int64_t n_pts, int64_t n_rays, float* weight,
                      float* T, float* alphainv_last, int64_t* i_start, int64_t* i_end) {
  for (int64_t i = 0; i < n_pts; ++i) {
    weight[i] = 0.f;
    T[i] = 1.f;
  }
  for (int64_t r = 0; r < n_rays; ++r) alphainv_last[r] = 1.f;
  segment_bounds(ray_id, n_pts, n_rays, i_start, i_end);
  if (n_pts == 0) return;
  for (int64_t r = 0; r < n_rays; ++r) {
    const int i_s = (int)i_start[r];
    const int i_e_max = (int)i_end[r];
    float T_cum = 1.;
    int i;
    for (i = i_s; i < i_e_max; ++i) {
      T[i] = T_cum;
      weight[i] = T_cum * alpha[i];
      T_cum *= (1. - alpha[i]);
      if (T_cum < 1e-3) {
        i += 1;
        break;
      }
    }
    i_end[r] = i;
    alphainv_last[r] = T_cum;
  }
}

/* render_utils_kernel.cu:653-707 (float, as the reference). */
void vxo_alpha2weight_backward(const float* alpha, const float* weight, const float* T, const float* alphainv_last,
                               const int64_t* i_start, const int64_t* i_end, int64_t n_pts, int64_t n_rays,
                               const float* grad_weights, const float* grad_last, float* grad) {
  for (int64_t i = 0; i < n_pts; ++i) grad[i] = 0.f;
  for (int64_t r = 0; r < n_rays; ++r) {
    const int i_s = (int)i_start[r];
    const int i_e = (int)i_end[r];
    float back_cum = grad_last[r] * alphainv_last[r];
    for (int i = i_e - 1; i >= i_s; --i) {
      grad[i] = grad_weights[i] * T[i] - back_cum / (1 - alpha[i] + 1e-10);
      back_cum = fmaf(grad_weights[i], weight[i], back_cum);
    }
  }
}

/* The same two scans in double (the FP64 model oracle). */
void vxo_alpha2weight_f64(const double* alpha, const int64_t* ray_id, int64_t n_pts, int64_t n_rays,
                          double* weight, double* T, double* alphainv_last, int64_t* i_start, int64_t* i_end) {
  for (int64_t i = 0; i < n_pts; ++i) {
    weight[i] = 0.;
    T[i] = 1.;
  }
  for (int64_t r = 0; r < n_rays; ++r) alphainv_last[r] = 1.;
  segment_bounds(ray_id, n_pts, n_rays, i_start, i_end);
  if (n_pts == 0) return;
  for (int64_t r = 0; r < n_rays; ++r) {
    const int64_t i_s = i_start[r], i_e_max = i_end[r];
    double T_cum = 1.;
    int64_t i;
    for (i = i_s; i < i_e_max; ++i) {
      T[i] = T_cum;
      weight[i] = T_cum * alpha[i];
      T_cum *= (1. - alpha[i]);
      if (T_cum < 1e-3) {
        i += 1;
        break;
      }
    }
    i_end[r] = i;
    alphainv_last[r] = T_cum;
  }
}

void vxo_alpha2weight_backward_f64(const double* alpha, const double* weight, const double* T,
                                   const double* alphainv_last, const int64_t* i_start, const int64_t* i_end,
                                   int64_t n_pts, int64_t n_rays, const double* grad_weights,
                                   const double* grad_last, double* grad) {
  for (int64_t i = 0; i < n_pts; ++i) grad[i] = 0.;
  for (int64_t r = 0; r < n_rays; ++r) {
    double back_cum = grad_last[r] * alphainv_last[r];
    for (int64_t i = i_end[r] - 1; i >= i_start[r]; --i) {
      grad[i] = grad_weights[i] * T[i] - back_cum / (1 - alpha[i] + 1e-10);
      back_cum += grad_weights[i] * weight[i];
    }
  }
}

/* ---- total_variation_kernel.cu:14-66 ------------------------------------- */
static float clampf1(float v) { return fminf(fmaxf(v, -1.f), 1.f); }

/* Flat (C, X, Y, Z) or (X, Y, Z, C) grid; masked != 0 selects the _new
 * variant.  wx, wy, wz are the host weights before the /6. */
void vxo_tv_add_grad(const float* param, float* grad, const float* mask, float wx, float wy, float wz,
                     int dense_mode, int64_t C, int64_t X, int64_t Y, int64_t Z, int channel_last) {
  wx /= 6;
  wy /= 6;
  wz /= 6;
  const int64_t sk = channel_last ? C : 1, sj = Z * sk, si = Y * sj;
  const int64_t n = C * X * Y * Z;
  /* The reference kernel reads `param` only and adds into `grad`, every
   * element independent: a serial sweep is equivalent. */
  for (int64_t idx = 0; idx < n; ++idx) {
    if (!(dense_mode || grad[idx] != 0)) continue;
    int64_t i, j, k;
    if (channel_last) {
      int64_t v = idx / C;
      k = v % Z; j = (v / Z) % Y; i = v / (Z * Y);
    } else {
      k = idx % Z; j = (idx / Z) % Y; i = (idx / (Z * Y)) % X;
    }
    const float c = param[idx];
    float g = 0;
    if (!mask) {
      g += (k == 0 ? 0 : wz * clampf1(c - param[idx - sk]));
      g += (k == Z - 1 ? 0 : wz * clampf1(c - param[idx + sk]));
      g += (j == 0 ? 0 : wy * clampf1(c - param[idx - sj]));
      g += (j == Y - 1 ? 0 : wy * clampf1(c - param[idx + sj]));
      g += (i == 0 ? 0 : wz * clampf1(c - param[idx - si]));
      g += (i == X - 1 ? 0 : wz * clampf1(c - param[idx + si]));
    } else {
      const float m = mask[idx];
      g += (k == 0 ? 0 : wx * clampf1(c - param[idx - sk]) * m * mask[idx - sk]);
      g += (k == Z - 1 ? 0 : wx * clampf1(c - param[idx + sk]) * m * mask[idx + sk]);
      g += (j == 0 ? 0 : wy * clampf1(c - param[idx - sj]) * m * mask[idx - sj]);
      g += (j == Y - 1 ? 0 : wy * clampf1(c - param[idx + sj]) * m * mask[idx + sj]);
      g += (i == 0 ? 0 : wz * clampf1(c - param[idx - si]) * m * mask[idx - si]);
      g += (i == X - 1 ? 0 : wz * clampf1(c - param[idx + si]) * m * mask[idx + si]);
    }
    grad[idx] += g;
  }
}

/* ---- adam_upd_kernel.cu:9-133 ---------------------------------------------- */
void vxo_adam_upd(int mode, float* param, const float* grad, float* exp_avg, float* exp_avg_sq, const float* perlr,
                  int64_t n, int step, float beta1, float beta2, float lr, float eps) {
  const float step_size = lr * sqrtf(1 - powf(beta2, (float)step)) / (1 - powf(beta1, (float)step));
  for (int64_t i = 0; i < n; ++i) {
    if (mode == 1 && grad[i] == 0) continue;
    exp_avg[i] = fmaf(beta1, exp_avg[i], (1 - beta1) * grad[i]);
    exp_avg_sq[i] = fmaf(beta2, exp_avg_sq[i], (1 - beta2) * grad[i] * grad[i]);
    if (mode == 2)
      param[i] -= step_size * perlr[i] * exp_avg[i] / (sqrtf(exp_avg_sq[i]) + eps);
    else
      param[i] -= step_size * exp_avg[i] / (sqrtf(exp_avg_sq[i]) + eps);
  }
}

/* ---- ub360_utils_kernel.cu:13-31 (cumdist_thres) ----------------------------- */
void vxo_cumdist_thres(const float* dist, int64_t n_rays, int64_t n_pts, float thres, uint8_t* mask) {
  for (int64_t r = 0; r < n_rays; ++r) {
    float cum = 0.f;
    for (int64_t i = r * n_pts; i < (r + 1) * n_pts; ++i) {
      cum += dist[i];
      const int over = cum > thres;
      cum *= (float)(!over);
      mask[i] = (uint8_t)over;
    }
  }
}

/* |v| as torch's norm reduction forms it (fused multiply-add accumulation). */
static float norm3_fma(float x, float y, float z) { return sqrtf(fmaf(z, z, fmaf(y, y, x * x))); }

/* ---- background samples, lib/voxurf_womask_fine.py:789-818 (sample_ray_ori),
 * :820-825 (outside_sphere_trans, filtered), :857-868 (bg_mask with the
 * cumdist_thres of consecutive inverted points); coarse variant
 * voxurf_womask_coarse.py:633-646 (outbbox_only).  Dense outputs over all
 * [n_rays, n_samples] candidates: pts [.,3], inv [.,3], keep [.]. */
void vxo_bg_samples(const float* rays_o, const float* rays_d, const float* jitter, const float* mn, const float* mx,
                    float near, float far, float stepdist, float dist_thres, int n_samples, int outbbox_only,
                    int64_t n_rays, float* pts, float* inv, uint8_t* keep) {
  for (int64_t r = 0; r < n_rays; ++r) {
    const float* o = rays_o + 3 * r;
    const float* d = rays_d + 3 * r;
    float tmin = -INFINITY, tmax = INFINITY;
    for (int i = 0; i < 3; ++i) {
      const float v = d[i] == 0.f ? 1e-6f : d[i];
      const float ra = (mx[i] - o[i]) / v;
      const float rb = (mn[i] - o[i]) / v;
      tmin = fmaxf(tmin, fminf(ra, rb));
      tmax = fminf(tmax, fmaxf(ra, rb));
    }
    tmin = fminf(fmaxf(tmin, near), far);
    tmax = fminf(fmaxf(tmax, near), far);
    const int miss = tmax <= tmin;
    const float dn = norm3_fma(d[0], d[1], d[2]);
    float cum = 0.f;
    for (int k = 0; k < n_samples; ++k) {
      const int64_t s = r * n_samples + k;
      const float rng = jitter ? (float)k + jitter[r] : (float)k;
      const float t = tmin + (stepdist * rng) / dn;
      float* p = pts + 3 * s;
      float* q = inv + 3 * s;
      for (int i = 0; i < 3; ++i) p[i] = o[i] + d[i] * t;
      const float n = norm3_fma(p[0], p[1], p[2]);
      const float n2 = n * n;
      for (int i = 0; i < 3; ++i) q[i] = p[i] / n2;
      int kp = !(n < 1.f);
      if (outbbox_only) {
        int out = miss;
        for (int i = 0; i < 3; ++i) out = out || (mn[i] > p[i]) || (p[i] > mx[i]);
        kp = kp && out;
      }
      if (k > 0) {
        const float* qp = q - 3;
        const float dx = q[0] - qp[0], dy = q[1] - qp[1], dz = q[2] - qp[2];
        cum += norm3_fma(dx, dy, dz);
        const int over = cum > dist_thres;
        cum *= (float)(!over);
        kp = kp && over;
      }
      keep[s] = (uint8_t)kp;
    }
  }
}

/* ---- correctly rounded a*b+c, elementwise ------------------------------------
 * C99 fmaf rounds once.  The contracted forms of the reference's float
 * expressions (nvcc's default --fmad=true turns a*b+c into one fused
 * multiply-add where it applies) are built from this in oracle/fma_forms.py. */
void vxo_fmaf(const float* a, const float* b, const float* c, float* out, int64_t n) {
  for (int64_t i = 0; i < n; ++i) out[i] = fmaf(a[i], b[i], c[i]);
}
