// The maskless fine model (lib/voxurf_womask_fine.py:833-1071): the pieces
// of its forward and backward that the masked fine model's kernels do not
// cover.  The foreground and background sample sets come from
// vx_bg_samples_* (inner mode for the foreground); alpha2weight, the feature
// rows of the foreground (vx_fine_features / vx_fine_backward) and the MLPs
// are shared with the fine model.
//
//   foreground alpha   sdf + finite-difference gradient on the smoothed SDF
//                      grid (grid_sampler(..., sample_grad=True, displace=1),
//                      :876) and the NeuS alpha (neus_alpha_from_sdf_scatter,
//                      use_mid, :879-880); backward through the same adjoint
//                      as the fine model's march;
//   background alpha   bg_density trilinear at the inverted points and
//                      activate_density: 1 - exp(-softplus(d + act_shift) *
//                      interval) (:898-900, :542-544);
//   background rows    [bg_k0 (12, trilinear at the inverted points),
//                      PE(normalised original point), PE(view)] (:955-970);
//   compositing        in = clamp(sum w sigmoid(logit)), bg = clamp(sum
//                      w_bg sigmoid(bg_logit)), rgb = clamp(in + (1 - sum w)
//                      bg), for the rgbnet and the k-branch (:972-1012), and
//                      its backward by hand.
#include "common.cuh"
#include "fine_device.cuh"
#include "trilinear.cuh"

namespace vx {
namespace {

GridGeom wm_geom(const vx_grid_geom* gg) {
  GridGeom g;
  g.X = (int)gg->X;
  g.Y = (int)gg->Y;
  g.Z = (int)gg->Z;
  for (int a = 0; a < 3; ++a) {
    g.mn[a] = gg->xyz_min[a];
    g.mx[a] = gg->xyz_max[a];
  }
  return g;
}

template <typename T>
__device__ __forceinline__ float elem(const T* row, int c);
template <>
__device__ __forceinline__ float elem<float>(const float* row, int c) { return row[c]; }
template <>
__device__ __forceinline__ float elem<__nv_bfloat16>(const __nv_bfloat16* row, int c) {
  return __bfloat162float(row[c]);
}

inline unsigned wm_blocks(int64_t n, int threads = 256) {
  const int64_t per_wave = (int64_t)sm_count() * 8;
  int64_t b = (n + threads - 1) / threads;
  if (b > per_wave * 4) b = per_wave * 4;
  return (unsigned)(b < 1 ? 1 : b);
}

// ---- foreground alpha --------------------------------------------------------
struct FgAlphaParams {
  int64_t n;
  const float* pts;
  const int64_t* ray_id;
  const float* viewdirs;
  GridGeom g;
  const float* sdf;
  float voxel_size, inv_s, dist;
  float* alpha;
  const float* d_alpha;
  float* d_sdf;
};

template <bool BWD>
__global__ void __launch_bounds__(256) fg_alpha_kernel(FgAlphaParams P) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += (int64_t)gridDim.x * blockDim.x) {
    float d = 0.f;
    if (BWD) {
      d = P.d_alpha[i];
      if (d == 0.f) continue;
    }
    const float p[3] = {P.pts[3 * i], P.pts[3 * i + 1], P.pts[3 * i + 2]};
    const int64_t r = P.ray_id[i];
    const float v[3] = {__ldg(P.viewdirs + 3 * r), __ldg(P.viewdirs + 3 * r + 1), __ldg(P.viewdirs + 3 * r + 2)};
    float ind[3];
    to_index(P.g, p, ind);
    if (BWD) {
      neus_alpha_adjoint_scatter(d, ind, v, P.inv_s, P.dist, P.sdf, P.g, P.voxel_size, P.d_sdf);
    } else {
      float s, gr[3];
      sdf_and_grad(P.sdf, P.g, P.voxel_size, ind, &s, gr);
      P.alpha[i] = neus_alpha(s, gr, v, P.inv_s, P.dist).alpha;
    }
  }
}

// ---- background alpha ---------------------------------------------------------
struct BgAlphaParams {
  int64_t n;
  const float* pts;
  GridGeom g;
  const float* dens;
  float shift, interval;
  float* alpha;
  const float* d_alpha;
  float* d_dens;
};

template <bool BWD>
__global__ void __launch_bounds__(256) bg_alpha_kernel(BgAlphaParams P) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += (int64_t)gridDim.x * blockDim.x) {
    const float p[3] = {P.pts[3 * i], P.pts[3 * i + 1], P.pts[3 * i + 2]};
    float ind[3];
    to_index(P.g, p, ind);
    const Corners c = corners_of(P.g, ind[0], ind[1], ind[2]);
    const float x = gather1(P.dens, c) + P.shift;
    // F.softplus (beta 1, threshold 20)
    const float sp = x > 20.f ? x : log1pf(expf(x));
    const float e = expf(-sp * P.interval);
    if (!BWD) {
      P.alpha[i] = 1.f - e;
    } else {
      const float da = P.d_alpha[i];
      if (da == 0.f) continue;
      // d alpha / d sp = exp(-sp * interval) * interval; softplus' = sigmoid
      // (as torch's softplus backward: z / (z + 1), z = exp(x); 1 above 20)
      float dsp = da * e * P.interval;
      if (!(x > 20.f)) {
        const float z = expf(x);
        dsp = dsp * z / (z + 1.f);
      }
      scatter1(P.d_dens, c, dsp);
    }
  }
}

// ---- background feature rows ------------------------------------------------
struct BgFeatParams {
  int64_t n;
  const float* outer_pts;   // inverted points (bg_k0 lookup)
  const float* pts_org;     // original points (positional encoding)
  const int64_t* ray_id;
  const float* viewdirs;
  GridGeom g;
  const float* k0;          // [X,Y,Z,12] or null (no bg_k0)
  float xyz_min[3], xyz_max[3];
  int pos_pe, view_pe;      // < 0: not used
  int ld, cols;
  void* X;
  int bf16;
  const void* dX;
  float* d_k0;
};

template <typename T>
__global__ void __launch_bounds__(128) bg_features_kernel(BgFeatParams P) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  T* row = reinterpret_cast<T*>(P.X) + i * P.ld;
  int c = 0;
  if (P.k0) {
    const float q[3] = {P.outer_pts[3 * i], P.outer_pts[3 * i + 1], P.outer_pts[3 * i + 2]};
    float ind[3];
    to_index(P.g, q, ind);
    float f[12];
    gatherC<12>(P.k0, corners_of(P.g, ind[0], ind[1], ind[2]), f);
#pragma unroll
    for (int ch = 0; ch < 12; ++ch) put(row, ch, f[ch]);
    c = 12;
  }
  if (P.pos_pe >= 0) {
    float x[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
      x[a] = fdiv(fsub(P.pts_org[3 * i + a], P.xyz_min[a]), fsub(P.xyz_max[a], P.xyz_min[a]));
    c = put_pe(row, c, x, P.pos_pe);
  }
  if (P.view_pe >= 0) {
    const int64_t r = P.ray_id[i];
    const float v[3] = {__ldg(P.viewdirs + 3 * r), __ldg(P.viewdirs + 3 * r + 1), __ldg(P.viewdirs + 3 * r + 2)};
    c = put_pe(row, c, v, P.view_pe);
  }
  for (; c < P.ld; ++c) put(row, c, 0.f);
}

// bg_k0 gradient: columns 0-11 of dX scattered to the eight corners (a
// warp's rows are consecutive samples of a ray; runs sharing a corner are
// summed first).
template <typename T>
__global__ void __launch_bounds__(128) bg_features_bwd_kernel(BgFeatParams P) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < P.n;
  if (__all_sync(0xffffffffu, !live)) return;
  float ind[3] = {0.f, 0.f, 0.f}, d[12];
#pragma unroll
  for (int ch = 0; ch < 12; ++ch) d[ch] = 0.f;
  if (live) {
    const float q[3] = {P.outer_pts[3 * i], P.outer_pts[3 * i + 1], P.outer_pts[3 * i + 2]};
    to_index(P.g, q, ind);
    const T* row = reinterpret_cast<const T*>(P.dX) + i * P.ld;
#pragma unroll
    for (int ch = 0; ch < 12; ++ch) d[ch] = elem(row, ch);
  }
  scatter12_warp(P.d_k0, P.g, ind[0], ind[1], ind[2], d, live);
}

// ---- fg/bg compositing ----------------------------------------------------------
struct WmCompParams {
  int n_rays;
  const int64_t* fg_off;
  const float* w;
  const float* logit;
  const float* kout;      // null: no k-branch
  const int64_t* bg_off;
  const float* bw;
  const float* blogit;
  float* stats;           // [N,10]: sum w sig(logit) (3), sum w sig(k logit) (3), sum w_bg sig(bg logit) (3), sum w
  float* rgb0;            // [N,3] rgb_marched of the rgbnet (rgb_marched0 with a k-branch)
  float* rgbk;            // [N,3] rgb_marched of the k-branch (or null)
  float* ainv;            // [N]   1 - sum w
  float* in_marched;      // [N,3] (k-branch's when present)
  float* bg_marched;      // [N,3]
  const float* g_rgb0;
  const float* g_rgbk;
  const float* g_ainv;
  float* d_logit;
  float* d_kout;
  float* d_w;
  float* d_blogit;
  float* d_bw;
  int k_into_logit;
  int unclamped_parts;    // 1: the in/bg sums enter unclamped (the coarse model)
};

__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.f), 1.f); }
__device__ __forceinline__ bool in01(float x) { return x >= 0.f && x <= 1.f; }
// a per-branch sum as it enters the final mix: clamped (fine model) or not
__device__ __forceinline__ float part(const WmCompParams& P, float x) { return P.unclamped_parts ? x : clamp01(x); }
__device__ __forceinline__ bool part_live(const WmCompParams& P, float x) { return P.unclamped_parts || in01(x); }

__global__ void __launch_bounds__(256) wm_composite_kernel(WmCompParams P) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  float s0[3] = {0.f, 0.f, 0.f}, sk[3] = {0.f, 0.f, 0.f}, sb[3] = {0.f, 0.f, 0.f}, cum = 0.f;
  for (int64_t i = P.fg_off[r] + lane; i < P.fg_off[r + 1]; i += 32) {
    const float w = P.w[i];
    cum += w;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float l = P.logit[3 * i + c];
      s0[c] += w * sigmoidf_(l);
      if (P.kout) sk[c] += w * sigmoidf_(l + P.kout[3 * i + c]);
    }
  }
  for (int64_t j = P.bg_off[r] + lane; j < P.bg_off[r + 1]; j += 32) {
    const float w = P.bw[j];
#pragma unroll
    for (int c = 0; c < 3; ++c) sb[c] += w * sigmoidf_(P.blogit[3 * j + c]);
  }
  cum = warp_sum(cum);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    s0[c] = warp_sum(s0[c]);
    sk[c] = warp_sum(sk[c]);
    sb[c] = warp_sum(sb[c]);
  }
  if (lane == 0) {
    const float one_m = 1.f - cum;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float bgm = part(P, sb[c]);
      const float in0 = part(P, s0[c]);
      P.rgb0[3 * r + c] = clamp01(in0 + one_m * bgm);
      P.bg_marched[3 * r + c] = bgm;
      float inm = in0;
      if (P.kout) {
        const float ink = part(P, sk[c]);
        P.rgbk[3 * r + c] = clamp01(ink + one_m * bgm);
        inm = ink;
      }
      P.in_marched[3 * r + c] = inm;
      P.stats[10 * r + c] = s0[c];
      P.stats[10 * r + 3 + c] = sk[c];
      P.stats[10 * r + 6 + c] = sb[c];
    }
    P.stats[10 * r + 9] = cum;
    P.ainv[r] = one_m;
  }
}

__global__ void __launch_bounds__(256) wm_composite_bwd_kernel(WmCompParams P) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  const float* st = P.stats + 10 * r;
  const float cum = st[9], one_m = 1.f - cum;
  float g_s0[3], g_sk[3], g_sb[3], g_onem = P.g_ainv ? P.g_ainv[r] : 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float bgm = part(P, st[6 + c]);
    float g_bgm = 0.f;
    // rgbnet: rgb0 = clamp(part(s0) + (1 - cum) * part(sb))
    const float in0 = part(P, st[c]);
    const float g_u0 = (P.g_rgb0 && in01(in0 + one_m * bgm)) ? P.g_rgb0[3 * r + c] : 0.f;
    g_s0[c] = part_live(P, st[c]) ? g_u0 : 0.f;
    g_onem += g_u0 * bgm;
    g_bgm += g_u0 * one_m;
    g_sk[c] = 0.f;
    if (P.kout) {
      const float ink = part(P, st[3 + c]);
      const float g_uk = (P.g_rgbk && in01(ink + one_m * bgm)) ? P.g_rgbk[3 * r + c] : 0.f;
      g_sk[c] = part_live(P, st[3 + c]) ? g_uk : 0.f;
      g_onem += g_uk * bgm;
      g_bgm += g_uk * one_m;
    }
    g_sb[c] = part_live(P, st[6 + c]) ? g_bgm : 0.f;
  }
  const float g_cum = -g_onem;
  for (int64_t i = P.fg_off[r] + lane; i < P.fg_off[r + 1]; i += 32) {
    const float w = P.w[i];
    float dw = g_cum;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float l = P.logit[3 * i + c];
      const float y0 = sigmoidf_(l);
      const float dl0 = (w * g_s0[c]) * (1.f - y0) * y0;
      dw += g_s0[c] * y0;
      float dlk = 0.f;
      if (P.kout) {
        const float yk = sigmoidf_(l + P.kout[3 * i + c]);
        dlk = (w * g_sk[c]) * (1.f - yk) * yk;
        dw += g_sk[c] * yk;
        P.d_kout[3 * i + c] = dlk;
      }
      P.d_logit[3 * i + c] = P.k_into_logit ? dl0 + dlk : dl0;
    }
    P.d_w[i] = dw;
  }
  for (int64_t j = P.bg_off[r] + lane; j < P.bg_off[r + 1]; j += 32) {
    const float w = P.bw[j];
    float dw = 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float y = sigmoidf_(P.blogit[3 * j + c]);
      P.d_blogit[3 * j + c] = (w * g_sb[c]) * (1.f - y) * y;
      dw += g_sb[c] * y;
    }
    P.d_bw[j] = dw;
  }
}

inline unsigned warp_grid(int64_t n_rays) { return (unsigned)((n_rays + 7) / 8); }

}  // namespace
}  // namespace vx

using namespace vx;

extern "C" {

int vx_womask_fg_alpha(const vx_womask_fg_alpha_args* a, void* stream) {
  if (!a || a->n < 0) return VX_ERR_ARG;
  if (a->n == 0) return VX_OK;
  const bool bwd = a->d_alpha != nullptr;
  if (!a->pts || !a->ray_id || !a->viewdirs || !a->sdf_smooth || (bwd ? !a->d_sdf_smooth : !a->alpha))
    return VX_ERR_ARG;
  FgAlphaParams P{};
  P.n = a->n;
  P.pts = a->pts;
  P.ray_id = a->ray_id;
  P.viewdirs = a->viewdirs;
  P.g = wm_geom(&a->grid);
  P.sdf = a->sdf_smooth;
  P.voxel_size = a->voxel_size;
  P.inv_s = a->inv_s;
  P.dist = a->dist;
  P.alpha = a->alpha;
  P.d_alpha = a->d_alpha;
  P.d_sdf = a->d_sdf_smooth;
  if (bwd)
    fg_alpha_kernel<true><<<wm_blocks(a->n), 256, 0, as_stream(stream)>>>(P);
  else
    fg_alpha_kernel<false><<<wm_blocks(a->n), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

int vx_womask_bg_alpha(const vx_womask_bg_alpha_args* a, void* stream) {
  if (!a || a->n < 0) return VX_ERR_ARG;
  if (a->n == 0) return VX_OK;
  const bool bwd = a->d_alpha != nullptr;
  if (!a->pts || !a->density || (bwd ? !a->d_density : !a->alpha)) return VX_ERR_ARG;
  BgAlphaParams P{};
  P.n = a->n;
  P.pts = a->pts;
  P.g = wm_geom(&a->grid);
  P.dens = a->density;
  P.shift = a->act_shift;
  P.interval = a->interval;
  P.alpha = a->alpha;
  P.d_alpha = a->d_alpha;
  P.d_dens = a->d_density;
  if (bwd)
    bg_alpha_kernel<true><<<wm_blocks(a->n), 256, 0, as_stream(stream)>>>(P);
  else
    bg_alpha_kernel<false><<<wm_blocks(a->n), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

int vx_womask_bg_features(const vx_womask_bg_features_args* a, void* stream) {
  if (!a || a->n < 0) return VX_ERR_ARG;
  if (a->n == 0) return VX_OK;
  const bool bwd = a->dX != nullptr;
  const int k0c = a->bg_k0 ? 12 : 0;
  const int cols = k0c + (a->posbase_pe >= 0 ? 3 + 6 * (int)a->posbase_pe : 0) +
                   (a->viewbase_pe >= 0 ? 3 + 6 * (int)a->viewbase_pe : 0);
  if (!a->outer_pts || (!bwd && (!a->X || (a->posbase_pe >= 0 && !a->pts_org) ||
                                 (a->viewbase_pe >= 0 && (!a->ray_id || !a->viewdirs)))))
    return VX_ERR_ARG;
  if (bwd && (!a->bg_k0 || !a->d_bg_k0)) return VX_ERR_ARG;
  if (a->ld < cols || a->posbase_pe > 16 || a->viewbase_pe > 16) return VX_ERR_ARG;
  if (a->n > (int64_t)INT32_MAX * 128) return VX_ERR_TOO_LARGE;
  BgFeatParams P{};
  P.n = a->n;
  P.outer_pts = a->outer_pts;
  P.pts_org = a->pts_org;
  P.ray_id = a->ray_id;
  P.viewdirs = a->viewdirs;
  P.g = wm_geom(&a->grid);
  P.k0 = a->bg_k0;
  for (int i = 0; i < 3; ++i) {
    P.xyz_min[i] = a->grid.xyz_min[i];
    P.xyz_max[i] = a->grid.xyz_max[i];
  }
  P.pos_pe = (int)a->posbase_pe;
  P.view_pe = (int)a->viewbase_pe;
  P.ld = (int)a->ld;
  P.cols = cols;
  P.X = a->X;
  P.bf16 = a->bf16;
  P.dX = a->dX;
  P.d_k0 = a->d_bg_k0;
  const unsigned b = (unsigned)((a->n + 127) / 128);
  cudaStream_t st = as_stream(stream);
  if (bwd) {
    if (a->bf16)
      bg_features_bwd_kernel<__nv_bfloat16><<<b, 128, 0, st>>>(P);
    else
      bg_features_bwd_kernel<float><<<b, 128, 0, st>>>(P);
  } else {
    if (a->bf16)
      bg_features_kernel<__nv_bfloat16><<<b, 128, 0, st>>>(P);
    else
      bg_features_kernel<float><<<b, 128, 0, st>>>(P);
  }
  return launch_status();
}

int vx_womask_composite(const vx_womask_composite_args* a, void* stream) {
  if (!a || a->n_rays < 0) return VX_ERR_ARG;
  if (a->n_rays == 0) return VX_OK;
  if (a->n_rays > INT32_MAX / 32) return VX_ERR_TOO_LARGE;
  const bool bwd = a->d_w != nullptr;
  if (!a->fg_off || !a->bg_off || !a->stats) return VX_ERR_ARG;
  if (!bwd && (!a->rgb0 || !a->ainv || !a->in_marched || !a->bg_marched || (a->kout && !a->rgbk))) return VX_ERR_ARG;
  if (bwd && (!a->d_logit || !a->d_blogit || !a->d_bw || (a->kout && !a->d_kout))) return VX_ERR_ARG;
  WmCompParams P{};
  P.n_rays = (int)a->n_rays;
  P.fg_off = a->fg_off;
  P.w = a->w;
  P.logit = a->logit;
  P.kout = a->kout;
  P.bg_off = a->bg_off;
  P.bw = a->bw;
  P.blogit = a->blogit;
  P.stats = a->stats;
  P.rgb0 = a->rgb0;
  P.rgbk = a->rgbk;
  P.ainv = a->ainv;
  P.in_marched = a->in_marched;
  P.bg_marched = a->bg_marched;
  P.g_rgb0 = a->g_rgb0;
  P.g_rgbk = a->g_rgbk;
  P.g_ainv = a->g_ainv;
  P.d_logit = a->d_logit;
  P.d_kout = a->d_kout;
  P.d_w = a->d_w;
  P.d_blogit = a->d_blogit;
  P.d_bw = a->d_bw;
  P.k_into_logit = a->k_into_logit;
  P.unclamped_parts = a->unclamped_parts != 0;
  if (bwd)
    wm_composite_bwd_kernel<<<warp_grid(a->n_rays), 256, 0, as_stream(stream)>>>(P);
  else
    wm_composite_kernel<<<warp_grid(a->n_rays), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

}  // extern "C"
