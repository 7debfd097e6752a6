// Fused per-ray volume rendering of the Voxurf fine model
// (lib/voxurf_fine.py:620-802) and its hand-written backward.
//
// Forward, one warp per ray, 32 samples per iteration:
//   march    : bbox clip + sample positions (render_utils_kernel.cu:12-194,
//              bit-identical to sample_pts_on_rays), mask lookup
//              (render_utils_kernel.cu:374-392), SDF + 6 finite-difference
//              probes on the smoothed grid (voxurf_fine.py:502-577 with
//              displace 1.0), NeuS alpha (voxurf_fine.py:463-500), the
//              alpha > thres compaction (:647-654), the transmittance scan
//              with the T < 1e-3 stop (render_utils_kernel.cu:577-605, FP64
//              carry) and the weight > thres flag (:668-676).  Survivors go to
//              per-ray slots; nothing is written for culled samples.
//   compact  : per-ray survivors of the weight test -> dense rows (ray-major,
//              near-to-far, the order of the reference's masked tensors).
//   features : per shaded row, centre SDF, hierarchical probes (6K values,
//              normalised gradients), k0 trilinear (channel-last, FP32 or
//              BF16 storage), positional encodings -> the two MLP inputs.
//   composite: per ray, sum w*sigmoid(logit) + alphainv_last*bg, k-branch
//              clamped (voxurf_fine.py:753-763).
// Backward recomputes every interpolated value (no per-sample activations
// are stored besides alpha, T, w) and scatters into dense FP32 gradient grids
// with red.global.add (vectorised .v4 for k0).
#include <math.h>
#include "common.cuh"
#include "fine_device.cuh"
#include "trilinear.cuh"

namespace vx {

struct MarchParams {
  const float* rays_o;
  const float* rays_d;
  const float* viewdirs;
  int n_rays;
  float near, stepdist;
  float bmin[3], bmax[3];  // model xyz_min/xyz_max
  GridGeom g;              // SDF grid geometry (same bbox)
  const float* sdf;        // smoothed SDF grid [X,Y,Z]
  float voxel_size;
  const uint8_t* mask;     // optional bool grid for maskcache_lookup semantics
  int mX, mY, mZ;
  float mscale[3], mshift[3];
  int unit_sphere;         // keep only |p| < 1 (the maskless coarse model)
  float inv_s, dist, thres;
  int max_steps;
  // outputs
  float4* rec;        // [n_rays*max_steps] {step|s2flag<<31, alpha, T, w}
  float* dw_slot;     // zeroed at every written slot
  int* n1;            // survivors of alpha > thres up to the stop, per ray
  int* n2;            // of which weight > thres
  float* alphainv_last;
  int* err;
  DensityMask dm;     // optional MaskCache density mask (DENS instantiation)
};

__device__ __forceinline__ bool mask_hit(const MarchParams& P, const float p[3]) {
  return mask_lookup(P.mask, P.mX, P.mY, P.mZ, P.mscale, P.mshift, p);
}

// The march of one ray after its setup; Acc (float or double) carries the
// transmittance product.
template <bool DENS, typename Acc>
__device__ __forceinline__ void march_fine_ray(const MarchParams& P, int r, const RayFrame& f, int64_t n_steps,
                                               const float (&v)[3]) {
  const int lane = lane_id();
  const unsigned lt_mask = (1u << lane) - 1u;
  const int64_t slot0 = (int64_t)r * P.max_steps;
  Acc carry = 1;
  int cnt1 = 0, cnt2 = 0;
  bool stopped = false;
  Acc last = 1;
  for (int base = 0; base < n_steps && !stopped; base += 32) {
    const int k = base + lane;
    bool keep = false;
    float alpha = 0.f;
    if (k < n_steps) {
      float p[3];
      sample_point(f, P.stepdist, k, p);
      bool inb = !outside_bbox(p, P.bmin, P.bmax);
      if (inb && P.unit_sphere) inb = norm3(p[0], p[1], p[2]) < 1.f;
      if (inb && P.mask) inb = mask_hit(P, p);
      if (DENS && inb) inb = density_mask_hit(P.dm, p);
      if (inb) {
        float ind[3], s, gr[3];
        to_index(P.g, p, ind);
        sdf_and_grad(P.sdf, P.g, P.voxel_size, ind, &s, gr);
        alpha = neus_alpha(s, gr, v, P.inv_s, P.dist).alpha;
        keep = alpha > P.thres;
      }
    }
    const unsigned keep_mask = __ballot_sync(0xffffffffu, keep);
    if (keep_mask == 0u) continue;
    const Acc fct = keep ? Acc(1) - (Acc)alpha : Acc(1);
    const Acc incl = warp_inclusive_prod(fct) * carry;
    Acc excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = carry;
    const unsigned stop_mask = __ballot_sync(0xffffffffu, keep && incl < Acc(1e-3));
    unsigned live = keep_mask;
    if (stop_mask) {
      const int ks = __ffs(stop_mask) - 1;
      live &= (ks == 31) ? 0xffffffffu : ((2u << ks) - 1u);
      last = __shfl_sync(0xffffffffu, incl, ks);
      stopped = true;
    }
    const bool mine = (live >> lane) & 1u;
    const float T = (float)excl;
    const float w = T * alpha;
    const bool s2 = mine && (w > P.thres);
    if (mine) {
      const int64_t slot = slot0 + cnt1 + __popc(live & lt_mask);
      const unsigned tag = (unsigned)k | (s2 ? 0x80000000u : 0u);
      P.rec[slot] = make_float4(__uint_as_float(tag), alpha, T, w);
      P.dw_slot[slot] = 0.f;
    }
    cnt1 += __popc(live);
    cnt2 += __popc(__ballot_sync(0xffffffffu, s2));
    if (!stopped) carry = __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) {
    P.n1[r] = cnt1;
    P.n2[r] = cnt2;
    P.alphainv_last[r] = (float)(stopped ? last : carry);
  }
}

template <bool DENS>
__global__ void __launch_bounds__(256, 4) march_fine_kernel(MarchParams P) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  float o[3], d[3], v[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = __ldg(P.rays_o + 3 * r + a);
    d[a] = __ldg(P.rays_d + 3 * r + a);
    v[a] = __ldg(P.viewdirs + 3 * r + a);
  }
  const RayFrame f = ray_frame(o, d, P.bmin, P.bmax, P.near, P.stepdist);
  int64_t n_steps = f.n_steps;
  if (n_steps > P.max_steps) {
    if (lane == 0) set_device_error(P.err, VX_ERR_CAPACITY);
    n_steps = P.max_steps;
  }
  if (f.n_steps > VX_FP32_SCAN_MAX_STEPS)
    march_fine_ray<DENS, double>(P, r, f, n_steps, v);
  else
    march_fine_ray<DENS, float>(P, r, f, n_steps, v);
}

// ---- compaction of the shaded samples -------------------------------------
struct CompactParams {
  const float* rays_o;
  const float* rays_d;
  int n_rays;
  float near, stepdist;
  float bmin[3], bmax[3];
  int max_steps;
  const float4* rec;
  const int* n1;
  const int64_t* s2_off;  // exclusive scan of n2, [n_rays+1]
  // outputs, one row per shaded sample
  int* ray2;
  int* step2;
  int* slot2;
  float* w2;
  float* alpha2;
  float* pts2;  // [S2, 3]
};

__global__ void __launch_bounds__(256) compact_fine_kernel(CompactParams P) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  const int n = P.n1[r];
  int64_t row = P.s2_off[r];
  if (P.s2_off[r + 1] == row) return;
  float o[3], d[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = __ldg(P.rays_o + 3 * r + a);
    d[a] = __ldg(P.rays_d + 3 * r + a);
  }
  const RayFrame f = ray_frame(o, d, P.bmin, P.bmax, P.near, P.stepdist);
  const int64_t slot0 = (int64_t)r * P.max_steps;
  for (int base = 0; base < n; base += 32) {
    const int j = base + lane;
    float4 rc = make_float4(0.f, 0.f, 0.f, 0.f);
    bool s2 = false;
    if (j < n) {
      rc = P.rec[slot0 + j];
      s2 = (__float_as_uint(rc.x) & 0x80000000u) != 0u;
    }
    const unsigned m = __ballot_sync(0xffffffffu, s2);
    if (s2) {
      const int64_t o2 = row + __popc(m & ((1u << lane) - 1u));
      const int k = (int)(__float_as_uint(rc.x) & 0x7fffffffu);
      float p[3];
      sample_point(f, P.stepdist, k, p);
      P.ray2[o2] = r;
      P.step2[o2] = k;
      P.slot2[o2] = (int)(slot0 + j);
      P.w2[o2] = rc.w;
      P.alpha2[o2] = rc.y;
      P.pts2[3 * o2 + 0] = p[0];
      P.pts2[3 * o2 + 1] = p[1];
      P.pts2[3 * o2 + 2] = p[2];
    }
    row += __popc(m);
  }
}

// ---- features of the shaded samples ----------------------------------------
struct FeatParams {
  int64_t n_rows;
  const int* ray2;
  const float* pts2;
  const float* viewdirs;
  GridGeom g;
  const float* sdf;  // smoothed
  float voxel_size;
  const float* k0f;            // [X,Y,Z,12] FP32 (or null)
  const __nv_bfloat16* k0h;    // [X,Y,Z,12] BF16 (or null)
  FeatLayout L;
  int ld1, ld2;                // row strides of X1, X2
  void* X1;
  void* X2;
  int out_bf16;
  // optional per-row outputs for the render path
  float* normal_out;   // [S2,3] gradient (xyz, unnormalised) or null
  int cols1, cols2;    // columns written; [cols, ld) is zero-filled
  const int64_t* n_rows_dev;  // optional device row count (rows beyond it are skipped)
};

// STAGE: the block's rows are assembled in shared memory (bank-conflict-free
// padded stride) and written out one row per warp in coalesced words.
template <typename T, int KK, bool STAGE>
__global__ void __launch_bounds__(128) features_fine_kernel(FeatParams P) {
  extern __shared__ __align__(16) unsigned char feat_stage[];
  const int64_t row0 = (int64_t)blockIdx.x * blockDim.x;
  const int64_t row = row0 + threadIdx.x;
  int64_t n = P.n_rows;
  if (P.n_rows_dev) n = min(n, *P.n_rows_dev);
  const bool valid = row < n;
  T* s1 = reinterpret_cast<T*>(feat_stage);
  const int64_t sl1 = stage_ld<T>(P.ld1), sl2 = stage_ld<T>(P.ld2);
  T* s2 = s1 + (int64_t)blockDim.x * sl1;
  if (valid) {
    const int r = P.ray2[row];
    const float p[3] = {P.pts2[3 * row], P.pts2[3 * row + 1], P.pts2[3 * row + 2]};
    const float v[3] = {__ldg(P.viewdirs + 3 * r), __ldg(P.viewdirs + 3 * r + 1), __ldg(P.viewdirs + 3 * r + 2)};
    T* x1 = STAGE ? s1 + (int64_t)threadIdx.x * sl1 : reinterpret_cast<T*>(P.X1) + row * P.ld1;
    T* x2 = STAGE ? s2 + (int64_t)threadIdx.x * sl2 : reinterpret_cast<T*>(P.X2) + row * P.ld2;
    float g1[3];
    fine_feature_rows<T, KK, STAGE>(P.sdf, P.g, P.voxel_size, P.k0f, P.k0h, P.L, p, v, x1, x2, g1);
    for (int c = P.cols1; c < P.ld1; ++c) put(x1, c, 0.f);
    for (int c = P.cols2; c < P.ld2; ++c) put(x2, c, 0.f);
    if (P.normal_out) {
      P.normal_out[3 * row + 0] = g1[0];
      P.normal_out[3 * row + 1] = g1[1];
      P.normal_out[3 * row + 2] = g1[2];
    }
  }
  if (STAGE) {
    __syncthreads();
    const int nv = (int)max((int64_t)0, min((int64_t)blockDim.x, n - row0));
    copy_rows_out(s1, reinterpret_cast<T*>(P.X1) + row0 * P.ld1, nv, P.ld1);
    copy_rows_out(s2, reinterpret_cast<T*>(P.X2) + row0 * P.ld2, nv, P.ld2);
  }
}

// ---- compositing ------------------------------------------------------------
struct CompositeParams {
  int n_rays;
  const int64_t* s2_off;
  const float* w2;
  const float* logit;    // [S2,3] rgbnet output
  const float* klogit;   // [S2,3] rgb_logit + k_rgbnet output (or null)
  const float* alphainv_last;
  float bg;
  float* rgb0;     // [N,3] sum w*sigmoid(logit) + alphainv*bg
  float* rgbk;     // [N,3] clamp(sum w*sigmoid(klogit) + alphainv*bg, 0, 1) (if klogit)
  float* rgbk_raw; // [N,3] before the clamp
  // optional render extras
  const float* normal2;  // [S2,3] or null
  const int* step2;
  float dist;
  float* normal_out;     // [N,3]
  float* depth_out;      // [N]
  float* wsum_out;       // [N]
  int has_k;             // k-branch present (an empty klogit has a null pointer)
};

__global__ void __launch_bounds__(256) composite_fine_kernel(CompositeParams P) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  const int64_t b = P.s2_off[r], e = P.s2_off[r + 1];
  float a0[3] = {0.f, 0.f, 0.f}, ak[3] = {0.f, 0.f, 0.f}, an[3] = {0.f, 0.f, 0.f};
  float dep = 0.f, ws = 0.f;
  for (int64_t i = b + lane; i < e; i += 32) {
    const float w = P.w2[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      a0[c] += w * sigmoidf_(P.logit[3 * i + c]);
      if (P.has_k) ak[c] += w * sigmoidf_(P.klogit[3 * i + c]);
    }
    ws += w;
    if (P.normal2) {
      const float nx = P.normal2[3 * i], ny = P.normal2[3 * i + 1], nz = P.normal2[3 * i + 2];
      const float inv = 1.f / (sqrtf(nx * nx + ny * ny + nz * nz) + 1e-6f);
      an[0] += w * nx * inv;
      an[1] += w * ny * inv;
      an[2] += w * nz * inv;
    }
    if (P.depth_out) dep += w * ((float)P.step2[i] * P.dist);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    a0[c] = warp_sum(a0[c]);
    ak[c] = warp_sum(ak[c]);
    an[c] = warp_sum(an[c]);
  }
  dep = warp_sum(dep);
  ws = warp_sum(ws);
  if (lane == 0) {
    const float bgt = P.alphainv_last[r] * P.bg;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      P.rgb0[3 * r + c] = a0[c] + bgt;
      if (P.has_k) {
        const float raw = ak[c] + bgt;
        P.rgbk_raw[3 * r + c] = raw;
        P.rgbk[3 * r + c] = fminf(fmaxf(raw, 0.f), 1.f);
      }
      if (P.normal_out) P.normal_out[3 * r + c] = an[c];
    }
    if (P.depth_out) P.depth_out[r] = dep;
    if (P.wsum_out) P.wsum_out[r] = ws;
  }
}

struct CompositeBwdParams {
  int n_rays;
  const int64_t* s2_off;
  const float* w2;
  const float* logit;
  const float* klogit;
  const float* rgbk_raw;
  const float* g_rgb0;  // [N,3] or null
  const float* g_rgbk;  // [N,3] or null
  float bg;
  const float* g_last_in;  // [N] extra grad of alphainv_last (e.g. entropy) or null
  float* d_logit;   // [S2,3]
  float* d_klogit;  // [S2,3] or null
  float* d_w2;      // [S2]
  float* d_last;    // [N]
  int has_k;
};

__global__ void __launch_bounds__(256) composite_fine_bwd_kernel(CompositeBwdParams P) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  float g0[3] = {0.f, 0.f, 0.f}, gk[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (P.g_rgb0) g0[c] = P.g_rgb0[3 * r + c];
    if (P.g_rgbk && P.has_k) {
      const float raw = P.rgbk_raw[3 * r + c];
      gk[c] = (raw >= 0.f && raw <= 1.f) ? P.g_rgbk[3 * r + c] : 0.f;  // clamp backward
    }
  }
  const int64_t b = P.s2_off[r], e = P.s2_off[r + 1];
  for (int64_t i = b + lane; i < e; i += 32) {
    const float w = P.w2[i];
    float dw = 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float y0 = sigmoidf_(P.logit[3 * i + c]);
      P.d_logit[3 * i + c] = (w * g0[c]) * (1.f - y0) * y0;
      dw += g0[c] * y0;
      if (P.has_k) {
        const float yk = sigmoidf_(P.klogit[3 * i + c]);
        P.d_klogit[3 * i + c] = (w * gk[c]) * (1.f - yk) * yk;
        dw += gk[c] * yk;
      }
    }
    P.d_w2[i] = dw;
  }
  if (lane == 0) {
    float dl = P.bg * (g0[0] + g0[1] + g0[2] + gk[0] + gk[1] + gk[2]);
    if (P.g_last_in) dl += P.g_last_in[r];
    P.d_last[r] = dl;
  }
}

// ---- compositing + photometric loss + compositing backward (training) -------
// One warp per ray.  The forward sums of composite_fine_kernel, the loss
// gradient of the ray's colours (known as soon as they are), then the
// backward of composite_fine_bwd_kernel from registers: run.py:604-610 and
// 627 (weight_main * mse(rgb_marched) + weight_rgb0 * mse(rgb_marched0) +
// weight_entropy_last * entropy(alphainv_cum[-1])) differentiated by hand.
// The k-branch logit is logit + kout (voxurf_fine.py:746, FP32 add).  Each
// block leaves its two squared-error sums (rays in warp order) for
// composite_loss_sum_kernel.
struct CompositeLossParams {
  int n_rays;
  const int64_t* s2_off;
  const float* w2;
  const float* logit;
  const float* kout;
  const float* alphainv_last;
  const float* target;
  float bg;
  float g_scale_k, g_scale_0;   // 2 w / (3N) for rgb_marched and rgb_marched0
  float w_entropy;
  float* rgb0;
  float* rgbk;
  float* d_logit;
  float* d_kout;
  float* d_w2;
  float* d_last;
  float2* part;                 // [gridDim.x] (sum dk^2, sum d0^2)
  float* entropy;               // [1] entropy term of the last ray (before its weight)
  int k_into_logit;
};

__global__ void __launch_bounds__(256) composite_loss_fine_kernel(CompositeLossParams P) {
  __shared__ float2 wpart[8];
  const int wib = threadIdx.x >> 5;
  const int r = blockIdx.x * (blockDim.x >> 5) + wib;
  const int lane = lane_id();
  float sk = 0.f, s0 = 0.f;
  if (r < P.n_rays) {
    const int64_t b = P.s2_off[r], e = P.s2_off[r + 1];
    float a0[3] = {0.f, 0.f, 0.f}, ak[3] = {0.f, 0.f, 0.f};
    for (int64_t i = b + lane; i < e; i += 32) {
      const float w = P.w2[i];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float l = P.logit[3 * i + c];
        a0[c] += w * sigmoidf_(l);
        ak[c] += w * sigmoidf_(l + P.kout[3 * i + c]);
      }
    }
    float g0[3], gk[3];
    const float last = P.alphainv_last[r];
    const float bgt = last * P.bg;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float t = P.target[3 * r + c];
      const float rgb0 = warp_sum(a0[c]) + bgt;
      const float raw = warp_sum(ak[c]) + bgt;
      const float rgbk = fminf(fmaxf(raw, 0.f), 1.f);
      const float d0 = rgb0 - t, dk = rgbk - t;
      s0 += d0 * d0;
      sk += dk * dk;
      g0[c] = d0 * P.g_scale_0;
      gk[c] = (raw >= 0.f && raw <= 1.f) ? dk * P.g_scale_k : 0.f;   // clamp backward
      if (lane == 0) {
        P.rgb0[3 * r + c] = rgb0;
        P.rgbk[3 * r + c] = rgbk;
      }
    }
    for (int64_t i = b + lane; i < e; i += 32) {
      const float w = P.w2[i];
      float dw = 0.f;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float l = P.logit[3 * i + c];
        const float y0 = sigmoidf_(l);
        const float yk = sigmoidf_(l + P.kout[3 * i + c]);
        const float dl0 = (w * g0[c]) * (1.f - y0) * y0;
        const float dlk = (w * gk[c]) * (1.f - yk) * yk;
        P.d_logit[3 * i + c] = P.k_into_logit ? dl0 + dlk : dl0;
        P.d_kout[3 * i + c] = dlk;
        dw += g0[c] * y0;
        dw += gk[c] * yk;
      }
      P.d_w2[i] = dw;
    }
    if (lane == 0) {
      float dl = P.bg * (g0[0] + g0[1] + g0[2] + gk[0] + gk[1] + gk[2]);
      if (r == P.n_rays - 1 && P.w_entropy > 0.f) {
        // pout = clamp(alphainv_last, 1e-6, 1 - 1e-6); d/dp of -(p log p + (1-p) log(1-p)) = log(1-p) - log p
        const float lo = 1e-6f, hi = (float)(1.0 - 1e-6);
        const float pc = fminf(fmaxf(last, lo), hi);
        const float lp = logf(pc), lq = logf(1.f - pc);
        P.entropy[0] = -(pc * lp + (1.f - pc) * lq);
        if (last >= lo && last <= hi) dl += P.w_entropy * (lq - lp);
      }
      P.d_last[r] = dl;
    }
  }
  if (lane == 0) wpart[wib] = make_float2(sk, s0);
  __syncthreads();
  if (threadIdx.x == 0) {
    float2 t = make_float2(0.f, 0.f);
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      t.x += wpart[w].x;
      t.y += wpart[w].y;
    }
    P.part[blockIdx.x] = t;
  }
}

// loss = w_main * sum_k / (3N) + w_rgb0 * sum_0 / (3N) + w_entropy * entropy,
// the block partials added in a fixed order (each thread a contiguous run,
// then the 256 run sums in thread order).
__global__ void __launch_bounds__(256) composite_loss_sum_kernel(const float2* part, int n_part, const float* entropy,
                                                                 float w_main, float w_rgb0, float w_entropy,
                                                                 float inv_numel, float* loss) {
  __shared__ float2 s[256];
  const int per = (n_part + 255) / 256, k0 = threadIdx.x * per, k1 = min(n_part, k0 + per);
  float2 t = make_float2(0.f, 0.f);
  for (int k = k0; k < k1; ++k) {
    t.x += part[k].x;
    t.y += part[k].y;
  }
  s[threadIdx.x] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    float2 a = make_float2(0.f, 0.f);
    for (int i = 0; i < 256; ++i) {
      a.x += s[i].x;
      a.y += s[i].y;
    }
    float l = w_main * (a.x * inv_numel) + w_rgb0 * (a.y * inv_numel);
    if (w_entropy > 0.f) l += w_entropy * entropy[0];
    loss[0] = l;
  }
}

// ---- backward: features of shaded rows -> dense gradient grids ---------------
struct FeatBwdParams {
  int64_t n_rows;
  const float* pts2;
  GridGeom g;
  const float* sdf;  // smoothed (recompute)
  float voxel_size;
  int K;
  float disp[MAX_K];
  int k_unit;
  int pos_pe, view_pe, kpos_pe, kview_pe;
  int center_sdf, use_rgbnet_k0, k_center_sdf;
  int ld1, ld2;
  const void* dX1;
  const void* dX2;
  int in_bf16;
  const float* dw2;      // [S2] weight grads (scattered to slots)
  const int* slot2;
  float* dw_slot;
  float* d_sdf;          // [X,Y,Z] grad of the smoothed grid
  float* d_k0;           // [X,Y,Z,12] channel-last
  const int64_t* n_rows_dev;  // optional device row count (rows beyond it are skipped)
  uint8_t* k0_touched;        // optional [X*Y*Z] marks of the k0 voxels scattered to
};

template <typename T>
__device__ __forceinline__ float get(const T* row, int c);
template <>
__device__ __forceinline__ float get<float>(const float* row, int c) { return row[c]; }
template <>
__device__ __forceinline__ float get<__nv_bfloat16>(const __nv_bfloat16* row, int c) {
  return __bfloat162float(row[c]);
}

// Thread per shaded row.  Scatters: the centre value and every probe of the
// SDF go through per-axis plane accumulators (PlaneAcc: the 8 + 48 K corner
// additions of a row become about 20 per axis), k0 through the warp's
// segmented reduction over runs of lanes sharing a corner (scatter12_warp).
template <typename T>
__global__ void __launch_bounds__(128) features_fine_bwd_kernel(FeatBwdParams P) {
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = row < P.n_rows && !(P.n_rows_dev && row >= *P.n_rows_dev);
  if (__all_sync(0xffffffffu, !live)) return;
  float ind[3] = {0.f, 0.f, 0.f};
  float dk0[12];
#pragma unroll
  for (int ch = 0; ch < 12; ++ch) dk0[ch] = 0.f;
  const T* dx1 = nullptr;
  const T* dx2 = nullptr;
  float d_center = 0.f, dgx = 0.f, dgy = 0.f, dgz = 0.f;
  int feat_col = 0, grad_col = 0;
  if (live) {
    if (P.dw_slot) P.dw_slot[P.slot2[row]] = P.dw2[row];
    const float p[3] = {P.pts2[3 * row], P.pts2[3 * row + 1], P.pts2[3 * row + 2]};
    to_index(P.g, p, ind);
    dx1 = reinterpret_cast<const T*>(P.dX1) + row * P.ld1;
    dx2 = reinterpret_cast<const T*>(P.dX2) + row * P.ld2;
    // column layout (must mirror features_fine_kernel)
    int c1 = (P.use_rgbnet_k0 ? 12 : 0) + (3 + 6 * P.pos_pe) + (3 + 6 * P.view_pe);
    if (P.center_sdf) d_center += get(dx1, c1++);
    feat_col = c1;
    grad_col = c1 + 6 * P.K;
    int c2 = 12 + (3 + 6 * P.kpos_pe) + (3 + 6 * P.kview_pe);
    dgx = get(dx2, c2);
    dgy = get(dx2, c2 + 1);
    dgz = get(dx2, c2 + 2);
    c2 += 3;
    if (P.k_center_sdf) d_center += get(dx2, c2++);
#pragma unroll
    for (int ch = 0; ch < 12; ++ch) dk0[ch] = get(dx2, ch);
    if (P.use_rgbnet_k0)
#pragma unroll
      for (int ch = 0; ch < 12; ++ch) dk0[ch] += get(dx1, ch);
  }
  scatter12_warp(P.d_k0, P.g, ind[0], ind[1], ind[2], dk0, live);
  if (!live) return;
  if (P.k0_touched) mark_corners(P.k0_touched, corners_of(P.g, ind[0], ind[1], ind[2]));
  PlaneAcc acc[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) plane_acc_init(acc[a], ind[a]);
  plane_acc_add(acc[0], P.d_sdf, P.g, ind, 0, ind[0], d_center);
  // hierarchical probes
  for (int kk = 0; kk < P.K; ++kk) {
    float fm[3], fp[3], invd[3], gr[3], xm[3], xp[3];
#pragma unroll
    for (int pair = 0; pair < 3; ++pair) {
      Probe pr;
      const int axis = 2 - pair;
      probe_axis(P.sdf, P.g, ind, axis, P.disp[kk], pr, false);
      fm[pair] = pr.fm;
      fp[pair] = pr.fp;
      invd[pair] = pr.inv_diff;
      gr[pair] = ((pr.fp - pr.fm) * pr.inv_diff) / P.voxel_size;
      const float hi = (float)(gsize(P.g, axis) - 1);
      xm[pair] = fminf(fmaxf(ind[axis] - P.disp[kk], 0.f), hi);
      xp[pair] = fminf(fmaxf(ind[axis] + P.disp[kk], 0.f), hi);
    }
    // d of the normalised gradient: n = g / (|g| + eps)
    const float sn = sqrtf(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
    const float den = sn + 1e-5f;
    float dn[3], dg[3];
#pragma unroll
    for (int pair = 0; pair < 3; ++pair) dn[pair] = get(dx1, grad_col + pair * P.K + kk);
    const float gdn = gr[0] * dn[0] + gr[1] * dn[1] + gr[2] * dn[2];
    const float corr = sn > 0.f ? gdn / (sn * den * den) : 0.f;
#pragma unroll
    for (int pair = 0; pair < 3; ++pair) dg[pair] = dn[pair] / den - gr[pair] * corr;
    if (kk == P.k_unit) {
      dg[0] += dgz;  // pairs are z, y, x
      dg[1] += dgy;
      dg[2] += dgx;
    }
#pragma unroll
    for (int pair = 0; pair < 3; ++pair) {
      const float dfd = dg[pair] * invd[pair] / P.voxel_size;  // d(fp - fm)
      const float dfm = get(dx1, feat_col + (2 * pair + 0) * P.K + kk) - dfd;
      const float dfp = get(dx1, feat_col + (2 * pair + 1) * P.K + kk) + dfd;
      const int axis = 2 - pair;
      plane_acc_add(acc[axis], P.d_sdf, P.g, ind, axis, xm[pair], dfm);
      plane_acc_add(acc[axis], P.d_sdf, P.g, ind, axis, xp[pair], dfp);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) plane_acc_flush(acc[a], P.d_sdf, P.g, ind, a);
}

// ---- backward: transmittance scan + NeuS alpha, per ray ----------------------
struct GeomBwdParams {
  const float* rays_o;
  const float* rays_d;
  const float* viewdirs;
  int n_rays;
  float near, stepdist;
  float bmin[3], bmax[3];
  GridGeom g;
  const float* sdf;
  float voxel_size;
  float inv_s, dist;
  int max_steps;
  const float4* rec;
  const float* dw_slot;
  const int* n1;
  const float* alphainv_last;
  const float* d_last;
  float* d_sdf;
  const float* inv_s_dev;  // optional device copy of inv_s (overrides inv_s)
};

__global__ void __launch_bounds__(256) geometry_fine_bwd_kernel(GeomBwdParams P) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  const int n = P.n1[r];
  if (n == 0) return;
  const float inv_s = P.inv_s_dev ? *P.inv_s_dev : P.inv_s;
  float o[3], d[3], v[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = __ldg(P.rays_o + 3 * r + a);
    d[a] = __ldg(P.rays_d + 3 * r + a);
    v[a] = __ldg(P.viewdirs + 3 * r + a);
  }
  const RayFrame f = ray_frame(o, d, P.bmin, P.bmax, P.near, P.stepdist);
  const int64_t slot0 = (int64_t)r * P.max_steps;
  // suffix sums of the transmittance backward: FP64 for rays of more than
  // 512 samples (as the forward's products), FP32 otherwise
  const bool wide = f.n_steps > VX_FP32_SCAN_MAX_STEPS;
  double carry_d = (double)(P.d_last[r] * P.alphainv_last[r]);
  float carry_f = P.d_last[r] * P.alphainv_last[r];
  for (int top = n; top > 0; top -= 32) {
    const int j = top - 32 + lane;
    const bool valid = j >= 0;
    float4 rc = make_float4(0.f, 0.f, 0.f, 0.f);
    float gw = 0.f;
    if (valid) {
      rc = P.rec[slot0 + j];
      gw = P.dw_slot[slot0 + j];
    }
    const float alpha = rc.y, T = rc.z, w = rc.w;
    float d_alpha;
    if (wide) {
      const double term = valid ? (double)(gw * w) : 0.0;
      const double suffix = warp_inclusive_suffix_sum(term);
      double after = __shfl_down_sync(0xffffffffu, suffix, 1);
      if (lane == 31) after = 0.0;
      const double back = carry_d + after;
      carry_d += __shfl_sync(0xffffffffu, suffix, 0);
      d_alpha = (float)((double)(gw * T) - back / ((double)(1.f - alpha) + 1e-10));
    } else {
      const float term = valid ? gw * w : 0.f;
      const float suffix = warp_inclusive_suffix_sum(term);
      float after = __shfl_down_sync(0xffffffffu, suffix, 1);
      if (lane == 31) after = 0.f;
      const float back = carry_f + after;
      carry_f += __shfl_sync(0xffffffffu, suffix, 0);
      d_alpha = gw * T - back / ((1.f - alpha) + 1e-10f);
    }
    if (!valid) continue;
    if (d_alpha == 0.f) continue;
    const int k = (int)(__float_as_uint(rc.x) & 0x7fffffffu);
    float p[3], ind[3];
    sample_point(f, P.stepdist, k, p);
    to_index(P.g, p, ind);
    neus_alpha_adjoint_scatter(d_alpha, ind, v, inv_s, P.dist, P.sdf, P.g, P.voxel_size, P.d_sdf);
  }
}

// =============================================================================
// Coarse model (lib/voxurf_coarse.py:513-619)
//   sdf      : trilinear on the (smoothed) SDF grid
//   gradient : trilinear on the central-difference gradient grid of the RAW
//              SDF (neus_sdf_gradient, :323-332), stored [X,Y,Z,4]
//   alpha    : as the fine model
//   weights  : Alphas2Weights over all in-bbox samples (:540) only decides the
//              weight > thres set; a second Alphas2Weights over that set
//              (:550) gives the weights that are rendered and differentiated.
// =============================================================================

__device__ __forceinline__ void gather_grad4(const float* __restrict__ G4, const Corners& c, float g[3]) {
  g[0] = g[1] = g[2] = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (c.off[q] < 0) continue;
    const float4 v = __ldg(reinterpret_cast<const float4*>(G4) + c.off[q]);
    g[0] += c.w[q] * v.x;
    g[1] += c.w[q] * v.y;
    g[2] += c.w[q] * v.z;
  }
}

__device__ __forceinline__ void scatter_grad4(float* __restrict__ dG4, const Corners& c, const float d[3]) {
  if (d[0] == 0.f && d[1] == 0.f && d[2] == 0.f) return;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (c.off[q] < 0 || c.w[q] == 0.f) continue;
    red_add_v4(dG4 + 4 * (int64_t)c.off[q], c.w[q] * d[0], c.w[q] * d[1], c.w[q] * d[2], 0.f);
  }
}

struct CoarseMarchParams {
  MarchParams m;       // rays, frame, grids, mask, alpha constants, outputs
  const float* G4;     // [X,Y,Z,4] gradient grid of the raw SDF
  int* n2b;            // records up to the second scan's stop (backward range)
};

// The coarse march of one ray after its setup; Acc (float or double)
// carries the two transmittance products.
template <bool DENS, typename Acc>
__device__ __forceinline__ void march_coarse_ray(const CoarseMarchParams& C, int r, const RayFrame& f,
                                                 int64_t n_steps, const float (&v)[3]) {
  const MarchParams& P = C.m;
  const int lane = lane_id();
  const unsigned lt_mask = (1u << lane) - 1u;
  const int64_t slot0 = (int64_t)r * P.max_steps;
  Acc carry1 = 1, carry2 = 1, last2 = 1;
  bool stop1 = false, stop2 = false;
  int cnt = 0, cnt_b = 0;
  for (int base = 0; base < n_steps && !stop1; base += 32) {
    const int k = base + lane;
    bool inb = false;
    float alpha = 0.f;
    if (k < n_steps) {
      float p[3];
      sample_point(f, P.stepdist, k, p);
      inb = !outside_bbox(p, P.bmin, P.bmax);
      if (inb && P.unit_sphere) inb = norm3(p[0], p[1], p[2]) < 1.f;
      if (inb && P.mask) inb = mask_hit(P, p);
      if (DENS && inb) inb = density_mask_hit(P.dm, p);
      if (inb) {
        float ind[3], gr[3];
        to_index(P.g, p, ind);
        const Corners c = corners_of(P.g, ind[0], ind[1], ind[2]);
        const float s = gather1(P.sdf, c);
        gather_grad4(C.G4, c, gr);
        alpha = neus_alpha(s, gr, v, P.inv_s, P.dist).alpha;
      }
    }
    const unsigned in_mask = __ballot_sync(0xffffffffu, inb);
    if (in_mask == 0u) continue;
    // first scan: every in-bbox sample
    const Acc f1 = inb ? Acc(1) - (Acc)alpha : Acc(1);
    const Acc incl1 = warp_inclusive_prod(f1) * carry1;
    Acc excl1 = __shfl_up_sync(0xffffffffu, incl1, 1);
    if (lane == 0) excl1 = carry1;
    const unsigned s1 = __ballot_sync(0xffffffffu, inb && incl1 < Acc(1e-3));
    unsigned live1 = in_mask;
    if (s1) {
      const int ks = __ffs(s1) - 1;
      live1 &= (ks == 31) ? 0xffffffffu : ((2u << ks) - 1u);
      stop1 = true;
    } else {
      carry1 = __shfl_sync(0xffffffffu, incl1, 31);
    }
    const float w1 = (float)excl1 * alpha;
    const bool sel = ((live1 >> lane) & 1u) && (w1 > P.thres);
    const unsigned sel_mask = __ballot_sync(0xffffffffu, sel);
    if (sel_mask == 0u) continue;
    // second scan: the selected samples only
    float T2 = 1.f, w2 = 0.f;
    unsigned live2 = 0u;
    if (!stop2) {
      const Acc f2 = sel ? Acc(1) - (Acc)alpha : Acc(1);
      const Acc incl2 = warp_inclusive_prod(f2) * carry2;
      Acc excl2 = __shfl_up_sync(0xffffffffu, incl2, 1);
      if (lane == 0) excl2 = carry2;
      const unsigned s2 = __ballot_sync(0xffffffffu, sel && incl2 < Acc(1e-3));
      live2 = sel_mask;
      if (s2) {
        const int ks = __ffs(s2) - 1;
        live2 &= (ks == 31) ? 0xffffffffu : ((2u << ks) - 1u);
        last2 = __shfl_sync(0xffffffffu, incl2, ks);
        stop2 = true;
      } else {
        carry2 = __shfl_sync(0xffffffffu, incl2, 31);
      }
      if ((live2 >> lane) & 1u) {
        T2 = (float)excl2;
        w2 = T2 * alpha;
      }
    }
    if (sel) {
      const int64_t slot = slot0 + cnt + __popc(sel_mask & lt_mask);
      const unsigned tag = (unsigned)k | 0x80000000u;
      P.rec[slot] = make_float4(__uint_as_float(tag), alpha, T2, w2);
      P.dw_slot[slot] = 0.f;
    }
    cnt += __popc(sel_mask);
    cnt_b += __popc(live2);
  }
  if (lane == 0) {
    P.n1[r] = cnt;
    P.n2[r] = cnt;
    C.n2b[r] = cnt_b;
    P.alphainv_last[r] = (float)(stop2 ? last2 : carry2);
  }
}

template <bool DENS>
__global__ void __launch_bounds__(256) march_coarse_kernel(CoarseMarchParams C) {
  const MarchParams& P = C.m;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  float o[3], d[3], v[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = __ldg(P.rays_o + 3 * r + a);
    d[a] = __ldg(P.rays_d + 3 * r + a);
    v[a] = __ldg(P.viewdirs + 3 * r + a);
  }
  const RayFrame f = ray_frame(o, d, P.bmin, P.bmax, P.near, P.stepdist);
  int64_t n_steps = f.n_steps;
  if (n_steps > P.max_steps) {
    if (lane == 0) set_device_error(P.err, VX_ERR_CAPACITY);
    n_steps = P.max_steps;
  }
  if (f.n_steps > VX_FP32_SCAN_MAX_STEPS)
    march_coarse_ray<DENS, double>(C, r, f, n_steps, v);
  else
    march_coarse_ray<DENS, float>(C, r, f, n_steps, v);
}

struct CoarseFeatParams {
  int64_t n_rows;
  const int* ray2;
  const float* pts2;
  const float* viewdirs;
  GridGeom g;
  const float* G4;
  const float* k0f;
  const __nv_bfloat16* k0h;
  int use_k0, pos_pe, view_pe, geo_rgb_dim;
  int ld;
  void* X;
  float* normal_out;  // [S2,3] interpolated gradient (unnormalised)
};

template <typename T>
__global__ void __launch_bounds__(128) features_coarse_kernel(CoarseFeatParams P) {
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= P.n_rows) return;
  const int r = P.ray2[row];
  const float p[3] = {P.pts2[3 * row], P.pts2[3 * row + 1], P.pts2[3 * row + 2]};
  const float v[3] = {__ldg(P.viewdirs + 3 * r), __ldg(P.viewdirs + 3 * r + 1), __ldg(P.viewdirs + 3 * r + 2)};
  float ind[3];
  to_index(P.g, p, ind);
  const Corners c = corners_of(P.g, ind[0], ind[1], ind[2]);
  T* x = reinterpret_cast<T*>(P.X) + row * P.ld;
  int col = 0;
  if (P.use_k0) {
    float k0v[12];
    if (P.k0h)
      gatherC<12>(P.k0h, c, k0v);
    else
      gatherC<12>(P.k0f, c, k0v);
    for (int ch = 0; ch < 12; ++ch) put(x, col++, k0v[ch]);
  }
  float xyzn[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) xyzn[a] = (p[a] - P.g.mn[a]) / (P.g.mx[a] - P.g.mn[a]);
  col = put_pe(x, col, xyzn, P.pos_pe);
  col = put_pe(x, col, v, P.view_pe);
  float gr[3];
  gather_grad4(P.G4, c, gr);
  if (P.geo_rgb_dim == 3) {
    const float inv = 1.f / (sqrtf(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]) + 1e-5f);
    put(x, col++, gr[0] * inv);
    put(x, col++, gr[1] * inv);
    put(x, col++, gr[2] * inv);
  }
  for (; col < P.ld; ++col) put(x, col, 0.f);   // pad columns of the MLP row stride
  if (P.normal_out) {
    P.normal_out[3 * row + 0] = gr[0];
    P.normal_out[3 * row + 1] = gr[1];
    P.normal_out[3 * row + 2] = gr[2];
  }
}

// rgb = clamp(sum w*sigmoid(logit) + (1 - sum w)*bg, 0, 1) (voxurf_coarse.py:575-584)
struct CoarseCompositeParams {
  int n_rays;
  const int64_t* s2_off;
  const float* w2;
  const float* logit;
  float bg;
  float* rgb;
  float* rgb_raw;
  const float* normal2;
  const int* step2;
  float dist;
  float* normal_out;
  float* depth_out;
  float* wsum_out;
};

__global__ void __launch_bounds__(256) composite_coarse_kernel(CoarseCompositeParams P) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  const int64_t b = P.s2_off[r], e = P.s2_off[r + 1];
  float a0[3] = {0.f, 0.f, 0.f}, an[3] = {0.f, 0.f, 0.f}, ws = 0.f, dep = 0.f;
  for (int64_t i = b + lane; i < e; i += 32) {
    const float w = P.w2[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) a0[c] += w * sigmoidf_(P.logit[3 * i + c]);
    ws += w;
    if (P.normal2) {
      const float nx = P.normal2[3 * i], ny = P.normal2[3 * i + 1], nz = P.normal2[3 * i + 2];
      const float inv = 1.f / (sqrtf(nx * nx + ny * ny + nz * nz) + 1e-6f);
      an[0] += w * nx * inv;
      an[1] += w * ny * inv;
      an[2] += w * nz * inv;
    }
    if (P.depth_out) dep += w * ((float)P.step2[i] * P.dist);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    a0[c] = warp_sum(a0[c]);
    an[c] = warp_sum(an[c]);
  }
  ws = warp_sum(ws);
  dep = warp_sum(dep);
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float raw = a0[c] + (1.f - ws) * P.bg;
      P.rgb_raw[3 * r + c] = raw;
      P.rgb[3 * r + c] = fminf(fmaxf(raw, 0.f), 1.f);
      if (P.normal_out) P.normal_out[3 * r + c] = an[c];
    }
    if (P.wsum_out) P.wsum_out[r] = ws;
    if (P.depth_out) P.depth_out[r] = dep;
  }
}

struct CoarseCompositeBwdParams {
  int n_rays;
  const int64_t* s2_off;
  const float* w2;
  const float* logit;
  const float* rgb_raw;
  const float* g_rgb;
  float bg;
  float* d_logit;
  float* d_w2;
};

__global__ void __launch_bounds__(256) composite_coarse_bwd_kernel(CoarseCompositeBwdParams P) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  float g[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float raw = P.rgb_raw[3 * r + c];
    g[c] = (raw >= 0.f && raw <= 1.f) ? P.g_rgb[3 * r + c] : 0.f;
  }
  const float gbg = P.bg * (g[0] + g[1] + g[2]);
  const int64_t b = P.s2_off[r], e = P.s2_off[r + 1];
  for (int64_t i = b + lane; i < e; i += 32) {
    const float w = P.w2[i];
    float dw = -gbg;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float y = sigmoidf_(P.logit[3 * i + c]);
      P.d_logit[3 * i + c] = (w * g[c]) * (1.f - y) * y;
      dw += g[c] * y;
    }
    P.d_w2[i] = dw;
  }
}

struct CoarseBwdParams {
  GeomBwdParams gb;     // rays, frame, grid, sdf (smoothed), alpha constants, records
  const int* n2b;       // backward range per ray
  const float* G4;
  float* dG4;           // [X,Y,Z,4] gradient of the gradient grid
  // per-row feature backward
  int64_t n_rows;
  const float* pts2;
  const int* slot2;
  const float* dw2;
  float* dw_slot;
  int use_k0, pos_pe, view_pe, geo_rgb_dim, ld, in_bf16;
  const void* dX;
  float* d_k0;
  const float* d_grad2;  // optional [S2,3] gradient of the raw interpolated gradient
};

template <typename T>
__global__ void __launch_bounds__(128) features_coarse_bwd_kernel(CoarseBwdParams P) {
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= P.n_rows) return;
  P.dw_slot[P.slot2[row]] = P.dw2[row];
  const float p[3] = {P.pts2[3 * row], P.pts2[3 * row + 1], P.pts2[3 * row + 2]};
  float ind[3];
  to_index(P.gb.g, p, ind);
  const Corners c = corners_of(P.gb.g, ind[0], ind[1], ind[2]);
  const T* dx = reinterpret_cast<const T*>(P.dX) + row * P.ld;
  if (P.use_k0) {
    float dk0[12];
#pragma unroll
    for (int ch = 0; ch < 12; ++ch) dk0[ch] = get(dx, ch);
    scatterC<12>(P.d_k0, c, dk0);
  }
  float dg[3] = {0.f, 0.f, 0.f};
  if (P.geo_rgb_dim == 3) {
    const int col = (P.use_k0 ? 12 : 0) + (3 + 6 * P.pos_pe) + (3 + 6 * P.view_pe);
    float gr[3];
    gather_grad4(P.G4, c, gr);
    const float sn = sqrtf(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
    const float den = sn + 1e-5f;
    const float dn[3] = {get(dx, col), get(dx, col + 1), get(dx, col + 2)};
    const float gdn = gr[0] * dn[0] + gr[1] * dn[1] + gr[2] * dn[2];
    const float corr = sn > 0.f ? gdn / (sn * den * den) : 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) dg[a] = dn[a] / den - gr[a] * corr;
  }
  if (P.d_grad2) {
#pragma unroll
    for (int a = 0; a < 3; ++a) dg[a] += P.d_grad2[3 * row + a];
  }
  scatter_grad4(P.dG4, c, dg);
}

__global__ void __launch_bounds__(256) geometry_coarse_bwd_kernel(CoarseBwdParams C) {
  const GeomBwdParams& P = C.gb;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  const int n = C.n2b[r];
  if (n == 0) return;
  float o[3], d[3], v[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = __ldg(P.rays_o + 3 * r + a);
    d[a] = __ldg(P.rays_d + 3 * r + a);
    v[a] = __ldg(P.viewdirs + 3 * r + a);
  }
  const RayFrame f = ray_frame(o, d, P.bmin, P.bmax, P.near, P.stepdist);
  const int64_t slot0 = (int64_t)r * P.max_steps;
  // suffix sums of the transmittance backward: FP64 for rays of more than
  // 512 samples (as the forward's products), FP32 otherwise
  const bool wide = f.n_steps > VX_FP32_SCAN_MAX_STEPS;
  double carry_d = (double)(P.d_last[r] * P.alphainv_last[r]);
  float carry_f = P.d_last[r] * P.alphainv_last[r];
  for (int top = n; top > 0; top -= 32) {
    const int j = top - 32 + lane;
    const bool valid = j >= 0;
    float4 rc = make_float4(0.f, 0.f, 0.f, 0.f);
    float gw = 0.f;
    if (valid) {
      rc = P.rec[slot0 + j];
      gw = P.dw_slot[slot0 + j];
    }
    const float alpha = rc.y, T = rc.z, w = rc.w;
    float d_alpha;
    if (wide) {
      const double term = valid ? (double)(gw * w) : 0.0;
      const double suffix = warp_inclusive_suffix_sum(term);
      double after = __shfl_down_sync(0xffffffffu, suffix, 1);
      if (lane == 31) after = 0.0;
      const double back = carry_d + after;
      carry_d += __shfl_sync(0xffffffffu, suffix, 0);
      d_alpha = (float)((double)(gw * T) - back / ((double)(1.f - alpha) + 1e-10));
    } else {
      const float term = valid ? gw * w : 0.f;
      const float suffix = warp_inclusive_suffix_sum(term);
      float after = __shfl_down_sync(0xffffffffu, suffix, 1);
      if (lane == 31) after = 0.f;
      const float back = carry_f + after;
      carry_f += __shfl_sync(0xffffffffu, suffix, 0);
      d_alpha = gw * T - back / ((1.f - alpha) + 1e-10f);
    }
    if (!valid) continue;
    if (d_alpha == 0.f) continue;
    const int k = (int)(__float_as_uint(rc.x) & 0x7fffffffu);
    float p[3], ind[3], gr[3];
    sample_point(f, P.stepdist, k, p);
    to_index(P.g, p, ind);
    const Corners c = corners_of(P.g, ind[0], ind[1], ind[2]);
    const float s = gather1(P.sdf, c);
    gather_grad4(C.G4, c, gr);
    const AlphaState a = neus_alpha(s, gr, v, P.inv_s, P.dist);
    if (!(a.raw >= 0.f && a.raw <= 1.f)) continue;
    const float den = a.P + 1e-5f;
    const float dP = d_alpha * a.Q / (den * den);
    const float dQ = -d_alpha / den;
    const float d_prev = dP * a.P * a.nP * P.inv_s;
    const float d_next = dQ * a.Q * a.nQ * P.inv_s;
    const float d_ic = (d_next - d_prev) * P.dist * 0.5f;
    const float d_cos = a.cosv < 0.f ? d_ic : 0.f;
    scatter1(P.d_sdf, c, d_prev + d_next);
    const float dg[3] = {d_cos * v[0], d_cos * v[1], d_cos * v[2]};
    scatter_grad4(C.dG4, c, dg);
  }
}

inline unsigned warp_blocks(int64_t n_items, int warps_per_block = 8) {
  return (unsigned)((n_items + warps_per_block - 1) / warps_per_block);
}

// ---- generic DenseGrid.forward (lib/grid.py:47-58) and its adjoint ------------
__global__ void grid_sample_kernel(const float* __restrict__ grid, int C, int channel_last, GridGeom g,
                                   const float* __restrict__ xyz, int64_t n, float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float p[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
  float ind[3];
  to_index(g, p, ind);
  const Corners c = corners_of(g, ind[0], ind[1], ind[2]);
  const int64_t vox = (int64_t)g.X * g.Y * g.Z;
  for (int ch = 0; ch < C; ++ch) {
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (c.off[q] < 0) continue;
      const int64_t o = channel_last ? (int64_t)c.off[q] * C + ch : (int64_t)ch * vox + c.off[q];
      acc += c.w[q] * __ldg(grid + o);
    }
    out[i * C + ch] = acc;
  }
}

__global__ void grid_sample_bwd_kernel(const float* __restrict__ grad_out, int C, int channel_last, GridGeom g,
                                       const float* __restrict__ xyz, int64_t n, float* __restrict__ grad_grid) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float p[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
  float ind[3];
  to_index(g, p, ind);
  const Corners c = corners_of(g, ind[0], ind[1], ind[2]);
  const int64_t vox = (int64_t)g.X * g.Y * g.Z;
  for (int ch = 0; ch < C; ++ch) {
    const float d = grad_out[i * C + ch];
    if (d == 0.f) continue;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (c.off[q] < 0 || c.w[q] == 0.f) continue;
      const int64_t o = channel_last ? (int64_t)c.off[q] * C + ch : (int64_t)ch * vox + c.off[q];
      atomicAdd(grad_grid + o, c.w[q] * d);
    }
  }
}

}  // namespace vx

using namespace vx;

// The C ABI below takes the parameter structs declared in voxurf_gb300.h;
// they mirror the device structs field by field.
extern "C" {

static GridGeom geom_from(const vx_grid_geom* gg) {
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

int vx_grid_sample(const float* grid, int64_t C, int channel_last, const vx_grid_geom* geom, const float* xyz,
                   int64_t n_pts, float* out, void* stream) {
  if (!geom || C <= 0 || n_pts < 0) return VX_ERR_ARG;
  if (n_pts == 0) return VX_OK;
  if (!grid || !xyz || !out) return VX_ERR_ARG;
  if (geom->X * geom->Y * geom->Z > INT32_MAX) return VX_ERR_ARG;
  grid_sample_kernel<<<grid_for(n_pts, 128), 128, 0, as_stream(stream)>>>(grid, (int)C, channel_last,
                                                                         geom_from(geom), xyz, n_pts, out);
  return launch_status();
}

int vx_grid_sample_backward(const float* grad_out, int64_t C, int channel_last, const vx_grid_geom* geom,
                            const float* xyz, int64_t n_pts, float* grad_grid, void* stream) {
  if (!geom || C <= 0 || n_pts < 0) return VX_ERR_ARG;
  if (n_pts == 0) return VX_OK;
  if (!grad_out || !xyz || !grad_grid) return VX_ERR_ARG;
  if (geom->X * geom->Y * geom->Z > INT32_MAX) return VX_ERR_ARG;
  grid_sample_bwd_kernel<<<grid_for(n_pts, 128), 128, 0, as_stream(stream)>>>(grad_out, (int)C, channel_last,
                                                                             geom_from(geom), xyz, n_pts, grad_grid);
  return launch_status();
}

int vx_fine_march(const vx_fine_march_args* A, void* stream) {
  if (!A || A->n_rays < 0 || A->max_steps <= 0) return VX_ERR_ARG;
  if (A->n_rays == 0) return VX_OK;
  if (!A->rays_o || !A->rays_d || !A->viewdirs || !A->sdf_smooth || !A->rec || !A->dw_slot || !A->n1 || !A->n2 ||
      !A->alphainv_last)
    return VX_ERR_ARG;
  if ((int64_t)A->n_rays * A->max_steps > INT32_MAX) return VX_ERR_ARG;
  MarchParams P{};
  P.rays_o = A->rays_o;
  P.rays_d = A->rays_d;
  P.viewdirs = A->viewdirs;
  P.n_rays = (int)A->n_rays;
  P.near = A->near;
  P.stepdist = A->stepdist;
  for (int a = 0; a < 3; ++a) {
    P.bmin[a] = A->grid.xyz_min[a];
    P.bmax[a] = A->grid.xyz_max[a];
  }
  P.g = geom_from(&A->grid);
  P.sdf = A->sdf_smooth;
  P.voxel_size = A->voxel_size;
  P.mask = A->mask;
  P.mX = (int)A->mask_X;
  P.mY = (int)A->mask_Y;
  P.mZ = (int)A->mask_Z;
  for (int a = 0; a < 3; ++a) {
    P.mscale[a] = A->mask_scale[a];
    P.mshift[a] = A->mask_shift[a];
  }
  P.unit_sphere = A->unit_sphere != 0;
  P.inv_s = A->inv_s;
  P.dist = A->dist;
  P.thres = A->fast_color_thres;
  P.max_steps = (int)A->max_steps;
  P.rec = reinterpret_cast<float4*>(A->rec);
  P.dw_slot = A->dw_slot;
  P.n1 = A->n1;
  P.n2 = A->n2;
  P.alphainv_last = A->alphainv_last;
  P.err = device_error_ptr();
  const int s = fill_density_mask(A->mask_density, A->mask_dgrid, A->mask_act_shift, A->mask_voxel_size_ratio,
                                  A->mask_thres, A->mask != nullptr, P.dm);
  if (s) return s;
  if (P.dm.dens)
    march_fine_kernel<true><<<warp_blocks(A->n_rays), 256, 0, as_stream(stream)>>>(P);
  else
    march_fine_kernel<false><<<warp_blocks(A->n_rays), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

int vx_fine_compact(const vx_fine_compact_args* A, void* stream) {
  if (!A || A->n_rays < 0) return VX_ERR_ARG;
  if (A->n_rays == 0) return VX_OK;
  CompactParams P{};
  P.rays_o = A->rays_o;
  P.rays_d = A->rays_d;
  P.n_rays = (int)A->n_rays;
  P.near = A->near;
  P.stepdist = A->stepdist;
  for (int a = 0; a < 3; ++a) {
    P.bmin[a] = A->xyz_min[a];
    P.bmax[a] = A->xyz_max[a];
  }
  P.max_steps = (int)A->max_steps;
  P.rec = reinterpret_cast<const float4*>(A->rec);
  P.n1 = A->n1;
  P.s2_off = A->s2_off;
  P.ray2 = A->ray2;
  P.step2 = A->step2;
  P.slot2 = A->slot2;
  P.w2 = A->w2;
  P.alpha2 = A->alpha2;
  P.pts2 = A->pts2;
  compact_fine_kernel<<<warp_blocks(A->n_rays), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

static int fill_feat_common(const vx_fine_feature_cfg* c, int& K, float* disp, int& k_unit) {
  FeatLayout L;
  const int s = fill_feat_layout(c, L);
  if (s) return s;
  K = L.K;
  for (int i = 0; i < K; ++i) disp[i] = L.disp[i];
  k_unit = L.k_unit;
  return VX_OK;
}

int vx_fine_features(const vx_fine_features_args* A, void* stream) {
  if (!A || A->n_rows < 0) return VX_ERR_ARG;
  if (A->n_rows == 0) return VX_OK;
  FeatParams P{};
  int s = fill_feat_layout(&A->cfg, P.L);
  if (s) return s;
  if ((!A->k0_f32 && !A->k0_bf16) || !A->sdf_smooth || !A->X1 || !A->X2) return VX_ERR_ARG;
  if (A->ld1 < x1_cols(&A->cfg) || A->ld2 < x2_cols(&A->cfg)) return VX_ERR_ARG;
  P.cols1 = (int)x1_cols(&A->cfg);
  P.cols2 = (int)x2_cols(&A->cfg);
  P.n_rows_dev = A->n_rows_dev;
  P.n_rows = A->n_rows;
  P.ray2 = A->ray2;
  P.pts2 = A->pts2;
  P.viewdirs = A->viewdirs;
  P.g = geom_from(&A->grid);
  P.sdf = A->sdf_smooth;
  P.voxel_size = A->voxel_size;
  P.k0f = A->k0_f32;
  P.k0h = reinterpret_cast<const __nv_bfloat16*>(A->k0_bf16);
  P.ld1 = (int)A->ld1;
  P.ld2 = (int)A->ld2;
  P.X1 = A->X1;
  P.X2 = A->X2;
  P.out_bf16 = A->out_bf16;
  P.normal_out = A->normal_out;
  const unsigned b = (unsigned)((A->n_rows + 127) / 128);
  cudaStream_t st = as_stream(stream);
  // staged rows: strides of 16-byte multiples, aligned bases, <= 48 KB of shared memory
  const size_t esz = A->out_bf16 ? 2 : 4;
  const size_t shm = 128 * (size_t)(A->ld1 + A->ld2 + 2 * (4 / esz)) * esz;
  const bool stage = (A->ld1 * esz) % 4 == 0 && (A->ld2 * esz) % 4 == 0 && shm <= 48 * 1024 &&
                     ((reinterpret_cast<uintptr_t>(A->X1) | reinterpret_cast<uintptr_t>(A->X2)) & 3) == 0;
#define VX_FEAT_LAUNCH(T, KK)                                           \
  if (stage)                                                            \
    features_fine_kernel<T, KK, true><<<b, 128, shm, st>>>(P);          \
  else                                                                  \
    features_fine_kernel<T, KK, false><<<b, 128, 0, st>>>(P)
#define VX_FEAT_SWITCH(T)        \
  switch (P.L.K) {               \
    case 1: VX_FEAT_LAUNCH(T, 1); break; \
    case 2: VX_FEAT_LAUNCH(T, 2); break; \
    case 3: VX_FEAT_LAUNCH(T, 3); break; \
    default: VX_FEAT_LAUNCH(T, 4); break; \
  }
  if (A->out_bf16) {
    VX_FEAT_SWITCH(__nv_bfloat16)
  } else {
    VX_FEAT_SWITCH(float)
  }
#undef VX_FEAT_SWITCH
#undef VX_FEAT_LAUNCH
  return launch_status();
}

int vx_fine_composite(const vx_fine_composite_args* A, void* stream) {
  if (!A || A->n_rays < 0) return VX_ERR_ARG;
  if (A->n_rays == 0) return VX_OK;
  CompositeParams P{};
  P.n_rays = (int)A->n_rays;
  P.s2_off = A->s2_off;
  P.w2 = A->w2;
  P.logit = A->logit;
  P.klogit = A->klogit;
  P.alphainv_last = A->alphainv_last;
  P.bg = A->bg;
  P.rgb0 = A->rgb0;
  P.rgbk = A->rgbk;
  P.rgbk_raw = A->rgbk_raw;
  P.normal2 = A->normal2;
  P.step2 = A->step2;
  P.dist = A->dist;
  P.normal_out = A->normal_out;
  P.depth_out = A->depth_out;
  P.wsum_out = A->wsum_out;
  P.has_k = A->has_k;
  composite_fine_kernel<<<warp_blocks(A->n_rays), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

int vx_fine_composite_backward(const vx_fine_composite_bwd_args* A, void* stream) {
  if (!A || A->n_rays < 0) return VX_ERR_ARG;
  if (A->n_rays == 0) return VX_OK;
  CompositeBwdParams P{};
  P.n_rays = (int)A->n_rays;
  P.s2_off = A->s2_off;
  P.w2 = A->w2;
  P.logit = A->logit;
  P.klogit = A->klogit;
  P.rgbk_raw = A->rgbk_raw;
  P.g_rgb0 = A->g_rgb0;
  P.g_rgbk = A->g_rgbk;
  P.bg = A->bg;
  P.g_last_in = A->g_last_in;
  P.d_logit = A->d_logit;
  P.d_klogit = A->d_klogit;
  P.d_w2 = A->d_w2;
  P.d_last = A->d_last;
  P.has_k = A->has_k;
  composite_fine_bwd_kernel<<<warp_blocks(A->n_rays), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

size_t vx_fine_composite_loss_scratch_bytes(int64_t n_rays) {
  return (size_t)(warp_blocks(n_rays > 0 ? n_rays : 1) + 2) * sizeof(float2);
}

int vx_fine_composite_loss(const vx_fine_composite_loss_args* A, void* stream) {
  if (!A || A->n_rays <= 0) return VX_ERR_ARG;
  // the per-row buffers (w2, logit, kout, d_logit, d_kout, d_w2) are read
  // only for rows that s2_off gives; they may be NULL when there are none
  if (!A->s2_off || !A->alphainv_last || !A->target || !A->rgb0 || !A->rgbk || !A->d_last || !A->loss ||
      !A->scratch)
    return VX_ERR_ARG;
  if (A->n_rays > INT32_MAX / 32) return VX_ERR_TOO_LARGE;
  if (A->scratch_bytes < vx_fine_composite_loss_scratch_bytes(A->n_rays)) return VX_ERR_ARG;
  CompositeLossParams P{};
  P.n_rays = (int)A->n_rays;
  P.s2_off = A->s2_off;
  P.w2 = A->w2;
  P.logit = A->logit;
  P.kout = A->kout;
  P.alphainv_last = A->alphainv_last;
  P.target = A->target;
  P.bg = A->bg;
  const double numel = 3.0 * (double)A->n_rays;
  P.g_scale_k = (float)(2.0 * (double)A->w_main / numel);
  P.g_scale_0 = (float)(2.0 * (double)A->w_rgb0 / numel);
  P.w_entropy = A->w_entropy_last;
  P.rgb0 = A->rgb0;
  P.rgbk = A->rgbk;
  P.d_logit = A->d_logit;
  P.d_kout = A->d_kout;
  P.d_w2 = A->d_w2;
  P.d_last = A->d_last;
  const unsigned blocks = warp_blocks(A->n_rays);
  P.part = reinterpret_cast<float2*>(A->scratch);
  P.entropy = reinterpret_cast<float*>(P.part + blocks + 1);
  P.k_into_logit = A->k_into_logit;
  cudaStream_t st = as_stream(stream);
  composite_loss_fine_kernel<<<blocks, 256, 0, st>>>(P);
  composite_loss_sum_kernel<<<1, 256, 0, st>>>(P.part, (int)blocks, P.entropy, A->w_main, A->w_rgb0,
                                                 A->w_entropy_last, (float)(1.0 / numel), A->loss);
  return launch_status();
}

int vx_fine_backward(const vx_fine_backward_args* A, void* stream) {
  if (!A || A->n_rays < 0 || A->n_rows < 0) return VX_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (A->n_rows > 0) {
    FeatBwdParams F{};
    int s = fill_feat_common(&A->cfg, F.K, F.disp, F.k_unit);
    if (s) return s;
    if (A->ld1 < x1_cols(&A->cfg) || A->ld2 < x2_cols(&A->cfg)) return VX_ERR_ARG;
    F.n_rows = A->n_rows;
    F.n_rows_dev = A->n_rows_dev;
    F.k0_touched = A->k0_touched;
    F.pts2 = A->pts2;
    F.g = geom_from(&A->grid);
    F.sdf = A->sdf_smooth;
    F.voxel_size = A->voxel_size;
    F.pos_pe = (int)A->cfg.posbase_pe;
    F.view_pe = (int)A->cfg.viewbase_pe;
    F.kpos_pe = (int)A->cfg.k_posbase_pe;
    F.kview_pe = (int)A->cfg.k_viewbase_pe;
    F.center_sdf = A->cfg.center_sdf;
    F.use_rgbnet_k0 = A->cfg.use_rgbnet_k0;
    F.k_center_sdf = A->cfg.k_center_sdf;
    F.ld1 = (int)A->ld1;
    F.ld2 = (int)A->ld2;
    F.dX1 = A->dX1;
    F.dX2 = A->dX2;
    F.in_bf16 = A->in_bf16;
    F.dw2 = A->dw2;
    F.slot2 = A->slot2;
    F.dw_slot = A->dw_slot;
    F.d_sdf = A->d_sdf_smooth;
    F.d_k0 = A->d_k0;
    const unsigned b = (unsigned)((A->n_rows + 127) / 128);
    if (A->in_bf16)
      features_fine_bwd_kernel<__nv_bfloat16><<<b, 128, 0, st>>>(F);
    else
      features_fine_bwd_kernel<float><<<b, 128, 0, st>>>(F);
    s = launch_status();
    if (s) return s;
  }
  if (A->n_rays == 0) return VX_OK;
  GeomBwdParams G{};
  G.rays_o = A->rays_o;
  G.rays_d = A->rays_d;
  G.viewdirs = A->viewdirs;
  G.n_rays = (int)A->n_rays;
  G.near = A->near;
  G.stepdist = A->stepdist;
  for (int a = 0; a < 3; ++a) {
    G.bmin[a] = A->grid.xyz_min[a];
    G.bmax[a] = A->grid.xyz_max[a];
  }
  G.g = geom_from(&A->grid);
  G.sdf = A->sdf_smooth;
  G.voxel_size = A->voxel_size;
  G.inv_s = A->inv_s;
  G.dist = A->dist;
  G.max_steps = (int)A->max_steps;
  G.rec = reinterpret_cast<const float4*>(A->rec);
  G.dw_slot = A->dw_slot;
  G.n1 = A->n1;
  G.alphainv_last = A->alphainv_last;
  G.d_last = A->d_last;
  G.d_sdf = A->d_sdf_smooth;
  G.inv_s_dev = A->inv_s_dev;
  geometry_fine_bwd_kernel<<<warp_blocks(A->n_rays), 256, 0, st>>>(G);
  return launch_status();
}

// ---- coarse model ------------------------------------------------------------

int vx_coarse_march(const vx_coarse_march_args* A, void* stream) {
  if (!A) return VX_ERR_ARG;
  const vx_fine_march_args* M = &A->march;
  if (M->n_rays < 0 || M->max_steps <= 0) return VX_ERR_ARG;
  if (M->n_rays == 0) return VX_OK;
  if (!M->rays_o || !M->rays_d || !M->viewdirs || !M->sdf_smooth || !A->grad4 || !M->rec || !M->dw_slot ||
      !M->n1 || !M->n2 || !A->n2b || !M->alphainv_last)
    return VX_ERR_ARG;
  if ((int64_t)M->n_rays * M->max_steps > INT32_MAX || (((uintptr_t)A->grad4) & 15)) return VX_ERR_ARG;
  CoarseMarchParams C{};
  MarchParams& P = C.m;
  P.rays_o = M->rays_o;
  P.rays_d = M->rays_d;
  P.viewdirs = M->viewdirs;
  P.n_rays = (int)M->n_rays;
  P.near = M->near;
  P.stepdist = M->stepdist;
  for (int a = 0; a < 3; ++a) {
    P.bmin[a] = M->grid.xyz_min[a];
    P.bmax[a] = M->grid.xyz_max[a];
    P.mscale[a] = M->mask_scale[a];
    P.mshift[a] = M->mask_shift[a];
  }
  P.g = geom_from(&M->grid);
  P.sdf = M->sdf_smooth;
  P.voxel_size = M->voxel_size;
  P.mask = M->mask;
  P.mX = (int)M->mask_X;
  P.mY = (int)M->mask_Y;
  P.mZ = (int)M->mask_Z;
  P.unit_sphere = M->unit_sphere != 0;
  P.inv_s = M->inv_s;
  P.dist = M->dist;
  P.thres = M->fast_color_thres;
  P.max_steps = (int)M->max_steps;
  P.rec = reinterpret_cast<float4*>(M->rec);
  P.dw_slot = M->dw_slot;
  P.n1 = M->n1;
  P.n2 = M->n2;
  P.alphainv_last = M->alphainv_last;
  P.err = device_error_ptr();
  C.G4 = A->grad4;
  C.n2b = A->n2b;
  const int s = fill_density_mask(M->mask_density, M->mask_dgrid, M->mask_act_shift, M->mask_voxel_size_ratio,
                                  M->mask_thres, M->mask != nullptr, P.dm);
  if (s) return s;
  if (P.dm.dens)
    march_coarse_kernel<true><<<warp_blocks(M->n_rays), 256, 0, as_stream(stream)>>>(C);
  else
    march_coarse_kernel<false><<<warp_blocks(M->n_rays), 256, 0, as_stream(stream)>>>(C);
  return launch_status();
}

static int64_t coarse_cols(const vx_coarse_feature_cfg* c) {
  return (c->use_k0 ? 12 : 0) + (3 + 6 * c->posbase_pe) + (3 + 6 * c->viewbase_pe) + (c->geo_rgb_dim == 3 ? 3 : 0);
}

static bool coarse_cfg_ok(const vx_coarse_feature_cfg* c) {
  return c->posbase_pe >= 0 && c->posbase_pe <= 16 && c->viewbase_pe >= 0 && c->viewbase_pe <= 16 &&
         (c->geo_rgb_dim == 0 || c->geo_rgb_dim == 3);
}

int vx_coarse_features(const vx_coarse_features_args* A, void* stream) {
  if (!A || A->n_rows < 0 || !coarse_cfg_ok(&A->cfg)) return VX_ERR_ARG;
  if (A->n_rows == 0) return VX_OK;
  if (A->ld < coarse_cols(&A->cfg) || !A->X || !A->grad4 || (A->cfg.use_k0 && !A->k0_f32 && !A->k0_bf16))
    return VX_ERR_ARG;
  CoarseFeatParams P{};
  P.n_rows = A->n_rows;
  P.ray2 = A->ray2;
  P.pts2 = A->pts2;
  P.viewdirs = A->viewdirs;
  P.g = geom_from(&A->grid);
  P.G4 = A->grad4;
  P.k0f = A->k0_f32;
  P.k0h = reinterpret_cast<const __nv_bfloat16*>(A->k0_bf16);
  P.use_k0 = A->cfg.use_k0;
  P.pos_pe = (int)A->cfg.posbase_pe;
  P.view_pe = (int)A->cfg.viewbase_pe;
  P.geo_rgb_dim = A->cfg.geo_rgb_dim;
  P.ld = (int)A->ld;
  P.X = A->X;
  P.normal_out = A->normal_out;
  const unsigned b = (unsigned)((A->n_rows + 127) / 128);
  if (A->out_bf16)
    features_coarse_kernel<__nv_bfloat16><<<b, 128, 0, as_stream(stream)>>>(P);
  else
    features_coarse_kernel<float><<<b, 128, 0, as_stream(stream)>>>(P);
  return launch_status();
}

int vx_coarse_composite(const vx_coarse_composite_args* A, void* stream) {
  if (!A || A->n_rays < 0) return VX_ERR_ARG;
  if (A->n_rays == 0) return VX_OK;
  CoarseCompositeParams P{};
  P.n_rays = (int)A->n_rays;
  P.s2_off = A->s2_off;
  P.w2 = A->w2;
  P.logit = A->logit;
  P.bg = A->bg;
  P.rgb = A->rgb;
  P.rgb_raw = A->rgb_raw;
  P.normal2 = A->normal2;
  P.step2 = A->step2;
  P.dist = A->dist;
  P.normal_out = A->normal_out;
  P.depth_out = A->depth_out;
  P.wsum_out = A->wsum_out;
  composite_coarse_kernel<<<warp_blocks(A->n_rays), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

int vx_coarse_composite_backward(const vx_coarse_composite_bwd_args* A, void* stream) {
  if (!A || A->n_rays < 0) return VX_ERR_ARG;
  if (A->n_rays == 0) return VX_OK;
  CoarseCompositeBwdParams P{};
  P.n_rays = (int)A->n_rays;
  P.s2_off = A->s2_off;
  P.w2 = A->w2;
  P.logit = A->logit;
  P.rgb_raw = A->rgb_raw;
  P.g_rgb = A->g_rgb;
  P.bg = A->bg;
  P.d_logit = A->d_logit;
  P.d_w2 = A->d_w2;
  composite_coarse_bwd_kernel<<<warp_blocks(A->n_rays), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

int vx_coarse_backward(const vx_coarse_backward_args* A, void* stream) {
  if (!A || A->n_rays < 0 || A->n_rows < 0 || !coarse_cfg_ok(&A->cfg)) return VX_ERR_ARG;
  if (A->n_rows > 0 && A->ld < coarse_cols(&A->cfg)) return VX_ERR_ARG;
  if ((((uintptr_t)A->grad4) | ((uintptr_t)A->d_grad4)) & 15) return VX_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  CoarseBwdParams C{};
  GeomBwdParams& G = C.gb;
  G.rays_o = A->rays_o;
  G.rays_d = A->rays_d;
  G.viewdirs = A->viewdirs;
  G.n_rays = (int)A->n_rays;
  G.near = A->near;
  G.stepdist = A->stepdist;
  for (int a = 0; a < 3; ++a) {
    G.bmin[a] = A->grid.xyz_min[a];
    G.bmax[a] = A->grid.xyz_max[a];
  }
  G.g = geom_from(&A->grid);
  G.sdf = A->sdf_smooth;
  G.voxel_size = A->voxel_size;
  G.inv_s = A->inv_s;
  G.dist = A->dist;
  G.max_steps = (int)A->max_steps;
  G.rec = reinterpret_cast<const float4*>(A->rec);
  G.dw_slot = A->dw_slot;
  G.n1 = A->n2b;
  G.alphainv_last = A->alphainv_last;
  G.d_last = A->d_last;
  G.d_sdf = A->d_sdf_smooth;
  C.n2b = A->n2b;
  C.G4 = A->grad4;
  C.dG4 = A->d_grad4;
  C.n_rows = A->n_rows;
  C.pts2 = A->pts2;
  C.slot2 = A->slot2;
  C.dw2 = A->dw2;
  C.dw_slot = A->dw_slot;
  C.use_k0 = A->cfg.use_k0;
  C.pos_pe = (int)A->cfg.posbase_pe;
  C.view_pe = (int)A->cfg.viewbase_pe;
  C.geo_rgb_dim = A->cfg.geo_rgb_dim;
  C.ld = (int)A->ld;
  C.in_bf16 = A->in_bf16;
  C.dX = A->dX;
  C.d_k0 = A->d_k0;
  C.d_grad2 = A->d_grad2;
  if (A->n_rows > 0) {
    const unsigned b = (unsigned)((A->n_rows + 127) / 128);
    if (A->in_bf16)
      features_coarse_bwd_kernel<__nv_bfloat16><<<b, 128, 0, st>>>(C);
    else
      features_coarse_bwd_kernel<float><<<b, 128, 0, st>>>(C);
    int s = launch_status();
    if (s) return s;
  }
  if (A->n_rays == 0) return VX_OK;
  geometry_coarse_bwd_kernel<<<warp_blocks(A->n_rays), 256, 0, st>>>(C);
  return launch_status();
}

}  // extern "C"
