// Dense per-voxel sweeps: total-variation add-grad and Adam.
//
// Drop-ins:
//   total_variation_cuda.total_variation_add_grad[_new]
//     (total_variation.cpp:29-32; total_variation_kernel.cu:14-66, 68-134)
//   adam_upd_cuda.adam_upd / masked_adam_upd / adam_upd_with_perlr
//     (adam_upd.cpp:79-86; adam_upd_kernel.cu:9-57, 59-133)
// plus the update rule of the optimizer the reference actually trains with,
// lib/utils.py:Adam (utils.py:154-199), and one fused sweep that applies TV,
// Adam and the gradient reset in a single pass over a grid (the reference
// needs a TV launch plus ~6 elementwise torch launches per parameter).
//
// Grids are addressed through (C, X, Y, Z) + a layout flag so the same
// kernels serve the reference's channel-first [1,C,X,Y,Z] tensors and the
// channel-last [X,Y,Z,C] storage used by the fused renderer.
#include <math.h>
#include "common.cuh"

namespace vx {

struct GridShape {
  int64_t C, X, Y, Z;
  int channel_last;
};

// Strides (in elements) of the three spatial axes and the decomposition of
// a flat index into (i, j, k).
struct GridIndex {
  int64_t i, j, k;
  int64_t si, sj, sk;
};

__device__ __forceinline__ GridIndex decompose(const GridShape& g, int64_t idx) {
  GridIndex r;
  if (g.channel_last) {
    const int64_t v = idx / g.C;
    r.k = v % g.Z;
    r.j = (v / g.Z) % g.Y;
    r.i = v / (g.Z * g.Y);
    r.sk = g.C;
  } else {
    r.k = idx % g.Z;
    r.j = (idx / g.Z) % g.Y;
    r.i = (idx / (g.Z * g.Y)) % g.X;
    r.sk = 1;
  }
  r.sj = g.Z * r.sk;
  r.si = g.Y * r.sj;
  return r;
}

__device__ __forceinline__ float clamp1(float v) { return fminf(fmaxf(v, -1.f), 1.f); }

// Sum of the six clamped differences, in the reference's order
// (k-1, k+1, j-1, j+1, i-1, i+1), with per-axis weights wk, wj, wi
// already divided by 6.
__device__ __forceinline__ float tv_term(const float* __restrict__ p, int64_t idx, const GridShape& g,
                                         const GridIndex& q, float wk, float wj, float wi) {
  const float c = p[idx];
  float s = 0.f;
  s = fadd(s, q.k == 0 ? 0.f : fmul(wk, clamp1(fsub(c, p[idx - q.sk]))));
  s = fadd(s, q.k == g.Z - 1 ? 0.f : fmul(wk, clamp1(fsub(c, p[idx + q.sk]))));
  s = fadd(s, q.j == 0 ? 0.f : fmul(wj, clamp1(fsub(c, p[idx - q.sj]))));
  s = fadd(s, q.j == g.Y - 1 ? 0.f : fmul(wj, clamp1(fsub(c, p[idx + q.sj]))));
  s = fadd(s, q.i == 0 ? 0.f : fmul(wi, clamp1(fsub(c, p[idx - q.si]))));
  s = fadd(s, q.i == g.X - 1 ? 0.f : fmul(wi, clamp1(fsub(c, p[idx + q.si]))));
  return s;
}

// Masked variant: each term is (w*clamp(d))*m[idx]*m[nbr]
// (total_variation_kernel.cu:237-242).
__device__ __forceinline__ float tv_term_masked(const float* __restrict__ p, const float* __restrict__ m,
                                                int64_t idx, const GridShape& g, const GridIndex& q, float wk,
                                                float wj, float wi) {
  const float c = p[idx];
  const float mc = m[idx];
  float s = 0.f;
  s = fadd(s, q.k == 0 ? 0.f : fmul(fmul(fmul(wk, clamp1(fsub(c, p[idx - q.sk]))), mc), m[idx - q.sk]));
  s = fadd(s, q.k == g.Z - 1 ? 0.f : fmul(fmul(fmul(wk, clamp1(fsub(c, p[idx + q.sk]))), mc), m[idx + q.sk]));
  s = fadd(s, q.j == 0 ? 0.f : fmul(fmul(fmul(wj, clamp1(fsub(c, p[idx - q.sj]))), mc), m[idx - q.sj]));
  s = fadd(s, q.j == g.Y - 1 ? 0.f : fmul(fmul(fmul(wj, clamp1(fsub(c, p[idx + q.sj]))), mc), m[idx + q.sj]));
  s = fadd(s, q.i == 0 ? 0.f : fmul(fmul(fmul(wi, clamp1(fsub(c, p[idx - q.si]))), mc), m[idx - q.si]));
  s = fadd(s, q.i == g.X - 1 ? 0.f : fmul(fmul(fmul(wi, clamp1(fsub(c, p[idx + q.si]))), mc), m[idx + q.si]));
  return s;
}

template <bool DENSE, bool MASKED>
__global__ void tv_add_grad_kernel(const float* __restrict__ param, float* __restrict__ grad,
                                   const float* __restrict__ mask, GridShape g, float wk, float wj, float wi,
                                   int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += stride) {
    const float gv = grad[idx];
    if (!DENSE && gv == 0.f) continue;
    const GridIndex q = decompose(g, idx);
    const float add = MASKED ? tv_term_masked(param, mask, idx, g, q, wk, wj, wi)
                             : tv_term(param, idx, g, q, wk, wj, wi);
    grad[idx] = fadd(gv, add);
  }
}

// ---- Adam ------------------------------------------------------------------

// adam_upd_kernel.cu:9-57.  MODE 0 plain, 1 masked (grad != 0), 2 per-lr.
template <int MODE>
__global__ void adam_upd_kernel(float* __restrict__ param, const float* __restrict__ grad,
                                float* __restrict__ exp_avg, float* __restrict__ exp_avg_sq,
                                const float* __restrict__ perlr, int64_t n, float step_size, float beta1,
                                float beta2, float eps) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float g = grad[i];
    if (MODE == 1 && g == 0.f) continue;
    // the reference's compiled kernel fuses beta1*m and beta2*v into the sums
    const float m = __fmaf_rn(beta1, exp_avg[i], fmul(fsub(1.f, beta1), g));
    const float v = __fmaf_rn(beta2, exp_avg_sq[i], fmul(fmul(fsub(1.f, beta2), g), g));
    exp_avg[i] = m;
    exp_avg_sq[i] = v;
    const float num = (MODE == 2) ? fmul(fmul(step_size, perlr[i]), m) : fmul(step_size, m);
    param[i] = fsub(param[i], fdiv(num, fadd(__fsqrt_rn(v), eps)));
  }
}

// lib/utils.py:184-199 in FP32:
//   m = m*b1 + g*(1-b1);  v = v*b2 + (1-b2)*g*g
//   denom = sqrt(v)/sqrt(bc2) + eps;  p += -step_size * (m [*per_lr]) / denom
struct AdamParams {
  float beta1, beta2, one_m_beta1, one_m_beta2, step_size, sqrt_bc2, eps;
};

__device__ __forceinline__ float adam_update(float p, float g, float& m, float& v, float plr, bool has_plr,
                                             const AdamParams& a) {
  m = fadd(fmul(m, a.beta1), fmul(g, a.one_m_beta1));
  v = fadd(fmul(v, a.beta2), fmul(fmul(a.one_m_beta2, g), g));
  const float denom = fadd(fdiv(__fsqrt_rn(v), a.sqrt_bc2), a.eps);
  const float num = has_plr ? fmul(m, plr) : m;
  return fadd(p, fmul(-a.step_size, fdiv(num, denom)));
}

// Vectorised elementwise Adam (4 elements/thread) with optional gradient
// reset; used for the MLP parameters and for grids without TV.
__global__ void adam_step_kernel(float* __restrict__ param, float* __restrict__ grad, float* __restrict__ exp_avg,
                                 float* __restrict__ exp_avg_sq, const float* __restrict__ per_lr, int64_t n,
                                 AdamParams a, int zero_grad) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const bool vec = ((((uintptr_t)param) | ((uintptr_t)grad) | ((uintptr_t)exp_avg) | ((uintptr_t)exp_avg_sq) |
                     ((uintptr_t)per_lr)) & 15) == 0;
  if (vec) {
    const int64_t n4 = n >> 2;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += stride) {
      float4 p = reinterpret_cast<const float4*>(param)[q];
      float4 g = reinterpret_cast<const float4*>(grad)[q];
      float4 m = reinterpret_cast<const float4*>(exp_avg)[q];
      float4 v = reinterpret_cast<const float4*>(exp_avg_sq)[q];
      float4 l = per_lr ? reinterpret_cast<const float4*>(per_lr)[q] : make_float4(1.f, 1.f, 1.f, 1.f);
      const bool h = per_lr != nullptr;
      p.x = adam_update(p.x, g.x, m.x, v.x, l.x, h, a);
      p.y = adam_update(p.y, g.y, m.y, v.y, l.y, h, a);
      p.z = adam_update(p.z, g.z, m.z, v.z, l.z, h, a);
      p.w = adam_update(p.w, g.w, m.w, v.w, l.w, h, a);
      reinterpret_cast<float4*>(param)[q] = p;
      reinterpret_cast<float4*>(exp_avg)[q] = m;
      reinterpret_cast<float4*>(exp_avg_sq)[q] = v;
      if (zero_grad) reinterpret_cast<float4*>(grad)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int64_t i = (n4 << 2) + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
      float m = exp_avg[i], v = exp_avg_sq[i];
      param[i] = adam_update(param[i], grad[i], m, v, per_lr ? per_lr[i] : 1.f, per_lr != nullptr, a);
      exp_avg[i] = m;
      exp_avg_sq[i] = v;
      if (zero_grad) grad[i] = 0.f;
    }
  } else {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
      float m = exp_avg[i], v = exp_avg_sq[i];
      param[i] = adam_update(param[i], grad[i], m, v, per_lr ? per_lr[i] : 1.f, per_lr != nullptr, a);
      exp_avg[i] = m;
      exp_avg_sq[i] = v;
      if (zero_grad) grad[i] = 0.f;
    }
  }
}

// Fused grid sweep: TV add-grad (reference semantics, read from the OLD
// parameter buffer) -> Adam -> write the NEW parameter buffer (+ optional
// BF16 shadow copy) -> reset the gradient.  param_in and param_out must be
// different buffers when TV is on, because TV reads neighbours that other
// threads are updating.  Four consecutive elements per thread (float4
// streams for g, m, v, p); TV neighbours come through L1/L2.
template <bool TV, bool DENSE, bool SHADOW>
__global__ void __launch_bounds__(256) grid_tv_adam_kernel(const float* __restrict__ param_in,
                                                          float* __restrict__ param_out, float* __restrict__ grad,
                                                          float* __restrict__ exp_avg,
                                                          float* __restrict__ exp_avg_sq,
                                                          const float* __restrict__ per_lr,
                                                          __nv_bfloat16* __restrict__ shadow, GridShape g,
                                                          float wk, float wj, float wi, AdamParams a,
                                                          int zero_grad, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n4 = n >> 2;
  const bool h = per_lr != nullptr;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += stride) {
    const int64_t base = q << 2;
    float4 p = reinterpret_cast<const float4*>(param_in)[q];
    float4 gr = reinterpret_cast<const float4*>(grad)[q];
    float4 m = reinterpret_cast<const float4*>(exp_avg)[q];
    float4 v = reinterpret_cast<const float4*>(exp_avg_sq)[q];
    float4 l = h ? reinterpret_cast<const float4*>(per_lr)[q] : make_float4(1.f, 1.f, 1.f, 1.f);
    float pv[4] = {p.x, p.y, p.z, p.w};
    float gv[4] = {gr.x, gr.y, gr.z, gr.w};
    float mv[4] = {m.x, m.y, m.z, m.w};
    float vv[4] = {v.x, v.y, v.z, v.w};
    float lv[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (TV && (DENSE || gv[e] != 0.f)) {
        const int64_t idx = base + e;
        const GridIndex qi = decompose(g, idx);
        gv[e] = fadd(gv[e], tv_term(param_in, idx, g, qi, wk, wj, wi));
      }
      pv[e] = adam_update(pv[e], gv[e], mv[e], vv[e], lv[e], h, a);
    }
    reinterpret_cast<float4*>(param_out)[q] = make_float4(pv[0], pv[1], pv[2], pv[3]);
    reinterpret_cast<float4*>(exp_avg)[q] = make_float4(mv[0], mv[1], mv[2], mv[3]);
    reinterpret_cast<float4*>(exp_avg_sq)[q] = make_float4(vv[0], vv[1], vv[2], vv[3]);
    if (zero_grad) reinterpret_cast<float4*>(grad)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (SHADOW) {
      __nv_bfloat162 lo = __floats2bfloat162_rn(pv[0], pv[1]);
      __nv_bfloat162 hi = __floats2bfloat162_rn(pv[2], pv[3]);
      uint2 packed;
      packed.x = *reinterpret_cast<uint32_t*>(&lo);
      packed.y = *reinterpret_cast<uint32_t*>(&hi);
      reinterpret_cast<uint2*>(shadow)[q] = packed;
    }
  }
  // Tail (n not a multiple of 4).
  for (int64_t idx = (n4 << 2) + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += stride) {
    float gv = grad[idx];
    if (TV && (DENSE || gv != 0.f)) {
      const GridIndex qi = decompose(g, idx);
      gv = fadd(gv, tv_term(param_in, idx, g, qi, wk, wj, wi));
    }
    float m = exp_avg[idx], v = exp_avg_sq[idx];
    const float pn = adam_update(param_in[idx], gv, m, v, h ? per_lr[idx] : 1.f, h, a);
    param_out[idx] = pn;
    exp_avg[idx] = m;
    exp_avg_sq[idx] = v;
    if (zero_grad) grad[idx] = 0.f;
    if (SHADOW) shadow[idx] = __float2bfloat16_rn(pn);
  }
}

// Row-structured variant of the fused sweep for the layouts the models use:
// channel-last with C % 4 == 0 (k0, C = 12) and single-channel grids (sdf).
// One CTA per (i, j) row: blockIdx.x = j, blockIdx.y = i, threads walk the
// row's Z*C/4 float4 quads, so (i, j, k, c) need no integer division and
// every TV neighbour is one float4 load (k +- 1 from the same row through
// L1, j +- 1 and i +- 1 from rows other CTAs are streaming through L2).
// Same operation order as grid_tv_adam_kernel, hence bit-identical results.
template <int C>
__device__ __forceinline__ float4 ld4(const float* __restrict__ p, int64_t q) {
  return __ldg(reinterpret_cast<const float4*>(p) + q);
}

__device__ __forceinline__ float tv1(float c, float n, float w) { return fmul(w, clamp1(fsub(c, n))); }

template <int C, bool TV, bool DENSE, bool SHADOW>
__global__ void __launch_bounds__(256) grid_tv_adam_row_kernel(const float* __restrict__ param_in,
                                                              float* __restrict__ param_out,
                                                              float* __restrict__ grad,
                                                              float* __restrict__ exp_avg,
                                                              float* __restrict__ exp_avg_sq,
                                                              const float* __restrict__ per_lr,
                                                              __nv_bfloat16* __restrict__ shadow, int X, int Y,
                                                              int Z, float wk, float wj, float wi, AdamParams a,
                                                              int zero_grad, const uint8_t* __restrict__ touched) {
  const int j = blockIdx.x, i = blockIdx.y;
  const int row_q = Z * C / 4;  // float4 quads per row
  const int64_t row0 = ((int64_t)i * Y + j) * row_q;
  const int64_t sj = row_q, si = (int64_t)Y * row_q;
  const bool h = per_lr != nullptr;
  const int64_t vox0 = ((int64_t)i * Y + j) * Z;  // first voxel of the row
  for (int t = threadIdx.x; t < row_q; t += blockDim.x) {
    const int64_t q = row0 + t;
    const float4 p = ld4<C>(param_in, q);
    // touched map: the gradient is zero outside the marked voxels, so
    // unmarked quads are not read
    bool use_g = true;
    if (touched) {
      if (C == 1)
        use_g = *reinterpret_cast<const uint32_t*>(touched + vox0 + 4 * t) != 0u;
      else
        use_g = touched[vox0 + t / (C >= 4 ? C / 4 : 1)] != 0;
    }
    float4 gr = use_g ? reinterpret_cast<const float4*>(grad)[q] : make_float4(0.f, 0.f, 0.f, 0.f);
    float gv[4] = {gr.x, gr.y, gr.z, gr.w};
    const float pv[4] = {p.x, p.y, p.z, p.w};
    if (TV) {
      // neighbours of the 4 elements along each axis
      float km[4], kp[4];
      int kk[4];
      if (C == 1) {
        const float4 L = t > 0 ? ld4<C>(param_in, q - 1) : p;
        const float4 Rr = t < row_q - 1 ? ld4<C>(param_in, q + 1) : p;
        km[0] = L.w; km[1] = p.x; km[2] = p.y; km[3] = p.z;
        kp[0] = p.y; kp[1] = p.z; kp[2] = p.w; kp[3] = Rr.x;
#pragma unroll
        for (int e = 0; e < 4; ++e) kk[e] = 4 * t + e;
      } else {
        constexpr int QPV = C >= 4 ? C / 4 : 1;  // float4 quads per voxel
        const int k = t / QPV;
        const float4 L = k > 0 ? ld4<C>(param_in, q - QPV) : p;
        const float4 Rr = k < Z - 1 ? ld4<C>(param_in, q + QPV) : p;
        km[0] = L.x; km[1] = L.y; km[2] = L.z; km[3] = L.w;
        kp[0] = Rr.x; kp[1] = Rr.y; kp[2] = Rr.z; kp[3] = Rr.w;
#pragma unroll
        for (int e = 0; e < 4; ++e) kk[e] = k;
      }
      const float4 jm = j > 0 ? ld4<C>(param_in, q - sj) : p;
      const float4 jp = j < Y - 1 ? ld4<C>(param_in, q + sj) : p;
      const float4 im = i > 0 ? ld4<C>(param_in, q - si) : p;
      const float4 ip = i < X - 1 ? ld4<C>(param_in, q + si) : p;
      const float jmv[4] = {jm.x, jm.y, jm.z, jm.w}, jpv[4] = {jp.x, jp.y, jp.z, jp.w};
      const float imv[4] = {im.x, im.y, im.z, im.w}, ipv[4] = {ip.x, ip.y, ip.z, ip.w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (!(DENSE || gv[e] != 0.f)) continue;
        const float c = pv[e];
        float s = 0.f;
        s = fadd(s, kk[e] == 0 ? 0.f : tv1(c, km[e], wk));
        s = fadd(s, kk[e] == Z - 1 ? 0.f : tv1(c, kp[e], wk));
        s = fadd(s, j == 0 ? 0.f : tv1(c, jmv[e], wj));
        s = fadd(s, j == Y - 1 ? 0.f : tv1(c, jpv[e], wj));
        s = fadd(s, i == 0 ? 0.f : tv1(c, imv[e], wi));
        s = fadd(s, i == X - 1 ? 0.f : tv1(c, ipv[e], wi));
        gv[e] = fadd(gv[e], s);
      }
    }
    float4 m = reinterpret_cast<const float4*>(exp_avg)[q];
    float4 v = reinterpret_cast<const float4*>(exp_avg_sq)[q];
    const float4 l = h ? ld4<C>(per_lr, q) : make_float4(1.f, 1.f, 1.f, 1.f);
    float mv[4] = {m.x, m.y, m.z, m.w}, vv[4] = {v.x, v.y, v.z, v.w};
    const float lv[4] = {l.x, l.y, l.z, l.w};
    float out[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) out[e] = adam_update(pv[e], gv[e], mv[e], vv[e], lv[e], h, a);
    reinterpret_cast<float4*>(param_out)[q] = make_float4(out[0], out[1], out[2], out[3]);
    reinterpret_cast<float4*>(exp_avg)[q] = make_float4(mv[0], mv[1], mv[2], mv[3]);
    reinterpret_cast<float4*>(exp_avg_sq)[q] = make_float4(vv[0], vv[1], vv[2], vv[3]);
    if (zero_grad && use_g) reinterpret_cast<float4*>(grad)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (SHADOW) {
      __nv_bfloat162 lo = __floats2bfloat162_rn(out[0], out[1]);
      __nv_bfloat162 hi = __floats2bfloat162_rn(out[2], out[3]);
      uint2 packed;
      packed.x = *reinterpret_cast<uint32_t*>(&lo);
      packed.y = *reinterpret_cast<uint32_t*>(&hi);
      reinterpret_cast<uint2*>(shadow)[q] = packed;
    }
  }
}

// Multi-tensor utils.Adam: up to VX_ADAM_MULTI_MAX small tensors (the MLP
// weights and biases) in one launch.  The table is a by-value kernel
// parameter; CTA b works on chunk b, mapped to (tensor, offset) through the
// chunk prefix.
constexpr int ADAM_MULTI_MAX = 48;
constexpr int ADAM_CHUNK = 4096;

struct AdamMultiTable {
  int n;
  float* p[ADAM_MULTI_MAX];
  float* g[ADAM_MULTI_MAX];
  float* m[ADAM_MULTI_MAX];
  float* v[ADAM_MULTI_MAX];
  int64_t len[ADAM_MULTI_MAX];
  int chunk0[ADAM_MULTI_MAX + 1];
  float step_size[ADAM_MULTI_MAX];
  float sqrt_bc2[ADAM_MULTI_MAX];
  float beta1, beta2, one_m_beta1, one_m_beta2, eps;
};

__global__ void __launch_bounds__(256) adam_multi_kernel(const AdamMultiTable T) {
  const int b = blockIdx.x;
  int t = 0;
  while (t + 1 < T.n && T.chunk0[t + 1] <= b) ++t;
  const int64_t off = (int64_t)(b - T.chunk0[t]) * ADAM_CHUNK;
  const int64_t end = min(off + ADAM_CHUNK, T.len[t]);
  AdamParams a;
  a.beta1 = T.beta1;
  a.beta2 = T.beta2;
  a.one_m_beta1 = T.one_m_beta1;
  a.one_m_beta2 = T.one_m_beta2;
  a.step_size = T.step_size[t];
  a.sqrt_bc2 = T.sqrt_bc2[t];
  a.eps = T.eps;
  float* p = T.p[t];
  float* g = T.g[t];
  float* m = T.m[t];
  float* v = T.v[t];
  for (int64_t i = off + threadIdx.x; i < end; i += blockDim.x) {
    float mi = m[i], vi = v[i];
    p[i] = adam_update(p[i], g[i], mi, vi, 1.f, false, a);
    m[i] = mi;
    v[i] = vi;
  }
}

// Resets a gradient grid that is nonzero only at marked voxels: zeroes the
// C values of every marked voxel and clears the marks (16 marks per thread
// and chunk; unmarked chunks cost one 16-byte read).
__global__ void __launch_bounds__(256) clear_touched_kernel(float* __restrict__ grad, uint8_t* __restrict__ touched,
                                                           int64_t n_vox, int C) {
  const int64_t chunks = (n_vox + 15) / 16;
  for (int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ch < chunks;
       ch += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v0 = ch * 16;
    if (v0 + 16 <= n_vox) {
      const uint4 m = reinterpret_cast<const uint4*>(touched)[ch];
      if ((m.x | m.y | m.z | m.w) == 0u) continue;
      const uint32_t w[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
      for (int b = 0; b < 16; ++b) {
        if (((w[b >> 2] >> (8 * (b & 3))) & 0xffu) == 0u) continue;
        float* g = grad + (v0 + b) * C;
        for (int c = 0; c < C; ++c) g[c] = 0.f;
      }
      reinterpret_cast<uint4*>(touched)[ch] = make_uint4(0u, 0u, 0u, 0u);
    } else {
      for (int64_t v = v0; v < n_vox; ++v) {
        if (!touched[v]) continue;
        for (int c = 0; c < C; ++c) grad[v * C + c] = 0.f;
        touched[v] = 0;
      }
    }
  }
}

inline unsigned sweep_blocks(int64_t work_items) {
  // Persistent-style grid: a multiple of the SM count, capped by the work.
  const int64_t per_wave = (int64_t)sm_count() * 8;  // 8 x 256-thread CTAs per SM
  int64_t b = (work_items + 255) / 256;
  if (b > per_wave * 4) b = per_wave * 4;
  if (b < 1) b = 1;
  return (unsigned)b;
}

inline bool shape_ok(int64_t C, int64_t X, int64_t Y, int64_t Z) { return C > 0 && X > 0 && Y > 0 && Z > 0; }

}  // namespace vx

using namespace vx;

extern "C" {

int vx_total_variation_add_grad(const float* param, float* grad, float wx, float wy, float wz, int dense_mode,
                                int64_t C, int64_t X, int64_t Y, int64_t Z, int channel_last, void* stream) {
  if (!shape_ok(C, X, Y, Z) || !param || !grad) return VX_ERR_ARG;
  // Host-side weight scaling as total_variation_kernel.cu:76-78; the
  // reference kernel applies wz to both the k and i axes and ignores wx.
  (void)wx;
  wy /= 6;
  wz /= 6;
  GridShape g{C, X, Y, Z, channel_last};
  const int64_t n = C * X * Y * Z;
  cudaStream_t st = as_stream(stream);
  if (dense_mode)
    tv_add_grad_kernel<true, false><<<sweep_blocks(n), 256, 0, st>>>(param, grad, nullptr, g, wz, wy, wz, n);
  else
    tv_add_grad_kernel<false, false><<<sweep_blocks(n), 256, 0, st>>>(param, grad, nullptr, g, wz, wy, wz, n);
  return launch_status();
}

int vx_total_variation_add_grad_new(const float* param, float* grad, const float* mask, float wx, float wy, float wz,
                                    int dense_mode, int64_t C, int64_t X, int64_t Y, int64_t Z, int channel_last,
                                    void* stream) {
  if (!shape_ok(C, X, Y, Z) || !param || !grad || !mask) return VX_ERR_ARG;
  wx /= 6;
  wy /= 6;
  wz /= 6;
  GridShape g{C, X, Y, Z, channel_last};
  const int64_t n = C * X * Y * Z;
  cudaStream_t st = as_stream(stream);
  if (dense_mode)
    tv_add_grad_kernel<true, true><<<sweep_blocks(n), 256, 0, st>>>(param, grad, mask, g, wx, wy, wz, n);
  else
    tv_add_grad_kernel<false, true><<<sweep_blocks(n), 256, 0, st>>>(param, grad, mask, g, wx, wy, wz, n);
  return launch_status();
}

static float adam_upd_step_size(int step, float beta1, float beta2, float lr) {
  // adam_upd_kernel.cu:72 (float pow/sqrt on the host).
  return lr * sqrtf(1.f - powf(beta2, (float)step)) / (1.f - powf(beta1, (float)step));
}

static int adam_upd_common(int mode, float* param, const float* grad, float* exp_avg, float* exp_avg_sq,
                           const float* perlr, int64_t n, int step, float beta1, float beta2, float lr, float eps,
                           void* stream) {
  if (n < 0) return VX_ERR_ARG;
  if (n == 0) return VX_OK;
  if (!param || !grad || !exp_avg || !exp_avg_sq || (mode == 2 && !perlr)) return VX_ERR_ARG;
  const float ss = adam_upd_step_size(step, beta1, beta2, lr);
  cudaStream_t st = as_stream(stream);
  const unsigned b = sweep_blocks(n);
  if (mode == 0)
    adam_upd_kernel<0><<<b, 256, 0, st>>>(param, grad, exp_avg, exp_avg_sq, perlr, n, ss, beta1, beta2, eps);
  else if (mode == 1)
    adam_upd_kernel<1><<<b, 256, 0, st>>>(param, grad, exp_avg, exp_avg_sq, perlr, n, ss, beta1, beta2, eps);
  else
    adam_upd_kernel<2><<<b, 256, 0, st>>>(param, grad, exp_avg, exp_avg_sq, perlr, n, ss, beta1, beta2, eps);
  return launch_status();
}

int vx_adam_upd(float* param, const float* grad, float* exp_avg, float* exp_avg_sq, int64_t n, int step,
                float beta1, float beta2, float lr, float eps, void* stream) {
  return adam_upd_common(0, param, grad, exp_avg, exp_avg_sq, nullptr, n, step, beta1, beta2, lr, eps, stream);
}

int vx_masked_adam_upd(float* param, const float* grad, float* exp_avg, float* exp_avg_sq, int64_t n, int step,
                       float beta1, float beta2, float lr, float eps, void* stream) {
  return adam_upd_common(1, param, grad, exp_avg, exp_avg_sq, nullptr, n, step, beta1, beta2, lr, eps, stream);
}

int vx_adam_upd_with_perlr(float* param, const float* grad, float* exp_avg, float* exp_avg_sq, const float* perlr,
                           int64_t n, int step, float beta1, float beta2, float lr, float eps, void* stream) {
  return adam_upd_common(2, param, grad, exp_avg, exp_avg_sq, perlr, n, step, beta1, beta2, lr, eps, stream);
}

int vx_adam_step(float* param, float* grad, float* exp_avg, float* exp_avg_sq, const float* per_lr, int64_t n,
                 double lr, double beta1, double beta2, double eps, int64_t step, int zero_grad, void* stream) {
  if (n < 0 || step < 1) return VX_ERR_ARG;
  if (n == 0) return VX_OK;
  if (!param || !grad || !exp_avg || !exp_avg_sq) return VX_ERR_ARG;
  // Scalars exactly as lib/utils.py:177-194 derives them in Python double,
  // then cast to the tensor dtype.
  const double bc1 = 1.0 - pow(beta1, (double)step);
  const double bc2 = 1.0 - pow(beta2, (double)step);
  AdamParams a;
  a.beta1 = (float)beta1;
  a.beta2 = (float)beta2;
  a.one_m_beta1 = (float)(1.0 - beta1);
  a.one_m_beta2 = (float)(1.0 - beta2);
  a.step_size = (float)(lr / bc1);
  a.sqrt_bc2 = (float)sqrt(bc2);
  a.eps = (float)eps;
  adam_step_kernel<<<sweep_blocks((n + 3) / 4), 256, 0, as_stream(stream)>>>(param, grad, exp_avg, exp_avg_sq,
                                                                           per_lr, n, a, zero_grad);
  return launch_status();
}

int vx_adam_step_multi(int n_tensors, float* const* params, float* const* grads, float* const* exp_avgs,
                       float* const* exp_avg_sqs, const int64_t* sizes, const double* lrs, const int64_t* steps,
                       double beta1, double beta2, double eps, void* stream) {
  if (n_tensors < 0 || n_tensors > ADAM_MULTI_MAX) return VX_ERR_ARG;
  if (n_tensors == 0) return VX_OK;
  if (!params || !grads || !exp_avgs || !exp_avg_sqs || !sizes || !lrs || !steps) return VX_ERR_ARG;
  AdamMultiTable T;
  T.n = n_tensors;
  T.beta1 = (float)beta1;
  T.beta2 = (float)beta2;
  T.one_m_beta1 = (float)(1.0 - beta1);
  T.one_m_beta2 = (float)(1.0 - beta2);
  T.eps = (float)eps;
  int64_t chunks = 0;
  for (int t = 0; t < n_tensors; ++t) {
    if (!params[t] || !grads[t] || !exp_avgs[t] || !exp_avg_sqs[t] || sizes[t] < 0 || steps[t] < 1)
      return VX_ERR_ARG;
    T.p[t] = params[t];
    T.g[t] = grads[t];
    T.m[t] = exp_avgs[t];
    T.v[t] = exp_avg_sqs[t];
    T.len[t] = sizes[t];
    T.chunk0[t] = (int)chunks;
    chunks += (sizes[t] + ADAM_CHUNK - 1) / ADAM_CHUNK;
    // utils.py:177-194 scalars in double, cast to float
    const double bc1 = 1.0 - pow(beta1, (double)steps[t]);
    const double bc2 = 1.0 - pow(beta2, (double)steps[t]);
    T.step_size[t] = (float)(lrs[t] / bc1);
    T.sqrt_bc2[t] = (float)sqrt(bc2);
  }
  T.chunk0[n_tensors] = (int)chunks;
  if (chunks == 0) return VX_OK;
  if (chunks > INT32_MAX) return VX_ERR_ARG;
  adam_multi_kernel<<<(unsigned)chunks, 256, 0, as_stream(stream)>>>(T);
  return launch_status();
}

static int grid_tv_adam_impl(const float* param_in, float* param_out, float* grad, float* exp_avg,
                             float* exp_avg_sq, const float* per_lr, void* shadow_bf16, int64_t C, int64_t X,
                             int64_t Y, int64_t Z, int channel_last, int tv_enabled, float tv_weight,
                             int tv_dense_mode, double lr, double beta1, double beta2, double eps, int64_t step,
                             int zero_grad, const uint8_t* touched, void* stream) {
  if (!shape_ok(C, X, Y, Z) || step < 1) return VX_ERR_ARG;
  if (!param_in || !param_out || !grad || !exp_avg || !exp_avg_sq) return VX_ERR_ARG;
  if (tv_enabled && param_in == param_out) return VX_ERR_ARG;
  const uintptr_t al = ((uintptr_t)param_in) | ((uintptr_t)param_out) | ((uintptr_t)grad) | ((uintptr_t)exp_avg) |
                       ((uintptr_t)exp_avg_sq) | ((uintptr_t)per_lr);
  if ((al & 15) || (((uintptr_t)shadow_bf16) & 7) || (((uintptr_t)touched) & 3)) return VX_ERR_ARG;
  const double bc1 = 1.0 - pow(beta1, (double)step);
  const double bc2 = 1.0 - pow(beta2, (double)step);
  AdamParams a;
  a.beta1 = (float)beta1;
  a.beta2 = (float)beta2;
  a.one_m_beta1 = (float)(1.0 - beta1);
  a.one_m_beta2 = (float)(1.0 - beta2);
  a.step_size = (float)(lr / bc1);
  a.sqrt_bc2 = (float)sqrt(bc2);
  a.eps = (float)eps;
  // DenseGrid.total_variation_add_grad(w, w, w, dense) with equal weights
  // (voxurf_fine.py:403-405): every axis gets w/6.
  const float w6 = tv_weight / 6;
  GridShape g{C, X, Y, Z, channel_last};
  const int64_t n = C * X * Y * Z;
  cudaStream_t st = as_stream(stream);
  __nv_bfloat16* sh = reinterpret_cast<__nv_bfloat16*>(shadow_bf16);
  // Row-structured kernel for k0 (channel-last, 12 channels) and 1-channel grids.
  const bool row_c12 = channel_last && C == 12;
  const bool row_c1 = C == 1 && (Z % 4) == 0;
  if ((row_c12 || row_c1) && X <= 65535 && Y <= 2147483647LL && Z * C <= (1LL << 30)) {
    const int row_q = (int)(Z * C / 4);
    const int threads = row_q >= 256 ? 256 : ((row_q + 31) / 32) * 32;
    dim3 grid((unsigned)Y, (unsigned)X);
#define VX_ROW(CC, TV, DENSE, SH)                                                                             \
  grid_tv_adam_row_kernel<CC, TV, DENSE, SH><<<grid, threads, 0, st>>>(param_in, param_out, grad, exp_avg,       \
                                                                      exp_avg_sq, per_lr, sh, (int)X, (int)Y,   \
                                                                      (int)Z, w6, w6, w6, a, zero_grad, touched)
#define VX_ROW_C(CC)                                                                                       \
  if (tv_enabled) {                                                                                           \
    if (tv_dense_mode) {                                                                                      \
      if (sh) VX_ROW(CC, true, true, true); else VX_ROW(CC, true, true, false);                               \
    } else {                                                                                                  \
      if (sh) VX_ROW(CC, true, false, true); else VX_ROW(CC, true, false, false);                             \
    }                                                                                                         \
  } else {                                                                                                    \
    if (sh) VX_ROW(CC, false, false, true); else VX_ROW(CC, false, false, false);                             \
  }
    if (row_c12) {
      VX_ROW_C(12)
    } else {
      VX_ROW_C(1)
    }
#undef VX_ROW_C
#undef VX_ROW
    return launch_status();
  }
  if (touched) return VX_ERR_UNSUPPORTED;  // the map is read by the row kernel only
  const unsigned b = sweep_blocks((n + 3) / 4);
#define VX_LAUNCH_TVA(TV, DENSE, SH) \
  grid_tv_adam_kernel<TV, DENSE, SH><<<b, 256, 0, st>>>(param_in, param_out, grad, exp_avg, exp_avg_sq, per_lr, sh, \
                                                        g, w6, w6, w6, a, zero_grad, n)
  if (tv_enabled) {
    if (tv_dense_mode) {
      if (sh) VX_LAUNCH_TVA(true, true, true); else VX_LAUNCH_TVA(true, true, false);
    } else {
      if (sh) VX_LAUNCH_TVA(true, false, true); else VX_LAUNCH_TVA(true, false, false);
    }
  } else {
    if (sh) VX_LAUNCH_TVA(false, false, true); else VX_LAUNCH_TVA(false, false, false);
  }
#undef VX_LAUNCH_TVA
  return launch_status();
}

int vx_grid_tv_adam_step(const float* param_in, float* param_out, float* grad, float* exp_avg, float* exp_avg_sq,
                         const float* per_lr, void* shadow_bf16, int64_t C, int64_t X, int64_t Y, int64_t Z,
                         int channel_last, int tv_enabled, float tv_weight, int tv_dense_mode, double lr,
                         double beta1, double beta2, double eps, int64_t step, int zero_grad, void* stream) {
  return grid_tv_adam_impl(param_in, param_out, grad, exp_avg, exp_avg_sq, per_lr, shadow_bf16, C, X, Y, Z,
                           channel_last, tv_enabled, tv_weight, tv_dense_mode, lr, beta1, beta2, eps, step,
                           zero_grad, nullptr, stream);
}

int vx_grid_tv_adam_step_touched(const float* param_in, float* param_out, float* grad, float* exp_avg,
                                 float* exp_avg_sq, const float* per_lr, void* shadow_bf16, int64_t C, int64_t X,
                                 int64_t Y, int64_t Z, int channel_last, int tv_enabled, float tv_weight,
                                 int tv_dense_mode, double lr, double beta1, double beta2, double eps, int64_t step,
                                 int zero_grad, const uint8_t* touched, void* stream) {
  if (!touched) return VX_ERR_ARG;
  return grid_tv_adam_impl(param_in, param_out, grad, exp_avg, exp_avg_sq, per_lr, shadow_bf16, C, X, Y, Z,
                           channel_last, tv_enabled, tv_weight, tv_dense_mode, lr, beta1, beta2, eps, step,
                           zero_grad, touched, stream);
}

int vx_grid_clear_touched(float* grad, uint8_t* touched, int64_t n_vox, int64_t C, void* stream) {
  if (n_vox < 0 || C < 1 || C > 64) return VX_ERR_ARG;
  if (n_vox == 0) return VX_OK;
  if (!grad || !touched || (((uintptr_t)touched) & 15)) return VX_ERR_ARG;
  const int64_t chunks = (n_vox + 15) / 16;
  clear_touched_kernel<<<sweep_blocks(chunks), 256, 0, as_stream(stream)>>>(grad, touched, n_vox, (int)C);
  return launch_status();
}

}  // extern "C"
