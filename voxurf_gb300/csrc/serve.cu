// Render-server kernels: the inference form of the fine model's forward
// (lib/voxurf_fine.py:620-802 with global_step = None) over the rays of one
// tick, which mixes requests for several resident scenes.  Every stage is
// one launch for the whole tick; the scene of a ray selects its grids and
// constants from a table that each block copies into shared memory.
//
//   rays      : per ray, its view chunk (binary search) -> get_rays.
//   first     : per ray (one thread), the first sample that can lie in the
//               mask, from the mask's block occupancy (scenes that have one).
//   march     : per ray (one warp, 32 samples per iteration), exact samples,
//               mask, SDF + FD normal, NeuS alpha, transmittance scan with the
//               T < 1e-3 stop; only shaded samples (weight > thres) are kept,
//               as 8-byte (step, weight) records.
//   rows      : row -> ray map of the dense shaded rows.
//   features  : MLP input rows (fine_feature_rows), BF16 or FP32.
//   mlp_head  : the 192 -> 3 output layer with FP32 accumulation, for the
//               FP32 scenes whose hidden layers are GEMMs issued by the host
//               (BF16 scenes run the whole MLP in the fused tcgen05 kernel).
//   composite : per ray, sum w*sigmoid(logit) + alphainv_last*bg (clamped in
//               the k-branch) and depth, written into the output images.
#include <math.h>
#include "common.cuh"
#include "fine_device.cuh"
#include "trilinear.cuh"

namespace vx {

struct SceneK {
  GridGeom g;
  const float* sdf;
  const float* k0f;
  const __nv_bfloat16* k0h;
  const uint8_t* mask;
  int mX, mY, mZ;
  float mscale[3], mshift[3];
  float vs, inv_s, stepdist, near, bg, thres;
  const uint8_t* occ;  // optional block occupancy of the mask (padded by one cell)
  int oX, oY, oZ, oB;
  DensityMask dm;      // optional MaskCache density mask (dm.dens null: none)
};

struct SceneTable {
  SceneK s[VX_SERVE_MAX_SCENES];
  int n;
};

static_assert(sizeof(SceneK) % 4 == 0, "scene table is copied as 32-bit words");

// Cooperative copy of the (by-value) scene table into shared memory.
__device__ __forceinline__ void load_scenes(const SceneTable& T, SceneK* sh) {
  const int words = T.n * (int)(sizeof(SceneK) / 4);
  const int* src = reinterpret_cast<const int*>(T.s);
  int* dst = reinterpret_cast<int*>(sh);
  for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  __syncthreads();
}

// ---- rays of a tick ---------------------------------------------------------
__global__ void serve_rays_kernel(const vx_view_chunk* __restrict__ ch, int n_chunks, int64_t n_rays,
                                  float* __restrict__ rays_o, float* __restrict__ rays_d,
                                  float* __restrict__ viewdirs, int* __restrict__ ray_scene,
                                  int64_t* __restrict__ ray_out) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  int lo = 0, hi = n_chunks - 1;  // last chunk with ray0 <= r
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (ch[mid].ray0 <= r) lo = mid; else hi = mid - 1;
  }
  const vx_view_chunk& c = ch[lo];
  const int64_t pix = c.pix0 + (r - c.ray0);
  const float i = (float)(pix % c.W) + 0.5f, j = (float)(pix / c.W) + 0.5f;
  float o[3], d[3], v[3];
  pinhole_ray(c.c2w, c.fx, c.fy, c.cx, c.cy, c.inverse_y, i, j, o, d, v);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    rays_o[3 * r + a] = o[a];
    rays_d[3 * r + a] = d[a];
    viewdirs[3 * r + a] = v[a];
  }
  ray_scene[r] = c.scene;
  ray_out[r] = c.out0 + (r - c.ray0);
}

__global__ void camera_rays_kernel(vx_view_chunk c, int64_t n, float* __restrict__ rays_o,
                                   float* __restrict__ rays_d, float* __restrict__ viewdirs) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float i = (float)(p % c.W) + 0.5f, j = (float)(p / c.W) + 0.5f;
  float o[3], d[3], v[3];
  pinhole_ray(c.c2w, c.fx, c.fy, c.cx, c.cy, c.inverse_y, i, j, o, d, v);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    rays_o[3 * p + a] = o[a];
    rays_d[3 * p + a] = d[a];
    viewdirs[3 * p + a] = v[a];
  }
}

// ---- empty-space skipping ------------------------------------------------------
// Block occupancy: padded cell (I,J,K) <- any mask voxel in
// [B(I-1) - 1, B I + 1) x ... (the block widened by one voxel).
__global__ void mask_occupancy_kernel(const uint8_t* __restrict__ mask, int mX, int mY, int mZ, int B,
                                      uint8_t* __restrict__ occ, int oX, int oY, int oZ) {
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= (int64_t)oX * oY * oZ) return;
  const int K = (int)(cell % oZ), J = (int)((cell / oZ) % oY), I = (int)(cell / ((int64_t)oY * oZ));
  const int i0 = max(B * (I - 1) - 1, 0), i1 = min(B * I + 1, mX);
  const int j0 = max(B * (J - 1) - 1, 0), j1 = min(B * J + 1, mY);
  const int k0 = max(B * (K - 1) - 1, 0), k1 = min(B * K + 1, mZ);
  uint8_t any = 0;
  for (int i = i0; i < i1 && !any; ++i)
    for (int j = j0; j < j1 && !any; ++j)
      for (int k = k0; k < k1; ++k)
        if (mask[((int64_t)i * mY + j) * mZ + k]) {
          any = 1;
          break;
        }
  occ[cell] = any;
}

// Mask-index coordinates of sample k on a float model of the march:
// u(k) = u0 + du * k (the exact positions differ by far less than a voxel).
struct SkipModel {
  float u0[3], du[3];
};

__device__ __forceinline__ SkipModel skip_model(const RayFrame& f, const SceneK& S) {
  SkipModel m;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    m.u0[a] = f.st[a] * S.mscale[a] + S.mshift[a];
    m.du[a] = f.dr[a] * S.stepdist * S.mscale[a];
  }
  return m;
}

// First k' >= k whose sample the model places in an occupied cell (cells
// outside the padded grid are empty), or n_steps.  Every sample skipped lies
// in an empty widened cell, so its mask lookup would have been false.
__device__ __forceinline__ int skip_empty(const SkipModel& m, int k, int n_steps, const SceneK& S) {
  const int dims[3] = {S.oX, S.oY, S.oZ};
  const float invB = 1.f / (float)S.oB;
  for (int it = 0; it < 4096 && k < n_steps; ++it) {
    int c[3];
    bool inside = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float u = m.u0[a] + m.du[a] * (float)k;
      const float cf = floorf((u + 0.5f) * invB) + 1.f;
      // beyond the padded grid and moving away from it: no later sample can hit the mask
      if ((cf < 0.f && m.du[a] <= 0.f) || (cf >= (float)dims[a] && m.du[a] >= 0.f)) return n_steps;
      c[a] = (int)fminf(fmaxf(cf, -1.f), (float)dims[a]);
      inside &= (c[a] >= 0) & (c[a] < dims[a]);
    }
    if (inside && __ldg(S.occ + ((int64_t)c[0] * S.oY + c[1]) * S.oZ + c[2])) return k;
    float t = 3.0e9f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (m.du[a] > 0.f)
        t = fminf(t, ((float)(S.oB * c[a]) - 0.5f - m.u0[a]) / m.du[a]);
      else if (m.du[a] < 0.f)
        t = fminf(t, ((float)(S.oB * (c[a] - 1)) - 0.5f - m.u0[a]) / m.du[a]);
    }
    if (!(t < (float)n_steps)) return n_steps;
    k = max(k + 1, (int)ceilf(t));
  }
  return k;
}

// ---- march ------------------------------------------------------------------
struct ServeMarchParams {
  SceneTable T;
  const float* rays_o;
  const float* rays_d;
  const float* viewdirs;
  const int* ray_scene;
  int n_rays;
  int max_steps;
  uint2* rec;  // [n_rays*max_steps] {step, weight bits} of the shaded samples
  int* n2;
  float* alphainv_last;
  int* err;
};

// First and last sample of each ray that can lie in its scene's mask
// (scenes with an occupancy grid), written to n2[r] and (as int bits)
// alphainv_last[r] for the march to start and end at; both outputs are
// overwritten by the march.  One thread per ray: the block walk is serial
// per ray, so 32 rays share a warp's instruction stream (a warp-per-ray walk
// would spend 32x the issue slots).  Exact: skip_empty only passes cells of
// the one-voxel-widened occupancy that hold no mask voxel, and either walk's
// float model is within far less than the widening of the exact samples.
__global__ void __launch_bounds__(256) serve_first_kernel(ServeMarchParams P) {
  __shared__ SceneK sh[VX_SERVE_MAX_SCENES];
  load_scenes(P.T, sh);
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= P.n_rays) return;
  const int sc = P.ray_scene[r];
  if (sc < 0 || sc >= P.T.n) return;  // reported by the march
  const SceneK& S = sh[sc];
  if (!S.occ) {
    P.n2[r] = 0;
    return;
  }
  float o[3], d[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = __ldg(P.rays_o + 3 * r + a);
    d[a] = __ldg(P.rays_d + 3 * r + a);
  }
  const RayFrame f = ray_frame(o, d, S.g.mn, S.g.mx, S.near, S.stepdist);
  const int n_steps = (int)min(f.n_steps, (int64_t)P.max_steps);
  const SkipModel fwd = skip_model(f, S);
  const int first = skip_empty(fwd, 0, n_steps, S);
  // last possible sample: the same walk from the far end (model reversed)
  int last = -1;
  if (first < n_steps) {
    SkipModel rev;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      rev.u0[a] = fwd.u0[a] + fwd.du[a] * (float)(n_steps - 1);
      rev.du[a] = -fwd.du[a];
    }
    last = (n_steps - 1) - skip_empty(rev, 0, n_steps - first, S);
  }
  P.n2[r] = first;
  P.alphainv_last[r] = __int_as_float(last);  // stashed for the march, which overwrites it
}

template <bool DENS>  // some scene carries a MaskCache density mask
__global__ void __launch_bounds__(256, 4) serve_march_kernel(ServeMarchParams P) {
  __shared__ SceneK sh[VX_SERVE_MAX_SCENES];
  load_scenes(P.T, sh);
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  const unsigned lt_mask = (1u << lane) - 1u;
  const int sc = P.ray_scene[r];
  if (sc < 0 || sc >= P.T.n) {
    if (lane == 0) {
      set_device_error(P.err, VX_ERR_BOUNDS);
      P.n2[r] = 0;
      P.alphainv_last[r] = 1.f;
    }
    return;
  }
  const SceneK& S = sh[sc];
  float o[3], d[3], v[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = __ldg(P.rays_o + 3 * r + a);
    d[a] = __ldg(P.rays_d + 3 * r + a);
    v[a] = __ldg(P.viewdirs + 3 * r + a);
  }
  const RayFrame f = ray_frame(o, d, S.g.mn, S.g.mx, S.near, S.stepdist);
  int64_t n_steps = f.n_steps;
  if (n_steps > P.max_steps) {
    if (lane == 0) set_device_error(P.err, VX_ERR_CAPACITY);
    n_steps = P.max_steps;
  }
  uint2* rec = P.rec + (int64_t)r * P.max_steps;
  // transmittance product: FP64 for rays of more than 512 samples, FP32 otherwise
  const bool wide = f.n_steps > VX_FP32_SCAN_MAX_STEPS;
  double carry_d = 1.0, last_d = 1.0;
  float carry_f = 1.f, last_f = 1.f;
  int cnt2 = 0;
  bool stopped = false;
  // with an occupancy grid, serve_first_kernel left the first and the last
  // sample that can lie in the mask in n2[r] and alphainv_last[r]: every
  // sample outside [k0, kl] is masked out
  const int k0 = S.occ ? P.n2[r] : 0;
  const int kl = S.occ ? __float_as_int(P.alphainv_last[r]) : INT_MAX;
  for (int base = k0; !stopped && base <= kl; base += 32) {
    if (base >= n_steps) break;
    const int k = base + lane;
    bool keep = false;
    float alpha = 0.f;
    if (k < n_steps) {
      float p[3];
      sample_point(f, S.stepdist, k, p);
      bool inb = !outside_bbox(p, S.g.mn, S.g.mx);
      if (inb && S.mask) inb = mask_lookup(S.mask, S.mX, S.mY, S.mZ, S.mscale, S.mshift, p);
      if (DENS && inb && S.dm.dens) inb = density_mask_hit(S.dm, p);
      if (inb) {
        float ind[3], s, gr[3];
        to_index(S.g, p, ind);
        sdf_and_grad(S.sdf, S.g, S.vs, ind, &s, gr);
        alpha = neus_alpha(s, gr, v, S.inv_s, S.stepdist).alpha;
        keep = alpha > S.thres;
      }
    }
    const unsigned keep_mask = __ballot_sync(0xffffffffu, keep);
    if (keep_mask == 0u) continue;
    float T;
    const unsigned live = wide ? transmittance_step<double>(keep, alpha, carry_d, last_d, stopped, T)
                               : transmittance_step<float>(keep, alpha, carry_f, last_f, stopped, T);
    const bool mine = (live >> lane) & 1u;
    const float w = T * alpha;
    const bool s2 = mine && (w > S.thres);
    const unsigned s2_mask = __ballot_sync(0xffffffffu, s2);
    if (s2) rec[cnt2 + __popc(s2_mask & lt_mask)] = make_uint2((unsigned)k, __float_as_uint(w));
    cnt2 += __popc(s2_mask);
  }
  if (lane == 0) {
    P.n2[r] = cnt2;
    P.alphainv_last[r] = wide ? (float)(stopped ? last_d : carry_d) : (stopped ? last_f : carry_f);
  }
}

// ---- row -> ray --------------------------------------------------------------
// Thread per ray: a ray has a few shaded rows (about five at the fine
// shapes), so a warp per ray would leave most lanes idle.
__global__ void __launch_bounds__(256) serve_rows_kernel(const int64_t* __restrict__ s2_off, int n_rays,
                                                         int* __restrict__ ray2, int64_t capacity) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  const int64_t b = s2_off[r], e = min(s2_off[r + 1], capacity);
  for (int64_t i = b; i < e; ++i) ray2[i] = r;
}

// ---- features ----------------------------------------------------------------
struct ServeFeatParams {
  SceneTable T;
  FeatLayout L;
  const float* rays_o;
  const float* rays_d;
  const float* viewdirs;
  const int* ray_scene;
  int max_steps;
  const uint2* rec;
  const int64_t* s2_off;
  const int* ray2;
  int64_t n_rows;              // rows, or the capacity with n_rows_dev
  const int64_t* n_rows_dev;   // device row count or null
  int64_t ld1, ld2;
  int cols1, cols2;  // feature columns; X1 [cols1, ld1) and X2 [cols2 + 3, ld2) are zero-filled
  void* X1;
  void* X2;
};

// STAGE: rows assembled in shared memory (bank-conflict-free padded stride),
// written out one row per warp in coalesced words (the logit columns
// [cols2, cols2+3) are zero until the rgbnet output layer fills them).
// COMPACT (with STAGE, when x2's encodings equal x1's): the x2 stage holds
// only x2's own columns and the copy-out takes the encodings from the x1
// stage (27 instead of 38 KB per CTA at the fine layout: one CTA more per SM).
template <typename T, int KK, bool STAGE, bool COMPACT = false>
__global__ void __launch_bounds__(128) serve_features_kernel(ServeFeatParams P) {
  __shared__ SceneK sh[VX_SERVE_MAX_SCENES];
  extern __shared__ __align__(16) unsigned char feat_stage[];
  const int64_t n_rows = P.n_rows_dev ? min(*P.n_rows_dev, P.n_rows) : P.n_rows;
  const int64_t row0 = (int64_t)blockIdx.x * blockDim.x;
  if (row0 >= n_rows) return;  // uniform over the block
  load_scenes(P.T, sh);
  const int64_t row = row0 + threadIdx.x;
  T* s1 = reinterpret_cast<T*>(feat_stage);
  const int n_pe = (3 + 6 * P.L.pos_pe) + (3 + 6 * P.L.view_pe);
  const int shift2 = COMPACT ? n_pe : 0;
  const int64_t sl1 = stage_ld<T>(P.ld1), sl2 = COMPACT ? odd_words_ld<T>(P.ld2 - n_pe) : stage_ld<T>(P.ld2);
  T* s2 = s1 + (int64_t)blockDim.x * sl1;
  if (row < n_rows) {
    const int r = P.ray2[row];
    const SceneK& S = sh[P.ray_scene[r]];  // validated by the march
    const int j = (int)(row - P.s2_off[r]);
    const int k = (int)P.rec[(int64_t)r * P.max_steps + j].x;
    float o[3], d[3], v[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      o[a] = __ldg(P.rays_o + 3 * r + a);
      d[a] = __ldg(P.rays_d + 3 * r + a);
      v[a] = __ldg(P.viewdirs + 3 * r + a);
    }
    const RayFrame f = ray_frame(o, d, S.g.mn, S.g.mx, S.near, S.stepdist);
    float p[3];
    sample_point(f, S.stepdist, k, p);
    T* x1 = STAGE ? s1 + (int64_t)threadIdx.x * sl1 : reinterpret_cast<T*>(P.X1) + row * P.ld1;
    T* x2 = STAGE ? s2 + (int64_t)threadIdx.x * sl2 : reinterpret_cast<T*>(P.X2) + row * P.ld2;
    float g1[3];
    fine_feature_rows<T, KK, STAGE, COMPACT>(S.sdf, S.g, S.vs, S.k0f, S.k0h, P.L, p, v, x1, x2, g1);
    for (int c = P.cols1; c < P.ld1; ++c) put(x1, c, 0.f);
    for (int c = STAGE ? P.cols2 : P.cols2 + 3; c < P.ld2; ++c) put(x2, c - shift2, 0.f);
  }
  if (STAGE) {
    __syncthreads();
    const int nv = (int)max((int64_t)0, min((int64_t)blockDim.x, n_rows - row0));
    copy_rows_out(s1, reinterpret_cast<T*>(P.X1) + row0 * P.ld1, nv, P.ld1);
    if (COMPACT)
      copy_rows_out_compact(s1, sl1, s2, sl2, reinterpret_cast<T*>(P.X2) + row0 * P.ld2, nv, P.ld2,
                            P.L.use_rgbnet_k0 ? 12 : 0, n_pe);
    else
      copy_rows_out(s2, reinterpret_cast<T*>(P.X2) + row0 * P.ld2, nv, P.ld2);
  }
}

// ---- output layer ------------------------------------------------------------
constexpr int HEAD_MAX_WIDTH = 256;

__device__ __forceinline__ float to_f(float x) { return x; }
__device__ __forceinline__ float to_f(__nv_bfloat16 x) { return __bfloat162float(x); }

// 16-byte row chunks: 8 BF16 or 4 FP32 values.
__device__ __forceinline__ void chunk_to_f(const uint4& u, const __nv_bfloat16*, float x[8]) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 f = __bfloat1622float2(h[i]);
    x[2 * i] = f.x;
    x[2 * i + 1] = f.y;
  }
}
__device__ __forceinline__ void chunk_to_f(const uint4& u, const float*, float x[8]) {
  x[0] = __uint_as_float(u.x);
  x[1] = __uint_as_float(u.y);
  x[2] = __uint_as_float(u.z);
  x[3] = __uint_as_float(u.w);
}

// One thread per row; the 3 x width weights in shared memory (broadcast
// reads); VEC: rows read in 16-byte chunks (width and the row stride are
// multiples of the chunk, the base 16-byte aligned).
template <typename T, bool VEC>
__global__ void __launch_bounds__(256) mlp_head_kernel(const T* __restrict__ H, int64_t n_rows, int width,
                                                       int64_t ldh, const float* __restrict__ W,
                                                       const float* __restrict__ b, const float* __restrict__ add,
                                                       float* __restrict__ out, void* cols, int64_t ld_cols,
                                                       int cols_bf16) {
  __shared__ float sw[3 * HEAD_MAX_WIDTH];
  for (int i = threadIdx.x; i < 3 * width; i += blockDim.x) sw[i] = W[i];
  __syncthreads();
  constexpr int PER = 16 / (int)sizeof(T);
  const float b0 = b ? b[0] : 0.f, b1 = b ? b[1] : 0.f, b2 = b ? b[2] : 0.f;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < n_rows; row += stride) {
    const T* h = H + row * ldh;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    if (VEC) {
      const uint4* hv = reinterpret_cast<const uint4*>(h);
      for (int c0 = 0; c0 < width; c0 += PER) {
        float x[8];
        chunk_to_f(__ldg(hv + c0 / PER), h, x);
#pragma unroll
        for (int i = 0; i < PER; ++i) {
          a0 += x[i] * sw[c0 + i];
          a1 += x[i] * sw[width + c0 + i];
          a2 += x[i] * sw[2 * width + c0 + i];
        }
      }
    } else {
      for (int c = 0; c < width; ++c) {
        const float x = to_f(h[c]);
        a0 += x * sw[c];
        a1 += x * sw[width + c];
        a2 += x * sw[2 * width + c];
      }
    }
    a0 += b0;
    a1 += b1;
    a2 += b2;
    if (add) {
      a0 += add[3 * row + 0];
      a1 += add[3 * row + 1];
      a2 += add[3 * row + 2];
    }
    out[3 * row + 0] = a0;
    out[3 * row + 1] = a1;
    out[3 * row + 2] = a2;
    if (cols) {
      if (cols_bf16) {
        __nv_bfloat16* cp = reinterpret_cast<__nv_bfloat16*>(cols) + row * ld_cols;
        cp[0] = __float2bfloat16_rn(a0);
        cp[1] = __float2bfloat16_rn(a1);
        cp[2] = __float2bfloat16_rn(a2);
      } else {
        float* cp = reinterpret_cast<float*>(cols) + row * ld_cols;
        cp[0] = a0;
        cp[1] = a1;
        cp[2] = a2;
      }
    }
  }
}

// ---- composite -----------------------------------------------------------------
struct ServeCompositeParams {
  SceneTable T;
  const int* ray_scene;
  int n_rays;
  int max_steps;
  const uint2* rec;
  const int64_t* s2_off;
  const float* logit;
  const float* klogit;  // null: no k-branch
  const float* alphainv_last;
  const int64_t* ray_out;
  float* out_rgb;
  float* out_depth;
};

// Thread per ray (a few shaded rows each), the ray's rows summed in order.
__global__ void __launch_bounds__(256) serve_composite_kernel(ServeCompositeParams P) {
  __shared__ SceneK sh[VX_SERVE_MAX_SCENES];
  load_scenes(P.T, sh);
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= P.n_rays) return;
  const int sc = P.ray_scene[r];
  if (sc < 0 || sc >= P.T.n) return;  // reported by the march
  const SceneK& S = sh[sc];
  const int64_t b = P.s2_off[r], e = P.s2_off[r + 1];
  const uint2* rec = P.rec + (int64_t)r * P.max_steps;
  const float* lg = P.klogit ? P.klogit : P.logit;
  float acc[3] = {0.f, 0.f, 0.f}, dep = 0.f;
  for (int64_t i = b; i < e; ++i) {
    const uint2 rc = rec[i - b];
    const float w = __uint_as_float(rc.y);
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[c] += w * sigmoidf_(lg[3 * i + c]);
    dep += w * ((float)rc.x * S.stepdist);
  }
  {
    const float bgt = P.alphainv_last[r] * S.bg;
    const int64_t o = P.ray_out[r];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float x = acc[c] + bgt;
      P.out_rgb[3 * o + c] = P.klogit ? fminf(fmaxf(x, 0.f), 1.f) : x;
    }
    if (P.out_depth) P.out_depth[o] = dep;
  }
}

// ---- host helpers ----------------------------------------------------------------
static int scene_table(const vx_scene_desc* D, int n, SceneTable& T) {
  if (!D || n < 1 || n > VX_SERVE_MAX_SCENES) return VX_ERR_ARG;
  T.n = n;
  for (int i = 0; i < n; ++i) {
    const vx_scene_desc& d = D[i];
    SceneK& s = T.s[i];
    if (!d.sdf_smooth || !d.k0 || d.grid.X < 2 || d.grid.Y < 2 || d.grid.Z < 2) return VX_ERR_ARG;
    if (d.grid.X > INT32_MAX / d.grid.Y / d.grid.Z) return VX_ERR_TOO_LARGE;
    if (!(d.stepdist > 0.f) || !(d.voxel_size > 0.f)) return VX_ERR_ARG;
    s.g.X = (int)d.grid.X;
    s.g.Y = (int)d.grid.Y;
    s.g.Z = (int)d.grid.Z;
    for (int a = 0; a < 3; ++a) {
      s.g.mn[a] = d.grid.xyz_min[a];
      s.g.mx[a] = d.grid.xyz_max[a];
      s.mscale[a] = d.mask_scale[a];
      s.mshift[a] = d.mask_shift[a];
    }
    s.sdf = d.sdf_smooth;
    s.k0f = d.k0_bf16 ? nullptr : reinterpret_cast<const float*>(d.k0);
    s.k0h = d.k0_bf16 ? reinterpret_cast<const __nv_bfloat16*>(d.k0) : nullptr;
    s.mask = d.mask;
    s.mX = (int)d.mask_X;
    s.mY = (int)d.mask_Y;
    s.mZ = (int)d.mask_Z;
    s.vs = d.voxel_size;
    s.inv_s = d.inv_s;
    s.stepdist = d.stepdist;
    s.near = d.near;
    s.bg = d.bg;
    s.thres = d.fast_color_thres;
    s.occ = d.occ;
    s.oX = (int)d.occ_X;
    s.oY = (int)d.occ_Y;
    s.oZ = (int)d.occ_Z;
    s.oB = d.occ_block;
    if (d.occ && (!d.mask || d.occ_block < 1 || d.occ_X != (d.mask_X + d.occ_block - 1) / d.occ_block + 2 ||
                  d.occ_Y != (d.mask_Y + d.occ_block - 1) / d.occ_block + 2 ||
                  d.occ_Z != (d.mask_Z + d.occ_block - 1) / d.occ_block + 2))
      return VX_ERR_ARG;
    const int sd = fill_density_mask(d.mask_density, d.mask_dgrid, d.mask_act_shift, d.mask_voxel_size_ratio,
                                     d.mask_thres, d.mask != nullptr, s.dm);
    if (sd) return sd;
  }
  for (int i = n; i < VX_SERVE_MAX_SCENES; ++i) T.s[i] = T.s[0];
  return VX_OK;
}

static unsigned warp_blocks(int64_t n_warps) { return (unsigned)((n_warps + 7) / 8); }

}  // namespace vx

using namespace vx;

extern "C" {

int vx_camera_rays(const float* c2w_host, float fx, float fy, float cx, float cy, int64_t H, int64_t W,
                   int inverse_y, float* rays_o, float* rays_d, float* viewdirs, void* stream) {
  if (!c2w_host || H < 0 || W < 0 || H * W > INT32_MAX) return VX_ERR_ARG;
  if (H * W == 0) return VX_OK;
  if (!rays_o || !rays_d || !viewdirs) return VX_ERR_ARG;
  vx_view_chunk c = {};
  for (int q = 0; q < 12; ++q) c.c2w[q] = c2w_host[q];
  c.fx = fx;
  c.fy = fy;
  c.cx = cx;
  c.cy = cy;
  c.W = (int32_t)W;
  c.inverse_y = inverse_y;
  camera_rays_kernel<<<grid_for(H * W), VX_THREADS, 0, as_stream(stream)>>>(c, H * W, rays_o, rays_d, viewdirs);
  return launch_status();
}

int vx_serve_rays(const vx_view_chunk* chunks, int32_t n_chunks, int64_t n_rays, float* rays_o, float* rays_d,
                  float* viewdirs, int32_t* ray_scene, int64_t* ray_out, void* stream) {
  if (n_rays < 0 || n_rays > INT32_MAX) return VX_ERR_ARG;
  if (n_rays == 0) return VX_OK;
  if (!chunks || n_chunks < 1 || !rays_o || !rays_d || !viewdirs || !ray_scene || !ray_out) return VX_ERR_ARG;
  serve_rays_kernel<<<grid_for(n_rays), VX_THREADS, 0, as_stream(stream)>>>(chunks, n_chunks, n_rays, rays_o, rays_d,
                                                                           viewdirs, ray_scene, ray_out);
  return launch_status();
}

int vx_serve_march(const vx_scene_desc* scenes_host, int32_t n_scenes, const float* rays_o, const float* rays_d,
                   const float* viewdirs, const int32_t* ray_scene, int64_t n_rays, int64_t max_steps, void* rec,
                   int32_t* n2, float* alphainv_last, void* stream) {
  if (n_rays < 0 || n_rays > INT32_MAX || max_steps < 1 || max_steps > INT32_MAX) return VX_ERR_ARG;
  if (n_rays == 0) return VX_OK;
  ServeMarchParams P{};
  int s = scene_table(scenes_host, n_scenes, P.T);
  if (s) return s;
  if (!rays_o || !rays_d || !viewdirs || !ray_scene || !rec || !n2 || !alphainv_last) return VX_ERR_ARG;
  P.rays_o = rays_o;
  P.rays_d = rays_d;
  P.viewdirs = viewdirs;
  P.ray_scene = ray_scene;
  P.n_rays = (int)n_rays;
  P.max_steps = (int)max_steps;
  P.rec = reinterpret_cast<uint2*>(rec);
  P.n2 = n2;
  P.alphainv_last = alphainv_last;
  P.err = device_error_ptr();
  bool dens = false, occ = false;
  for (int i = 0; i < P.T.n; ++i) {
    dens |= P.T.s[i].dm.dens != nullptr;
    occ |= P.T.s[i].occ != nullptr;
  }
  if (occ) {
    serve_first_kernel<<<(unsigned)((n_rays + 255) / 256), 256, 0, as_stream(stream)>>>(P);
    s = launch_status();
    if (s) return s;
  }
  if (dens)
    serve_march_kernel<true><<<warp_blocks(n_rays), 256, 0, as_stream(stream)>>>(P);
  else
    serve_march_kernel<false><<<warp_blocks(n_rays), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

int vx_mask_occupancy(const uint8_t* mask, int64_t mX, int64_t mY, int64_t mZ, int32_t block, uint8_t* occ,
                      void* stream) {
  if (!mask || !occ || mX < 1 || mY < 1 || mZ < 1 || block < 1 || block > 64) return VX_ERR_ARG;
  if (mX > INT32_MAX / mY / mZ) return VX_ERR_TOO_LARGE;
  const int oX = (int)((mX + block - 1) / block + 2), oY = (int)((mY + block - 1) / block + 2),
            oZ = (int)((mZ + block - 1) / block + 2);
  const int64_t n = (int64_t)oX * oY * oZ;
  mask_occupancy_kernel<<<grid_for(n), VX_THREADS, 0, as_stream(stream)>>>(mask, (int)mX, (int)mY, (int)mZ, block, occ,
                                                                          oX, oY, oZ);
  return launch_status();
}

int vx_serve_rows(const int64_t* s2_off, int64_t n_rays, int32_t* ray2, int64_t capacity, void* stream) {
  if (n_rays < 0 || n_rays > INT32_MAX || capacity < 0) return VX_ERR_ARG;
  if (n_rays == 0) return VX_OK;
  if (!s2_off || !ray2) return VX_ERR_ARG;
  serve_rows_kernel<<<(unsigned)((n_rays + 255) / 256), 256, 0, as_stream(stream)>>>(s2_off, (int)n_rays, ray2,
                                                                                  capacity);
  return launch_status();
}

int vx_serve_features(const vx_scene_desc* scenes_host, int32_t n_scenes, const vx_fine_feature_cfg* cfg,
                      const float* rays_o, const float* rays_d, const float* viewdirs, const int32_t* ray_scene,
                      int64_t max_steps, const void* rec, const int64_t* s2_off, const int32_t* ray2, int64_t n_rows,
                      const int64_t* n_rows_dev, int64_t ld1, int64_t ld2, void* X1, void* X2, int32_t out_bf16,
                      int32_t staging, void* stream) {
  if (n_rows < 0 || !cfg || max_steps < 1 || max_steps > INT32_MAX || staging < -1 || staging > 1)
    return VX_ERR_ARG;
  if (n_rows == 0) return VX_OK;
  ServeFeatParams P{};
  int s = scene_table(scenes_host, n_scenes, P.T);
  if (s) return s;
  s = fill_feat_layout(cfg, P.L);
  if (s) return s;
  if (ld1 < x1_cols(cfg) || ld2 < x2_cols(cfg) + 3) return VX_ERR_ARG;
  if (!rays_o || !rays_d || !viewdirs || !ray_scene || !rec || !s2_off || !ray2 || !X1 || !X2) return VX_ERR_ARG;
  P.rays_o = rays_o;
  P.rays_d = rays_d;
  P.viewdirs = viewdirs;
  P.ray_scene = ray_scene;
  P.max_steps = (int)max_steps;
  P.rec = reinterpret_cast<const uint2*>(rec);
  P.s2_off = s2_off;
  P.ray2 = ray2;
  P.n_rows = n_rows;
  P.n_rows_dev = n_rows_dev;
  P.ld1 = ld1;
  P.ld2 = ld2;
  P.cols1 = (int)x1_cols(cfg);
  P.cols2 = (int)x2_cols(cfg);
  P.X1 = X1;
  P.X2 = X2;
  const unsigned b = (unsigned)((n_rows + 127) / 128);
  cudaStream_t st = as_stream(stream);
  // staged rows: strides of 4-byte multiples, aligned bases, static + dynamic
  // shared memory within the default 48 KB
  const size_t esz = out_bf16 ? 2 : 4;
  const size_t shm = 128 * (size_t)(ld1 + ld2 + 2 * (4 / esz)) * esz;
  const bool stage_ok = ((size_t)ld1 * esz) % 4 == 0 && ((size_t)ld2 * esz) % 4 == 0 &&
                        shm + sizeof(SceneK) * VX_SERVE_MAX_SCENES <= 48 * 1024 &&
                        ((reinterpret_cast<uintptr_t>(X1) | reinterpret_cast<uintptr_t>(X2)) & 3) == 0;
  if (staging == 1 && !stage_ok) return VX_ERR_UNSUPPORTED;
  const bool stage = staging != 0 && stage_ok;
  // compact x2 staging: x2's encodings are x1's (same frequencies) and the
  // column groups are 4-byte aligned
  const int64_t n_pe = (3 + 6 * P.L.pos_pe) + (3 + 6 * P.L.view_pe);
  const int64_t epw = 4 / (int64_t)esz;
  const bool compact = stage && P.L.kpos_pe == P.L.pos_pe && P.L.kview_pe == P.L.view_pe && n_pe % epw == 0 &&
                       (P.L.use_rgbnet_k0 ? 12 : 0) % epw == 0 && 12 % epw == 0;
  // the strides of stage_ld and odd_words_ld, in elements
  const int64_t nc = ld2 - n_pe, sl2c = ((nc * (int64_t)esz / 4) % 2 == 1) ? nc : nc + epw;
  const size_t shm_c = 128 * (size_t)(ld1 + epw + sl2c) * esz;
#define VX_FEAT_LAUNCH(T, KK)                                          \
  if (compact)                                                         \
    serve_features_kernel<T, KK, true, true><<<b, 128, shm_c, st>>>(P); \
  else if (stage)                                                      \
    serve_features_kernel<T, KK, true><<<b, 128, shm, st>>>(P);        \
  else                                                                 \
    serve_features_kernel<T, KK, false><<<b, 128, 0, st>>>(P)
#define VX_FEAT_SWITCH(T)        \
  switch (P.L.K) {               \
    case 1: VX_FEAT_LAUNCH(T, 1); break; \
    case 2: VX_FEAT_LAUNCH(T, 2); break; \
    case 3: VX_FEAT_LAUNCH(T, 3); break; \
    default: VX_FEAT_LAUNCH(T, 4); break; \
  }
  if (out_bf16) {
    VX_FEAT_SWITCH(__nv_bfloat16)
  } else {
    VX_FEAT_SWITCH(float)
  }
#undef VX_FEAT_SWITCH
#undef VX_FEAT_LAUNCH
  return launch_status();
}

int vx_mlp_head(const void* H, int64_t n_rows, int64_t width, int64_t ldh, int32_t in_bf16, const float* W,
                const float* b, const float* add, float* out, void* cols, int64_t ld_cols, int32_t cols_bf16,
                void* stream) {
  if (n_rows < 0 || width < 1 || ldh < width) return VX_ERR_ARG;
  if (width > HEAD_MAX_WIDTH) return VX_ERR_UNSUPPORTED;
  if (n_rows == 0) return VX_OK;
  if (!H || !W || !out || (cols && ld_cols < 3)) return VX_ERR_ARG;
  const int64_t blocks_needed = (n_rows + 255) / 256;
  const unsigned blocks = (unsigned)(blocks_needed < (int64_t)sm_count() * 8 ? blocks_needed : sm_count() * 8);
  const int64_t esz = in_bf16 ? 2 : 4, per = 16 / esz;
  const bool vec = (width % per == 0) && (ldh % per == 0) && ((reinterpret_cast<uintptr_t>(H) & 15) == 0);
  cudaStream_t st = as_stream(stream);
  const int w = (int)width;
  if (in_bf16) {
    const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(H);
    if (vec)
      mlp_head_kernel<__nv_bfloat16, true><<<blocks, 256, 0, st>>>(h, n_rows, w, ldh, W, b, add, out, cols, ld_cols,
                                                                   cols_bf16);
    else
      mlp_head_kernel<__nv_bfloat16, false><<<blocks, 256, 0, st>>>(h, n_rows, w, ldh, W, b, add, out, cols, ld_cols,
                                                                    cols_bf16);
  } else {
    const float* h = reinterpret_cast<const float*>(H);
    if (vec)
      mlp_head_kernel<float, true><<<blocks, 256, 0, st>>>(h, n_rows, w, ldh, W, b, add, out, cols, ld_cols,
                                                           cols_bf16);
    else
      mlp_head_kernel<float, false><<<blocks, 256, 0, st>>>(h, n_rows, w, ldh, W, b, add, out, cols, ld_cols,
                                                            cols_bf16);
  }
  return launch_status();
}

int vx_serve_composite(const vx_scene_desc* scenes_host, int32_t n_scenes, const int32_t* ray_scene, int64_t n_rays,
                       int64_t max_steps, const void* rec, const int64_t* s2_off, const float* logit,
                       const float* klogit, const float* alphainv_last, const int64_t* ray_out, float* out_rgb,
                       float* out_depth, void* stream) {
  if (n_rays < 0 || n_rays > INT32_MAX || max_steps < 1 || max_steps > INT32_MAX) return VX_ERR_ARG;
  if (n_rays == 0) return VX_OK;
  ServeCompositeParams P{};
  int s = scene_table(scenes_host, n_scenes, P.T);
  if (s) return s;
  if (!ray_scene || !rec || !s2_off || !logit || !alphainv_last || !ray_out || !out_rgb) return VX_ERR_ARG;
  P.ray_scene = ray_scene;
  P.n_rays = (int)n_rays;
  P.max_steps = (int)max_steps;
  P.rec = reinterpret_cast<const uint2*>(rec);
  P.s2_off = s2_off;
  P.logit = logit;
  P.klogit = klogit;
  P.alphainv_last = alphainv_last;
  P.ray_out = ray_out;
  P.out_rgb = out_rgb;
  P.out_depth = out_depth;
  serve_composite_kernel<<<(unsigned)((n_rays + 255) / 256), 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

}  // extern "C"
