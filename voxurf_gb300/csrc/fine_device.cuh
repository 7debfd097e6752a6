// Device helpers shared by the training kernels (render.cu) and the render
// server kernels (serve.cu): exact ray sample positions, SDF probes, NeuS
// alpha and the MLP input encodings of the fine model.
#pragma once
#include <math.h>
#include "common.cuh"
#include "trilinear.cuh"

namespace vx {

constexpr int MAX_K = 4;  // hierarchical displacements (configs use <= 4)

// ---- exact sample positions (shared with sampling.cu semantics) ------------
struct RayFrame {
  float st[3], dr[3];
  int64_t n_steps;
};

__device__ __forceinline__ RayFrame ray_frame(const float* o, const float* d, const float* mn, const float* mx,
                                              float near, float stepdist) {
  const float far = 1e9f;  // voxurf_fine.py:605
  const float vx = (d[0] == 0.f) ? 1e-6f : d[0];
  const float vy = (d[1] == 0.f) ? 1e-6f : d[1];
  const float vz = (d[2] == 0.f) ? 1e-6f : d[2];
  const float ax = fdiv(fsub(mx[0], o[0]), vx), ay = fdiv(fsub(mx[1], o[1]), vy), az = fdiv(fsub(mx[2], o[2]), vz);
  const float bx = fdiv(fsub(mn[0], o[0]), vx), by = fdiv(fsub(mn[1], o[1]), vy), bz = fdiv(fsub(mn[2], o[2]), vz);
  const float t_min = fmaxf(fminf(fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz)), far), near);
  const float t_max = fmaxf(fminf(fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz)), far), near);
  const float rn = ray_norm3(d[0], d[1], d[2]);
  RayFrame f;
  const float c = ceilf(fdiv(fmul(fsub(t_max, t_min), rn), stepdist));
  f.n_steps = (int64_t)fmax((double)c, 1.0);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    f.st[a] = __fmaf_rn(d[a], t_min, o[a]);  // fused as in the reference's compiled kernel
    f.dr[a] = fdiv(d[a], rn);
  }
  return f;
}

__device__ __forceinline__ void sample_point(const RayFrame& f, float stepdist, int k, float p[3]) {
  const float dist = fmul(stepdist, (float)k);
#pragma unroll
  for (int a = 0; a < 3; ++a) p[a] = __fmaf_rn(f.dr[a], dist, f.st[a]);
}

// Pinhole ray through pixel centre (i, j) (+0.5 already added) of a camera
// with row-major 3x4 camera-to-world c2w (get_rays, voxurf_fine.py:1001-1029;
// viewdir = d/|d|, :1064).  inverse_y selects OpenCV axes (+y down, +z fwd).
// One rounding per operation, so the rays are reproducible bit for bit.
__device__ __forceinline__ void pinhole_ray(const float* c2w, float fx, float fy, float cx, float cy, int inverse_y,
                                            float i, float j, float o[3], float d[3], float v[3]) {
  float dir[3];
  dir[0] = fdiv(fsub(i, cx), fx);
  if (inverse_y) {
    dir[1] = fdiv(fsub(j, cy), fy);
    dir[2] = 1.f;
  } else {
    dir[1] = -fdiv(fsub(j, cy), fy);
    dir[2] = -1.f;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
    d[a] = fadd(fadd(fmul(dir[0], c2w[4 * a + 0]), fmul(dir[1], c2w[4 * a + 1])), fmul(dir[2], c2w[4 * a + 2]));
  const float nrm = __fsqrt_rn(fadd(fadd(fmul(d[0], d[0]), fmul(d[1], d[1])), fmul(d[2], d[2])));
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = c2w[4 * a + 3];
    v[a] = fdiv(d[a], nrm);
  }
}

// ---- SDF value + finite-difference gradient (sample_sdfs, one displacement) -
struct Probe {
  float fm, fp;     // values at index -d and +d (clamped)
  float inv_diff;   // 1 / (clamped index difference)
  Corners cm, cp;
};

__device__ __forceinline__ void probe_axis(const float* __restrict__ sdf, const GridGeom& g, const float ind[3],
                                           int axis, float d, Probe& pr, bool keep_corners) {
  float im[3] = {ind[0], ind[1], ind[2]};
  float ip[3] = {ind[0], ind[1], ind[2]};
  const float hi = (float)(gsize(g, axis) - 1);
  im[axis] = fminf(fmaxf(ind[axis] - d, 0.f), hi);
  ip[axis] = fminf(fmaxf(ind[axis] + d, 0.f), hi);
  Corners cm = corners_of(g, im[0], im[1], im[2]);
  Corners cp = corners_of(g, ip[0], ip[1], ip[2]);
  pr.fm = gather1(sdf, cm);
  pr.fp = gather1(sdf, cp);
  pr.inv_diff = 1.f / (ip[axis] - im[axis]);
  if (keep_corners) {
    pr.cm = cm;
    pr.cp = cp;
  }
}

__device__ __forceinline__ void to_index(const GridGeom& g, const float p[3], float ind[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) ind[a] = world_to_index(g, a, p[a]);
}

// SDF and gradient (xyz order) at one point: centre + 6 probes at +-1 voxel
// (each probe's coordinate clamped to the grid), as seven trilinear lookups.
// Away from the grid's faces a probe is the centre's lookup moved by one
// cell: when ind[a] +- 1 is exact in float (its fraction equals the
// centre's, which fails only where the sum crosses a power of two) and no
// probe is clamped or leaves the grid, every lookup uses the centre's eight
// weights, and the probes read the centre's corner values plus one new
// plane each.  The weights are the same floats corners_of forms and the sums
// run in the same corner order, so this fast path gives the seven lookups'
// values bit for bit; every other point takes the seven lookups.
__device__ __forceinline__ void sdf_and_grad(const float* __restrict__ sdf, const GridGeom& g, float voxel_size,
                                             const float ind[3], float* s, float gr[3]) {
  const int dims[3] = {g.X, g.Y, g.Z};
  float t[3];
  int i0[3];
  bool fast = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float f0 = floorf(ind[a]);
    i0[a] = (int)f0;
    t[a] = ind[a] - f0;
    const float qm = ind[a] - 1.f, qp = ind[a] + 1.f;
    const float fm = floorf(qm), fp = floorf(qp);
    fast = fast && (i0[a] >= 1) && (i0[a] + 2 <= dims[a] - 1) && (qm - fm == t[a]) && (qp - fp == t[a]) &&
           ((int)fm == i0[a] - 1) && ((int)fp == i0[a] + 1);
  }
  if (fast) {
    const int sx = g.Y * g.Z, sy = g.Z;
    const float* b = sdf + ((int64_t)i0[0] * g.Y + i0[1]) * g.Z + i0[2];
    const float wi[2] = {1.f - t[0], t[0]}, wj[2] = {1.f - t[1], t[1]}, wk[2] = {1.f - t[2], t[2]};
    float w[8], vc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int di = q >> 2, dj = (q >> 1) & 1, dk = q & 1;
      w[q] = wi[di] * wj[dj] * wk[dk];
      vc[q] = __ldg(b + di * sx + dj * sy + dk);
    }
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) acc += w[q] * vc[q];
    *s = acc;
    const int st[3] = {sx, sy, 1};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const int bit = 4 >> a;  // corner-index bit of axis a
      float fmv = 0.f, fpv = 0.f;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int di = q >> 2, dj = (q >> 1) & 1, dk = q & 1;
        const int off = di * sx + dj * sy + dk;
        // probe -1: its lower plane is new (i0 - 1), its upper plane is the centre's lower
        const float vm = (q & bit) ? vc[q & ~bit] : __ldg(b + off - st[a]);
        // probe +1: its lower plane is the centre's upper, its upper plane is new (i0 + 2)
        const float vp = (q & bit) ? __ldg(b + off + st[a]) : vc[q | bit];
        fmv += w[q] * vm;
        fpv += w[q] * vp;
      }
      gr[a] = ((fpv - fmv) * (1.f / ((ind[a] + 1.f) - (ind[a] - 1.f)))) / voxel_size;
    }
    return;
  }
  *s = sample1(sdf, g, ind[0], ind[1], ind[2]);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    Probe pr;
    probe_axis(sdf, g, ind, a, 1.f, pr, false);
    gr[a] = ((pr.fp - pr.fm) * pr.inv_diff) / voxel_size;
  }
}

__device__ __forceinline__ float sigmoidf_(float x) { return 1.f / (1.f + expf(-x)); }

// NeuS s-density alpha (voxurf_fine.py:475-499, cos_anneal_ratio = 1):
//   P = sigmoid(prev*inv_s), Q = sigmoid(next*inv_s),
//   alpha = clip((P - Q + 1e-5) / (P + 1e-5), 0, 1).
// Away from the surface P and Q both approach 1 and the literal P - Q loses
// all FP32 precision (about 1e-3 relative error at alpha ~ 1e-4, which flips
// the fast_color_thres decisions against an FP64 evaluation).  The same
// quantity is formed without cancellation:
//   P - Q = sigmoid(a) * sigmoid(-b) * (-expm1(b - a)),  a = prev*inv_s,
// b = next*inv_s (b <= a), and 1 - P, 1 - Q are taken as sigmoid(-a),
// sigmoid(-b) in the backward.
struct AlphaState {
  float alpha, raw, P, Q, nP, nQ, cosv;
};

__device__ __forceinline__ AlphaState neus_alpha(float s, const float gr[3], const float v[3], float inv_s,
                                                 float dist) {
  AlphaState a;
  a.cosv = v[0] * gr[0] + v[1] * gr[1] + v[2] * gr[2];
  const float ic = fminf(a.cosv, 0.f);  // -relu(-cos)
  const float h = ic * dist * 0.5f;
  const float next = s + h, prev = s - h;
  const float xa = prev * inv_s, xb = next * inv_s;
  a.P = sigmoidf_(xa);
  a.Q = sigmoidf_(xb);
  a.nP = sigmoidf_(-xa);
  a.nQ = sigmoidf_(-xb);
  const float pmq = -(a.P * a.nQ) * expm1f(xb - xa);
  a.raw = (pmq + 1e-5f) / (a.P + 1e-5f);
  a.alpha = fminf(fmaxf(a.raw, 0.f), 1.f);
  return a;
}

// Adjoint of neus_alpha at one sample (continuous grid index ind, view
// direction v) for an incoming d_alpha, scattered into the gradient of the
// (smoothed) SDF grid: the SDF and its +-1-voxel finite-difference gradient
// are recomputed, the clip passes the gradient only where the raw alpha lies
// in [0, 1], and the centre and the six probes are summed per plane of each
// axis before their reductions (the centre joins axis 0).
__device__ __forceinline__ void neus_alpha_adjoint_scatter(float d_alpha, const float ind[3], const float v[3],
                                                           float inv_s, float dist, const float* __restrict__ sdf,
                                                           const GridGeom& g, float voxel_size,
                                                           float* __restrict__ d_sdf) {
  float s, gr[3];
  sdf_and_grad(sdf, g, voxel_size, ind, &s, gr);
  const AlphaState a = neus_alpha(s, gr, v, inv_s, dist);
  if (!(a.raw >= 0.f && a.raw <= 1.f)) return;  // clip backward
  const float den = a.P + 1e-5f;
  const float dP = d_alpha * a.Q / (den * den);
  const float dQ = -d_alpha / den;
  const float d_prev = dP * a.P * a.nP * inv_s;
  const float d_next = dQ * a.Q * a.nQ * inv_s;
  const float d_s = d_prev + d_next;
  const float d_ic = (d_next - d_prev) * dist * 0.5f;
  const float d_cos = a.cosv < 0.f ? d_ic : 0.f;
#pragma unroll
  for (int axis = 0; axis < 3; ++axis) {
    const float dg = d_cos * v[axis];
    if (axis > 0 && dg == 0.f) continue;
    PlaneAcc acc;
    plane_acc_init(acc, ind[axis]);
    if (axis == 0) plane_acc_add(acc, d_sdf, g, ind, 0, ind[0], d_s);
    if (dg != 0.f) {
      const float hi = (float)(gsize(g, axis) - 1);
      const float xm = fminf(fmaxf(ind[axis] - 1.f, 0.f), hi);
      const float xp = fminf(fmaxf(ind[axis] + 1.f, 0.f), hi);
      const float dfd = dg / (xp - xm) / voxel_size;
      plane_acc_add(acc, d_sdf, g, ind, axis, xp, dfd);
      plane_acc_add(acc, d_sdf, g, ind, axis, xm, -dfd);
    }
    plane_acc_flush(acc, d_sdf, g, ind, axis);
  }
}

__device__ __forceinline__ bool outside_bbox(const float p[3], const float* mn, const float* mx) {
  return (mn[0] > p[0]) | (mn[1] > p[1]) | (mn[2] > p[2]) | (mx[0] < p[0]) | (mx[1] < p[1]) | (mx[2] < p[2]);
}

// maskcache_lookup semantics (render_utils_kernel.cu:374-392): nearest voxel
// of xyz*scale + shift (one fused multiply-add, as the reference's compiled
// kernel computes it), round half away from zero, false outside the grid.
__device__ __forceinline__ bool mask_lookup(const uint8_t* __restrict__ mask, int mX, int mY, int mZ,
                                            const float* scale, const float* shift, const float p[3]) {
  int ijk[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) ijk[a] = (int)roundf(__fmaf_rn(p[a], scale[a], shift[a]));
  if (ijk[0] < 0 || ijk[0] >= mX || ijk[1] < 0 || ijk[1] >= mY || ijk[2] < 0 || ijk[2] >= mZ) return false;
  return mask[((int64_t)ijk[0] * mY + ijk[1]) * mZ + ijk[2]] != 0;
}

// MaskCache (voxurf_fine.py:917-942, voxurf_coarse.py:671-696): the coarse
// model's density, max-pooled 3^3 at load time, sampled trilinearly
// (grid_sample, align_corners, zero padding) and thresholded as an alpha:
// 1 - exp(-softplus(d + act_shift) * voxel_size_ratio) >= thres, softplus
// with torch's default threshold 20.
struct DensityMask {
  const float* dens;  // [X,Y,Z]; null: no density mask
  GridGeom g;
  float shift, ratio, thres;
};

__device__ __forceinline__ bool density_mask_hit(const DensityMask& m, const float p[3]) {
  float ind[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) ind[a] = world_to_index(m.g, a, p[a]);
  const float d = sample1(m.dens, m.g, ind[0], ind[1], ind[2]);
  const float x = d + m.shift;
  const float sp = x > 20.f ? x : log1pf(expf(x));
  return 1.f - expf(-sp * m.ratio) >= m.thres;
}

// ---- MLP input encodings ----------------------------------------------------
template <typename T>
__device__ __forceinline__ void put(T* row, int c, float v);
template <>
__device__ __forceinline__ void put<float>(float* row, int c, float v) { row[c] = v; }
template <>
__device__ __forceinline__ void put<__nv_bfloat16>(__nv_bfloat16* row, int c, float v) {
  row[c] = __float2bfloat16_rn(v);
}

template <typename T>
__device__ __forceinline__ int put_pe(T* row, int c, const float x[3], int n_freq) {
  // [x, sin(x*2^f) (axis-major), cos(...)] as torch.cat([x, emb.sin(), emb.cos()])
  // with emb = (x.unsqueeze(-1) * freq).flatten(-2)  (voxurf_fine.py:694-698).
  // FP32 rows: sincosf of every frequency.  BF16 rows: sincosf of the base
  // frequency and the double-angle recurrence above it (error ~2^q ulp of
  // FP32 at frequency 2^q, far below the BF16 rounding of the row).
#pragma unroll
  for (int a = 0; a < 3; ++a) put(row, c + a, x[a]);
  c += 3;
  const int cs = c, cc = c + 3 * n_freq;
  for (int a = 0; a < 3; ++a) {
    if (sizeof(T) == 2) {
      float s, co;
      sincosf(x[a], &s, &co);
      for (int q = 0; q < n_freq; ++q) {
        put(row, cs + a * n_freq + q, s);
        put(row, cc + a * n_freq + q, co);
        const float s2 = 2.f * s * co, c2 = (co - s) * (co + s);
        s = s2;
        co = c2;
      }
    } else {
      for (int q = 0; q < n_freq; ++q) {
        float s, co;
        sincosf(x[a] * (float)(1 << q), &s, &co);
        put(row, cs + a * n_freq + q, s);
        put(row, cc + a * n_freq + q, co);
      }
    }
  }
  return cc + 3 * n_freq;
}

// Columns [c_src, c_src + n) of a staged row copied to [c_dst, ...) of another.
template <typename T>
__device__ __forceinline__ void copy_cols(const T* src, int c_src, T* dst, int c_dst, int n) {
  for (int i = 0; i < n; ++i) dst[c_dst + i] = src[c_src + i];
}

// Hierarchical features of one point: feat[6K] (dir-major: z-,z+,y-,y+,x-,x+
// each over K) and grad[3K] (pair-major z,y,x, normalised per K when
// use_grad_norm), and the unnormalised d=1 gradient in xyz order.
__device__ __forceinline__ void hier_features(const float* __restrict__ sdf, const GridGeom& g, float vs,
                                              const float ind[3], int K, const float* disp, float feat[6 * MAX_K],
                                              float graw[3 * MAX_K]) {
  for (int kk = 0; kk < K; ++kk) {
#pragma unroll
    for (int pair = 0; pair < 3; ++pair) {
      const int axis = 2 - pair;  // zyx
      Probe pr;
      probe_axis(sdf, g, ind, axis, disp[kk], pr, false);
      feat[(2 * pair + 0) * K + kk] = pr.fm;
      feat[(2 * pair + 1) * K + kk] = pr.fp;
      graw[pair * K + kk] = ((pr.fp - pr.fm) * pr.inv_diff) / vs;
    }
  }
}

// Column layout of the two colour-MLP inputs (voxurf_fine.py:694-739).
struct FeatLayout {
  int K;
  float disp[MAX_K];
  int k_unit;  // index of displacement 1.0 in disp
  int pos_pe, view_pe, kpos_pe, kview_pe;
  int center_sdf, use_rgbnet_k0, k_center_sdf;
  int planes;  // every displacement in (0, 2]: probes from shared planes
};

// Rows of a block staged in shared memory, written by one thread each, then
// copied to global memory one row per warp (coalesced 4-byte words; one
// thread per row writing 2-byte values straight to global memory would touch
// a different cache line per thread and per column).  The staged row stride
// is the global stride plus one 4-byte word: an odd number of words, so the
// 32 threads of a warp writing the same column of 32 rows hit 32 different
// banks.  Requires ld * sizeof(T) % 4 == 0 and a 4-byte aligned destination.
template <typename T>
__host__ __device__ constexpr int64_t stage_ld(int64_t ld) {
  return ld + 4 / (int64_t)sizeof(T);
}

template <typename T>
__device__ __forceinline__ void copy_rows_out(const T* stage, T* dst, int n_rows, int64_t ld) {
  const int words = (int)(ld * (int64_t)sizeof(T) / 4), swords = words + 1;
  const uint32_t* s = reinterpret_cast<const uint32_t*>(stage);
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int r = warp; r < n_rows; r += nw)
    for (int w = lane; w < words; w += 32) d[(int64_t)r * words + w] = s[r * swords + w];
}

// Host side: checks a feature configuration and converts it.
// Host side: the density mask of a march descriptor (none when dens is
// null; a bool mask and a density mask together are an argument error).
inline int fill_density_mask(const float* dens, const vx_grid_geom& g, float shift, float ratio, float thres,
                             bool has_bool_mask, DensityMask& m) {
  m.dens = dens;
  if (!dens) return VX_OK;
  if (has_bool_mask) return VX_ERR_ARG;
  if (g.X < 1 || g.Y < 1 || g.Z < 1 || g.X * g.Y * g.Z > INT32_MAX) return VX_ERR_ARG;
  m.g.X = (int)g.X;
  m.g.Y = (int)g.Y;
  m.g.Z = (int)g.Z;
  for (int a = 0; a < 3; ++a) {
    m.g.mn[a] = g.xyz_min[a];
    m.g.mx[a] = g.xyz_max[a];
  }
  m.shift = shift;
  m.ratio = ratio;
  m.thres = thres;
  return VX_OK;
}

inline int fill_feat_layout(const vx_fine_feature_cfg* c, FeatLayout& L) {
  L.K = (int)c->K;
  if (L.K < 1 || L.K > MAX_K) return VX_ERR_ARG;
  L.k_unit = -1;
  L.planes = 1;
  for (int i = 0; i < L.K; ++i) {
    L.disp[i] = c->disp[i];
    if (c->disp[i] == 1.0f) L.k_unit = i;
    if (!(c->disp[i] > 0.f && c->disp[i] <= 2.f)) L.planes = 0;
  }
  if (L.k_unit < 0) return VX_ERR_ARG;  // k_grad_feat = (1.0,) must be among the displacements
  if (c->k0_channels != 12) return VX_ERR_UNSUPPORTED;
  if (c->posbase_pe < 0 || c->posbase_pe > 16 || c->viewbase_pe < 0 || c->viewbase_pe > 16 ||
      c->k_posbase_pe < 0 || c->k_posbase_pe > 16 || c->k_viewbase_pe < 0 || c->k_viewbase_pe > 16)
    return VX_ERR_ARG;
  L.pos_pe = (int)c->posbase_pe;
  L.view_pe = (int)c->viewbase_pe;
  L.kpos_pe = (int)c->k_posbase_pe;
  L.kview_pe = (int)c->k_viewbase_pe;
  L.center_sdf = c->center_sdf;
  L.use_rgbnet_k0 = c->use_rgbnet_k0;
  L.k_center_sdf = c->k_center_sdf;
  return VX_OK;
}

// Column counts of the rows fine_feature_rows writes.
inline int64_t x1_cols(const vx_fine_feature_cfg* c) {
  return (c->use_rgbnet_k0 ? 12 : 0) + (3 + 6 * c->posbase_pe) + (3 + 6 * c->viewbase_pe) + (c->center_sdf ? 1 : 0) +
         9 * c->K;
}
inline int64_t x2_cols(const vx_fine_feature_cfg* c) {
  return 12 + (3 + 6 * c->k_posbase_pe) + (3 + 6 * c->k_viewbase_pe) + 3 + (c->k_center_sdf ? 1 : 0);
}

// ---- axis probes from shared planes -------------------------------------------
// Every probe of a point along axis a moves only that coordinate, so it is a
// linear interpolation between two planes perpendicular to a, each a
// bilinear interpolation at the point's other two coordinates.  The planes
// i0-2 .. i0+3 cover every probe at |d| <= 2: 6 planes x 4 voxels per axis
// instead of 8 voxels per probe.  Voxels outside the grid are zero
// (grid_sample padding 'zeros'); a probe at floor fl with fraction t reads
// planes fl and fl+1, as its own trilinear lookup would.
// The 2x2 cross-section of the point perpendicular to axis A: the flat
// offsets of its four voxels without the A term, their validity and
// bilinear weights, formed once and reused for every plane p along A (the
// flat index is p * stride(A) + off).
template <int A>
struct CrossSection {
  int off[4];
  bool ok[4];
  float w[4];
  int stride, n;

  __device__ __forceinline__ CrossSection(const GridGeom& g, const int i0[3], const float t[3]) {
    constexpr int B = A == 0 ? 1 : 0, C = A == 2 ? 1 : 2;
    const int strides[3] = {g.Y * g.Z, g.Z, 1};
    stride = strides[A];
    n = gsize(g, A);
#pragma unroll
    for (int db = 0; db < 2; ++db)
#pragma unroll
      for (int dc = 0; dc < 2; ++dc) {
        const int q = 2 * db + dc;
        const int ib = i0[B] + db, ic = i0[C] + dc;
        ok[q] = ib >= 0 && ib < gsize(g, B) && ic >= 0 && ic < gsize(g, C);
        off[q] = ib * strides[B] + ic * strides[C];
        w[q] = (db ? t[B] : 1.f - t[B]) * (dc ? t[C] : 1.f - t[C]);
      }
  }

  // bilinear value on plane p (zero outside the grid)
  __device__ __forceinline__ float plane(const float* __restrict__ sdf, int p) const {
    if (p < 0 || p >= n) return 0.f;
    const float* base = sdf + (int64_t)p * stride;
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (ok[q]) acc += w[q] * __ldg(base + off[q]);
    return acc;
  }
};

// Value at coordinate q along the axis from planes P[0..5] = i0-2 .. i0+3.
__device__ __forceinline__ float plane_lerp(const float P[6], int i0, float q) {
  const float fl = floorf(q);
  const float tq = q - fl;
  const int p = (int)fl - (i0 - 2);  // in [0, 4] for |q - coordinate| <= 2
  float lo = P[0], hi = P[1];
#pragma unroll
  for (int k = 1; k < 5; ++k)
    if (p == k) {
      lo = P[k];
      hi = P[k + 1];
    }
  return (1.f - tq) * lo + tq * hi;
}

// Centre value and the hierarchical probes of hier_features (same outputs:
// feat[6K] dir-major z-,z+,y-,y+,x-,x+; graw[3K] pair-major z,y,x) from
// shared planes; requires every displacement <= 2.
template <int KK>
__device__ __forceinline__ void hier_features_planes(const float* __restrict__ sdf, const GridGeom& g, float vs,
                                                     const float ind[3], const float* disp, float* s,
                                                     float feat[6 * KK], float graw[3 * KK]) {
  int i0[3];
  float t[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float fl = floorf(ind[a]);
    i0[a] = (int)fl;
    t[a] = ind[a] - fl;
  }
  float P[3][6];
  {
    const CrossSection<0> cs(g, i0, t);
#pragma unroll
    for (int p = 0; p < 6; ++p) P[0][p] = cs.plane(sdf, i0[0] - 2 + p);
  }
  {
    const CrossSection<1> cs(g, i0, t);
#pragma unroll
    for (int p = 0; p < 6; ++p) P[1][p] = cs.plane(sdf, i0[1] - 2 + p);
  }
  {
    const CrossSection<2> cs(g, i0, t);
#pragma unroll
    for (int p = 0; p < 6; ++p) P[2][p] = cs.plane(sdf, i0[2] - 2 + p);
  }
  *s = (1.f - t[0]) * P[0][2] + t[0] * P[0][3];
#pragma unroll
  for (int kk = 0; kk < KK; ++kk) {
#pragma unroll
    for (int pair = 0; pair < 3; ++pair) {
      const int axis = 2 - pair;  // zyx
      const float hi = (float)(gsize(g, axis) - 1);
      const float qm = fminf(fmaxf(ind[axis] - disp[kk], 0.f), hi);
      const float qp = fminf(fmaxf(ind[axis] + disp[kk], 0.f), hi);
      const float fm = plane_lerp(P[axis], i0[axis], qm);
      const float fp = plane_lerp(P[axis], i0[axis], qp);
      feat[(2 * pair + 0) * KK + kk] = fm;
      feat[(2 * pair + 1) * KK + kk] = fp;
      graw[pair * KK + kk] = ((fp - fm) * (1.f / (qp - qm))) / vs;
    }
  }
}

// hier_features with the number of displacements known at compile time, so
// the value arrays stay in registers.
template <int KK>
__device__ __forceinline__ void hier_features_k(const float* __restrict__ sdf, const GridGeom& g, float vs,
                                                const float ind[3], const float* disp, float feat[6 * KK],
                                                float graw[3 * KK]) {
#pragma unroll
  for (int kk = 0; kk < KK; ++kk) {
#pragma unroll
    for (int pair = 0; pair < 3; ++pair) {
      const int axis = 2 - pair;  // zyx
      Probe pr;
      probe_axis(sdf, g, ind, axis, disp[kk], pr, false);
      feat[(2 * pair + 0) * KK + kk] = pr.fm;
      feat[(2 * pair + 1) * KK + kk] = pr.fp;
      graw[pair * KK + kk] = ((pr.fp - pr.fm) * pr.inv_diff) / vs;
    }
  }
}

// One shaded point p seen along viewdir v: the rgbnet input row x1
// ([k0], PE(xyz_n), PE(v), [sdf], 6K hierarchical values, 3K normalised
// gradients) and the k_rgbnet input row x2 without its trailing logits
// (k0, PE(xyz_n), PE(v), d=1 gradient, [sdf]); g1 = the d=1 gradient (xyz).
// KK = L.K (instantiated per displacement count).  REUSE: x1 and x2 are
// rows staged in shared memory, so x2's positional encodings are copied
// from x1 when both use the same frequencies.
template <typename T, int KK, bool REUSE = false, bool COMPACT = false>
__device__ __forceinline__ void fine_feature_rows(const float* __restrict__ sdf, const GridGeom& g, float vs,
                                                  const float* __restrict__ k0f,
                                                  const __nv_bfloat16* __restrict__ k0h, const FeatLayout& L,
                                                  const float p[3], const float v[3], T* x1, T* x2, float g1[3]) {
  // Columns are written as soon as their values exist (k0, the encodings,
  // then the SDF features), so few of them are live at once.
  float ind[3];
  to_index(g, p, ind);
  {
    float k0v[12];
    const Corners c = corners_of(g, ind[0], ind[1], ind[2]);
    if (k0h)
      gatherC<12>(k0h, c, k0v);
    else
      gatherC<12>(k0f, c, k0v);
#pragma unroll
    for (int ch = 0; ch < 12; ++ch) put(x2, ch, k0v[ch]);
    if (L.use_rgbnet_k0) {
#pragma unroll
      for (int ch = 0; ch < 12; ++ch) put(x1, ch, k0v[ch]);
    }
  }
  int col = L.use_rgbnet_k0 ? 12 : 0;
  const int pe1 = col;  // the two encodings of x1 start here
  int col2 = 12;
  // COMPACT: x2 holds only its own columns (k0, then the gradient and the
  // tail): its encodings equal x1's and are taken from x1 when the rows are
  // copied out, so x2 column c >= 12 + n_pe lives at c - n_pe
  const int n_pe = (3 + 6 * L.pos_pe) + (3 + 6 * L.view_pe);
  const int shift2 = COMPACT ? n_pe : 0;
  {
    float xyzn[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) xyzn[a] = (p[a] - g.mn[a]) / (g.mx[a] - g.mn[a]);
    col = put_pe(x1, col, xyzn, L.pos_pe);
    col = put_pe(x1, col, v, L.view_pe);
    if (COMPACT) {
      col2 += n_pe;
    } else if (REUSE && L.kpos_pe == L.pos_pe && L.kview_pe == L.view_pe) {
      // same encodings as x1 (rows staged in shared memory): copy, do not recompute
      copy_cols(x1, pe1, x2, col2, n_pe);
      col2 += n_pe;
    } else {
      col2 = put_pe(x2, col2, xyzn, L.kpos_pe);
      col2 = put_pe(x2, col2, v, L.kview_pe);
    }
  }
  float s;
  float feat[6 * KK], graw[3 * KK];
  float disp[KK];
#pragma unroll
  for (int kk = 0; kk < KK; ++kk) disp[kk] = L.disp[kk];
  if (L.planes) {
    hier_features_planes<KK>(sdf, g, vs, ind, disp, &s, feat, graw);
  } else {
    s = sample1(sdf, g, ind[0], ind[1], ind[2]);
    hier_features_k<KK>(sdf, g, vs, ind, disp, feat, graw);
  }
  // gradient for k_rgbnet: unnormalised, displacement 1.0, xyz order
  float gu[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int kk = 0; kk < KK; ++kk)
    if (kk == L.k_unit) {
      gu[0] = graw[2 * KK + kk];
      gu[1] = graw[1 * KK + kk];
      gu[2] = graw[0 * KK + kk];
    }
  g1[0] = gu[0];
  g1[1] = gu[1];
  g1[2] = gu[2];
  if (L.center_sdf) put(x1, col++, s);
#pragma unroll
  for (int q = 0; q < 6 * KK; ++q) put(x1, col + q, feat[q]);
  col += 6 * KK;
#pragma unroll
  for (int kk = 0; kk < KK; ++kk) {
    const float a = graw[0 * KK + kk], b = graw[1 * KK + kk], cc = graw[2 * KK + kk];
    const float nrm = sqrtf(a * a + b * b + cc * cc) + 1e-5f;
    put(x1, col + 0 * KK + kk, a / nrm);
    put(x1, col + 1 * KK + kk, b / nrm);
    put(x1, col + 2 * KK + kk, cc / nrm);
  }
  put(x2, col2++ - shift2, g1[0]);
  put(x2, col2++ - shift2, g1[1]);
  put(x2, col2++ - shift2, g1[2]);
  if (L.k_center_sdf) put(x2, col2++ - shift2, s);
}

// Staged row stride of n elements: an odd number of 4-byte words (bank-
// conflict-free column writes by the 32 threads of a warp).
template <typename T>
__host__ __device__ constexpr int64_t odd_words_ld(int64_t n) {
  return ((n * (int64_t)sizeof(T) / 4) % 2 == 1) ? n : n + 4 / (int64_t)sizeof(T);
}

// Copy-out of compact x2 rows: x2 word w of a row comes from the x2 stage
// (its k0 words and, after the encodings, its tail) or from the x1 stage
// (the encodings, starting at x1 column pe1).  Columns 12, pe1 and n_pe are
// word-aligned (even for BF16).
template <typename T>
__device__ __forceinline__ void copy_rows_out_compact(const T* stage1, int64_t sl1, const T* stage2, int64_t sl2,
                                                      T* dst, int n_rows, int64_t ld2, int pe1, int n_pe) {
  constexpr int EPW = 4 / (int)sizeof(T);  // elements per word
  const int words = (int)(ld2 / EPW), k0w = 12 / EPW, pew = n_pe / EPW, pe1w = pe1 / EPW;
  const int sw1 = (int)(sl1 / EPW), sw2 = (int)(sl2 / EPW);
  const uint32_t* s1 = reinterpret_cast<const uint32_t*>(stage1);
  const uint32_t* s2 = reinterpret_cast<const uint32_t*>(stage2);
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int r = warp; r < n_rows; r += nw)
    for (int w = lane; w < words; w += 32) {
      uint32_t v;
      if (w < k0w)
        v = s2[r * sw2 + w];
      else if (w < k0w + pew)
        v = s1[r * sw1 + pe1w + (w - k0w)];
      else
        v = s2[r * sw2 + (w - pew)];
      d[(int64_t)r * words + w] = v;
    }
}

}  // namespace vx
