// Loss-form total variation of a dense grid over a voxel mask, the
// `total_variation(v, mask)` of the model files, and its gradient.
//
//   pairs along axis a: (p, p + e_a), both inside the grid and both in the
//   mask (the `mask[..., :-1] & mask[..., 1:]` selections); every channel of
//   the grid uses the voxel mask (`mask.repeat(1, C, 1, 1, 1)`).
//   S_a = sum over the selected pairs and channels of |v[p + e_a] - v[p]|,
//   P_a = C x (number of selected pairs), M = C x (number of mask voxels).
//   mode 0 (lib/voxurf_coarse.py:702-715): (S_0 + S_1 + S_2) / 3 / M
//   mode 1 (lib/voxurf_fine.py:956-969, voxurf_womask_fine.py:1242-1255,
//           voxurf_womask_coarse.py:858-871): (S_0/P_0 + S_1/P_1 + S_2/P_2) / 3
//   loss = weight x that.  d loss / d|diff| of one selected pair along axis
//   a is the same for every pair of the axis (axis_scale[a]); the gradient
//   of |x| is sign(x) with sign(0) = 0, as torch's abs.
//
// Forward: one grid-stride pass, each thread owns voxels and their three
// forward pairs; per-thread FP64 sums, per-block partials in a fixed order,
// then one block sums the partials in a fixed order (deterministic run to
// run).  Backward: one pass, each voxel gathers the signs of its (up to)
// six pairs.  Both are HBM-bound sweeps: the neighbours come from L1/L2.
#include "common.cuh"

namespace vx {
namespace {

constexpr int TV_THREADS = 256;
constexpr int TV_PARTS = 7;  // S_0..2, pairs_0..2, mask voxels

struct TvParams {
  const float* v;
  int C, X, Y, Z;
  int channel_last;
  const uint8_t* mask;
};

__device__ __forceinline__ int64_t tv_el(const TvParams& P, int64_t vox, int c, int64_t V) {
  return P.channel_last ? vox * P.C + c : (int64_t)c * V + vox;
}

__device__ __forceinline__ bool tv_in(const TvParams& P, int64_t vox) { return !P.mask || P.mask[vox] != 0; }

__device__ __forceinline__ float sgnf(float x) { return (float)((x > 0.f) - (x < 0.f)); }

unsigned tv_blocks(int64_t V) {
  int64_t b = (V + TV_THREADS - 1) / TV_THREADS;
  const int64_t cap = (int64_t)sm_count() * 8;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

__global__ void __launch_bounds__(TV_THREADS) tv_loss_kernel(TvParams P, double* __restrict__ partial) {
  const int64_t V = (int64_t)P.X * P.Y * P.Z;
  const int64_t st[3] = {(int64_t)P.Y * P.Z, (int64_t)P.Z, 1};
  double s[3] = {0.0, 0.0, 0.0};
  int64_t np[3] = {0, 0, 0}, nm = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t vox = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; vox < V; vox += stride) {
    if (!tv_in(P, vox)) continue;
    ++nm;
    const int c3[3] = {(int)(vox / st[0]), (int)((vox / st[1]) % P.Y), (int)(vox % P.Z)};
    const int len[3] = {P.X, P.Y, P.Z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (c3[a] + 1 >= len[a]) continue;
      const int64_t nb = vox + st[a];
      if (!tv_in(P, nb)) continue;
      ++np[a];
      float acc = 0.f;
      for (int c = 0; c < P.C; ++c) acc += fabsf(__ldg(P.v + tv_el(P, nb, c, V)) - __ldg(P.v + tv_el(P, vox, c, V)));
      s[a] += (double)acc;
    }
  }
  double q[TV_PARTS] = {s[0], s[1], s[2], (double)np[0], (double)np[1], (double)np[2], (double)nm};
  __shared__ double red[TV_PARTS][TV_THREADS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < TV_PARTS; ++i) {
    const double t = warp_sum(q[i]);
    if (lane == 0) red[i][w] = t;
  }
  __syncthreads();
  if (threadIdx.x < TV_PARTS) {
    double t = 0.0;
    for (int k = 0; k < TV_THREADS / 32; ++k) t += red[threadIdx.x][k];
    partial[(int64_t)blockIdx.x * TV_PARTS + threadIdx.x] = t;
  }
}

__global__ void __launch_bounds__(TV_THREADS) tv_loss_finish_kernel(const double* __restrict__ partial, int n_part,
                                                                    int C, int mode, float weight,
                                                                    float* __restrict__ loss,
                                                                    float* __restrict__ axis_scale) {
  double q[TV_PARTS];
#pragma unroll
  for (int i = 0; i < TV_PARTS; ++i) q[i] = 0.0;
  for (int b = threadIdx.x; b < n_part; b += TV_THREADS)
#pragma unroll
    for (int i = 0; i < TV_PARTS; ++i) q[i] += partial[(int64_t)b * TV_PARTS + i];
  __shared__ double red[TV_PARTS][TV_THREADS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < TV_PARTS; ++i) {
    const double t = warp_sum(q[i]);
    if (lane == 0) red[i][w] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot[TV_PARTS];
    for (int i = 0; i < TV_PARTS; ++i) {
      tot[i] = 0.0;
      for (int k = 0; k < TV_THREADS / 32; ++k) tot[i] += red[i][k];
    }
    const double wgt = (double)weight;
    double l;
    if (mode == 0) {
      // (S_0 + S_1 + S_2) / 3 / M; an empty mask divides by zero as torch does
      const double m = tot[6] * C;
      l = (tot[0] + tot[1] + tot[2]) / 3.0 / m;
      for (int a = 0; a < 3; ++a) axis_scale[a] = (float)(wgt / (3.0 * m));
    } else {
      // the mean of an empty selection is NaN in torch: 0/0 here as well
      l = 0.0;
      for (int a = 0; a < 3; ++a) {
        const double p = tot[3 + a] * C;
        l += tot[a] / p;
        axis_scale[a] = (float)(wgt / (3.0 * p));
      }
      l /= 3.0;
    }
    loss[0] = (float)(wgt * l);
  }
}

// grad (same layout as v) += g * sum over the voxel's selected pairs of
// axis_scale[a] * d|v[q] - v[p]| / dv
__global__ void __launch_bounds__(TV_THREADS) tv_loss_bwd_kernel(TvParams P, const float* __restrict__ axis_scale,
                                                                 const float* __restrict__ g_loss,
                                                                 float* __restrict__ grad) {
  const int64_t V = (int64_t)P.X * P.Y * P.Z;
  const int64_t st[3] = {(int64_t)P.Y * P.Z, (int64_t)P.Z, 1};
  const float g = g_loss[0];
  const float sc[3] = {g * axis_scale[0], g * axis_scale[1], g * axis_scale[2]};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t vox = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; vox < V; vox += stride) {
    if (!tv_in(P, vox)) continue;
    const int c3[3] = {(int)(vox / st[0]), (int)((vox / st[1]) % P.Y), (int)(vox % P.Z)};
    const int len[3] = {P.X, P.Y, P.Z};
    bool lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      lo[a] = c3[a] >= 1 && tv_in(P, vox - st[a]);
      hi[a] = c3[a] + 1 < len[a] && tv_in(P, vox + st[a]);
    }
    for (int c = 0; c < P.C; ++c) {
      const int64_t e = tv_el(P, vox, c, V);
      const float x = __ldg(P.v + e);
      float acc = 0.f;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (lo[a]) acc += sc[a] * sgnf(x - __ldg(P.v + tv_el(P, vox - st[a], c, V)));
        if (hi[a]) acc -= sc[a] * sgnf(__ldg(P.v + tv_el(P, vox + st[a], c, V)) - x);
      }
      grad[e] += acc;
    }
  }
}

int tv_check(const vx_tv_loss_args* a) {
  if (!a || !a->v || a->C <= 0 || a->X <= 0 || a->Y <= 0 || a->Z <= 0) return VX_ERR_ARG;
  if (a->mode != 0 && a->mode != 1) return VX_ERR_ARG;
  if (a->C > 4096 || a->X * a->Y * a->Z > ((int64_t)1 << 40)) return VX_ERR_TOO_LARGE;
  return VX_OK;
}

TvParams tv_params(const vx_tv_loss_args* a) {
  TvParams P{};
  P.v = a->v;
  P.C = (int)a->C;
  P.X = (int)a->X;
  P.Y = (int)a->Y;
  P.Z = (int)a->Z;
  P.channel_last = a->channel_last != 0 && a->C > 1;
  P.mask = a->mask;
  return P;
}

}  // namespace
}  // namespace vx

using namespace vx;

extern "C" {

size_t vx_tv_loss_scratch_bytes(int64_t X, int64_t Y, int64_t Z) {
  return (size_t)tv_blocks(X * Y * Z) * TV_PARTS * sizeof(double);
}

int vx_tv_loss(const vx_tv_loss_args* a, void* stream) {
  const int s = tv_check(a);
  if (s) return s;
  if (!a->loss || !a->axis_scale || !a->scratch) return VX_ERR_ARG;
  const unsigned nb = tv_blocks(a->X * a->Y * a->Z);
  if (a->scratch_bytes < (size_t)nb * TV_PARTS * sizeof(double)) return VX_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  double* part = static_cast<double*>(a->scratch);
  tv_loss_kernel<<<nb, TV_THREADS, 0, st>>>(tv_params(a), part);
  tv_loss_finish_kernel<<<1, TV_THREADS, 0, st>>>(part, (int)nb, (int)a->C, a->mode, a->weight, a->loss,
                                                  a->axis_scale);
  return launch_status();
}

int vx_tv_loss_backward(const vx_tv_loss_args* a, const float* g_loss, float* grad, void* stream) {
  const int s = tv_check(a);
  if (s) return s;
  if (!a->axis_scale || !g_loss || !grad) return VX_ERR_ARG;
  tv_loss_bwd_kernel<<<tv_blocks(a->X * a->Y * a->Z), TV_THREADS, 0, as_stream(stream)>>>(tv_params(a),
                                                                                         a->axis_scale, g_loss, grad);
  return launch_status();
}

}  // extern "C"
