// Gaussian smoothing of the SDF grid and its adjoint.
//
// Replaces nn.Conv3d(1,1,k,padding=k//2,padding_mode='replicate') with the
// normalised Gaussian of Voxurf._gaussian_3dconv (lib/voxurf_fine.py:246-258,
// applied every step at voxurf_fine.py:638; voxurf_coarse.py:180-198, 531).
// exp(-(x^2+y^2+z^2)/(2 s^2)) / sum factorises exactly into three normalised
// 1-D kernels, so the 125-tap convolution becomes three 5-tap passes with
// clamped (replicate) indices.  The backward is the exact adjoint of each
// clamped pass, applied in reverse order.
#include "common.cuh"

namespace vx {

struct Taps {
  float w[9];
  int h;  // half width, ksize = 2h+1 (<= 9)
};

// One separable pass along `axis` (0: X, stride Y*Z; 1: Y, stride Z; 2: Z).
template <bool ADJOINT, bool ACCUM>
__global__ void smooth_axis_kernel(const float* __restrict__ in, float* __restrict__ out, int X, int Y, int Z,
                                   int axis, Taps t) {
  const int64_t n = (int64_t)X * Y * Z;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t astride = axis == 0 ? (int64_t)Y * Z : (axis == 1 ? (int64_t)Z : 1);
  const int len = axis == 0 ? X : (axis == 1 ? Y : Z);
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += stride) {
    const int pos = (int)((idx / astride) % len);
    const float* base = in + (idx - (int64_t)pos * astride);
    float acc = 0.f;
    if (!ADJOINT) {
      // out[i] = sum_t w_t * in[clamp(i+t)]
      for (int tt = -t.h; tt <= t.h; ++tt) {
        int q = pos + tt;
        q = q < 0 ? 0 : (q > len - 1 ? len - 1 : q);
        acc += t.w[tt + t.h] * base[(int64_t)q * astride];
      }
    } else {
      // out[j] = sum_i sum_t w_t * g[i] * [clamp(i+t) == j]
      if (len == 1) {
        float s = 0.f;
        for (int tt = -t.h; tt <= t.h; ++tt) s += t.w[tt + t.h];
        acc = s * base[0];
      } else if (pos == 0) {
        for (int i = 0; i <= t.h && i < len; ++i) {
          float s = 0.f;
          for (int tt = -t.h; tt <= -i; ++tt) s += t.w[tt + t.h];
          acc += s * base[(int64_t)i * astride];
        }
      } else if (pos == len - 1) {
        for (int i = (len - 1 - t.h > 0 ? len - 1 - t.h : 0); i < len; ++i) {
          float s = 0.f;
          for (int tt = len - 1 - i; tt <= t.h; ++tt) s += t.w[tt + t.h];
          acc += s * base[(int64_t)i * astride];
        }
      } else {
        for (int tt = -t.h; tt <= t.h; ++tt) {
          const int i = pos - tt;
          if (i >= 0 && i < len) acc += t.w[tt + t.h] * base[(int64_t)i * astride];
        }
      }
    }
    if (ACCUM)
      out[idx] += acc;
    else
      out[idx] = acc;
  }
}

// ---- single-pass tiled version ----------------------------------------------
// One CTA computes an 8 x 8 x 16 output tile: it stages the input tile plus a
// 2-voxel halo (12 x 12 x 20) in shared memory and applies the three 1-D
// passes there (z, then y, then x), so each voxel is read from DRAM about
// once and written once.  Forward: the halo is read at clamped coordinates
// (replicate padding).  Adjoint: the halo outside the grid is zero and each
// axis applies the adjoint of the clamped 1-D convolution (boundary voxels
// collect the taps that the forward clamped onto them).
constexpr int TX = 8, TY = 8, TZ = 16, HALO = 2;
constexpr int SX = TX + 2 * HALO, SY = TY + 2 * HALO, SZ = TZ + 2 * HALO;

// Adjoint of one clamped 1-D convolution at output position j of an axis of
// length n, reading the gradient through get(i) for i in [j-h, j+h] (zero
// outside [0, n)).
template <typename Get>
__device__ __forceinline__ float adjoint1d(const Taps& t, int j, int n, Get get) {
  float acc = 0.f;
  if (n == 1) {
    float s = 0.f;
    for (int tt = -t.h; tt <= t.h; ++tt) s += t.w[tt + t.h];
    return s * get(0);
  }
  if (j == 0) {
    for (int i = 0; i <= t.h && i < n; ++i) {
      float s = 0.f;
      for (int tt = -t.h; tt <= -i; ++tt) s += t.w[tt + t.h];
      acc += s * get(i);
    }
  } else if (j == n - 1) {
    for (int i = (n - 1 - t.h > 0 ? n - 1 - t.h : 0); i < n; ++i) {
      float s = 0.f;
      for (int tt = n - 1 - i; tt <= t.h; ++tt) s += t.w[tt + t.h];
      acc += s * get(i);
    }
  } else {
    for (int tt = -t.h; tt <= t.h; ++tt) {
      const int i = j - tt;
      if (i >= 0 && i < n) acc += t.w[tt + t.h] * get(i);
    }
  }
  return acc;
}

// 1-D pass at global position j of an axis of length n, reading the staged
// values through get(k) for k in [j-H, j+H] (staged coordinates are
// clamped for the forward, zero outside the grid for the adjoint).  The
// adjoint is the transposed convolution (flipped taps) except at the two
// boundary positions, which also collect the taps the forward clamped.
template <bool ADJOINT, int H, typename Get>
__device__ __forceinline__ float pass1d(const Taps& t, const float w[2 * H + 1], int j, int n, Get get) {
  float acc = 0.f;
  if (ADJOINT) {
    if (j == 0 || j == n - 1) return adjoint1d(t, j, n, get);
#pragma unroll
    for (int tt = H; tt >= -H; --tt) acc += w[H - tt] * get(j + tt);  // the order of adjoint1d
  } else {
#pragma unroll
    for (int tt = -H; tt <= H; ++tt) acc += w[tt + H] * get(j + tt);
  }
  return acc;
}

template <bool ADJOINT, bool ACCUM, int H>
__global__ void __launch_bounds__(256) smooth_tile_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                         int X, int Y, int Z, Taps t) {
  __shared__ float s_in[SX][SY][SZ];
  __shared__ float s_z[SX][SY][TZ];
  __shared__ float s_y[SX][TY][TZ];
  float w[2 * H + 1];
#pragma unroll
  for (int i = 0; i < 2 * H + 1; ++i) w[i] = t.w[i];
  const int x0 = blockIdx.z * TX, y0 = blockIdx.y * TY, z0 = blockIdx.x * TZ;
  const int tid = threadIdx.x;
  for (int e = tid; e < SX * SY * SZ; e += blockDim.x) {
    const int c = e % SZ, b = (e / SZ) % SY, a = e / (SZ * SY);
    int gx = x0 + a - HALO, gy = y0 + b - HALO, gz = z0 + c - HALO;
    float v;
    if (!ADJOINT) {
      gx = min(max(gx, 0), X - 1);
      gy = min(max(gy, 0), Y - 1);
      gz = min(max(gz, 0), Z - 1);
      v = in[((int64_t)gx * Y + gy) * Z + gz];
    } else {
      const bool inside = gx >= 0 && gx < X && gy >= 0 && gy < Y && gz >= 0 && gz < Z;
      v = inside ? in[((int64_t)gx * Y + gy) * Z + gz] : 0.f;
    }
    s_in[a][b][c] = v;
  }
  __syncthreads();
  // z pass over all (a, b) of the halo'd tile
  for (int e = tid; e < SX * SY * TZ; e += blockDim.x) {
    const int c = e % TZ, b = (e / TZ) % SY, a = e / (TZ * SY);
    s_z[a][b][c] = pass1d<ADJOINT, H>(t, w, z0 + c, Z, [&](int i) { return s_in[a][b][i - z0 + HALO]; });
  }
  __syncthreads();
  for (int e = tid; e < SX * TY * TZ; e += blockDim.x) {
    const int c = e % TZ, b = (e / TZ) % TY, a = e / (TZ * TY);
    s_y[a][b][c] = pass1d<ADJOINT, H>(t, w, y0 + b, Y, [&](int i) { return s_z[a][i - y0 + HALO][c]; });
  }
  __syncthreads();
  for (int e = tid; e < TX * TY * TZ; e += blockDim.x) {
    const int c = e % TZ, b = (e / TZ) % TY, a = e / (TZ * TY);
    const int gx = x0 + a, gy = y0 + b, gz = z0 + c;
    if (gx >= X || gy >= Y || gz >= Z) continue;
    const float acc = pass1d<ADJOINT, H>(t, w, gx, X, [&](int i) { return s_y[i - x0 + HALO][b][c]; });
    const int64_t o = ((int64_t)gx * Y + gy) * Z + gz;
    if (ACCUM)
      out[o] += acc;
    else
      out[o] = acc;
  }
}

template <bool ADJOINT, bool ACCUM>
static void launch_tile(const float* in, float* out, int X, int Y, int Z, const Taps& t, cudaStream_t st) {
  dim3 grid((unsigned)((Z + TZ - 1) / TZ), (unsigned)((Y + TY - 1) / TY), (unsigned)((X + TX - 1) / TX));
  if (t.h == 2)
    smooth_tile_kernel<ADJOINT, ACCUM, 2><<<grid, 256, 0, st>>>(in, out, X, Y, Z, t);
  else if (t.h == 1)
    smooth_tile_kernel<ADJOINT, ACCUM, 1><<<grid, 256, 0, st>>>(in, out, X, Y, Z, t);
  else
    smooth_tile_kernel<ADJOINT, ACCUM, 0><<<grid, 256, 0, st>>>(in, out, X, Y, Z, t);
}

static unsigned pass_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 16;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace vx

using namespace vx;

extern "C" {

int vx_smooth3d(const float* in, float* out, float* tmp1, float* tmp2, int64_t X, int64_t Y, int64_t Z,
                const float* taps_host, int ksize, void* stream) {
  if (X <= 0 || Y <= 0 || Z <= 0 || ksize < 1 || ksize > 9 || (ksize % 2) == 0) return VX_ERR_ARG;
  if (!in || !out || !tmp1 || !tmp2 || !taps_host) return VX_ERR_ARG;
  if (X * Y * Z > INT32_MAX) return VX_ERR_ARG;
  Taps t;
  t.h = ksize / 2;
  for (int i = 0; i < 9; ++i) t.w[i] = i < ksize ? taps_host[i] : 0.f;
  cudaStream_t st = as_stream(stream);
  if (t.h <= HALO) {
    launch_tile<false, false>(in, out, (int)X, (int)Y, (int)Z, t, st);
    return launch_status();
  }
  const unsigned b = pass_blocks(X * Y * Z);
  smooth_axis_kernel<false, false><<<b, 256, 0, st>>>(in, tmp1, (int)X, (int)Y, (int)Z, 0, t);
  int s = launch_status();
  if (s) return s;
  smooth_axis_kernel<false, false><<<b, 256, 0, st>>>(tmp1, tmp2, (int)X, (int)Y, (int)Z, 1, t);
  s = launch_status();
  if (s) return s;
  smooth_axis_kernel<false, false><<<b, 256, 0, st>>>(tmp2, out, (int)X, (int)Y, (int)Z, 2, t);
  return launch_status();
}

int vx_smooth3d_adjoint(const float* grad_out, float* grad_in, float* tmp1, float* tmp2, int64_t X, int64_t Y,
                        int64_t Z, const float* taps_host, int ksize, int accumulate, void* stream) {
  if (X <= 0 || Y <= 0 || Z <= 0 || ksize < 1 || ksize > 9 || (ksize % 2) == 0) return VX_ERR_ARG;
  if (!grad_out || !grad_in || !tmp1 || !tmp2 || !taps_host) return VX_ERR_ARG;
  if (X * Y * Z > INT32_MAX) return VX_ERR_ARG;
  Taps t;
  t.h = ksize / 2;
  for (int i = 0; i < 9; ++i) t.w[i] = i < ksize ? taps_host[i] : 0.f;
  cudaStream_t st = as_stream(stream);
  if (t.h <= HALO) {
    if (accumulate)
      launch_tile<true, true>(grad_out, grad_in, (int)X, (int)Y, (int)Z, t, st);
    else
      launch_tile<true, false>(grad_out, grad_in, (int)X, (int)Y, (int)Z, t, st);
    return launch_status();
  }
  const unsigned b = pass_blocks(X * Y * Z);
  smooth_axis_kernel<true, false><<<b, 256, 0, st>>>(grad_out, tmp1, (int)X, (int)Y, (int)Z, 2, t);
  int s = launch_status();
  if (s) return s;
  smooth_axis_kernel<true, false><<<b, 256, 0, st>>>(tmp1, tmp2, (int)X, (int)Y, (int)Z, 1, t);
  s = launch_status();
  if (s) return s;
  if (accumulate)
    smooth_axis_kernel<true, true><<<b, 256, 0, st>>>(tmp2, grad_in, (int)X, (int)Y, (int)Z, 0, t);
  else
    smooth_axis_kernel<true, false><<<b, 256, 0, st>>>(tmp2, grad_in, (int)X, (int)Y, (int)Z, 0, t);
  return launch_status();
}

}  // extern "C"
