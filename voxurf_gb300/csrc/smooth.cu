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
