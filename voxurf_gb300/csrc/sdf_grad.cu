// Dense SDF gradient grid (Voxurf.neus_sdf_gradient, 'interpolate' mode,
// lib/voxurf_fine.py:440-450, lib/voxurf_coarse.py:323-332) and its adjoint;
// the smooth_grad_tv regulariser built on it (voxurf_fine.py:412-421,
// run.py:621-622).
//
//   G[a](i,j,k) = (sdf[i+e_a] - sdf[i-e_a]) / 2 / voxel_size on interior
//                 points of axis a, 0 on the two boundary slabs of that axis.
#include "common.cuh"

namespace vx {

struct Dims {
  int X, Y, Z;
};

__device__ __forceinline__ void ijk_of(const Dims& d, int64_t idx, int& i, int& j, int& k) {
  k = (int)(idx % d.Z);
  j = (int)((idx / d.Z) % d.Y);
  i = (int)(idx / ((int64_t)d.Z * d.Y));
}

__device__ __forceinline__ float cdiff(const float* __restrict__ s, const Dims& d, int i, int j, int k, int a,
                                       float vs) {
  const int n = a == 0 ? d.X : (a == 1 ? d.Y : d.Z);
  const int c = a == 0 ? i : (a == 1 ? j : k);
  if (c < 1 || c > n - 2) return 0.f;
  const int64_t st = a == 0 ? (int64_t)d.Y * d.Z : (a == 1 ? (int64_t)d.Z : 1);
  const int64_t idx = ((int64_t)i * d.Y + j) * d.Z + k;
  return (s[idx + st] - s[idx - st]) / 2.f / vs;
}

// layout 0: [3, X, Y, Z]; layout 1: [X, Y, Z, 4] (4th channel zero)
__global__ void sdf_gradient_kernel(const float* __restrict__ sdf, float* __restrict__ G, Dims d, float vs,
                                    int layout) {
  const int64_t n = (int64_t)d.X * d.Y * d.Z;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += stride) {
    int i, j, k;
    ijk_of(d, idx, i, j, k);
    const float gx = cdiff(sdf, d, i, j, k, 0, vs);
    const float gy = cdiff(sdf, d, i, j, k, 1, vs);
    const float gz = cdiff(sdf, d, i, j, k, 2, vs);
    if (layout == 0) {
      G[idx] = gx;
      G[n + idx] = gy;
      G[2 * n + idx] = gz;
    } else {
      reinterpret_cast<float4*>(G)[idx] = make_float4(gx, gy, gz, 0.f);
    }
  }
}

__device__ __forceinline__ float gval(const float* __restrict__ G, int64_t n, int64_t idx, int a, int layout) {
  return layout == 0 ? G[a * n + idx] : G[4 * idx + a];
}

// d_sdf[m] (+)= sum_a ( dG_a[m - e_a] [m - e_a interior] - dG_a[m + e_a] [m + e_a interior] ) / 2 / vs
__global__ void sdf_gradient_adjoint_kernel(const float* __restrict__ dG, float* __restrict__ d_sdf, Dims d, float vs,
                                            int layout, int accumulate) {
  const int64_t n = (int64_t)d.X * d.Y * d.Z;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += stride) {
    int c[3];
    ijk_of(d, idx, c[0], c[1], c[2]);
    const int len[3] = {d.X, d.Y, d.Z};
    const int64_t st[3] = {(int64_t)d.Y * d.Z, (int64_t)d.Z, 1};
    float acc = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (c[a] - 1 >= 1 && c[a] - 1 <= len[a] - 2) acc += gval(dG, n, idx - st[a], a, layout) / 2.f / vs;
      if (c[a] + 1 >= 1 && c[a] + 1 <= len[a] - 2) acc -= gval(dG, n, idx + st[a], a, layout) / 2.f / vs;
    }
    if (accumulate)
      d_sdf[idx] += acc;
    else
      d_sdf[idx] = acc;
  }
}

// smooth_grad_tv: e = tv_smooth_conv(G) - G on the non-empty voxels, loss
// = weight * mean(e^2) over the 3 channels of the masked voxels
// (voxurf_fine.py:417-420; the smoothed term is detached).  tv_smooth_conv
// is the normalised 3x3x3 kernel [1,2,1]^3/64 with replicate padding
// (voxurf_fine.py:237-242 with sigma 0).  Writes dG = d loss / d G (the
// smoothed term carries no gradient) and block partial sums of e^2.
__global__ void smooth_grad_tv_kernel(const float* __restrict__ G, const uint8_t* __restrict__ mask, Dims d,
                                      float grad_scale, float* __restrict__ dG, double* __restrict__ partial) {
  const int64_t n = (int64_t)d.X * d.Y * d.Z;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double local = 0.0;
  const float w1[3] = {0.25f, 0.5f, 0.25f};
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += stride) {
    int i, j, k;
    ijk_of(d, idx, i, j, k);
    const float4 g = reinterpret_cast<const float4*>(G)[idx];
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!mask || mask[idx]) {
      float sx = 0.f, sy = 0.f, sz = 0.f;
      for (int a = -1; a <= 1; ++a) {
        const int ii = min(max(i + a, 0), d.X - 1);
        for (int b = -1; b <= 1; ++b) {
          const int jj = min(max(j + b, 0), d.Y - 1);
          for (int c = -1; c <= 1; ++c) {
            const int kk = min(max(k + c, 0), d.Z - 1);
            const float w = w1[a + 1] * w1[b + 1] * w1[c + 1];
            const float4 q = reinterpret_cast<const float4*>(G)[((int64_t)ii * d.Y + jj) * d.Z + kk];
            sx += w * q.x;
            sy += w * q.y;
            sz += w * q.z;
          }
        }
      }
      const float ex = sx - g.x, ey = sy - g.y, ez = sz - g.z;
      local += (double)ex * ex + (double)ey * ey + (double)ez * ez;
      // d/dG of mean((S(G).detach() - G)^2) = -2 e / count
      out = make_float4(-grad_scale * ex, -grad_scale * ey, -grad_scale * ez, 0.f);
    }
    reinterpret_cast<float4*>(dG)[idx] = out;
  }
  local = warp_sum(local);
  __shared__ double ws[8];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
    partial[blockIdx.x] = t;
  }
}

static unsigned dense_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 8;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace vx

using namespace vx;

extern "C" {

int vx_sdf_gradient_grid(const float* sdf, float* G, int64_t X, int64_t Y, int64_t Z, float voxel_size, int layout,
                         void* stream) {
  if (!sdf || !G || X <= 0 || Y <= 0 || Z <= 0 || (layout != 0 && layout != 1)) return VX_ERR_ARG;
  if (layout == 1 && (((uintptr_t)G) & 15)) return VX_ERR_ARG;
  Dims d{(int)X, (int)Y, (int)Z};
  sdf_gradient_kernel<<<dense_blocks(X * Y * Z), 256, 0, as_stream(stream)>>>(sdf, G, d, voxel_size, layout);
  return launch_status();
}

int vx_sdf_gradient_grid_adjoint(const float* dG, float* d_sdf, int64_t X, int64_t Y, int64_t Z, float voxel_size,
                                 int layout, int accumulate, void* stream) {
  if (!dG || !d_sdf || X <= 0 || Y <= 0 || Z <= 0 || (layout != 0 && layout != 1)) return VX_ERR_ARG;
  Dims d{(int)X, (int)Y, (int)Z};
  sdf_gradient_adjoint_kernel<<<dense_blocks(X * Y * Z), 256, 0, as_stream(stream)>>>(dG, d_sdf, d, voxel_size,
                                                                                     layout, accumulate);
  return launch_status();
}

size_t vx_smooth_grad_tv_scratch_bytes(int64_t X, int64_t Y, int64_t Z) {
  return (size_t)dense_blocks(X * Y * Z) * sizeof(double);
}

// G: [X,Y,Z,4] gradient grid (layout 1); mask: optional non-empty bytes;
// grad_scale = 2 * weight / count; dG out [X,Y,Z,4]; partial: per-block
// sums of e^2 (scratch, vx_smooth_grad_tv_scratch_bytes).
int vx_smooth_grad_tv(const float* G, const uint8_t* mask, int64_t X, int64_t Y, int64_t Z, float grad_scale,
                      float* dG, double* partial, void* stream) {
  if (!G || !dG || !partial || X <= 0 || Y <= 0 || Z <= 0) return VX_ERR_ARG;
  Dims d{(int)X, (int)Y, (int)Z};
  smooth_grad_tv_kernel<<<dense_blocks(X * Y * Z), 256, 0, as_stream(stream)>>>(G, mask, d, grad_scale, dG,
                                                                              partial);
  return launch_status();
}

}  // extern "C"
