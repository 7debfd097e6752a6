// Trilinear sampling of dense grids with F.grid_sample(align_corners=True,
// padding_mode='zeros') semantics, its adjoint (scatter), and the
// world -> continuous-index mapping of DenseGrid.forward / sample_sdfs
// (lib/grid.py:52-54, lib/voxurf_fine.py:544-547):
//     ind_norm = ((xyz - min) / (max - min)) * 2 - 1
//     index    = ((ind_norm + 1) / 2) * (size - 1)
// World axis a indexes grid dimension a (the flip(-1) and grid_sample's
// x->W, y->H, z->D ordering cancel).
#pragma once
#include "common.cuh"

namespace vx {

struct GridGeom {
  int X, Y, Z;
  float mn[3], mx[3];
};

__device__ __forceinline__ int gsize(const GridGeom& g, int a) { return a == 0 ? g.X : (a == 1 ? g.Y : g.Z); }

__device__ __forceinline__ float world_to_index(const GridGeom& g, int a, float x) {
  const float t = (x - g.mn[a]) / (g.mx[a] - g.mn[a]);
  const float u = t * 2.f - 1.f;
  return ((u + 1.f) * 0.5f) * (float)(gsize(g, a) - 1);
}

// Corner set of one trilinear lookup.  w[c] for corner c = (di<<2)|(dj<<1)|dk;
// off[c] is the flat voxel offset or -1 when the corner is outside the grid
// (zero padding).
struct Corners {
  float w[8];
  int off[8];
};

__device__ __forceinline__ Corners corners_of(const GridGeom& g, float fi, float fj, float fk) {
  Corners c;
  const float fi0 = floorf(fi), fj0 = floorf(fj), fk0 = floorf(fk);
  const int i0 = (int)fi0, j0 = (int)fj0, k0 = (int)fk0;
  const float ti = fi - fi0, tj = fj - fj0, tk = fk - fk0;
  const float wi[2] = {1.f - ti, ti}, wj[2] = {1.f - tj, tj}, wk[2] = {1.f - tk, tk};
#pragma unroll
  for (int di = 0; di < 2; ++di)
#pragma unroll
    for (int dj = 0; dj < 2; ++dj)
#pragma unroll
      for (int dk = 0; dk < 2; ++dk) {
        const int cidx = (di << 2) | (dj << 1) | dk;
        const int ii = i0 + di, jj = j0 + dj, kk = k0 + dk;
        const bool in = (ii >= 0) & (ii < g.X) & (jj >= 0) & (jj < g.Y) & (kk >= 0) & (kk < g.Z);
        c.w[cidx] = wi[di] * wj[dj] * wk[dk];
        c.off[cidx] = in ? ((ii * g.Y + jj) * g.Z + kk) : -1;
      }
  return c;
}

__device__ __forceinline__ float gather1(const float* __restrict__ grid, const Corners& c) {
  float acc = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q)
    if (c.off[q] >= 0) acc += c.w[q] * __ldg(grid + c.off[q]);
  return acc;
}

__device__ __forceinline__ float sample1(const float* __restrict__ grid, const GridGeom& g, float fi, float fj,
                                         float fk) {
  return gather1(grid, corners_of(g, fi, fj, fk));
}

// Adjoint: grid[corner] += w * d  (red.global.add.f32).
__device__ __forceinline__ void scatter1(float* __restrict__ grid, const Corners& c, float d) {
  if (d == 0.f) return;
#pragma unroll
  for (int q = 0; q < 8; ++q)
    if (c.off[q] >= 0 && c.w[q] != 0.f) atomicAdd(grid + c.off[q], c.w[q] * d);
}

// Channel-last C-channel gather (float or bf16 storage), accumulating in FP32.
template <int C>
__device__ __forceinline__ void gatherC(const float* __restrict__ grid, const Corners& c, float out[C]) {
#pragma unroll
  for (int ch = 0; ch < C; ++ch) out[ch] = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (c.off[q] < 0) continue;
    const float4* p = reinterpret_cast<const float4*>(grid + (int64_t)c.off[q] * C);
#pragma unroll
    for (int v = 0; v < C / 4; ++v) {
      const float4 x = __ldg(p + v);
      out[4 * v + 0] += c.w[q] * x.x;
      out[4 * v + 1] += c.w[q] * x.y;
      out[4 * v + 2] += c.w[q] * x.z;
      out[4 * v + 3] += c.w[q] * x.w;
    }
  }
}

template <int C>
__device__ __forceinline__ void gatherC(const __nv_bfloat16* __restrict__ grid, const Corners& c, float out[C]) {
#pragma unroll
  for (int ch = 0; ch < C; ++ch) out[ch] = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (c.off[q] < 0) continue;
    const uint2* p = reinterpret_cast<const uint2*>(grid + (int64_t)c.off[q] * C);
#pragma unroll
    for (int v = 0; v < C / 4; ++v) {
      const uint2 x = __ldg(p + v);
      const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&x.x));
      const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&x.y));
      out[4 * v + 0] += c.w[q] * a.x;
      out[4 * v + 1] += c.w[q] * a.y;
      out[4 * v + 2] += c.w[q] * b.x;
      out[4 * v + 3] += c.w[q] * b.y;
    }
  }
}

// Vector reduction into 4 consecutive floats (sm_90+: red.global.add.v4.f32).
__device__ __forceinline__ void red_add_v4(float* addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}

template <int C>
__device__ __forceinline__ void scatterC(float* __restrict__ grid, const Corners& c, const float d[C]) {
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (c.off[q] < 0 || c.w[q] == 0.f) continue;
    float* p = grid + (int64_t)c.off[q] * C;
    const float w = c.w[q];
#pragma unroll
    for (int v = 0; v < C / 4; ++v)
      red_add_v4(p + 4 * v, w * d[4 * v + 0], w * d[4 * v + 1], w * d[4 * v + 2], w * d[4 * v + 3]);
  }
}

// Marks the voxels scatterC adds to (every writer stores the same byte, so
// plain stores suffice).
__device__ __forceinline__ void mark_corners(uint8_t* __restrict__ touched, const Corners& c) {
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (c.off[q] < 0 || c.w[q] == 0.f) continue;
    touched[c.off[q]] = 1;
  }
}

}  // namespace vx
