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

// ---- aggregated scatters ----------------------------------------------------
// Probes of one point along one axis a (the finite differences of the SDF
// gradient and the hierarchical features) move only coordinate a: every
// probe's eight corners share the point's two b and two c corners, so their
// contributions are summed per a-plane in registers and each plane leaves
// with one reduction per (b, c) corner.  PlaneAcc covers the planes
// floor(ind_a) - 3 .. floor(ind_a) + 4 (probes up to 3 voxels away); a
// contribution outside that window goes straight to the grid.
constexpr int VX_PLANES = 8;

struct PlaneAcc {
  float v[VX_PLANES];
  int base;  // plane of slot 0
};

__device__ __forceinline__ void plane_acc_init(PlaneAcc& A, float ind_a) {
#pragma unroll
  for (int s = 0; s < VX_PLANES; ++s) A.v[s] = 0.f;
  A.base = (int)floorf(ind_a) - 3;
}

// Adds the contribution d of a trilinear lookup at ind with coordinate a
// replaced by x (the planes floor(x) and floor(x) + 1).
__device__ __forceinline__ void plane_acc_add(PlaneAcc& A, float* __restrict__ grid, const GridGeom& g,
                                              const float ind[3], int a, float x, float d) {
  if (d == 0.f) return;
  const float x0f = floorf(x);
  const int s0 = (int)x0f - A.base;
  if (s0 >= 0 && s0 + 1 < VX_PLANES) {
    const float t = x - x0f;
    // the slot is a run-time index: every slot takes a selected addend (zero
    // for all but two) so the accumulator stays in registers
#pragma unroll
    for (int s = 0; s < VX_PLANES; ++s) {
      const float add = (s == s0) ? d * (1.f - t) : ((s == s0 + 1) ? d * t : 0.f);
      A.v[s] += add;
    }
  } else {
    float p[3] = {ind[0], ind[1], ind[2]};
    p[a] = x;
    scatter1(grid, corners_of(g, p[0], p[1], p[2]), d);
  }
}

// One reduction per in-grid (plane, b, c) corner with a nonzero sum.
__device__ __forceinline__ void plane_acc_flush(const PlaneAcc& A, float* __restrict__ grid, const GridGeom& g,
                                                const float ind[3], int a) {
  const int b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;
  const float fb0 = floorf(ind[b]), fc0 = floorf(ind[c]);
  const int b0 = (int)fb0, c0 = (int)fc0;
  const float tb = ind[b] - fb0, tc = ind[c] - fc0;
  const float wb[2] = {1.f - tb, tb}, wc[2] = {1.f - tc, tc};
  const int na = gsize(g, a), nb = gsize(g, b), nc = gsize(g, c);
  const int64_t sa = a == 0 ? (int64_t)g.Y * g.Z : (a == 1 ? g.Z : 1);
  const int64_t sb = b == 0 ? (int64_t)g.Y * g.Z : (b == 1 ? g.Z : 1);
  const int64_t sc = c == 0 ? (int64_t)g.Y * g.Z : (c == 1 ? g.Z : 1);
#pragma unroll
  for (int s = 0; s < VX_PLANES; ++s) {
    const int pa = A.base + s;
    if (A.v[s] == 0.f || pa < 0 || pa >= na) continue;
#pragma unroll
    for (int db = 0; db < 2; ++db)
#pragma unroll
      for (int dc = 0; dc < 2; ++dc) {
        const int jb = b0 + db, jc = c0 + dc;
        const float w = wb[db] * wc[dc];
        if (jb < 0 || jb >= nb || jc < 0 || jc >= nc || w == 0.f) continue;
        atomicAdd(grid + pa * sa + jb * sb + jc * sc, A.v[s] * w);
      }
  }
}

// Channel-last 12-channel scatter of one trilinear lookup per lane (at
// continuous index fi, fj, fk), reduced over the lanes of a warp first: the
// rows of a warp are consecutive shaded samples (ray-major, 0.5 voxel
// apart), so runs of lanes share a corner voxel.  For each corner q the runs
// of equal voxel offsets are summed by a segmented reduction (five shuffle
// steps) and the run's first lane issues the three red.global.add.v4 of the
// sum.  All 32 lanes must call it; a lane without a lookup passes live =
// false.  Corner weights and offsets are those of corners_of.
__device__ __forceinline__ void scatter12_warp(float* __restrict__ grid, const GridGeom& g, float fi, float fj,
                                               float fk, const float d[12], bool live) {
  const unsigned full = 0xffffffffu;
  const int lane = lane_id();
  const float fi0 = floorf(fi), fj0 = floorf(fj), fk0 = floorf(fk);
  const int i0 = (int)fi0, j0 = (int)fj0, k0 = (int)fk0;
  const float ti = fi - fi0, tj = fj - fj0, tk = fk - fk0;
#pragma unroll 1
  for (int q = 0; q < 8; ++q) {
    const int di = q >> 2, dj = (q >> 1) & 1, dk = q & 1;
    const int ii = i0 + di, jj = j0 + dj, kk = k0 + dk;
    const bool in = (ii >= 0) & (ii < g.X) & (jj >= 0) & (jj < g.Y) & (kk >= 0) & (kk < g.Z);
    const float w = (di ? ti : 1.f - ti) * (dj ? tj : 1.f - tj) * (dk ? tk : 1.f - tk);
    const int key = (live && in && w != 0.f) ? (ii * g.Y + jj) * g.Z + kk : -1;
    if (__all_sync(full, key < 0)) continue;
    const int nxt = __shfl_down_sync(full, key, 1);
    const int prv = __shfl_up_sync(full, key, 1);
    const unsigned tails = __ballot_sync(full, lane == 31 || nxt != key);
    const int seg_end = lane + __ffs(tails >> lane) - 1;
    const float wq = key >= 0 ? w : 0.f;
    float v[12];
#pragma unroll
    for (int ch = 0; ch < 12; ++ch) v[ch] = wq * d[ch];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const bool take = lane + o <= seg_end;
#pragma unroll
      for (int ch = 0; ch < 12; ++ch) {
        const float t = __shfl_down_sync(full, v[ch], o);
        if (take) v[ch] += t;
      }
    }
    if ((lane == 0 || prv != key) && key >= 0) {
      float* p = grid + (int64_t)key * 12;
#pragma unroll
      for (int u = 0; u < 3; ++u) red_add_v4(p + 4 * u, v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
    }
  }
}

}  // namespace vx
