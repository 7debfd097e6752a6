// Dense SDF field query for mesh extraction.
//
// extract_fields (lib/dvgo_ori.py:679-693, called by Voxurf.extract_geometry,
// voxurf_fine.py:894-910 / voxurf_coarse.py:652-665) samples
// query_func = grid_sampler(pts, -sdf_grid) on the R^3 lattice
// torch.linspace(bound_min[a], bound_max[a], R) per axis (meshgrid 'ij'),
// in 64^3 chunks with a host copy per chunk.  Here one launch writes the
// whole [R, R, R] field on the device: a thread per lattice point, the
// lattice coordinate formed as torch.linspace forms it (start + step * i for
// the first half, end - step * (R - 1 - i) for the second), then the
// trilinear lookup (align_corners, zero padding) scaled by `sign`.
// Bound: HBM writes, 4 bytes per lattice point (the SDF grid is L2-resident
// at 256^3).  Marching cubes itself stays on the host.
#include <algorithm>

#include "common.cuh"
#include "fine_device.cuh"
#include "trilinear.cuh"

namespace vx {

// ---- MaskCache queries -------------------------------------------------------
__global__ void __launch_bounds__(256) density_mask_kernel(DensityMask m, const float* __restrict__ xyz, int64_t n,
                                                           uint8_t* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float p[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    out[i] = density_mask_hit(m, p) ? 1 : 0;
  }
}

struct HitParams {
  const float* rays_o;
  const float* rays_d;
  int n_rays;
  float near, stepdist;
  float bmin[3], bmax[3];
  const uint8_t* mask;
  int mX, mY, mZ;
  float mscale[3], mshift[3];
  DensityMask dm;
  uint8_t* hit;
};

// One warp per ray, 32 samples per step, stop at the first sample in the mask.
__global__ void __launch_bounds__(256) hit_coarse_geo_kernel(HitParams P) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= P.n_rays) return;
  const int lane = lane_id();
  float o[3], d[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = __ldg(P.rays_o + 3 * r + a);
    d[a] = __ldg(P.rays_d + 3 * r + a);
  }
  const RayFrame f = ray_frame(o, d, P.bmin, P.bmax, P.near, P.stepdist);
  bool any = false;
  for (int64_t base = 0; base < f.n_steps && !any; base += 32) {
    const int64_t k = base + lane;
    bool h = false;
    if (k < f.n_steps) {
      float p[3];
      sample_point(f, P.stepdist, (int)k, p);
      h = !outside_bbox(p, P.bmin, P.bmax);
      if (h) h = P.mask ? mask_lookup(P.mask, P.mX, P.mY, P.mZ, P.mscale, P.mshift, p) : density_mask_hit(P.dm, p);
    }
    any = __any_sync(0xffffffffu, h);
  }
  if (lane == 0) P.hit[r] = any ? 1 : 0;
}

// ---- dense field ---------------------------------------------------------------
struct FieldAxis {
  float start, end, step;
  int half;  // first index computed from the end
};

__device__ __forceinline__ float lattice(const FieldAxis& a, int i, int R) {
  return i < a.half ? fadd(a.start, fmul(a.step, (float)i)) : fsub(a.end, fmul(a.step, (float)(R - 1 - i)));
}

// One warp per lattice row (i, j): the x/y part of the trilinear lookup
// (floors, weights, the four row offsets and their bounds) is formed once
// per row, the lanes walk z (consecutive lattice points, coalesced stores).
// Corner order and weight products are those of corners_of / gather1, so a
// point's value is bit-identical to sample1 at the same index.
__global__ void __launch_bounds__(256) sdf_field_kernel(const float* __restrict__ sdf, GridGeom g, FieldAxis ax,
                                                        FieldAxis ay, FieldAxis az, int R, float sign,
                                                        float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t rows = (int64_t)R * R;
  const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < rows; row += wstride) {
    const int i = (int)(row / R), j = (int)(row - (int64_t)i * R);
    const float fi = world_to_index(g, 0, lattice(ax, i, R));
    const float fj = world_to_index(g, 1, lattice(ay, j, R));
    const float fi0 = floorf(fi), fj0 = floorf(fj);
    const int i0 = (int)fi0, j0 = (int)fj0;
    const float ti = fi - fi0, tj = fj - fj0;
    const float wi[2] = {1.f - ti, ti}, wj[2] = {1.f - tj, tj};
    int64_t rbase[2][2];
    bool rin[2][2];
#pragma unroll
    for (int di = 0; di < 2; ++di)
#pragma unroll
      for (int dj = 0; dj < 2; ++dj) {
        const int ii = i0 + di, jj = j0 + dj;
        rin[di][dj] = (ii >= 0) & (ii < g.X) & (jj >= 0) & (jj < g.Y);
        rbase[di][dj] = ((int64_t)ii * g.Y + jj) * g.Z;
      }
    float* orow = out + row * R;
    for (int k = lane; k < R; k += 32) {
      const float fk = world_to_index(g, 2, lattice(az, k, R));
      const float fk0 = floorf(fk);
      const int k0 = (int)fk0;
      const float tk = fk - fk0;
      const float wk[2] = {1.f - tk, tk};
      float acc = 0.f;
#pragma unroll
      for (int di = 0; di < 2; ++di)
#pragma unroll
        for (int dj = 0; dj < 2; ++dj)
#pragma unroll
          for (int dk = 0; dk < 2; ++dk) {
            const int kk = k0 + dk;
            if (rin[di][dj] && kk >= 0 && kk < g.Z)
              acc += (wi[di] * wj[dj] * wk[dk]) * __ldg(sdf + rbase[di][dj] + kk);
          }
      orow[k] = sign * acc;
    }
  }
}

static FieldAxis field_axis(float start, float end, int64_t R) {
  FieldAxis a;
  a.start = start;
  a.end = end;
  a.step = R > 1 ? (end - start) / (float)(R - 1) : 0.f;
  a.half = (int)(R / 2);
  return a;
}

}  // namespace vx

using namespace vx;

extern "C" {

int vx_sdf_field(const float* sdf, const vx_grid_geom* grid, const float* bound_min, const float* bound_max,
                 int64_t R, float sign, float* out, void* stream) {
  if (!sdf || !grid || !bound_min || !bound_max || !out) return VX_ERR_ARG;
  if (R < 1 || R > 2048) return VX_ERR_ARG;
  if (grid->X < 1 || grid->Y < 1 || grid->Z < 1) return VX_ERR_ARG;
  if ((int64_t)grid->X * grid->Y * grid->Z > INT32_MAX) return VX_ERR_ARG;
  GridGeom g;
  g.X = (int)grid->X;
  g.Y = (int)grid->Y;
  g.Z = (int)grid->Z;
  for (int a = 0; a < 3; ++a) {
    g.mn[a] = grid->xyz_min[a];
    g.mx[a] = grid->xyz_max[a];
  }
  const FieldAxis ax = field_axis(bound_min[0], bound_max[0], R), ay = field_axis(bound_min[1], bound_max[1], R),
                  az = field_axis(bound_min[2], bound_max[2], R);
  const int64_t rows = R * R;  // one warp per row, 8 warps per block
  const int64_t cap = (int64_t)sm_count() * 64;
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((rows + 7) / 8, cap));
  sdf_field_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(sdf, g, ax, ay, az, (int)R, sign, out);
  return launch_status();
}

int vx_density_mask(const float* density, const vx_grid_geom* dgrid, float act_shift, float voxel_size_ratio,
                    float thres, const float* xyz, int64_t n, uint8_t* out, void* stream) {
  if (n < 0 || !dgrid) return VX_ERR_ARG;
  if (n == 0) return VX_OK;
  if (!density || !xyz || !out) return VX_ERR_ARG;
  DensityMask m;
  const int s = fill_density_mask(density, *dgrid, act_shift, voxel_size_ratio, thres, false, m);
  if (s) return s;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 32);
  density_mask_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(m, xyz, n, out);
  return launch_status();
}

int vx_hit_coarse_geo(const vx_fine_march_args* A, uint8_t* hit, void* stream) {
  if (!A || A->n_rays < 0 || A->n_rays > INT32_MAX) return VX_ERR_ARG;
  if (A->n_rays == 0) return VX_OK;
  if (!A->rays_o || !A->rays_d || !hit || !(A->stepdist > 0.f)) return VX_ERR_ARG;
  if (!A->mask && !A->mask_density) return VX_ERR_ARG;
  HitParams P{};
  P.rays_o = A->rays_o;
  P.rays_d = A->rays_d;
  P.n_rays = (int)A->n_rays;
  P.near = A->near;
  P.stepdist = A->stepdist;
  for (int a = 0; a < 3; ++a) {
    P.bmin[a] = A->grid.xyz_min[a];
    P.bmax[a] = A->grid.xyz_max[a];
    P.mscale[a] = A->mask_scale[a];
    P.mshift[a] = A->mask_shift[a];
  }
  P.mask = A->mask;
  P.mX = (int)A->mask_X;
  P.mY = (int)A->mask_Y;
  P.mZ = (int)A->mask_Z;
  const int s = fill_density_mask(A->mask_density, A->mask_dgrid, A->mask_act_shift, A->mask_voxel_size_ratio,
                                  A->mask_thres, A->mask != nullptr, P.dm);
  if (s) return s;
  P.hit = hit;
  const int64_t blocks = (A->n_rays + 7) / 8;
  hit_coarse_geo_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(P);
  return launch_status();
}

}  // extern "C"
