// Ray-bbox clip, sample counts, point sampling and the mask-grid lookup.
//
// Drop-in for the `render_utils_cuda` ops infer_t_minmax, infer_n_samples,
// infer_ray_start_dir, sample_pts_on_rays and maskcache_lookup
// (render_utils.cpp:171-177; kernels at render_utils_kernel.cu:12-242 and
// 374-424).  Differences by design:
//   * sample_pts_on_rays is split into a count phase (clip + counts + device
//     scan, no host sync) and a fill phase (one warp per ray writes its
//     samples, coalesced), replacing six launches, two cumsums and the host
//     `.item()` of render_utils_kernel.cu:212;
//   * every float operation that feeds an index or a bbox/mask decision is
//     rounded once, except the multiply-adds that the reference's compiled
//     kernels fuse (ray norm, ray start, sample point, mask index), which
//     are one __fmaf_rn here too: the outputs equal the reference kernels'
//     and the CPU oracle's bit for bit.
#include <math.h>
#include <mutex>
#include "common.cuh"

namespace vx {

// Scan scratch of vx_sample_pts_count_noalloc: one int64 partial sum per
// 2048-ray tile plus the grand total, for at most VX_NOALLOC_MAX_RAYS rays
// (2049 entries, 16 KB).  Every GPU that loads the library holds this array
// until the process exits.  Host code must not hand the symbol itself to a
// kernel (on the host it is only a stand-in, not a device address); the
// device address comes from cudaGetSymbolAddress, looked up once per device.
static __device__ __align__(256) int64_t g_noalloc_scan[VX_NOALLOC_MAX_RAYS / 2048 + 8];

static std::mutex g_noalloc_mutex;
static void* g_noalloc_ptr[64] = {nullptr};

// Device address of g_noalloc_scan on the current device (set-up on first
// use per device).  Returns VX_OK or a CUDA error status.
static int noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e);
  if (dev < 0 || dev >= 64) return VX_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scan);
    if (e != cudaSuccess) return cuda_status(e);
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return VX_OK;
}

struct RayClip {
  float t_min, t_max;
};

// render_utils_kernel.cu:20-33
__device__ __forceinline__ RayClip clip_ray(const float* __restrict__ o, const float* __restrict__ d,
                                            const float* __restrict__ mn, const float* __restrict__ mx,
                                            float near, float far) {
  const float vx = (d[0] == 0.f) ? 1e-6f : d[0];
  const float vy = (d[1] == 0.f) ? 1e-6f : d[1];
  const float vz = (d[2] == 0.f) ? 1e-6f : d[2];
  const float ax = fdiv(fsub(mx[0], o[0]), vx);
  const float ay = fdiv(fsub(mx[1], o[1]), vy);
  const float az = fdiv(fsub(mx[2], o[2]), vz);
  const float bx = fdiv(fsub(mn[0], o[0]), vx);
  const float by = fdiv(fsub(mn[1], o[1]), vy);
  const float bz = fdiv(fsub(mn[2], o[2]), vz);
  RayClip c;
  c.t_min = fmaxf(fminf(fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz)), far), near);
  c.t_max = fmaxf(fminf(fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz)), far), near);
  return c;
}

// sqrt(dx*dx + dy*dy + dz*dz), render_utils_kernel.cu:48-51, in the form the
// reference's compiled kernel computes it: dx*dx and dz*dz fused into the
// sum, sqrt(fma(dz, dz, fma(dx, dx, dy*dy)))
__device__ __forceinline__ float ray_norm(const float* __restrict__ d) {
  return ray_norm3(d[0], d[1], d[2]);
}

// max(ceil((t_max-t_min)*|d|/stepdist), 1), render_utils_kernel.cu:53
__device__ __forceinline__ int64_t n_samples_of(float t_min, float t_max, float rnorm, float stepdist) {
  const float c = ceilf(fdiv(fmul(fsub(t_max, t_min), rnorm), stepdist));
  const double m = fmax((double)c, 1.0);
  return (int64_t)m;
}

__global__ void infer_t_minmax_kernel(const float* __restrict__ rays_o, const float* __restrict__ rays_d,
                                      const float* __restrict__ xyz_min, const float* __restrict__ xyz_max,
                                      float near, float far, int64_t n_rays, float* __restrict__ t_min,
                                      float* __restrict__ t_max) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  RayClip c = clip_ray(rays_o + 3 * r, rays_d + 3 * r, xyz_min, xyz_max, near, far);
  t_min[r] = c.t_min;
  t_max[r] = c.t_max;
}

__global__ void infer_n_samples_kernel(const float* __restrict__ rays_d, const float* __restrict__ t_min,
                                       const float* __restrict__ t_max, float stepdist, int64_t n_rays,
                                       int64_t* __restrict__ n_samples) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  n_samples[r] = n_samples_of(t_min[r], t_max[r], ray_norm(rays_d + 3 * r), stepdist);
}

__global__ void infer_ray_start_dir_kernel(const float* __restrict__ rays_o, const float* __restrict__ rays_d,
                                           const float* __restrict__ t_min, int64_t n_rays,
                                           float* __restrict__ rays_start, float* __restrict__ rays_dir) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  const float* o = rays_o + 3 * r;
  const float* d = rays_d + 3 * r;
  const float rn = ray_norm(d);
  const float t = t_min[r];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    rays_start[3 * r + a] = __fmaf_rn(d[a], t, o[a]);
    rays_dir[3 * r + a] = fdiv(d[a], rn);
  }
}

// Phase 1: clip + count for every ray (one thread per ray).
__global__ void sample_count_kernel(const float* __restrict__ rays_o, const float* __restrict__ rays_d,
                                    const float* __restrict__ xyz_min, const float* __restrict__ xyz_max,
                                    float near, float far, float stepdist, int64_t n_rays,
                                    float* __restrict__ t_min, float* __restrict__ t_max,
                                    int64_t* __restrict__ n_steps) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  RayClip c = clip_ray(rays_o + 3 * r, rays_d + 3 * r, xyz_min, xyz_max, near, far);
  t_min[r] = c.t_min;
  t_max[r] = c.t_max;
  n_steps[r] = n_samples_of(c.t_min, c.t_max, ray_norm(rays_d + 3 * r), stepdist);
}

// Phase 2: one warp per ray writes samples offsets[r] .. offsets[r+1]-1.
// Point: start + dir*(stepdist*k) with start = o + d*t_min, dir = d/|d|
// (render_utils_kernel.cu:72-77, 184-192).
__global__ void sample_fill_kernel(const float* __restrict__ rays_o, const float* __restrict__ rays_d,
                                   const float* __restrict__ xyz_min, const float* __restrict__ xyz_max,
                                   const float* __restrict__ t_min, const int64_t* __restrict__ offsets,
                                   float stepdist, int64_t n_rays, int64_t capacity,
                                   float* __restrict__ ray_pts, uint8_t* __restrict__ mask_outbbox,
                                   int64_t* __restrict__ ray_id, int64_t* __restrict__ step_id, int* err) {
  const int64_t warps_per_block = blockDim.x >> 5;
  const int64_t r = (int64_t)blockIdx.x * warps_per_block + (threadIdx.x >> 5);
  if (r >= n_rays) return;
  const int lane = threadIdx.x & 31;
  const float* o = rays_o + 3 * r;
  const float* d = rays_d + 3 * r;
  const float rn = ray_norm(d);
  const float t = t_min[r];
  float st[3], dr[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    st[a] = __fmaf_rn(d[a], t, o[a]);
    dr[a] = fdiv(d[a], rn);
  }
  const float mn0 = xyz_min[0], mn1 = xyz_min[1], mn2 = xyz_min[2];
  const float mx0 = xyz_max[0], mx1 = xyz_max[1], mx2 = xyz_max[2];
  const int64_t beg = offsets[r], end = offsets[r + 1];
  if (end > capacity) {
    if (lane == 0) set_device_error(err, VX_ERR_CAPACITY);
  }
  for (int64_t idx = beg + lane; idx < end; idx += 32) {
    if (idx >= capacity) break;
    const int64_t k = idx - beg;
    const float dist = fmul(stepdist, (float)k);
    const float px = __fmaf_rn(dr[0], dist, st[0]);
    const float py = __fmaf_rn(dr[1], dist, st[1]);
    const float pz = __fmaf_rn(dr[2], dist, st[2]);
    ray_pts[3 * idx + 0] = px;
    ray_pts[3 * idx + 1] = py;
    ray_pts[3 * idx + 2] = pz;
    mask_outbbox[idx] = (mn0 > px) | (mn1 > py) | (mn2 > pz) | (mx0 < px) | (mx1 < py) | (mx2 < pz);
    ray_id[idx] = r;
    step_id[idx] = k;
  }
}

// C `round` (half away from zero) of x*scale + shift
// (render_utils_kernel.cu:385-387), fused into one multiply-add as the
// reference's compiled kernel computes it.
__device__ __forceinline__ int mask_index(float x, float scale, float shift) {
  return (int)roundf(__fmaf_rn(x, scale, shift));
}

__global__ void maskcache_lookup_kernel(const uint8_t* __restrict__ world, const float* __restrict__ xyz,
                                        uint8_t* __restrict__ out, const float* __restrict__ scale,
                                        const float* __restrict__ shift, int sz_i, int sz_j, int sz_k,
                                        int64_t n_pts) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_pts) return;
  const int i = mask_index(xyz[3 * p + 0], scale[0], shift[0]);
  const int j = mask_index(xyz[3 * p + 1], scale[1], shift[1]);
  const int k = mask_index(xyz[3 * p + 2], scale[2], shift[2]);
  uint8_t v = 0;
  if (0 <= i && i < sz_i && 0 <= j && j < sz_j && 0 <= k && k < sz_k)
    v = world[((int64_t)i * sz_j + j) * sz_k + k] ? 1 : 0;
  out[p] = v;
}

}  // namespace vx

using namespace vx;

extern "C" {

int vx_infer_t_minmax(const float* rays_o, const float* rays_d, const float* xyz_min, const float* xyz_max,
                      float near, float far, int64_t n_rays, float* t_min, float* t_max, void* stream) {
  if (n_rays < 0) return VX_ERR_ARG;
  if (n_rays == 0) return VX_OK;
  if (!rays_o || !rays_d || !xyz_min || !xyz_max || !t_min || !t_max) return VX_ERR_ARG;
  infer_t_minmax_kernel<<<grid_for(n_rays), VX_THREADS, 0, as_stream(stream)>>>(rays_o, rays_d, xyz_min, xyz_max,
                                                                              near, far, n_rays, t_min, t_max);
  return launch_status();
}

int vx_infer_n_samples(const float* rays_d, const float* t_min, const float* t_max, float stepdist, int64_t n_rays,
                       int64_t* n_samples, void* stream) {
  if (n_rays < 0) return VX_ERR_ARG;
  if (n_rays == 0) return VX_OK;
  if (!rays_d || !t_min || !t_max || !n_samples) return VX_ERR_ARG;
  infer_n_samples_kernel<<<grid_for(n_rays), VX_THREADS, 0, as_stream(stream)>>>(rays_d, t_min, t_max, stepdist,
                                                                               n_rays, n_samples);
  return launch_status();
}

int vx_infer_ray_start_dir(const float* rays_o, const float* rays_d, const float* t_min, int64_t n_rays,
                           float* rays_start, float* rays_dir, void* stream) {
  if (n_rays < 0) return VX_ERR_ARG;
  if (n_rays == 0) return VX_OK;
  if (!rays_o || !rays_d || !t_min || !rays_start || !rays_dir) return VX_ERR_ARG;
  infer_ray_start_dir_kernel<<<grid_for(n_rays), VX_THREADS, 0, as_stream(stream)>>>(rays_o, rays_d, t_min, n_rays,
                                                                                   rays_start, rays_dir);
  return launch_status();
}

int vx_sample_pts_count(const float* rays_o, const float* rays_d, const float* xyz_min, const float* xyz_max,
                        float near, float far, float stepdist, int64_t n_rays, float* t_min, float* t_max,
                        int64_t* n_steps, int64_t* offsets, void* scratch, size_t scratch_bytes, void* stream) {
  if (n_rays < 0 || !offsets) return VX_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (n_rays > 0) {
    if (!rays_o || !rays_d || !xyz_min || !xyz_max || !t_min || !t_max || !n_steps) return VX_ERR_ARG;
    sample_count_kernel<<<grid_for(n_rays), VX_THREADS, 0, st>>>(rays_o, rays_d, xyz_min, xyz_max, near, far,
                                                               stepdist, n_rays, t_min, t_max, n_steps);
    int s = launch_status();
    if (s) return s;
  }
  return exclusive_scan<int64_t, int64_t>(n_steps, n_rays, offsets, scratch, scratch_bytes, st);
}

// Same results as vx_sample_pts_count, for callers that cannot allocate
// device memory: the scan scratch is the library's own static array.  The
// array is shared by every call on a device and keeps the last call's
// contents; every entry a call reads is written by that same call first, so
// nothing needs clearing.  Calls that overlap on the GPU (different streams,
// or threads without ordering) race on the array.
int vx_sample_pts_count_noalloc(const float* rays_o, const float* rays_d, const float* xyz_min,
                                const float* xyz_max, float near, float far, float stepdist, int64_t n_rays,
                                float* t_min, float* t_max, int64_t* n_steps, int64_t* offsets, void* stream) {
  if (n_rays < 0 || !offsets) return VX_ERR_ARG;
  if (n_rays > VX_NOALLOC_MAX_RAYS) return VX_ERR_TOO_LARGE;
  void* scratch = nullptr;
  int s = noalloc_scratch(&scratch);
  if (s) return s;
  const size_t bytes = (size_t)(scan_n_tiles(n_rays) + 1) * sizeof(int64_t);
  if (bytes > sizeof(g_noalloc_scan)) return VX_ERR_TOO_LARGE;
  cudaStream_t st = as_stream(stream);
  if (n_rays > 0) {
    if (!rays_o || !rays_d || !xyz_min || !xyz_max || !t_min || !t_max || !n_steps) return VX_ERR_ARG;
    sample_count_kernel<<<grid_for(n_rays), VX_THREADS, 0, st>>>(rays_o, rays_d, xyz_min, xyz_max, near, far,
                                                               stepdist, n_rays, t_min, t_max, n_steps);
    s = launch_status();
    if (s) return s;
  }
  return exclusive_scan<int64_t, int64_t>(n_steps, n_rays, offsets, scratch, bytes, st);
}

int vx_sample_pts_fill(const float* rays_o, const float* rays_d, const float* xyz_min, const float* xyz_max,
                       const float* t_min, const int64_t* offsets, float stepdist, int64_t n_rays, int64_t capacity,
                       float* ray_pts, uint8_t* mask_outbbox, int64_t* ray_id, int64_t* step_id, void* stream) {
  if (n_rays < 0 || capacity < 0) return VX_ERR_ARG;
  if (n_rays == 0 || capacity == 0) return VX_OK;
  if (!rays_o || !rays_d || !xyz_min || !xyz_max || !t_min || !offsets || !ray_pts || !mask_outbbox || !ray_id ||
      !step_id)
    return VX_ERR_ARG;
  const int warps_per_block = VX_THREADS / 32;
  const unsigned blocks = (unsigned)((n_rays + warps_per_block - 1) / warps_per_block);
  sample_fill_kernel<<<blocks, VX_THREADS, 0, as_stream(stream)>>>(rays_o, rays_d, xyz_min, xyz_max, t_min, offsets,
                                                                  stepdist, n_rays, capacity, ray_pts, mask_outbbox,
                                                                  ray_id, step_id, device_error_ptr());
  return launch_status();
}

int vx_maskcache_lookup(const uint8_t* world, int64_t sz_i, int64_t sz_j, int64_t sz_k, const float* xyz,
                        int64_t n_pts, const float* xyz2ijk_scale, const float* xyz2ijk_shift, uint8_t* out,
                        void* stream) {
  if (n_pts < 0 || sz_i < 0 || sz_j < 0 || sz_k < 0) return VX_ERR_ARG;
  if (sz_i > INT32_MAX || sz_j > INT32_MAX || sz_k > INT32_MAX) return VX_ERR_ARG;
  if (n_pts == 0) return VX_OK;
  if (!world || !xyz || !xyz2ijk_scale || !xyz2ijk_shift || !out) return VX_ERR_ARG;
  maskcache_lookup_kernel<<<grid_for(n_pts), VX_THREADS, 0, as_stream(stream)>>>(
      world, xyz, out, xyz2ijk_scale, xyz2ijk_shift, (int)sz_i, (int)sz_j, (int)sz_k, n_pts);
  return launch_status();
}

}  // extern "C"
