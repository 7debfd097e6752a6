// Background branch of the scenes without an object mask
// (lib/voxurf_womask_fine.py, lib/voxurf_womask_coarse.py):
//   * vx_cumdist_thres: the reference's ub360_utils_cuda.cumdist_thres
//     (lib/cuda/ub360_utils.cpp, kernel at ub360_utils_kernel.cu:13-31): a
//     per-ray running distance that marks a sample and restarts from zero
//     once it exceeds `thres`;
//   * vx_bg_samples_count / vx_bg_samples_fill: the whole background sample
//     generator of voxurf_womask_fine.py:857-870 (and of
//     voxurf_womask_coarse.py:633-650) in two launches: uniform samples from
//     the bbox entry (sample_ray_ori, voxurf_womask_fine.py:789-818), the
//     inversion x / |x|^2 (outside_sphere_trans with filtered=True, :820-825),
//     the distance between consecutive inverted samples, cumdist_thres over
//     it and the compaction of the kept samples.  The reference materialises
//     [N, S, 3] points, their norms, the inverted points, the [N, S-1]
//     distances and the masks in HBM (about 60 bytes per candidate sample)
//     before compacting with boolean indexing; here one warp walks one ray
//     in registers and only the kept samples are written.
// Every float operation is rounded as the reference's torch expressions
// round it (one rounding per elementwise operation; the norms accumulate with
// fused multiply-adds like torch's norm reduction), so the CPU restatement
// reproduces the outputs bit for bit.
#include <math.h>
#include "common.cuh"

namespace vx {
namespace {

// ---------------------------------------------------------------------------
// cumdist_thres.  A CTA of 32 threads owns 32 rays; the rows are moved
// through shared memory in [32 rays x 32 samples] tiles so that the loads
// and stores are coalesced (a thread walking its own row would touch a new
// 128-byte line per sample), and each thread scans its ray's row of the
// tile while the next tile is in flight.
constexpr int CD_RAYS = 32;
constexpr int CD_COLS = 32;

__global__ void __launch_bounds__(CD_RAYS) cumdist_thres_kernel(const float* __restrict__ dist, int64_t n_rays,
                                                                 int64_t n_pts, float thres,
                                                                 uint8_t* __restrict__ mask) {
  __shared__ float tile[CD_RAYS][CD_COLS + 1];
  __shared__ uint8_t over_t[CD_RAYS][CD_COLS + 4];
  const int lane = threadIdx.x;
  const int64_t r0 = (int64_t)blockIdx.x * CD_RAYS;
  float cum = 0.f;
  // the next tile's 32 values of this lane's column are loaded into
  // registers while the current tile is scanned
  float nxt[CD_RAYS];
#pragma unroll
  for (int rr = 0; rr < CD_RAYS; ++rr) {
    const int64_t r = r0 + rr;
    nxt[rr] = (r < n_rays && lane < n_pts) ? dist[r * n_pts + lane] : 0.f;
  }
  for (int64_t c0 = 0; c0 < n_pts; c0 += CD_COLS) {
    const int64_t c = c0 + lane;
#pragma unroll
    for (int rr = 0; rr < CD_RAYS; ++rr) tile[rr][lane] = nxt[rr];
    __syncwarp();
    const int64_t cn = c + CD_COLS;
#pragma unroll
    for (int rr = 0; rr < CD_RAYS; ++rr) {
      const int64_t r = r0 + rr;
      nxt[rr] = (r < n_rays && cn < n_pts) ? dist[r * n_pts + cn] : 0.f;
    }
    const int cols = n_pts - c0 < CD_COLS ? (int)(n_pts - c0) : CD_COLS;
    for (int j = 0; j < cols; ++j) {
      cum = fadd(cum, tile[lane][j]);
      const bool over = cum > thres;
      cum = fmul(cum, (float)(!over));
      over_t[lane][j] = over ? 1 : 0;
    }
    __syncwarp();
    for (int rr = 0; rr < CD_RAYS; ++rr) {
      const int64_t r = r0 + rr;
      if (r < n_rays && c < n_pts) mask[r * n_pts + c] = over_t[rr][lane];
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Background samples of one ray.

struct BgRay {
  float o[3], d[3];
  float t_min, d_norm, jit;
  bool miss;  // t_max <= t_min (the ray-level mask_outbbox of :803)
};

__device__ __forceinline__ BgRay bg_ray(const vx_bg_sample_args& a, int64_t r) {
  BgRay R;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    R.o[i] = a.rays_o[3 * r + i];
    R.d[i] = a.rays_d[3 * r + i];
  }
  // voxurf_womask_fine.py:797-803: slab clip with zero directions replaced
  // by 1e-6, clamp(min=near, max=far)
  float tmin = -INFINITY, tmax = INFINITY;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float v = R.d[i] == 0.f ? 1e-6f : R.d[i];
    const float ra = fdiv(fsub(a.xyz_max[i], R.o[i]), v);
    const float rb = fdiv(fsub(a.xyz_min[i], R.o[i]), v);
    tmin = fmaxf(tmin, fminf(ra, rb));
    tmax = fminf(tmax, fmaxf(ra, rb));
  }
  R.t_min = fminf(fmaxf(tmin, a.near), a.far);
  R.miss = fminf(fmaxf(tmax, a.near), a.far) <= R.t_min;
  R.d_norm = norm3(R.d[0], R.d[1], R.d[2]);
  R.jit = a.jitter ? a.jitter[r] : 0.f;
  return R;
}

// Sample k of the ray (sample_ray_ori :805-812) and its inversion; returns
// whether the point lies inside the unit sphere.
__device__ __forceinline__ bool bg_point(const vx_bg_sample_args& a, const BgRay& R, int k, float p[3],
                                         float q[3]) {
  const float rng = a.jitter ? fadd((float)k, R.jit) : (float)k;
  const float step = fmul(a.stepdist, rng);
  const float t = fadd(R.t_min, fdiv(step, R.d_norm));
#pragma unroll
  for (int i = 0; i < 3; ++i) p[i] = fadd(R.o[i], fmul(R.d[i], t));
  const float n = norm3(p[0], p[1], p[2]);
  const float n2 = fmul(n, n);
#pragma unroll
  for (int i = 0; i < 3; ++i) q[i] = fdiv(p[i], n2);
  return n < 1.f;
}

// One warp per ray; the lanes take 32 consecutive samples at a time.  Each
// lane forms its point, the inverted point and the distance to the previous
// inverted point (shuffled up from the neighbouring lane); the cumdist
// recurrence is serial along the ray, so every lane runs it over the 32
// shuffled distances in order (the running sum is identical in all lanes)
// and picks its own mark.  The kept samples of the 32 are compacted with a
// ballot, so the fill pass writes consecutive records from consecutive lanes.
constexpr int BG_THREADS = 256;

template <bool FILL>
__global__ void __launch_bounds__(BG_THREADS) bg_samples_kernel(
    const vx_bg_sample_args a, int64_t* __restrict__ counts, const int64_t* __restrict__ offsets, int64_t capacity,
    float* __restrict__ outer_pts, float* __restrict__ pts_org, int64_t* __restrict__ ray_id,
    int64_t* __restrict__ step_id, int* err) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * BG_THREADS + threadIdx.x) >> 5;
  if (r >= a.n_rays) return;  // r is uniform over the warp
  const BgRay R = bg_ray(a, r);
  int64_t idx = FILL ? offsets[r] : 0;
  const int64_t end = FILL ? offsets[r + 1] : 0;
  if (FILL && lane == 0 && end > capacity) set_device_error(err, VX_ERR_CAPACITY);
  int64_t n = 0;
  float cum = 0.f;
  float lastq[3] = {0.f, 0.f, 0.f};  // inverted point of the previous chunk's last sample
  for (int k0 = 0; k0 < a.n_samples; k0 += 32) {
    const int k = k0 + lane;
    const bool valid = k < a.n_samples;
    float p[3] = {0.f, 0.f, 0.f}, q[3] = {0.f, 0.f, 0.f};
    bool keep = false;
    if (valid) {
      const bool inside = bg_point(a, R, k, p, q);
      keep = a.inner ? inside : !inside;
      if (a.outbbox_only && !a.inner) {
        // voxurf_womask_coarse.py:641 keeps only samples outside the bbox
        // (sample_ray_ori's mask_outbbox, voxurf_womask_fine.py:814)
        bool out = R.miss;
#pragma unroll
        for (int i = 0; i < 3; ++i) out = out || (a.xyz_min[i] > p[i]) || (p[i] > a.xyz_max[i]);
        keep = keep && out;
      }
    }
    if (a.inner) {
      // foreground samples (voxurf_womask_fine.py:846-849): the points
      // inside the unit sphere, no inversion and no distance test
      const unsigned ball = __ballot_sync(FULL, keep);
      if (FILL) {
        if (keep) {
          const int64_t o = idx + __popc(ball & ((1u << lane) - 1u));
          if (o < capacity && o < end) {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              outer_pts[3 * o + i] = p[i];
              if (pts_org) pts_org[3 * o + i] = p[i];
            }
            ray_id[o] = r;
            step_id[o] = k;
          }
        }
        idx += __popc(ball);
      } else {
        n += __popc(ball);
      }
      continue;
    }
    // dist of :866 between this sample's and the previous inverted point
    float prevq[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float up = __shfl_up_sync(FULL, q[i], 1);
      prevq[i] = lane == 0 ? lastq[i] : up;
      lastq[i] = __shfl_sync(FULL, q[i], 31);
    }
    float dd = 0.f;
    if (valid && k > 0) dd = norm3(fsub(q[0], prevq[0]), fsub(q[1], prevq[1]), fsub(q[2], prevq[2]));
    // cumdist_thres over the chunk, in sample order
    const int cnt = a.n_samples - k0 < 32 ? a.n_samples - k0 : 32;
    unsigned marks = 0;
    for (int j = 0; j < cnt; ++j) {
      const float v = __shfl_sync(FULL, dd, j);
      if (k0 + j > 0) {
        cum = fadd(cum, v);
        const bool over = cum > a.dist_thres;
        cum = fmul(cum, (float)(!over));
        marks |= (unsigned)over << j;
      }
    }
    if (k > 0) keep = keep && ((marks >> lane) & 1u);
    const unsigned ball = __ballot_sync(FULL, keep);
    if (FILL) {
      if (keep) {
        const int64_t o = idx + __popc(ball & ((1u << lane) - 1u));
        if (o < capacity && o < end) {
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            outer_pts[3 * o + i] = q[i];
            pts_org[3 * o + i] = p[i];
          }
          ray_id[o] = r;
          step_id[o] = k;
        }
      }
      idx += __popc(ball);
    } else {
      n += __popc(ball);
    }
  }
  if (!FILL && lane == 0) counts[r] = n;
}

inline unsigned bg_blocks(int64_t n_rays) {
  return (unsigned)((n_rays * 32 + BG_THREADS - 1) / BG_THREADS);
}

bool bg_args_ok(const vx_bg_sample_args* a) {
  if (!a || a->n_rays < 0 || a->n_samples < 0) return false;
  if (a->n_rays > ((int64_t)INT32_MAX * BG_THREADS) / 32) return false;
  if (a->n_rays > 0 && (!a->rays_o || !a->rays_d)) return false;
  return true;
}

}  // namespace
}  // namespace vx

using namespace vx;

extern "C" {

int vx_cumdist_thres(const float* dist, int64_t n_rays, int64_t n_pts, float thres, uint8_t* mask, void* stream) {
  if (n_rays < 0 || n_pts < 0) return VX_ERR_ARG;
  if (n_rays == 0 || n_pts == 0) return VX_OK;
  if (!dist || !mask) return VX_ERR_ARG;
  const int64_t blocks = (n_rays + CD_RAYS - 1) / CD_RAYS;
  if (blocks > INT32_MAX) return VX_ERR_TOO_LARGE;
  cumdist_thres_kernel<<<(unsigned)blocks, CD_RAYS, 0, as_stream(stream)>>>(dist, n_rays, n_pts, thres, mask);
  return launch_status();
}

int vx_bg_samples_count(const vx_bg_sample_args* args, int64_t* counts, int64_t* offsets, void* scratch,
                        size_t scratch_bytes, void* stream) {
  if (!bg_args_ok(args) || !offsets) return VX_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (args->n_rays > 0) {
    if (!counts) return VX_ERR_ARG;
    bg_samples_kernel<false><<<bg_blocks(args->n_rays), BG_THREADS, 0, st>>>(*args, counts, nullptr, 0, nullptr,
                                                                              nullptr, nullptr, nullptr, nullptr);
    const int s = launch_status();
    if (s) return s;
  }
  return exclusive_scan<int64_t, int64_t>(counts, args->n_rays, offsets, scratch, scratch_bytes, st);
}

int vx_bg_samples_fill(const vx_bg_sample_args* args, const int64_t* offsets, int64_t capacity, float* outer_pts,
                       float* pts_org, int64_t* ray_id, int64_t* step_id, void* stream) {
  if (!bg_args_ok(args) || capacity < 0) return VX_ERR_ARG;
  if (args->n_rays == 0 || capacity == 0) return VX_OK;
  if (!offsets || !outer_pts || (!pts_org && !args->inner) || !ray_id || !step_id) return VX_ERR_ARG;
  bg_samples_kernel<true><<<bg_blocks(args->n_rays), BG_THREADS, 0, as_stream(stream)>>>(
      *args, nullptr, offsets, capacity, outer_pts, pts_org, ray_id, step_id, device_error_ptr());
  return launch_status();
}

}  // extern "C"
