// Per-ray transmittance / weight scan (alpha2weight) and its backward.
//
// Drop-in for render_utils_cuda.alpha2weight / alpha2weight_backward
// (render_utils.cpp:182-183; kernels render_utils_kernel.cu:577-707).  The
// reference walks each ray with one thread (8192 rays -> 32 CTAs on 152 SMs)
// and a serial loop.  Here one warp owns one ray and walks it 32 samples at a
// time with a warp prefix product; the running transmittance is carried in
// FP64 on segments of more than 512 samples (so the prefix stays accurate on
// rays of thousands of samples) and in FP32 on shorter ones, as the
// reference's float loop.  Semantics kept exactly:
//   T[i] = prod_{j<i} (1 - alpha[j]),  w[i] = T[i] * alpha[i],
//   stop after the first sample whose inclusive product drops below 1e-3,
//   samples after the stop keep w = 0, T = 1, grad = 0,
//   empty rays report i_start = i_end = 0 and alphainv_last = 1.
// Segment bounds come from a binary search in the sorted ray_id instead of
// the reference's scatter kernel + device-indexed host write (:607-635).
#include "common.cuh"

namespace vx {

// Segment [beg, end) of ray r in a sorted ray_id array.
__device__ __forceinline__ void ray_segment(const int64_t* __restrict__ ray_id, int64_t n_pts, int64_t r,
                                            int64_t* beg, int64_t* end) {
  // Lanes 0 and 1 search the two bounds concurrently.
  const int lane = lane_id();
  int64_t v = 0;
  if (lane < 2) v = lower_bound_i64(ray_id, 0, n_pts, r + lane);
  *beg = __shfl_sync(0xffffffffu, v, 0);
  *end = __shfl_sync(0xffffffffu, v, 1);
}

// Warp-level forward scan of one segment.  Writes weight/T for every sample
// of [beg, end); returns (via lane 0 convention, broadcast) i_end and
// alphainv_last.
template <typename Acc>
__device__ __forceinline__ void scan_segment_fwd(const float* __restrict__ alpha, int64_t beg, int64_t end,
                                                 float* __restrict__ weight, float* __restrict__ T,
                                                 int64_t* i_end_out, float* last_out) {
  const int lane = lane_id();
  Acc carry = 1;
  bool stopped = false;
  int64_t i_end = end;
  float last = 1.f;
  for (int64_t base = beg; base < end; base += 32) {
    const int64_t i = base + lane;
    const bool valid = i < end;
    if (stopped) {
      if (valid) {
        weight[i] = 0.f;
        T[i] = 1.f;
      }
      continue;
    }
    const float a = valid ? alpha[i] : 0.f;
    const Acc f = Acc(1) - (Acc)a;
    const Acc incl = warp_inclusive_prod(f) * carry;
    Acc excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = carry;
    const unsigned stop_mask = __ballot_sync(0xffffffffu, valid && incl < Acc(1e-3));
    if (stop_mask) {
      const int k = __ffs(stop_mask) - 1;  // first sample that drops below 1e-3
      const Acc incl_k = __shfl_sync(0xffffffffu, incl, k);
      if (valid) {
        if (lane <= k) {
          const float t = (float)excl;
          T[i] = t;
          weight[i] = t * a;
        } else {
          weight[i] = 0.f;
          T[i] = 1.f;
        }
      }
      stopped = true;
      i_end = base + k + 1;
      last = (float)incl_k;
    } else {
      if (valid) {
        const float t = (float)excl;
        T[i] = t;
        weight[i] = t * a;
      }
      carry = __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  if (!stopped) last = (float)carry;
  *i_end_out = i_end;
  *last_out = last;
}

__global__ void alpha2weight_kernel(const float* __restrict__ alpha, const int64_t* __restrict__ ray_id,
                                    int64_t n_pts, int64_t n_rays, float* __restrict__ weight,
                                    float* __restrict__ T, float* __restrict__ alphainv_last,
                                    int64_t* __restrict__ i_start, int64_t* __restrict__ i_end) {
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= n_rays) return;
  int64_t beg, end;
  ray_segment(ray_id, n_pts, r, &beg, &end);
  if (beg >= end) {
    if (lane_id() == 0) {
      i_start[r] = 0;
      i_end[r] = 0;
      alphainv_last[r] = 1.f;
    }
    return;
  }
  int64_t ie;
  float last;
  if (end - beg > VX_FP32_SCAN_MAX_STEPS)
    scan_segment_fwd<double>(alpha, beg, end, weight, T, &ie, &last);
  else
    scan_segment_fwd<float>(alpha, beg, end, weight, T, &ie, &last);
  if (lane_id() == 0) {
    i_start[r] = beg;
    i_end[r] = ie;
    alphainv_last[r] = last;
  }
}

// Reverse scan, render_utils_kernel.cu:671-675:
//   back = grad_last*alphainv_last;  for i = i_end-1 .. i_start:
//     grad[i] = gw[i]*T[i] - back/(1-alpha[i]+1e-10);  back += gw[i]*w[i]
// The running sum `back` is carried in Acc (FP64 on segments of more than
// 512 samples).
template <typename Acc>
__device__ __forceinline__ void scan_segment_bwd(const float* __restrict__ alpha, const float* __restrict__ weight,
                                                 const float* __restrict__ T, const float* __restrict__ grad_w,
                                                 int64_t beg, int64_t end, float back0,
                                                 float* __restrict__ grad) {
  const int lane = lane_id();
  Acc carry = (Acc)back0;
  for (int64_t top = end; top > beg; top -= 32) {
    const int64_t i = top - 32 + lane;
    const bool valid = i >= beg;
    float gw = 0.f, w = 0.f, t = 0.f, a = 0.f;
    if (valid) {
      gw = grad_w[i];
      w = weight[i];
      t = T[i];
      a = alpha[i];
    }
    const Acc term = valid ? (Acc)(gw * w) : Acc(0);
    const Acc suffix = warp_inclusive_suffix_sum(term);  // sum of lanes >= this lane
    Acc after = __shfl_down_sync(0xffffffffu, suffix, 1);
    if (lane == 31) after = 0;
    const Acc back = carry + after;
    if (valid) {
      const Acc denom = (Acc)(1.f - a) + Acc(1e-10);
      grad[i] = (float)((Acc)(gw * t) - back / denom);
    }
    carry += __shfl_sync(0xffffffffu, suffix, 0);
  }
}

__global__ void alpha2weight_backward_kernel(const float* __restrict__ alpha, const float* __restrict__ weight,
                                             const float* __restrict__ T,
                                             const float* __restrict__ alphainv_last,
                                             const int64_t* __restrict__ i_start,
                                             const int64_t* __restrict__ i_end, int64_t n_pts, int64_t n_rays,
                                             const float* __restrict__ grad_weights,
                                             const float* __restrict__ grad_last, float* __restrict__ grad,
                                             int* err) {
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= n_rays) return;
  const int64_t beg = i_start[r], end = i_end[r];
  if (beg >= end) return;
  if (beg < 0 || end > n_pts) {
    if (lane_id() == 0) set_device_error(err, VX_ERR_BOUNDS);
    return;
  }
  if (end - beg > VX_FP32_SCAN_MAX_STEPS)
    scan_segment_bwd<double>(alpha, weight, T, grad_weights, beg, end, grad_last[r] * alphainv_last[r], grad);
  else
    scan_segment_bwd<float>(alpha, weight, T, grad_weights, beg, end, grad_last[r] * alphainv_last[r], grad);
}

}  // namespace vx

using namespace vx;

extern "C" {

int vx_alpha2weight(const float* alpha, const int64_t* ray_id, int64_t n_pts, int64_t n_rays, float* weight,
                    float* T, float* alphainv_last, int64_t* i_start, int64_t* i_end, void* stream) {
  if (n_pts < 0 || n_rays < 0) return VX_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (n_rays == 0) return VX_OK;
  if (!alphainv_last || !i_start || !i_end) return VX_ERR_ARG;
  if (n_pts > 0 && (!alpha || !ray_id || !weight || !T)) return VX_ERR_ARG;
  const int wpb = VX_THREADS / 32;
  alpha2weight_kernel<<<(unsigned)((n_rays + wpb - 1) / wpb), VX_THREADS, 0, st>>>(
      alpha, ray_id, n_pts, n_rays, weight, T, alphainv_last, i_start, i_end);
  return launch_status();
}

int vx_alpha2weight_backward(const float* alpha, const float* weight, const float* T, const float* alphainv_last,
                             const int64_t* i_start, const int64_t* i_end, int64_t n_pts, int64_t n_rays,
                             const float* grad_weights, const float* grad_last, float* grad, void* stream) {
  if (n_pts < 0 || n_rays < 0) return VX_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (n_pts > 0) {
    if (!grad) return VX_ERR_ARG;
    int s = cuda_status(cudaMemsetAsync(grad, 0, (size_t)n_pts * sizeof(float), st));
    if (s) return s;
  }
  if (n_rays == 0 || n_pts == 0) return VX_OK;
  if (!alpha || !weight || !T || !alphainv_last || !i_start || !i_end || !grad_weights || !grad_last)
    return VX_ERR_ARG;
  const int wpb = VX_THREADS / 32;
  alpha2weight_backward_kernel<<<(unsigned)((n_rays + wpb - 1) / wpb), VX_THREADS, 0, st>>>(
      alpha, weight, T, alphainv_last, i_start, i_end, n_pts, n_rays, grad_weights, grad_last, grad,
      device_error_ptr());
  return launch_status();
}

}  // extern "C"
