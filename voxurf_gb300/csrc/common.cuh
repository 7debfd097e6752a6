// Shared helpers for the voxurf_gb300 CUDA library (sm_103a only).
//
// Every exported entry point is `extern "C"`, takes plain device pointers,
// sizes and a cudaStream_t, never allocates device memory, and returns an
// int status (VX_OK on success).  Launch errors are caught with
// cudaGetLastError() right after each launch, unlike the pybind11 ops they
// replace, which never check (render_utils.cpp:46-48 only checks inputs).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "voxurf_gb300.h"

#define VX_THREADS 256

namespace vx {

// Last CUDA error seen by any entry point of this library (host-side copy).
extern int g_last_cuda_error;
// Number of kernel launches issued by this library (every launch is
// followed by exactly one launch_status() call).
extern unsigned long long g_launch_count;

inline int launch_status() {
  __atomic_add_fetch(&g_launch_count, 1ull, __ATOMIC_RELAXED);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_last_cuda_error = (int)e;
    return VX_ERR_LAUNCH;
  }
  return VX_OK;
}

inline int cuda_status(cudaError_t e) {
  if (e != cudaSuccess) {
    g_last_cuda_error = (int)e;
    return VX_ERR_CUDA;
  }
  return VX_OK;
}

// Device-resident error word (one per device, in runtime.cu).  Kernels that
// detect an out-of-range index or an overflowing capacity record the first
// error code there (and skip the access) instead of faulting;
// vx_device_error() reads and clears it.  Host code passes its address to
// the kernels that may report (device_error_ptr()).
int* device_error_ptr();

__device__ __forceinline__ void set_device_error(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

inline unsigned int grid_for(int64_t n, int threads = VX_THREADS) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  return (unsigned int)b;
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per process).
int sm_count();

// Device-wide exclusive scan (scan.cu).  out has n+1 entries, out[n] = total.
int64_t scan_n_tiles(int64_t n);
template <typename Tin, typename Tout>
int exclusive_scan(const Tin* in, int64_t n, Tout* out, void* scratch, size_t scratch_bytes, cudaStream_t st);

// ---------------------------------------------------------------------------
// Uncontracted IEEE float arithmetic.  The index-producing stages (ray/bbox
// clip, sample counts, sample positions, mask rounding) round every
// operation once, except the multiply-adds that the reference's compiled
// kernels fuse (written as __fmaf_rn where they occur), so that the results
// equal the reference's kernels and a CPU restatement bit for bit.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// |v| as torch's norm reduction forms it: squares accumulated with fused
// multiply-adds in x, y, z order, then a correctly rounded square root.
__device__ __forceinline__ float norm3(float x, float y, float z) {
  return __fsqrt_rn(__fmaf_rn(z, z, __fmaf_rn(y, y, fmul(x, x))));
}

// |d| of a ray as the reference's compiled sampling kernels compute
// sqrt(dx*dx + dy*dy + dz*dz) (render_utils_kernel.cu:48-51, 67-70; nvcc's
// --fmad=true fuses dx*dx and then dz*dz into the sum).
__device__ __forceinline__ float ray_norm3(float x, float y, float z) {
  return __fsqrt_rn(__fmaf_rn(z, z, __fmaf_rn(x, x, fmul(y, y))));
}

// Transmittance precision: a ray of more samples than this carries its
// transmittance products (forward) and its suffix sums (backward) in FP64;
// shorter rays in FP32.  GB300 runs FP64 at a small fraction of its FP32
// rate, and at 512 factors an FP32 product is still within a few 1e-6 of
// the exact one.  The decision is per ray (warp-uniform).
constexpr int64_t VX_FP32_SCAN_MAX_STEPS = 512;

// Warp-wide helpers -----------------------------------------------------------
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Inclusive warp prefix product (Hillis-Steele; 5 shuffle rounds).
template <typename T>
__device__ __forceinline__ T warp_inclusive_prod(T v) {
  const int lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v *= u;
  }
  return v;
}

// Inclusive warp suffix sum: lane i gets sum of lanes i..31.
template <typename T>
__device__ __forceinline__ T warp_inclusive_suffix_sum(T v) {
  const int lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_down_sync(0xffffffffu, v, o);
    if (lane + o < 32) v += u;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_inclusive_sum(T v) {
  const int lane = lane_id();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

// One 32-sample step of a ray's transmittance scan with the T < 1e-3 stop
// (render_utils_kernel.cu:577-605): the lanes with `keep` multiply in
// (1 - alpha) in Acc.  T = this lane's exclusive product (FP32); returns the
// lanes up to and including the first whose inclusive product drops below
// 1e-3 (all kept lanes when none does).  carry advances to the next step
// unless the ray stops here, in which case last = the stopping product.
template <typename Acc>
__device__ __forceinline__ unsigned transmittance_step(bool keep, float alpha, Acc& carry, Acc& last, bool& stopped,
                                                       float& T) {
  const int lane = lane_id();
  const unsigned keep_mask = __ballot_sync(0xffffffffu, keep);
  const Acc fct = keep ? Acc(1) - (Acc)alpha : Acc(1);
  const Acc incl = warp_inclusive_prod(fct) * carry;
  Acc excl = __shfl_up_sync(0xffffffffu, incl, 1);
  if (lane == 0) excl = carry;
  const unsigned stop_mask = __ballot_sync(0xffffffffu, keep && incl < Acc(1e-3));
  unsigned live = keep_mask;
  if (stop_mask) {
    const int ks = __ffs(stop_mask) - 1;
    live &= (ks == 31) ? 0xffffffffu : ((2u << ks) - 1u);
    last = __shfl_sync(0xffffffffu, incl, ks);
    stopped = true;
  }
  T = (float)excl;
  if (!stopped) carry = __shfl_sync(0xffffffffu, incl, 31);
  return live;
}

// First index i in [lo, hi) with a[i] >= key (a sorted ascending).
__device__ __forceinline__ int64_t lower_bound_i64(const int64_t* a, int64_t lo, int64_t hi, int64_t key) {
  while (lo < hi) {
    int64_t mid = lo + ((hi - lo) >> 1);
    if (a[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

}  // namespace vx
