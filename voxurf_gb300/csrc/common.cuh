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
// clip, sample counts, sample positions, mask rounding) are computed with
// one rounding per operation so that the results are reproducible bit for
// bit by a CPU restatement with the same operation order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

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

// First index i in [lo, hi) with a[i] >= key (a sorted ascending).
__device__ __forceinline__ int64_t lower_bound_i64(const int64_t* a, int64_t lo, int64_t hi, int64_t key) {
  while (lo < hi) {
    int64_t mid = lo + ((hi - lo) >> 1);
    if (a[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

}  // namespace vx
