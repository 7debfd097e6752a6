// Elementwise parts of the colour-MLP backward (rgbnet / k_rgbnet,
// lib/voxurf_fine.py:132-187, lib/voxurf_coarse.py:116-123), fused:
//   dz = dh * (h > 0)      (ReLU backward, h = the layer's post-ReLU output)
//   db += sum_rows dz      (bias gradient, FP32 accumulation)
// One pass over dh/h instead of torch's threshold_backward + a strided
// column reduction.  The GEMMs (dW = dz^T x, dx = dz W) stay in cuBLAS.
#include "common.cuh"

namespace vx {

template <typename T>
__device__ __forceinline__ float ldf(const T* p, int64_t i);
template <>
__device__ __forceinline__ float ldf<float>(const float* p, int64_t i) { return p[i]; }
template <>
__device__ __forceinline__ float ldf<__nv_bfloat16>(const __nv_bfloat16* p, int64_t i) {
  return __bfloat162float(p[i]);
}
template <typename T>
__device__ __forceinline__ void stf(T* p, int64_t i, float v);
template <>
__device__ __forceinline__ void stf<float>(float* p, int64_t i, float v) { p[i] = v; }
template <>
__device__ __forceinline__ void stf<__nv_bfloat16>(__nv_bfloat16* p, int64_t i, float v) {
  p[i] = __float2bfloat16_rn(v);
}

constexpr int ROWS_PER_BLOCK = 128;

// blockDim.x threads own columns tid, tid + blockDim.x, ...; each block walks
// ROWS_PER_BLOCK rows (coalesced along the row), then one atomic per column.
template <typename T, bool RELU>
__global__ void relu_bwd_colsum_kernel(const T* __restrict__ dh, const T* __restrict__ h, int64_t M, int N,
                                       T* __restrict__ dz, float* __restrict__ colsum) {
  const int64_t r0 = (int64_t)blockIdx.x * ROWS_PER_BLOCK;
  const int64_t r1 = min(r0 + ROWS_PER_BLOCK, M);
  for (int c = threadIdx.x; c < N; c += blockDim.x) {
    float s = 0.f;
#pragma unroll 4
    for (int64_t r = r0; r < r1; ++r) {
      const int64_t i = r * N + c;
      float v = ldf(dh, i);
      if (RELU) {
        v = ldf(h, i) > 0.f ? v : 0.f;
        stf(dz, i, v);
      }
      s += v;
    }
    atomicAdd(colsum + c, s);
  }
}

}  // namespace vx

using namespace vx;

extern "C" {

// dtype: 0 float32, 1 bfloat16 (dh, h, dz).  h == NULL: no ReLU (dz unused),
// only the column sums.  colsum [N] is accumulated (callers zero it).
int vx_relu_bwd_colsum(const void* dh, const void* h, int64_t M, int64_t N, int dtype, void* dz, float* colsum,
                       void* stream) {
  if (M < 0 || N <= 0 || N > INT32_MAX || !colsum || (dtype != 0 && dtype != 1)) return VX_ERR_ARG;
  if (M == 0) return VX_OK;
  if (!dh || (h && !dz)) return VX_ERR_ARG;
  const unsigned blocks = (unsigned)((M + ROWS_PER_BLOCK - 1) / ROWS_PER_BLOCK);
  const int threads = N >= 256 ? 256 : (int)((N + 31) / 32) * 32;
  cudaStream_t st = as_stream(stream);
  if (dtype == 0) {
    if (h)
      relu_bwd_colsum_kernel<float, true><<<blocks, threads, 0, st>>>(
          (const float*)dh, (const float*)h, M, (int)N, (float*)dz, colsum);
    else
      relu_bwd_colsum_kernel<float, false><<<blocks, threads, 0, st>>>((const float*)dh, nullptr, M, (int)N, nullptr,
                                                                      colsum);
  } else {
    using B = __nv_bfloat16;
    if (h)
      relu_bwd_colsum_kernel<B, true><<<blocks, threads, 0, st>>>((const B*)dh, (const B*)h, M, (int)N, (B*)dz,
                                                                 colsum);
    else
      relu_bwd_colsum_kernel<B, false><<<blocks, threads, 0, st>>>((const B*)dh, nullptr, M, (int)N, nullptr, colsum);
  }
  return launch_status();
}

}  // extern "C"
