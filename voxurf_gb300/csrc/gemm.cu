// FP32 GEMM entry point for the colour-MLP backward (weight and input
// gradients of the 192-wide layers, lib/voxurf_fine.py:132-187 under
// autograd).  A plain library GEMM: cuBLAS SGEMM on the caller's stream with
// the caller's workspace, optionally in cuBLAS's BF16x9 FP32 emulation
// (CUBLAS_FP32_EMULATED_BF16X9_MATH: each FP32 operand split into three BF16
// parts on the tensor cores, FP32 accumulation; cuBLAS uses it where it is
// faster than its CUDA-core kernels).  Column-major, as cublasSgemm.
#include <cublas_v2.h>
#include <mutex>
#include "common.cuh"

namespace {

constexpr int kMaxDevices = 64;
cublasHandle_t g_handles[kMaxDevices] = {};
std::mutex g_mutex;

int handle_for_current_device(cublasHandle_t* out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return VX_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_handles[dev] && cublasCreate(&g_handles[dev]) != CUBLAS_STATUS_SUCCESS) {
    g_handles[dev] = nullptr;
    return VX_ERR_CUDA;
  }
  *out = g_handles[dev];
  return VX_OK;
}

// out[i] = sum over b of part[b * n + i], b in order.
__global__ void sum_partials_kernel(const float* __restrict__ part, int64_t n, int nb, float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float acc = 0.f;
  for (int b = 0; b < nb; ++b) acc += part[(int64_t)b * n + i];
  out[i] = acc;
}

}  // namespace

using namespace vx;

extern "C" {

int vx_gemm_f32(int transa, int transb, int64_t m, int64_t n, int64_t k, float alpha, const float* A, int64_t lda,
                const float* B, int64_t ldb, float beta, float* C, int64_t ldc, int emulate, void* workspace,
                size_t workspace_bytes, void* stream) {
  if (m < 0 || n < 0 || k < 0) return VX_ERR_ARG;
  if (m == 0 || n == 0) return VX_OK;
  if ((k > 0 && (!A || !B)) || !C) return VX_ERR_ARG;
  if (m > INT32_MAX || n > INT32_MAX || k > INT32_MAX || lda > INT32_MAX || ldb > INT32_MAX || ldc > INT32_MAX)
    return VX_ERR_ARG;
  cublasHandle_t h = nullptr;
  int s = handle_for_current_device(&h);
  if (s) return s;
  std::lock_guard<std::mutex> lock(g_mutex);  // the handle's stream / workspace / mode are per call
  if (cublasSetStream(h, reinterpret_cast<cudaStream_t>(stream)) != CUBLAS_STATUS_SUCCESS) return VX_ERR_CUDA;
  if (workspace && workspace_bytes &&
      cublasSetWorkspace(h, workspace, workspace_bytes) != CUBLAS_STATUS_SUCCESS)
    return VX_ERR_CUDA;
  const cublasMath_t mode = emulate ? CUBLAS_FP32_EMULATED_BF16X9_MATH : CUBLAS_DEFAULT_MATH;
  if (cublasSetMathMode(h, mode) != CUBLAS_STATUS_SUCCESS) return VX_ERR_UNSUPPORTED;
  // k = 0: C = beta C (A and B are not read)
  const cublasStatus_t st =
      cublasSgemm(h, transa ? CUBLAS_OP_T : CUBLAS_OP_N, transb ? CUBLAS_OP_T : CUBLAS_OP_N, (int)m, (int)n, (int)k,
                  &alpha, A, (int)lda, B, (int)ldb, &beta, C, (int)ldc);
  if (st != CUBLAS_STATUS_SUCCESS) return st == CUBLAS_STATUS_NOT_SUPPORTED ? VX_ERR_UNSUPPORTED : VX_ERR_CUDA;
  return VX_OK;
}

int vx_gemm_f32_wgrad(const float* dz, const float* h, int64_t S, int64_t n_out, int64_t k_in, int64_t rows_per_chunk,
                      float* partials, float* dW, int emulate, void* stream) {
  if (S < 0 || n_out <= 0 || k_in <= 0 || rows_per_chunk <= 0 || !dW) return VX_ERR_ARG;
  if (S <= rows_per_chunk)
    return vx_gemm_f32(0, 1, k_in, n_out, S, 1.f, h, k_in, dz, n_out, 0.f, dW, k_in, emulate, nullptr, 0, stream);
  if (!dz || !h || !partials) return VX_ERR_ARG;
  const int64_t nb = S / rows_per_chunk, rem = S - nb * rows_per_chunk, n = n_out * k_in;
  if (nb + 1 > INT32_MAX || rows_per_chunk > INT32_MAX || n_out > INT32_MAX || k_in > INT32_MAX) return VX_ERR_ARG;
  cublasHandle_t hd = nullptr;
  int s = handle_for_current_device(&hd);
  if (s) return s;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (cublasSetStream(hd, reinterpret_cast<cudaStream_t>(stream)) != CUBLAS_STATUS_SUCCESS) return VX_ERR_CUDA;
    if (cublasSetMathMode(hd, emulate ? CUBLAS_FP32_EMULATED_BF16X9_MATH : CUBLAS_DEFAULT_MATH) !=
        CUBLAS_STATUS_SUCCESS)
      return VX_ERR_UNSUPPORTED;
    const float one = 1.f, zero = 0.f;
    // chunk b: partials[b] (k_in x n_out, column-major) = h_b^T dz_b
    cublasStatus_t st = cublasSgemmStridedBatched(
        hd, CUBLAS_OP_N, CUBLAS_OP_T, (int)k_in, (int)n_out, (int)rows_per_chunk, &one, h, (int)k_in,
        rows_per_chunk * k_in, dz, (int)n_out, rows_per_chunk * n_out, &zero, partials, (int)k_in, n, (int)nb);
    if (st == CUBLAS_STATUS_SUCCESS && rem > 0)
      st = cublasSgemm(hd, CUBLAS_OP_N, CUBLAS_OP_T, (int)k_in, (int)n_out, (int)rem, &one,
                       h + nb * rows_per_chunk * k_in, (int)k_in, dz + nb * rows_per_chunk * n_out, (int)n_out,
                       &zero, partials + nb * n, (int)k_in);
    if (st != CUBLAS_STATUS_SUCCESS) return st == CUBLAS_STATUS_NOT_SUPPORTED ? VX_ERR_UNSUPPORTED : VX_ERR_CUDA;
  }
  const int parts = (int)(nb + (rem > 0 ? 1 : 0));
  sum_partials_kernel<<<grid_for(n), VX_THREADS, 0, as_stream(stream)>>>(partials, n, parts, dW);
  return launch_status();
}

}  // extern "C"
