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

}  // namespace

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

}  // extern "C"
