// Library-level bookkeeping: status strings, the device error word, SM count.
#include <stdio.h>
#include "common.cuh"

namespace vx {

int g_last_cuda_error = 0;
unsigned long long g_launch_count = 0;
static __device__ int g_device_error = 0;

int* device_error_ptr() {
  static int* cached[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!cached[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_device_error) != cudaSuccess) return nullptr;
    cached[dev] = reinterpret_cast<int*>(p);
  }
  return cached[dev];
}

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (cached[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
    cached[dev] = n;
  }
  return cached[dev];
}

}  // namespace vx

extern "C" {

int vx_version(void) { return VX_ABI_VERSION; }

const char* vx_status_string(int status) {
  switch (status) {
    case VX_OK: return "ok";
    case VX_ERR_ARG: return "invalid argument";
    case VX_ERR_CAPACITY: return "output capacity exceeded";
    case VX_ERR_BOUNDS: return "index out of bounds";
    case VX_ERR_LAUNCH: return "kernel launch failed";
    case VX_ERR_CUDA: return "CUDA runtime error";
    case VX_ERR_UNSUPPORTED: return "unsupported configuration";
    case VX_ERR_TOO_LARGE: return "size above the fixed maximum of the no-allocation entry point";
    case VX_ERR_TIMEOUT: return "bounded device wait expired";
    default: return "unknown status";
  }
}

int vx_last_cuda_error(void) { return vx::g_last_cuda_error; }

unsigned long long vx_launch_count(void) { return __atomic_load_n(&vx::g_launch_count, __ATOMIC_RELAXED); }

const char* vx_cuda_error_string(int code) { return cudaGetErrorString((cudaError_t)code); }

int vx_device_error(void* stream, int* out_code) {
  // Reads and clears the device error word on `stream` (synchronises it).
  if (!out_code) return VX_ERR_ARG;
  cudaStream_t st = vx::as_stream(stream);
  int host = 0;
  cudaError_t e = cudaMemcpyFromSymbolAsync(&host, vx::g_device_error, sizeof(int), 0, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return vx::cuda_status(e);
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return vx::cuda_status(e);
  *out_code = host;
  if (host != 0) {
    const int zero = 0;
    e = cudaMemcpyToSymbolAsync(vx::g_device_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return vx::cuda_status(e);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return vx::cuda_status(e);
  }
  return VX_OK;
}

}  // extern "C"
