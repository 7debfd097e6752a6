// Elementwise parts of the colour-MLP backward (rgbnet / k_rgbnet,
// lib/voxurf_fine.py:132-187, lib/voxurf_coarse.py:116-123), fused:
//   dz = dh * (h > 0)      (ReLU backward, h = the layer's post-ReLU output)
//   db += sum_rows dz      (bias gradient, FP32 accumulation)
// One pass over dh/h instead of torch's threshold_backward + a strided
// column reduction, for callers that run the layer GEMMs themselves (the
// library's own training engines fuse this step into their kernels:
// mlp_train.cu, mlp_f32.cu).
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

// Vectorised form for rows of 16-byte chunks (N % (16/sizeof(T)) == 0, 16-byte
// aligned rows): thread (rl, g) of a block of G*RL threads owns chunk g of the
// rows r0 + rl, r0 + rl + RL, ...; the RL partial sums of a column are added
// in shared memory, then one atomic per column and block.
__device__ __forceinline__ void unpack16(const uint4& u, const float*, float x[4]) {
  x[0] = __uint_as_float(u.x);
  x[1] = __uint_as_float(u.y);
  x[2] = __uint_as_float(u.z);
  x[3] = __uint_as_float(u.w);
}
__device__ __forceinline__ void unpack16(const uint4& u, const __nv_bfloat16*, float x[8]) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 f = __bfloat1622float2(h[i]);
    x[2 * i] = f.x;
    x[2 * i + 1] = f.y;
  }
}
__device__ __forceinline__ uint4 pack16(const float x[4], const float*) {
  return make_uint4(__float_as_uint(x[0]), __float_as_uint(x[1]), __float_as_uint(x[2]), __float_as_uint(x[3]));
}
__device__ __forceinline__ uint4 pack16(const float x[8], const __nv_bfloat16*) {
  uint32_t w[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x[2 * i], x[2 * i + 1]);
    w[i] = *reinterpret_cast<const uint32_t*>(&h);
  }
  return make_uint4(w[0], w[1], w[2], w[3]);
}

constexpr int VEC_ROWS_PER_BLOCK = 256;

template <typename T, bool RELU>
__global__ void relu_bwd_colsum_vec_kernel(const T* __restrict__ dh, const T* __restrict__ h, int64_t M, int N,
                                           T* __restrict__ dz, float* __restrict__ colsum) {
  constexpr int PER = 16 / (int)sizeof(T);
  extern __shared__ float part[];  // [RL][N]
  const int G = N / PER, RL = blockDim.x / G;
  const int tid = threadIdx.x, rl = tid / G, g = tid % G;
  float s[PER];
#pragma unroll
  for (int e = 0; e < PER; ++e) s[e] = 0.f;
  if (rl < RL) {
    const int64_t r0 = (int64_t)blockIdx.x * VEC_ROWS_PER_BLOCK;
    const int64_t r1 = min(r0 + VEC_ROWS_PER_BLOCK, M);
    for (int64_t r = r0 + rl; r < r1; r += RL) {
      const int64_t i = r * (N / PER) + g;
      float v[PER];
      unpack16(__ldg(reinterpret_cast<const uint4*>(dh) + i), dh, v);
      if (RELU) {
        float hv[PER];
        unpack16(__ldg(reinterpret_cast<const uint4*>(h) + i), h, hv);
#pragma unroll
        for (int e = 0; e < PER; ++e) v[e] = hv[e] > 0.f ? v[e] : 0.f;
        reinterpret_cast<uint4*>(dz)[i] = pack16(v, dz);
      }
#pragma unroll
      for (int e = 0; e < PER; ++e) s[e] += v[e];
    }
#pragma unroll
    for (int e = 0; e < PER; ++e) part[rl * N + g * PER + e] = s[e];
  }
  __syncthreads();
  for (int c = tid; c < N; c += blockDim.x) {
    float acc = 0.f;
    for (int q = 0; q < RL; ++q) acc += part[q * N + c];
    atomicAdd(colsum + c, acc);
  }
}

// Backward of the 3-output layer of a colour MLP fused with the ReLU backward
// of the hidden layer feeding it (out = W h + b, h = relu(.)):
//   dW[j][c] += sum_rows g_j h_c,  db[j] += sum_rows g_j,
//   dz_c = (h_c > 0) * sum_j g_j W[j][c],  db_prev[c] += sum_rows dz_c.
// g = dout [M,3] FP32; h, dz [M,N] (T); W [3,N] FP32.  Replaces three GEMMs
// with a 3-wide dimension (which map to slow unaligned kernels), a ReLU
// backward and a bias reduction.  Rows in 16-byte chunks as the kernel above.
constexpr int HEAD_MAX_N = 256;

template <typename T>
__global__ void head_backward_kernel(const float* __restrict__ dout, const T* __restrict__ h,
                                     const float* __restrict__ W, int64_t M, int N, T* __restrict__ dz,
                                     float* __restrict__ dW, float* __restrict__ db, float* __restrict__ db_prev) {
  constexpr int PER = 16 / (int)sizeof(T);
  extern __shared__ float sh[];  // W [3][N] | partials [RL][4][N] | db partials [RL][3]
  const int G = N / PER, RL = blockDim.x / G;
  const int tid = threadIdx.x, rl = tid / G, g = tid % G;
  float* Ws = sh;
  float* part = sh + 3 * N;
  float* dbp = part + (size_t)RL * 4 * N;
  for (int i = tid; i < 3 * N; i += blockDim.x) Ws[i] = W[i];
  __syncthreads();
  float w[3][PER], aw[3][PER], ab[PER], a3[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int e = 0; e < PER; ++e) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      w[j][e] = Ws[j * N + g * PER + e];
      aw[j][e] = 0.f;
    }
    ab[e] = 0.f;
  }
  if (rl < RL) {
    const int64_t r0 = (int64_t)blockIdx.x * VEC_ROWS_PER_BLOCK;
    const int64_t r1 = min(r0 + VEC_ROWS_PER_BLOCK, M);
    for (int64_t r = r0 + rl; r < r1; r += RL) {
      const float g0 = dout[3 * r], g1 = dout[3 * r + 1], g2 = dout[3 * r + 2];
      const int64_t i = r * (N / PER) + g;
      float hv[PER], d[PER];
      unpack16(__ldg(reinterpret_cast<const uint4*>(h) + i), h, hv);
#pragma unroll
      for (int e = 0; e < PER; ++e) {
        aw[0][e] += g0 * hv[e];
        aw[1][e] += g1 * hv[e];
        aw[2][e] += g2 * hv[e];
        const float dh = g0 * w[0][e] + g1 * w[1][e] + g2 * w[2][e];
        d[e] = hv[e] > 0.f ? dh : 0.f;
        ab[e] += d[e];
      }
      reinterpret_cast<uint4*>(dz)[i] = pack16(d, dz);
      if (g == 0) {
        a3[0] += g0;
        a3[1] += g1;
        a3[2] += g2;
      }
    }
#pragma unroll
    for (int e = 0; e < PER; ++e) {
      const int c = g * PER + e;
#pragma unroll
      for (int j = 0; j < 3; ++j) part[((size_t)rl * 4 + j) * N + c] = aw[j][e];
      part[((size_t)rl * 4 + 3) * N + c] = ab[e];
    }
    if (g == 0) {
      dbp[3 * rl + 0] = a3[0];
      dbp[3 * rl + 1] = a3[1];
      dbp[3 * rl + 2] = a3[2];
    }
  }
  __syncthreads();
  for (int k = tid; k < 4 * N; k += blockDim.x) {
    const int j = k / N, c = k % N;
    float acc = 0.f;
    for (int q = 0; q < RL; ++q) acc += part[((size_t)q * 4 + j) * N + c];
    if (j < 3)
      atomicAdd(dW + j * N + c, acc);
    else
      atomicAdd(db_prev + c, acc);
  }
  if (tid < 3) {
    float acc = 0.f;
    for (int q = 0; q < RL; ++q) acc += dbp[3 * q + tid];
    atomicAdd(db + tid, acc);
  }
}

}  // namespace vx

namespace vx {

// Several FP32 -> BF16 row-block copies in one launch (the per-step casts of
// the colour-MLP weights and biases in the mixed-precision step).  Block b
// belongs to the job whose [first_block, first_block + blocks) holds b.
struct CastJobs {
  vx_cast_job job[VX_CAST_MAX_JOBS];
  int first_block[VX_CAST_MAX_JOBS + 1];
  int n;
};

__global__ void __launch_bounds__(256) cast_rows_bf16_kernel(const CastJobs J) {
  int j = 0;
  while (j + 1 < J.n && (int)blockIdx.x >= J.first_block[j + 1]) ++j;
  const vx_cast_job& c = J.job[j];
  const int64_t i = (int64_t)(blockIdx.x - J.first_block[j]) * blockDim.x + threadIdx.x;
  if (i >= (int64_t)c.rows * c.cols) return;
  const int64_t r = i / c.cols, k = i - r * c.cols;
  reinterpret_cast<__nv_bfloat16*>(c.dst)[r * c.dst_ld + k] = __float2bfloat16_rn(c.src[r * c.src_ld + k]);
}

}  // namespace vx

using namespace vx;

extern "C" {

int vx_cast_rows_bf16(const vx_cast_job* jobs_host, int32_t n_jobs, void* stream) {
  if (n_jobs < 0 || n_jobs > VX_CAST_MAX_JOBS || (n_jobs > 0 && !jobs_host)) return VX_ERR_ARG;
  CastJobs J{};
  int blocks = 0;
  for (int j = 0; j < n_jobs; ++j) {
    const vx_cast_job& c = jobs_host[j];
    if (c.rows < 0 || c.cols < 0 || c.src_ld < c.cols || c.dst_ld < c.cols) return VX_ERR_ARG;
    if (c.rows > 0 && c.cols > 0 && (!c.src || !c.dst)) return VX_ERR_ARG;
    J.job[j] = c;
    J.first_block[j] = blocks;
    blocks += (int)((((int64_t)c.rows * c.cols) + 255) / 256);
  }
  J.first_block[n_jobs] = blocks;
  J.n = n_jobs;
  if (blocks == 0) return VX_OK;
  cast_rows_bf16_kernel<<<blocks, 256, 0, as_stream(stream)>>>(J);
  return launch_status();
}


int vx_mlp_head_backward(const float* dout, const void* h, const float* W, int64_t M, int64_t N, int dtype, void* dz,
                         float* dW, float* db, float* db_prev, void* stream) {
  if (M < 0 || N <= 0 || N > HEAD_MAX_N || (dtype != 0 && dtype != 1)) return VX_ERR_ARG;
  if (!dW || !db || !db_prev || !W) return VX_ERR_ARG;
  if (M == 0) return VX_OK;
  if (!dout || !h || !dz) return VX_ERR_ARG;
  const int per = dtype == 0 ? 4 : 8;
  if (N % per || ((reinterpret_cast<uintptr_t>(h) | reinterpret_cast<uintptr_t>(dz)) & 15)) return VX_ERR_UNSUPPORTED;
  const int G = (int)(N / per), RL = 256 / G, threads = RL * G;
  const size_t shm = ((size_t)3 * N + (size_t)RL * 4 * N + 3 * RL) * sizeof(float);
  const unsigned blocks = (unsigned)((M + VEC_ROWS_PER_BLOCK - 1) / VEC_ROWS_PER_BLOCK);
  cudaStream_t st = as_stream(stream);
  if (dtype == 0)
    head_backward_kernel<float><<<blocks, threads, shm, st>>>(dout, (const float*)h, W, M, (int)N, (float*)dz, dW, db,
                                                              db_prev);
  else
    head_backward_kernel<__nv_bfloat16><<<blocks, threads, shm, st>>>(
        dout, (const __nv_bfloat16*)h, W, M, (int)N, (__nv_bfloat16*)dz, dW, db, db_prev);
  return launch_status();
}

// dtype: 0 float32, 1 bfloat16 (dh, h, dz).  h == NULL: no ReLU (dz unused),
// only the column sums.  colsum [N] is accumulated (callers zero it).
int vx_relu_bwd_colsum(const void* dh, const void* h, int64_t M, int64_t N, int dtype, void* dz, float* colsum,
                       void* stream) {
  if (M < 0 || N <= 0 || N > INT32_MAX || !colsum || (dtype != 0 && dtype != 1)) return VX_ERR_ARG;
  if (M == 0) return VX_OK;
  if (!dh || (h && !dz)) return VX_ERR_ARG;
  {
    const int per = dtype == 0 ? 4 : 8;
    const uintptr_t al = reinterpret_cast<uintptr_t>(dh) | reinterpret_cast<uintptr_t>(h) |
                         reinterpret_cast<uintptr_t>(dz);
    const int G = (int)(N / per);
    if (N % per == 0 && (al & 15) == 0 && G <= 256) {
      const int RL = 256 / G;  // row lanes per block
      const int threads = RL * G;
      const size_t shm = (size_t)RL * N * sizeof(float);
      if (shm <= 48 * 1024) {
        const unsigned vb = (unsigned)((M + VEC_ROWS_PER_BLOCK - 1) / VEC_ROWS_PER_BLOCK);
        cudaStream_t vst = as_stream(stream);
        using B = __nv_bfloat16;
        if (dtype == 0) {
          if (h)
            relu_bwd_colsum_vec_kernel<float, true><<<vb, threads, shm, vst>>>((const float*)dh, (const float*)h, M,
                                                                                (int)N, (float*)dz, colsum);
          else
            relu_bwd_colsum_vec_kernel<float, false><<<vb, threads, shm, vst>>>((const float*)dh, nullptr, M, (int)N,
                                                                                 nullptr, colsum);
        } else {
          if (h)
            relu_bwd_colsum_vec_kernel<B, true><<<vb, threads, shm, vst>>>((const B*)dh, (const B*)h, M, (int)N,
                                                                            (B*)dz, colsum);
          else
            relu_bwd_colsum_vec_kernel<B, false><<<vb, threads, shm, vst>>>((const B*)dh, nullptr, M, (int)N,
                                                                             nullptr, colsum);
        }
        return launch_status();
      }
    }
  }
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
