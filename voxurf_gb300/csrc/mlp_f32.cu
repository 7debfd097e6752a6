// Colour-MLP training in plain FP32 on the CUDA cores: the hidden layers of
// rgbnet / k_rgbnet (lib/voxurf_fine.py:132-187) and of the coarse rgbnet
// (lib/voxurf_coarse.py:116-123), forward and backward, with FP32 operands
// and FP32 fused multiply-adds (the arithmetic of the reference's FP32
// nn.Linear under autograd).  The 3-wide output layer has kernels of its own
// (vx_mlp_head, vx_mlp_head_backward in mlp_ops.cu).
//
//   rowgemm_kernel   C[m][n] = sum_k A[m][k] Bt[k][n] over a 64-row tile and
//                    all N columns (N = 16 TN), with one of three epilogues:
//                    +bias and ReLU (forward), times the ReLU mask of the
//                    layer's activation plus per-CTA column sums (backward,
//                    hidden layer), none (backward, input gradient).  Bt is
//                    the layer's weight, transposed or not, zero-padded to
//                    [Kp][Np] by vx_mlp_train_pack (mode 3).
//   wgrad_kernel     D[m][n] = sum over a CTA's rows of A[r][m] B[r][n] (the
//                    weight gradient dz^T h, summed over rows), one FP32
//                    partial per CTA; vx_mlp_f32_reduce sums the partials in a
//                    fixed order.
#include <algorithm>

#include "common.cuh"

namespace vx {
namespace mf {

constexpr int BM = 64;       // rows per rowgemm tile
constexpr int KC = 16;       // K per shared-memory stage
constexpr int THREADS = 256; // 16 x 16 threads

struct RowGemmParams {
  const float* A;            // [M, lda]
  int64_t lda;
  int64_t M;
  const int64_t* m_dev;      // optional device row count (<= M)
  int K;                     // columns of A used
  const float* Bt;           // [Kp][Np] (Kp = round_up(K, 16), zero rows beyond K)
  int Np;
  int mode;                  // 0: relu(acc + bias); 1: acc * [H > 0] + column sums; 2: acc
  const float* bias;         // mode 0: [Np]
  const float* H;            // mode 1: [M, ldh] post-ReLU activation of the layer
  int64_t ldh;
  float* C;                  // [M, ldc], columns < n_store
  int64_t ldc;
  int n_store;
  float* colsum;             // mode 1: [gridDim.x][Np] per-CTA column sums
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// 16-byte asynchronous global -> shared copy, zero fill beyond src_bytes.
__device__ __forceinline__ void cp16(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ int64_t rows_of(int64_t n, const int64_t* n_dev) {
  if (n_dev) {
    const int64_t d = *n_dev;
    if (d < n) n = d < 0 ? 0 : d;
  }
  return n;
}

// 4-byte asynchronous copy (rows whose stride is not a multiple of 4 floats).
__device__ __forceinline__ void cp4(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_addr(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
template <int N>
__device__ __forceinline__ void cp_wait_group() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

constexpr int RG_STAGES = 3;   // shared-memory ring of the row GEMM
constexpr int AS_LD = KC + 4;  // A stage row stride (floats): 16-byte rows, no bank conflicts

// A 64-row tile of C = A Bt: each thread owns 4 rows x TN columns.  Stages of
// KC columns of A ([64][KC] row-major) and KC rows of Bt ([KC][NP]) arrive by
// cp.async in a three-deep ring, so the copies of the next two stages are in
// flight while one is computed; A is read as float4 along k (one load per 4
// k steps and row), Bt as float4 along n.
template <int TN>
__global__ void __launch_bounds__(THREADS, 2) rowgemm_kernel(RowGemmParams P) {
  constexpr int NP = 16 * TN;
  // dynamic shared memory: the A ring, the Bt ring; the column-sum scratch of
  // the epilogue reuses the A ring
  extern __shared__ __align__(16) float rg_smem[];
  auto As = reinterpret_cast<float (*)[BM][AS_LD]>(rg_smem);
  auto Bs = reinterpret_cast<float (*)[KC][NP]>(rg_smem + RG_STAGES * BM * AS_LD);
  auto red = reinterpret_cast<float (*)[NP]>(rg_smem);
  static_assert(16 * NP <= RG_STAGES * BM * AS_LD, "column-sum scratch fits the A ring");
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t M = rows_of(P.M, P.m_dev);
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  if (m0 >= M && P.mode != 1) return;
  const int nk = (P.K + KC - 1) / KC;
  const bool avec = (P.lda & 3) == 0 && (reinterpret_cast<uintptr_t>(P.A) & 15) == 0;

  auto load_stage = [&](int kt, int slot) {
    const int k0 = kt * KC;
    if (avec) {
      // 64 rows x 4 pieces of 16 bytes: one piece per thread
      const int r = tid >> 2, c = 4 * (tid & 3);
      const int64_t row = m0 + r;
      const int valid = (row < M) ? max(0, min(4, P.K - (k0 + c))) : 0;
      cp16(&As[slot][r][c], valid ? P.A + row * P.lda + k0 + c : P.A, (uint32_t)(4 * valid));
    } else {
      for (int i = tid; i < BM * KC; i += THREADS) {
        const int r = i / KC, c = i % KC;
        const int64_t row = m0 + r;
        const bool ok = row < M && k0 + c < P.K;
        cp4(&As[slot][r][c], ok ? P.A + row * P.lda + k0 + c : P.A, ok ? 4u : 0u);
      }
    }
    const float* src = P.Bt + (int64_t)kt * KC * NP;
    float* dst = &Bs[slot][0][0];
    for (int i = tid; i < KC * NP / 4; i += THREADS) cp16(dst + 4 * i, src + 4 * i, 16u);
  };

  float acc[4][TN];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;

#pragma unroll
  for (int s = 0; s < RG_STAGES - 1; ++s) {
    if (s < nk) load_stage(s, s);
    cp_commit();
  }
  for (int kt = 0; kt < nk; ++kt) {
    cp_wait_group<RG_STAGES - 2>();   // stage kt has landed (this thread's copies)
    __syncthreads();                  // ... everyone's; slot (kt - 1) % S is free
    if (kt + RG_STAGES - 1 < nk) load_stage(kt + RG_STAGES - 1, (kt + RG_STAGES - 1) % RG_STAGES);
    cp_commit();
    const int slot = kt % RG_STAGES;
#pragma unroll
    for (int k = 0; k < KC; k += 4) {
      float a[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float4 v = *reinterpret_cast<const float4*>(&As[slot][4 * ty + i][k]);
        a[i][0] = v.x; a[i][1] = v.y; a[i][2] = v.z; a[i][3] = v.w;
      }
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        float b[TN];
        if constexpr (TN % 4 == 0) {
#pragma unroll
          for (int j = 0; j < TN / 4; ++j) {
            const float4 b4 = *reinterpret_cast<const float4*>(&Bs[slot][k + kk][TN * tx + 4 * j]);
            b[4 * j] = b4.x; b[4 * j + 1] = b4.y; b[4 * j + 2] = b4.z; b[4 * j + 3] = b4.w;
          }
        } else {
#pragma unroll
          for (int j = 0; j < TN; ++j) b[j] = Bs[slot][k + kk][TN * tx + j];
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i][kk], b[j], acc[i][j]);
      }
    }
  }
  cp_wait_group<0>();
  // epilogue
  float cs[TN];
#pragma unroll
  for (int j = 0; j < TN; ++j) cs[j] = 0.f;
  const int n0 = TN * tx;
  const bool cvec = (P.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(P.C) & 15) == 0;
  const bool hvec = P.mode == 1 && (P.ldh & 3) == 0 && (reinterpret_cast<uintptr_t>(P.H) & 15) == 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t m = m0 + 4 * ty + i;
    if (m >= M) continue;
    float v[TN];
#pragma unroll
    for (int j = 0; j < TN; ++j) v[j] = acc[i][j];
    if (P.mode == 0) {
#pragma unroll
      for (int j = 0; j < TN; ++j) v[j] = fmaxf(v[j] + __ldg(P.bias + n0 + j), 0.f);
    } else if (P.mode == 1) {
      const float* hrow = P.H + m * P.ldh + n0;
      bool done = false;
      if constexpr (TN % 4 == 0) {
        if (hvec) {
#pragma unroll
          for (int j = 0; j < TN; j += 4) {
            const float4 h = __ldg(reinterpret_cast<const float4*>(hrow + j));
            v[j] = h.x > 0.f ? v[j] : 0.f;
            v[j + 1] = h.y > 0.f ? v[j + 1] : 0.f;
            v[j + 2] = h.z > 0.f ? v[j + 2] : 0.f;
            v[j + 3] = h.w > 0.f ? v[j + 3] : 0.f;
          }
          done = true;
        }
      }
      if (!done) {
#pragma unroll
        for (int j = 0; j < TN; ++j) v[j] = hrow[j] > 0.f ? v[j] : 0.f;
      }
#pragma unroll
      for (int j = 0; j < TN; ++j) cs[j] += v[j];
    }
    float* crow = P.C + m * P.ldc;
    bool stored = false;
    if constexpr (TN % 4 == 0) {
      if (n0 + TN <= P.n_store && cvec) {
#pragma unroll
        for (int j = 0; j < TN; j += 4)
          *reinterpret_cast<float4*>(crow + n0 + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
        stored = true;
      }
    }
    if (!stored) {
#pragma unroll
      for (int j = 0; j < TN; ++j)
        if (n0 + j < P.n_store) crow[n0 + j] = v[j];
    }
  }
  if (P.mode == 1) {
    __syncthreads();   // every thread is done with the A ring
#pragma unroll
    for (int j = 0; j < TN; ++j) red[ty][n0 + j] = cs[j];
    __syncthreads();
    for (int n = tid; n < NP; n += THREADS) {
      float s = 0.f;
      for (int r = 0; r < 16; ++r) s += red[r][n];
      P.colsum[(int64_t)blockIdx.x * NP + n] = s;
    }
  }
}

// ---------------------------------------------------------------------------
struct WgradParams {
  const float* A;            // [rows, lda] (dz of the layer's output), columns < M
  int64_t lda;
  const float* B;            // [rows, ldb] (the layer's input), columns < N
  int64_t ldb;
  int M, N;                  // N <= 16 TN, M <= 16 TM
  int64_t rows;
  const int64_t* rows_dev;
  float* part;               // [gridDim.x][16 TM][16 TN]
};

constexpr int WG_KC = 16;    // rows per stage

template <int TM, int TN>
__global__ void __launch_bounds__(THREADS, 1) wgrad_kernel(WgradParams P) {
  constexpr int MP = 16 * TM, NP = 16 * TN;
  __shared__ __align__(16) float As[2][WG_KC][MP];
  __shared__ __align__(16) float Bs[2][WG_KC][NP];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t rows = rows_of(P.rows, P.rows_dev);
  // this CTA's rows: a contiguous range, in stages of WG_KC
  const int64_t per = (rows + gridDim.x - 1) / gridDim.x;
  const int64_t r0 = std::min<int64_t>(rows, (int64_t)blockIdx.x * per);
  const int64_t r1 = std::min<int64_t>(rows, r0 + per);
  const int nst = (int)((r1 - r0 + WG_KC - 1) / WG_KC);

  // rows of A and B -> the stage, 16-byte asynchronous pieces (zero past the
  // CTA's rows and past M / N) when the rows are 16-byte aligned, otherwise
  // plain element copies
  const bool vec = (P.lda & 3) == 0 && (P.ldb & 3) == 0 && ((reinterpret_cast<uintptr_t>(P.A) |
                                                              reinterpret_cast<uintptr_t>(P.B)) & 15) == 0;
  auto load = [&](int st, int s) {
    const int64_t rb = r0 + (int64_t)st * WG_KC;
    if (vec) {
      for (int i = tid; i < WG_KC * MP / 4; i += THREADS) {
        const int rr = i / (MP / 4), c = 4 * (i % (MP / 4));
        const int64_t r = rb + rr;
        const int valid = (r < r1) ? max(0, min(4, P.M - c)) : 0;
        cp16(&As[s][rr][c], valid ? P.A + r * P.lda + c : P.A, (uint32_t)(4 * valid));
      }
      for (int i = tid; i < WG_KC * NP / 4; i += THREADS) {
        const int rr = i / (NP / 4), c = 4 * (i % (NP / 4));
        const int64_t r = rb + rr;
        const int valid = (r < r1) ? max(0, min(4, P.N - c)) : 0;
        cp16(&Bs[s][rr][c], valid ? P.B + r * P.ldb + c : P.B, (uint32_t)(4 * valid));
      }
      cp_commit();
      return;
    }
    for (int i = tid; i < WG_KC * MP; i += THREADS) {
      const int rr = i / MP, c = i % MP;
      const int64_t r = rb + rr;
      As[s][rr][c] = (r < r1 && c < P.M) ? P.A[r * P.lda + c] : 0.f;
    }
    for (int i = tid; i < WG_KC * NP; i += THREADS) {
      const int rr = i / NP, c = i % NP;
      const int64_t r = rb + rr;
      Bs[s][rr][c] = (r < r1 && c < P.N) ? P.B[r * P.ldb + c] : 0.f;
    }
  };

  float acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;
  if (nst > 0) load(0, 0);
  cp_wait_all();
  __syncthreads();
  for (int st = 0; st < nst; ++st) {
    const int s = st & 1;
    if (st + 1 < nst) load(st + 1, s ^ 1);   // lands while this stage is computed
#pragma unroll 4
    for (int k = 0; k < WG_KC; ++k) {
      float a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[s][k][TM * ty + i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[s][k][TN * tx + j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    cp_wait_all();
    __syncthreads();
  }
  float* part = P.part + (size_t)blockIdx.x * MP * NP;
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) part[(TM * ty + i) * NP + TN * tx + j] = acc[i][j];
}

struct SumJob {
  const float* part;         // [n_part][part_stride], element (m, n) at m * part_ld + n
  int64_t n_part, part_stride, part_ld;
  int64_t rows, cols;
  float* out;                // out[m * out_ld + n]
  int64_t out_ld;
};
constexpr int MAX_SUM_JOBS = 16;
struct SumJobs {
  SumJob j[MAX_SUM_JOBS];
  int n;
};

// A block of 256 threads sums 32 consecutive outputs (lane = output): warp w
// adds the partials of its contiguous eighth of k, then the eight warp sums
// are added in warp order.  The order is fixed, so the result does not
// depend on timing.
__global__ void __launch_bounds__(256) sum_partials_kernel(SumJobs J) {
  const SumJob& S = J.j[blockIdx.y];
  __shared__ float red[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t total = S.rows * S.cols;
  const int64_t per = (S.n_part + 7) / 8, k0 = per * warp, k1 = min(S.n_part, k0 + per);
  for (int64_t base = (int64_t)blockIdx.x * 32; base < total; base += (int64_t)gridDim.x * 32) {
    const int64_t i = base + lane;
    float s = 0.f;
    if (i < total) {
      const int64_t m = i / S.cols, n = i % S.cols;
      const float* p = S.part + m * S.part_ld + n;
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
      int64_t k = k0;
      for (; k + 4 <= k1; k += 4) {
        a0 += p[k * S.part_stride];
        a1 += p[(k + 1) * S.part_stride];
        a2 += p[(k + 2) * S.part_stride];
        a3 += p[(k + 3) * S.part_stride];
      }
      for (; k < k1; ++k) a0 += p[k * S.part_stride];
      s = (a0 + a1) + (a2 + a3);
    }
    red[warp][lane] = s;
    __syncthreads();
    if (warp == 0 && i < total) {
      float t = 0.f;
      for (int w = 0; w < 8; ++w) t += red[w][lane];
      const int64_t m = i / S.cols, n = i % S.cols;
      S.out[m * S.out_ld + n] = t;
    }
    __syncthreads();
  }
}

}  // namespace mf
}  // namespace vx

using namespace vx;
using namespace vx::mf;

extern "C" {

size_t vx_mlp_f32_rowgemm_grid(int64_t M) { return (size_t)std::max<int64_t>(1, (M + BM - 1) / BM); }

int vx_mlp_f32_rowgemm(const vx_mlp_f32_rowgemm_args* a, void* stream) {
  if (!a || a->M < 0 || a->K < 1 || !a->Bt) return VX_ERR_ARG;
  // rows of an empty batch may have no storage (null pointers)
  if (a->M > 0 && (!a->A || !a->C || (a->mode == 1 && !a->H))) return VX_ERR_ARG;
  if (a->mode < 0 || a->mode > 2 || a->lda < a->K || a->n_store < 1 || a->n_store > a->Np || a->ldc < a->n_store)
    return VX_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(a->Bt) & 15) || (a->mode == 0 && !a->bias) ||
      (a->mode == 1 && (!a->colsum || a->ldh < a->Np ||
                        a->colsum_cap < (int64_t)vx_mlp_f32_rowgemm_grid(a->M) * a->Np)))
    return VX_ERR_ARG;
  if (a->M == 0 && a->mode != 1) return VX_OK;   // mode 1 still writes its (zero) column sums
  RowGemmParams P{};
  P.A = a->A;
  P.lda = a->lda;
  P.M = a->M;
  P.m_dev = a->m_dev;
  P.K = (int)a->K;
  P.Bt = a->Bt;
  P.Np = (int)a->Np;
  P.mode = a->mode;
  P.bias = a->bias;
  P.H = a->H;
  P.ldh = a->ldh;
  P.C = a->C;
  P.ldc = a->ldc;
  P.n_store = (int)a->n_store;
  P.colsum = a->colsum;
  const unsigned grid = (unsigned)vx_mlp_f32_rowgemm_grid(a->M);
  cudaStream_t st = as_stream(stream);
  auto launch = [&](auto kernel, int np) -> int {
    const size_t smem = sizeof(float) * ((size_t)RG_STAGES * BM * AS_LD + (size_t)RG_STAGES * KC * np);
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
    kernel<<<grid, THREADS, smem, st>>>(P);
    return launch_status();
  };
  switch (a->Np) {
    case 32: return launch(rowgemm_kernel<2>, 32);
    case 64: return launch(rowgemm_kernel<4>, 64);
    case 80: return launch(rowgemm_kernel<5>, 80);
    case 128: return launch(rowgemm_kernel<8>, 128);
    case 192: return launch(rowgemm_kernel<12>, 192);
    default: return VX_ERR_UNSUPPORTED;
  }
}

size_t vx_mlp_f32_wgrad_grid(int64_t rows) {
  // at least 256 rows per CTA, at most one CTA per SM
  return (size_t)std::max<int64_t>(1, std::min<int64_t>(sm_count(), (rows + 255) / 256));
}

int vx_mlp_f32_wgrad(const vx_mlp_f32_wgrad_args* a, void* stream) {
  if (!a || a->rows < 0 || !a->part || a->M < 1 || a->N < 1 || a->lda < a->M || a->ldb < a->N) return VX_ERR_ARG;
  if (a->rows > 0 && (!a->A || !a->B)) return VX_ERR_ARG;   // an empty batch writes zero partials
  auto pad = [](int64_t x) -> int64_t { return x <= 32 ? 32 : x <= 64 ? 64 : x <= 80 ? 80 : x <= 128 ? 128 : x <= 192 ? 192 : -1; };
  const int64_t MP = pad(a->M), NP = pad(a->N);
  if (MP < 0 || NP < 0) return VX_ERR_UNSUPPORTED;
  const unsigned grid = (unsigned)vx_mlp_f32_wgrad_grid(a->rows);
  if (a->part_cap < (int64_t)grid * MP * NP) return VX_ERR_ARG;
  WgradParams P{};
  P.A = a->A;
  P.lda = a->lda;
  P.B = a->B;
  P.ldb = a->ldb;
  P.M = (int)a->M;
  P.N = (int)a->N;
  P.rows = a->rows;
  P.rows_dev = a->rows_dev;
  P.part = a->part;
  cudaStream_t st = as_stream(stream);
#define VX_WG(TM_, TN_)                                            \
  if (MP == 16 * TM_ && NP == 16 * TN_) {                          \
    wgrad_kernel<TM_, TN_><<<grid, THREADS, 0, st>>>(P);           \
    return launch_status();                                        \
  }
  VX_WG(12, 12) VX_WG(12, 5) VX_WG(12, 4) VX_WG(8, 8) VX_WG(8, 5) VX_WG(8, 4) VX_WG(4, 4) VX_WG(4, 5) VX_WG(2, 2)
  VX_WG(2, 5) VX_WG(2, 4) VX_WG(4, 2)
#undef VX_WG
  return VX_ERR_UNSUPPORTED;
}

int vx_mlp_f32_reduce(const vx_mlp_sum_job* jobs, int n_jobs, void* stream) {
  if (!jobs || n_jobs < 1 || n_jobs > MAX_SUM_JOBS) return VX_ERR_ARG;
  SumJobs J{};
  for (int i = 0; i < n_jobs; ++i) {
    const vx_mlp_sum_job& s = jobs[i];
    if (!s.part || !s.out || s.n_part < 1 || s.rows < 1 || s.cols < 1 || s.part_ld < s.cols || s.out_ld < s.cols)
      return VX_ERR_ARG;
    J.j[i] = SumJob{s.part, s.n_part, s.part_stride, s.part_ld, s.rows, s.cols, s.out, s.out_ld};
  }
  J.n = n_jobs;
  int64_t most = 1;
  for (int i = 0; i < n_jobs; ++i) most = std::max<int64_t>(most, jobs[i].rows * jobs[i].cols);
  dim3 grid((unsigned)std::min<int64_t>((most + 31) / 32, 2048), (unsigned)n_jobs);
  sum_partials_kernel<<<grid, 256, 0, as_stream(stream)>>>(J);
  return launch_status();
}

}  // extern "C"
