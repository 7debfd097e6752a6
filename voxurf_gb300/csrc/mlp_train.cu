// Colour-MLP training on the 5th-generation tensor cores (tcgen05), BF16
// operands with FP32 accumulation: the rgbnet / k_rgbnet stacks of
// lib/voxurf_fine.py:132-187 and the coarse rgbnet of
// lib/voxurf_coarse.py:116-123 (Linear -> ReLU x L, then a 3-wide output
// layer), forward and backward, as run by torch autograd in the reference
// (voxurf_fine.py:718-752 under run.py:615's loss.backward()).
//
//   h_1 = relu(X W_0^T + b_0),  h_{l+1} = relu(h_l W_l^T + b_l),  y = h_L Wh^T + bh
//   dz_L = (dy Wh) * [h_L > 0],  dz_l = (dz_{l+1} W_l) * [h_l > 0],  dX = dz_1 W_0
//   dW_l = dz_{l+1}^T h_l,  db_l = sum_rows dz_{l+1},  dWh = dy^T h_L,  dbh = sum_rows dy
//
// Four kernels, all persistent over 128-row tiles:
//   mlp_fwd_kernel    forward; hidden activations stay in tensor memory
//                     between layers and also leave, per tile, as "T-tiles"
//                     (below) plus one ReLU bit per element;
//   mlp_bwd_kernel    the input-gradient chain: dz_L on the CUDA cores from
//                     dy, Wh and the ReLU bits, then one MMA per layer with
//                     A = dz in tensor memory; writes each dz_l as T-tiles
//                     and dX as rows;
//   mlp_wgrad_kernel  one weight gradient (D = A^T B summed over rows) per
//                     launch: A and B tiles arrive by bulk copy (two stages),
//                     the MMA reads both MN-major, the sum over a CTA's rows
//                     stays in tensor memory, and an extra N=16 MMA against
//                     a ones tile gives the bias gradient; one FP32 partial
//                     per CTA;
//   mlp_reduce_kernel the partials of all CTAs summed in a fixed order (the
//                     result does not depend on timing).
//
// T-tile: the rows [128 t, 128 t + 128) of a [rows, C] BF16 matrix as 16 x
// (C/8) core matrices of 8 rows x 8 columns, K-chunk (8 rows) major:
//   element (r, c) of tile t at  t*128*C + ((r/8)*(C/8) + c/8)*64 + (r%8)*8 + c%8.
// It is the MN-major operand layout of a GEMM whose K dimension is the rows
// (LBO = C*16 bytes, SBO = 128 bytes), so the weight-gradient kernel loads a
// whole tile with one bulk copy; a producer thread that owns a row writes
// 16-byte pieces, and the 8 threads of 8 consecutive rows fill one 128-byte
// line.
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "tcgen05.cuh"

namespace vx {
namespace mt {

using namespace tc;
using bf16 = __nv_bfloat16;

constexpr int TM = 128;             // rows per tile (one cta_group::1 MMA)
constexpr int EPI_WARPS = 8;        // warps w, w + 4 share TMEM lanes 32 (w % 4) ..
constexpr int THREADS = 32 * (EPI_WARPS + 1);   // + the MMA warp
constexpr int MAX_K0 = 80;

// Epilogue hand-off: a layer's W output columns are converted in STEPS
// steps of SW columns; the two threads of a row take CPW columns each.
template <int W>
struct Geo {
  static constexpr int STEPS = W >= 64 ? W / 64 : 1;
  static constexpr int SW = W / STEPS;
  static constexpr int CPW = SW / 2;
  static constexpr int KPS = SW / 16;   // MMA K steps per hand-off step
  static_assert(W % 32 == 0 && W <= 192, "hidden width");
  static_assert(CPW == 32 || CPW == 16, "epilogue split");
};

__host__ __device__ inline int64_t tt_off(int r, int c, int C) {
  return ((int64_t)((r >> 3) * (C >> 3) + (c >> 3)) << 6) + ((r & 7) << 3) + (c & 7);
}

__host__ __device__ inline uint32_t tmem_cols_for(int need) {
  uint32_t c = 32;
  while ((int)c < need) c <<= 1;
  return c;
}

__device__ __forceinline__ int64_t rows_of(int64_t n, const int64_t* n_dev) {
  if (n_dev) {
    const int64_t d = *n_dev;
    if (d < n) n = d < 0 ? 0 : d;
  }
  return n;
}

// K-major A tile in shared memory ([K/8][128][8]) x K-major B ([K/8][N][8]):
// MMAs of K steps [ks0, ks1).
__device__ __forceinline__ void mma_rows_ss(uint32_t d, uint32_t a_s, uint32_t b_s, int N, int ks0, int ks1,
                                            bool acc_first) {
  const uint32_t id = idesc(TM, N);
  for (int ks = ks0; ks < ks1; ++ks) {
    const uint64_t ad = desc(a_s + (uint32_t)(2 * ks) * (TM * 16), TM * 16, 128);
    const uint64_t bd = desc(b_s + (uint32_t)(2 * ks) * (uint32_t)(N * 16), (uint32_t)(N * 16), 128);
    mma_ss(d, ad, bd, id, acc_first || ks > 0);
  }
}

// A in tensor memory (8 columns per K step of 16), B K-major in shared memory.
__device__ __forceinline__ void mma_rows_ts(uint32_t d, uint32_t a_t, uint32_t b_s, int N, int ks0, int ks1) {
  const uint32_t id = idesc(TM, N);
  for (int ks = ks0; ks < ks1; ++ks) {
    const uint64_t bd = desc(b_s + (uint32_t)(2 * ks) * (uint32_t)(N * 16), (uint32_t)(N * 16), 128);
    mma_ts(d, a_t + (uint32_t)(8 * ks), bd, id, ks > 0);
  }
}

// ============================================================================
// Forward
// ============================================================================
struct FwdParams {
  const bf16* X;          // [n, ldx] rows, columns [K0, ldx) ignored (zero weights)
  int64_t ldx;
  int K0;                 // multiple of 16, <= MAX_K0
  int64_t n_rows;
  const int64_t* n_rows_dev;  // optional device row count (<= n_rows)
  const bf16* W0p;        // [K0/8][W][8]
  const bf16* Wp;         // hidden layers 1..L-1, [W/8][W][8] each, back to back
  const float* bias;      // [L][W]
  const bf16* Whp;        // [W/8][16][8]: output rows 0-2 hi, 3-5 lo parts
  const float* bh;        // [3]
  float* out;             // [n, 3] logits
  bf16* cols;             // optional BF16 copy of the logits at cols[row * ld_cols + 0..2]
  int64_t ld_cols;
  bf16* H;                // optional: T-tiles of h_1..h_L, h_l at (l-1) * h_stride
  uint16_t* relu;         // optional: ReLU bits [L][rows_cap][W/16]
  int64_t h_stride, relu_stride;
  int* err;
};

template <int W>
__device__ __forceinline__ void load_rows_tile(const bf16* X, int64_t ldx, int K0, int64_t n, bf16* Xs, int64_t row0,
                                               int tid, int nthreads) {
  const int chunks = K0 / 8;
  for (int i = tid; i < chunks * TM; i += nthreads) {
    const int c = i / TM, r = i % TM;
    const bool in = row0 + r < n;
    const bf16* src = X + (in ? (row0 + r) * ldx + 8 * c : 0);
    cp_async16(Xs + ((size_t)c * TM + r) * 8, src, in ? 16u : 0u);
  }
  cp_async_commit();
}

// Pipeline per tile (one tile in flight per CTA):
//   MMA warp:   layer 0 (A = X tile, shared memory) -> ACC0, commit bar_acc;
//               layers 1..L-1 -> ACC(l % 2) and the output layer -> HEAD:
//               for each hand-off step s, wait bar_a[s], issue its K steps;
//               commit.
//   epilogues:  per hidden layer: wait bar_acc; per step: tcgen05.ld, +bias,
//               ReLU, BF16 -> A operand (tcgen05.st) [-> T-tile + ReLU bits];
//               arrive bar_a[s].  Then the logits of the output layer.
template <int W, int L>
__global__ void __launch_bounds__(THREADS, 1) mlp_fwd_kernel(FwdParams P, uint32_t tmem_cols) {
  using G = Geo<W>;
  extern __shared__ __align__(1024) uint8_t smem[];
  const int K0 = P.K0;
  bf16* W0s = reinterpret_cast<bf16*>(smem);
  bf16* Ws = W0s + (size_t)K0 * W;                       // (L-1) x [W/8][W][8]
  bf16* Xs = Ws + (size_t)(L - 1) * W * W;               // [K0/8][128][8]
  bf16* WHs = Xs + (size_t)K0 * TM;                      // [W/8][16][8]
  float* bias_s = reinterpret_cast<float*>(WHs + (size_t)16 * W);   // [L][W]
  uint64_t* bar_w = reinterpret_cast<uint64_t*>(bias_s + L * W);
  uint64_t* bar_acc = bar_w + 1;
  uint64_t* bar_head = bar_w + 2;
  uint64_t* bar_x = bar_w + 3;
  uint64_t* bar_fin = bar_w + 4;
  uint64_t* bar_a = bar_w + 5;   // [STEPS]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_a + G::STEPS);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool mma_warp = warp == EPI_WARPS;
  const int quarter = warp & 3, part = (warp >> 2) & 1;
  const int epi_threads = 32 * EPI_WARPS;
  const int64_t n = rows_of(P.n_rows, P.n_rows_dev);
  const int64_t n_tiles = (n + TM - 1) / TM;
  const uint32_t ACC[2] = {0u, (uint32_t)W};
  const uint32_t TA = 2 * W, THEAD = 2 * W + W / 2;
  if (warp == 0) alloc(tmem_slot, tmem_cols);
  if (tid == 0) {
    mbar_init(bar_w, 1);
    mbar_init(bar_acc, 1);
    mbar_init(bar_head, 1);
    mbar_init(bar_x, EPI_WARPS);
    mbar_init(bar_fin, 1);
    for (int s = 0; s < G::STEPS; ++s) mbar_init(bar_a + s, EPI_WARPS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    const uint32_t w0b = (uint32_t)K0 * W * 2, wb = (uint32_t)W * W * 2, whb = 16u * W * 2, bb = (uint32_t)L * W * 4;
    mbar_expect_tx(bar_w, w0b + (L - 1) * wb + whb + bb);
    bulk_g2s(W0s, P.W0p, w0b, bar_w);
    for (int l = 0; l < L - 1; ++l) bulk_g2s(Ws + (size_t)l * W * W, P.Wp + (size_t)l * W * W, wb, bar_w);
    bulk_g2s(WHs, P.Whp, whb, bar_w);
    bulk_g2s(bias_s, P.bias, bb, bar_w);
  }
  if (!mma_warp && blockIdx.x < n_tiles) {
    load_rows_tile<W>(P.X, P.ldx, K0, n, Xs, (int64_t)blockIdx.x * TM, tid, epi_threads);
    cp_async_wait_all();
    fence_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(bar_x);
  }
  bool ok = mbar_wait(bar_w, 0);
  const float bh0 = __ldg(P.bh + 0), bh1 = __ldg(P.bh + 1), bh2 = __ldg(P.bh + 2);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t tmem_row = tmem + ((uint32_t)(32 * quarter) << 16);
  const uint32_t x_s = smem_u32(Xs), w0_s = smem_u32(W0s), ws_s = smem_u32(Ws), wh_s = smem_u32(WHs);

  if (mma_warp) {
    uint32_t ph_x = 0, ph_a = 0;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
      ok = mbar_wait(bar_x, ph_x);
      ph_x ^= 1u;
      fence_after();
      if (!ok) break;
      if (lane == 0) {
        mma_rows_ss(tmem + ACC[0], x_s, w0_s, W, 0, K0 / 16, false);
        commit(bar_acc);
      }
      __syncwarp();
#pragma unroll 1
      for (int layer = 1; layer <= L && ok; ++layer) {
        const bool head = layer == L;
        const uint32_t d = head ? THEAD : ACC[layer & 1];
        const uint32_t b = head ? wh_s : ws_s + (uint32_t)(layer - 1) * W * W * 2;
        const int N = head ? 16 : W;
#pragma unroll 1
        for (int s = 0; s < G::STEPS; ++s) {
          ok = mbar_wait(bar_a + s, ph_a);
          fence_after();
          if (!ok) break;
          if (lane == 0) mma_rows_ts(tmem + d, tmem + TA, b, N, G::KPS * s, G::KPS * (s + 1));
          __syncwarp();
        }
        ph_a ^= 1u;
        if (ok && lane == 0) commit(head ? bar_head : bar_acc);
        __syncwarp();
      }
    }
    if (lane == 0) {
      commit(bar_fin);
      if (!mbar_wait(bar_fin, 0)) ok = false;
    }
    __syncwarp();
  } else {
    uint32_t ph_acc = 0, ph_head = 0;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
      const int r = 32 * quarter + lane;             // row in the tile
      const int64_t row = tile * TM + r;
#pragma unroll 1
      for (int layer = 0; layer < L; ++layer) {
        ok = mbar_wait(bar_acc, ph_acc);
        ph_acc ^= 1u;
        fence_after();
        if (!ok) break;
        if (layer == 0) {
          const int64_t next = tile + gridDim.x;     // the X tile is consumed: prefetch the next one
          if (next < n_tiles) load_rows_tile<W>(P.X, P.ldx, K0, n, Xs, next * TM, tid, epi_threads);
        }
        const uint32_t acc = ACC[layer & 1];
        const float* bl = bias_s + layer * W;
        bf16* Ht = P.H ? P.H + layer * P.h_stride + tile * (int64_t)TM * W : nullptr;
        uint16_t* rl = P.relu ? P.relu + layer * P.relu_stride + row * (W / 16) : nullptr;
#pragma unroll 1
        for (int s = 0; s < G::STEPS; ++s) {
          const int col0 = G::SW * s + G::CPW * part;
          uint32_t v[G::CPW];
          ld_cols<G::CPW>(tmem_row + acc + (uint32_t)col0, v);
          uint32_t pk[G::CPW / 2];
          uint32_t bits = 0;
#pragma unroll
          for (int q = 0; q < G::CPW / 4; ++q) {
            const float4 bq = *reinterpret_cast<const float4*>(bl + col0 + 4 * q);
            const float h0 = fmaxf(__uint_as_float(v[4 * q + 0]) + bq.x, 0.f);
            const float h1 = fmaxf(__uint_as_float(v[4 * q + 1]) + bq.y, 0.f);
            const float h2 = fmaxf(__uint_as_float(v[4 * q + 2]) + bq.z, 0.f);
            const float h3 = fmaxf(__uint_as_float(v[4 * q + 3]) + bq.w, 0.f);
            pk[2 * q] = pack_bf16(h0, h1);
            pk[2 * q + 1] = pack_bf16(h2, h3);
            // ReLU bit of the stored (BF16) activation
            bits |= (uint32_t)((pk[2 * q] & 0x7FFFu) != 0) << (4 * q);
            bits |= (uint32_t)((pk[2 * q] & 0x7FFF0000u) != 0) << (4 * q + 1);
            bits |= (uint32_t)((pk[2 * q + 1] & 0x7FFFu) != 0) << (4 * q + 2);
            bits |= (uint32_t)((pk[2 * q + 1] & 0x7FFF0000u) != 0) << (4 * q + 3);
          }
          st_cols<G::CPW / 2>(tmem_row + TA + (uint32_t)(col0 / 2), pk);
          if (Ht) {
#pragma unroll
            for (int q = 0; q < G::CPW / 8; ++q)
              *reinterpret_cast<uint4*>(Ht + tt_off(r, col0 + 8 * q, W)) =
                  make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
          }
          if (rl) {
            if constexpr (G::CPW == 32) *reinterpret_cast<uint32_t*>(rl + col0 / 16) = bits;
            else rl[col0 / 16] = (uint16_t)bits;
          }
          wait_st();
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(bar_a + s);
        }
        if (layer == L - 1) {
          cp_async_wait_all();     // the next X tile (if any) is in shared memory
          fence_async_smem();
          __syncwarp();
          if (lane == 0) mbar_arrive(bar_x);
        }
      }
      if (!ok) break;
      if (part == 0) {
        ok = mbar_wait(bar_head, ph_head);
        fence_after();
        if (!ok) break;
        uint32_t hv[16];
        ld_cols<16>(tmem_row + THEAD, hv);
        if (row < n) {
          const float a0 = (__uint_as_float(hv[0]) + __uint_as_float(hv[3])) + bh0;
          const float a1 = (__uint_as_float(hv[1]) + __uint_as_float(hv[4])) + bh1;
          const float a2 = (__uint_as_float(hv[2]) + __uint_as_float(hv[5])) + bh2;
          P.out[3 * row + 0] = a0;
          P.out[3 * row + 1] = a1;
          P.out[3 * row + 2] = a2;
          if (P.cols) {
            bf16* cp = P.cols + row * P.ld_cols;
            cp[0] = __float2bfloat16_rn(a0);
            cp[1] = __float2bfloat16_rn(a1);
            cp[2] = __float2bfloat16_rn(a2);
          }
        }
        fence_before();
      }
      ph_head ^= 1u;
    }
    cp_async_wait_all();
  }
  if (!ok) set_device_error(P.err, VX_ERR_TIMEOUT);
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    dealloc(tmem, tmem_cols);
  }
}

// ============================================================================
// Backward: input-gradient chain
// ============================================================================
struct BwdParams {
  const float* dY;        // [n, 3]
  int64_t n_rows;
  const int64_t* n_rows_dev;
  const float* Wh;        // [3][W] output-layer weights (FP32)
  const uint16_t* relu;   // [L][rows_cap][W/16] ReLU bits of h_1..h_L
  int64_t relu_stride;
  const bf16* WTp;        // hidden layers 1..L-1 transposed: layer l at (l-1) W W, [W/8][W][8] of B[n=in][k=out]
  const bf16* W0Tp;       // [W/8][K0][8] of B[n=in][k=out]
  int K0;
  bf16* dZ;               // T-tiles of dz_1..dz_L, dz_l at (l-1) * dz_stride
  int64_t dz_stride;
  bf16* dYT;              // T-tiles (width 16) of [dy hi (3), dy lo (3), 0 ...]
  void* dX;               // [n, ld_dx] (columns < K0 written), BF16 or FP32
  int64_t ld_dx;
  int dx_bf16;
  float* dbh_part;        // [gridDim.x][4]: this CTA's column sums of dy
  int* err;
};

template <int W, int L>
__global__ void __launch_bounds__(THREADS, 1) mlp_bwd_kernel(BwdParams P, uint32_t tmem_cols) {
  using G = Geo<W>;
  extern __shared__ __align__(1024) uint8_t smem[];
  const int K0 = P.K0;
  const int AW = W > K0 ? W : K0;                    // accumulator width
  bf16* WTs = reinterpret_cast<bf16*>(smem);         // (L-1) x [W/8][W][8]
  bf16* W0Ts = WTs + (size_t)(L - 1) * W * W;        // [W/8][K0][8]
  float* Wh_s = reinterpret_cast<float*>(W0Ts + (size_t)K0 * W);   // [3][W]
  float* dbh_s = Wh_s + 3 * W;                       // [4 warps][4]
  uint64_t* bar_w = reinterpret_cast<uint64_t*>(dbh_s + 16);
  uint64_t* bar_acc = bar_w + 1;
  uint64_t* bar_fin = bar_w + 2;
  uint64_t* bar_a = bar_w + 3;   // [STEPS]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_a + G::STEPS);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool mma_warp = warp == EPI_WARPS;
  const int quarter = warp & 3, part = (warp >> 2) & 1;
  const int64_t n = rows_of(P.n_rows, P.n_rows_dev);
  const int64_t n_tiles = (n + TM - 1) / TM;
  const uint32_t ACC[2] = {0u, (uint32_t)AW};
  const uint32_t TA = 2 * AW;
  if (warp == 0) alloc(tmem_slot, tmem_cols);
  if (tid == 0) {
    mbar_init(bar_w, 1);
    mbar_init(bar_acc, 1);
    mbar_init(bar_fin, 1);
    for (int s = 0; s < G::STEPS; ++s) mbar_init(bar_a + s, EPI_WARPS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    const uint32_t wb = (uint32_t)W * W * 2, w0b = (uint32_t)K0 * W * 2, hb = 3u * W * 4;
    mbar_expect_tx(bar_w, (L - 1) * wb + w0b + hb);
    for (int l = 0; l < L - 1; ++l) bulk_g2s(WTs + (size_t)l * W * W, P.WTp + (size_t)l * W * W, wb, bar_w);
    bulk_g2s(W0Ts, P.W0Tp, w0b, bar_w);
    bulk_g2s(Wh_s, P.Wh, hb, bar_w);
  }
  bool ok = mbar_wait(bar_w, 0);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t tmem_row = tmem + ((uint32_t)(32 * quarter) << 16);
  const uint32_t wt_s = smem_u32(WTs), w0t_s = smem_u32(W0Ts);

  if (mma_warp) {
    uint32_t ph_a = 0;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
#pragma unroll 1
      for (int i = 0; i < L && ok; ++i) {
        // backward MMA i: dz_{L-i} (A, tensor memory) x W_{L-1-i} -> ACC(i % 2)
        const bool last = i == L - 1;
        const uint32_t b = last ? w0t_s : wt_s + (uint32_t)(L - 2 - i) * W * W * 2;
        const int N = last ? K0 : W;
#pragma unroll 1
        for (int s = 0; s < G::STEPS; ++s) {
          ok = mbar_wait(bar_a + s, ph_a);
          fence_after();
          if (!ok) break;
          if (lane == 0) mma_rows_ts(tmem + ACC[i & 1], tmem + TA, b, N, G::KPS * s, G::KPS * (s + 1));
          __syncwarp();
        }
        ph_a ^= 1u;
        if (ok && lane == 0) commit(bar_acc);
        __syncwarp();
      }
    }
    if (lane == 0) {
      commit(bar_fin);
      if (!mbar_wait(bar_fin, 0)) ok = false;
    }
    __syncwarp();
  } else {
    uint32_t ph_acc = 0;
    float sy0 = 0.f, sy1 = 0.f, sy2 = 0.f;    // this thread's rows' dy sums (part 0)
    const int r = 32 * quarter + lane;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
      const int64_t row = tile * TM + r;
      const bool live = row < n;
      // ---- output layer: dz_L = (dy Wh) * [h_L > 0] on the CUDA cores ----
      float y0 = 0.f, y1 = 0.f, y2 = 0.f;
      if (live) {
        y0 = P.dY[3 * row + 0];
        y1 = P.dY[3 * row + 1];
        y2 = P.dY[3 * row + 2];
      }
      if (part == 0) {
        sy0 += y0;
        sy1 += y1;
        sy2 += y2;
        // dy as BF16 hi + lo parts for the output layer's weight gradient
        const bf16 h0 = __float2bfloat16_rn(y0), h1 = __float2bfloat16_rn(y1), h2 = __float2bfloat16_rn(y2);
        const bf16 l0 = __float2bfloat16_rn(y0 - __bfloat162float(h0));
        const bf16 l1 = __float2bfloat16_rn(y1 - __bfloat162float(h1));
        const bf16 l2 = __float2bfloat16_rn(y2 - __bfloat162float(h2));
        __align__(16) bf16 c8[8] = {h0, h1, h2, l0, l1, l2, __float2bfloat16_rn(0.f), __float2bfloat16_rn(0.f)};
        bf16* yt = P.dYT + tile * (int64_t)TM * 16;
        *reinterpret_cast<uint4*>(yt + tt_off(r, 0, 16)) = *reinterpret_cast<const uint4*>(c8);
        *reinterpret_cast<uint4*>(yt + tt_off(r, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
      }
      {
        const uint16_t* rl = P.relu + (L - 1) * P.relu_stride + row * (W / 16);
        bf16* Zt = P.dZ + (L - 1) * P.dz_stride + tile * (int64_t)TM * W;
#pragma unroll 1
        for (int s = 0; s < G::STEPS; ++s) {
          const int col0 = G::SW * s + G::CPW * part;
          uint32_t bits = 0;
          if (live) {
            if constexpr (G::CPW == 32) bits = *reinterpret_cast<const uint32_t*>(rl + col0 / 16);
            else bits = rl[col0 / 16];
          }
          uint32_t pk[G::CPW / 2];
#pragma unroll
          for (int q = 0; q < G::CPW / 2; ++q) {
            const int c = col0 + 2 * q;
            float g0 = y0 * Wh_s[c] + y1 * Wh_s[W + c] + y2 * Wh_s[2 * W + c];
            float g1 = y0 * Wh_s[c + 1] + y1 * Wh_s[W + c + 1] + y2 * Wh_s[2 * W + c + 1];
            g0 = ((bits >> (2 * q)) & 1u) ? g0 : 0.f;
            g1 = ((bits >> (2 * q + 1)) & 1u) ? g1 : 0.f;
            pk[q] = pack_bf16(g0, g1);
          }
          st_cols<G::CPW / 2>(tmem_row + TA + (uint32_t)(col0 / 2), pk);
#pragma unroll
          for (int q = 0; q < G::CPW / 8; ++q)
            *reinterpret_cast<uint4*>(Zt + tt_off(r, col0 + 8 * q, W)) =
                make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
          wait_st();
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(bar_a + s);
        }
      }
      // ---- hidden layers and the input gradient ----
#pragma unroll 1
      for (int i = 0; i < L; ++i) {
        ok = mbar_wait(bar_acc, ph_acc);
        ph_acc ^= 1u;
        fence_after();
        if (!ok) break;
        const uint32_t acc = ACC[i & 1];
        if (i < L - 1) {
          const int l = L - 1 - i;      // dz_l = (dz_{l+1} W_l) * [h_l > 0]
          const uint16_t* rl = P.relu + (l - 1) * P.relu_stride + row * (W / 16);
          bf16* Zt = P.dZ + (l - 1) * P.dz_stride + tile * (int64_t)TM * W;
#pragma unroll 1
          for (int s = 0; s < G::STEPS; ++s) {
            const int col0 = G::SW * s + G::CPW * part;
            uint32_t v[G::CPW];
            ld_cols<G::CPW>(tmem_row + acc + (uint32_t)col0, v);
            uint32_t bits = 0;
            if (live) {
              if constexpr (G::CPW == 32) bits = *reinterpret_cast<const uint32_t*>(rl + col0 / 16);
              else bits = rl[col0 / 16];
            }
            uint32_t pk[G::CPW / 2];
#pragma unroll
            for (int q = 0; q < G::CPW / 2; ++q) {
              const float g0 = ((bits >> (2 * q)) & 1u) ? __uint_as_float(v[2 * q]) : 0.f;
              const float g1 = ((bits >> (2 * q + 1)) & 1u) ? __uint_as_float(v[2 * q + 1]) : 0.f;
              pk[q] = pack_bf16(g0, g1);
            }
            st_cols<G::CPW / 2>(tmem_row + TA + (uint32_t)(col0 / 2), pk);
#pragma unroll
            for (int q = 0; q < G::CPW / 8; ++q)
              *reinterpret_cast<uint4*>(Zt + tt_off(r, col0 + 8 * q, W)) =
                  make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
            wait_st();
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar_a + s);
          }
        } else {
          // dX = dz_1 W_0: this thread's half of the K0 columns, 8 at a time
          const int half = K0 / 2;
          for (int c0 = half * part; c0 < half * (part + 1); c0 += 8) {
            uint32_t v[8];
            ld_cols<8>(tmem_row + acc + (uint32_t)c0, v);
            if (live) {
              if (P.dx_bf16) {
                bf16* dst = reinterpret_cast<bf16*>(P.dX) + row * P.ld_dx + c0;
                *reinterpret_cast<uint4*>(dst) = make_uint4(
                    pack_bf16(__uint_as_float(v[0]), __uint_as_float(v[1])),
                    pack_bf16(__uint_as_float(v[2]), __uint_as_float(v[3])),
                    pack_bf16(__uint_as_float(v[4]), __uint_as_float(v[5])),
                    pack_bf16(__uint_as_float(v[6]), __uint_as_float(v[7])));
              } else {
                float* dst = reinterpret_cast<float*>(P.dX) + row * P.ld_dx + c0;
                *reinterpret_cast<uint4*>(dst) = make_uint4(v[0], v[1], v[2], v[3]);
                *reinterpret_cast<uint4*>(dst + 4) = make_uint4(v[4], v[5], v[6], v[7]);
              }
            }
          }
          fence_before();
        }
      }
    }
    if (part == 0) {
      sy0 = warp_sum(sy0);
      sy1 = warp_sum(sy1);
      sy2 = warp_sum(sy2);
      if (lane == 0) {
        dbh_s[4 * quarter + 0] = sy0;
        dbh_s[4 * quarter + 1] = sy1;
        dbh_s[4 * quarter + 2] = sy2;
      }
    }
  }
  if (!ok) set_device_error(P.err, VX_ERR_TIMEOUT);
  fence_before();
  __syncthreads();
  if (tid < 3) {   // fixed order over the four lane quarters
    P.dbh_part[4 * blockIdx.x + tid] = ((dbh_s[tid] + dbh_s[4 + tid]) + dbh_s[8 + tid]) + dbh_s[12 + tid];
  }
  if (warp == 0) {
    fence_after();
    dealloc(tmem, tmem_cols);
  }
}

// ============================================================================
// Weight gradient: D[m][n] = sum_rows A[row][m] B[row][n]  (+ ones: sum_rows A[row][m])
// ============================================================================
struct WgradParams {
  const bf16* A;          // T-tiles of width WA
  int WA;                 // multiple of 16, <= 256
  const bf16* B;          // T-tiles of width WB, or (b_rows) rows [n, ldb]
  int WB;                 // multiple of 16, <= 240
  int64_t ldb;
  int b_rows;
  int ones;               // 1: 16 more columns, column WB holds sum_rows A[row][m]
  int64_t n_rows;
  const int64_t* n_rows_dev;
  float* part;            // [gridDim.x][WA][WB + 16 ones]
  int* err;
};

// Several passes in one launch: CTAs [cta0[p], cta0[p+1]) run pass p (the
// passes of one or more MLPs stream their tiles side by side).
constexpr int MAX_WG_PASSES = 8;
struct WgradPasses {
  WgradParams p[MAX_WG_PASSES];
  int cta0[MAX_WG_PASSES + 1];
  int n;
};

constexpr int WG_LOADERS = 4;                    // warps 0-3: loads, write-out
constexpr int WG_THREADS = 32 * (WG_LOADERS + 1);
constexpr uint32_t WG_TAIL = 2048;               // readable bytes after each A stage (M-tile rows past WA)

__host__ __device__ inline size_t wg_a_bytes(int WA) { return (size_t)TM * WA * 2 + WG_TAIL; }
__host__ __device__ inline size_t wg_b_bytes(int WB) { return (size_t)TM * WB * 2; }

__global__ void __launch_bounds__(WG_THREADS, 1) mlp_wgrad_kernel(const __grid_constant__ WgradPasses PS) {
  extern __shared__ __align__(1024) uint8_t smem[];
  int pi = 0;
  while (pi + 1 < PS.n && PS.cta0[pi + 1] <= (int)blockIdx.x) ++pi;
  const WgradParams& P = PS.p[pi];
  const int cta = (int)blockIdx.x - PS.cta0[pi], n_cta = PS.cta0[pi + 1] - PS.cta0[pi];
  const int WA = P.WA, WB = P.WB;
  const int MT = (WA + TM - 1) / TM;
  const int NC = WB + (P.ones ? 16 : 0);
  const uint32_t tmem_cols = tmem_cols_for(MT * NC);
  const size_t ab = wg_a_bytes(WA), bbytes = wg_b_bytes(WB);
  uint8_t* As[2] = {smem, smem + ab};
  uint8_t* Bs[2] = {smem + 2 * ab, smem + 2 * ab + bbytes};
  bf16* ones_s = reinterpret_cast<bf16*>(smem + 2 * ab + 2 * bbytes);   // K-major [16][16][8], 4 KB
  uint64_t* bar_full = reinterpret_cast<uint64_t*>(ones_s + 16 * 16 * 8);   // [2]
  uint64_t* bar_empty = bar_full + 2;                                    // [2]
  uint64_t* bar_done = bar_full + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_full + 5);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool mma_warp = warp == WG_LOADERS;
  const int64_t n = rows_of(P.n_rows, P.n_rows_dev);
  const int64_t n_tiles = (n + TM - 1) / TM;
  if (warp == 0) alloc(tmem_slot, tmem_cols);
  // the ones tile: B[n][k] = 1 for n = 0
  for (int i = tid; i < 16 * 16 * 8; i += blockDim.x) {
    const int nn = (i >> 3) & 15;
    ones_s[i] = __float2bfloat16_rn(nn == 0 ? 1.f : 0.f);
  }
  // zero the tails past each A stage (read by the last M-tile's rows >= WA)
  for (int s = 0; s < 2; ++s)
    for (int i = tid; i < (int)(WG_TAIL / 16); i += blockDim.x)
      reinterpret_cast<uint4*>(As[s] + (size_t)TM * WA * 2)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    const uint32_t full_count = 1 + (P.b_rows ? WG_LOADERS : 0);
    for (int s = 0; s < 2; ++s) {
      mbar_init(bar_full + s, full_count);
      mbar_init(bar_empty + s, 1);
    }
    mbar_init(bar_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_async_smem();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;
  bool ok = true;
  int64_t done_tiles = 0;

  if (!mma_warp) {
    // ---- producers: tile t of this CTA into stage t % 2 ----
    int64_t t = 0;
    for (int64_t tile = cta; tile < n_tiles && ok; tile += n_cta, ++t) {
      const int s = (int)(t & 1);
      if (t >= 2) {
        ok = mbar_wait(bar_empty + s, (uint32_t)(((t >> 1) - 1) & 1));
        if (!ok) break;
      }
      if (tid == 0) {
        const uint32_t abytes = (uint32_t)TM * WA * 2;
        const uint32_t bb = P.b_rows ? 0u : (uint32_t)bbytes;
        mbar_expect_tx(bar_full + s, abytes + bb);
        bulk_g2s(As[s], P.A + tile * (int64_t)TM * WA, abytes, bar_full + s);
        if (!P.b_rows) bulk_g2s(Bs[s], P.B + tile * (int64_t)TM * WB, bb, bar_full + s);
      }
      if (P.b_rows) {
        // rows [n, ldb] -> T-tile layout, 16-byte pieces, zero past the last row
        const int chunks = WB / 8;
        bf16* dst = reinterpret_cast<bf16*>(Bs[s]);
        for (int i = tid; i < chunks * TM; i += 32 * WG_LOADERS) {
          const int rr = i / chunks, c = i % chunks;
          const int64_t row = tile * TM + rr;
          const bool in = row < n;
          const bf16* src = P.B + (in ? row * P.ldb + 8 * c : 0);
          cp_async16(dst + tt_off(rr, 8 * c, WB), src, in ? 16u : 0u);
        }
        cp_async_commit();
        cp_async_wait_all();
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(bar_full + s);
      }
    }
  } else {
    // ---- MMA warp ----
    const uint32_t a_lbo = (uint32_t)WA * 16, b_lbo = (uint32_t)WB * 16;
    const uint32_t id_w = idesc(TM, WB, 1, 1), id_1 = idesc(TM, 16, 1, 0);
    const uint32_t ones_a = smem_u32(ones_s);
    int64_t t = 0;
    for (int64_t tile = cta; tile < n_tiles && ok; tile += n_cta, ++t) {
      const int s = (int)(t & 1);
      ok = mbar_wait(bar_full + s, (uint32_t)((t >> 1) & 1));
      fence_after();
      if (!ok) break;
      if (lane == 0) {
        const uint32_t a_s = smem_u32(As[s]), b_s = smem_u32(Bs[s]);
        for (int mt = 0; mt < MT; ++mt) {
          const uint32_t d = tmem + (uint32_t)(mt * NC);
          for (int ks = 0; ks < TM / 16; ++ks) {
            const bool acc = t > 0 || ks > 0;
            const uint64_t ad = desc(a_s + (uint32_t)(2 * ks) * a_lbo + (uint32_t)mt * 16 * 128, a_lbo, 128);
            const uint64_t bd = desc(b_s + (uint32_t)(2 * ks) * b_lbo, b_lbo, 128);
            mma_ss(d, ad, bd, id_w, acc);
            if (P.ones) {
              const uint64_t od = desc(ones_a + (uint32_t)(2 * ks) * 256, 256, 128);
              mma_ss(d + (uint32_t)WB, ad, od, id_1, acc);
            }
          }
        }
        commit(bar_empty + s);
      }
      __syncwarp();
      ++done_tiles;
    }
    if (lane == 0) commit(bar_done);
    __syncwarp();
  }
  // ---- write-out: D rows (lane = m) of each M-tile ----
  if (!mma_warp) {
    const bool any = cta < n_tiles;
    bool okd = true;
    if (any) {
      okd = mbar_wait(bar_done, 0);
      fence_after();
    }
    float* part = P.part + (size_t)cta * WA * NC;
    for (int mt = 0; mt < MT && okd; ++mt) {
      const int m = mt * TM + 32 * warp + lane;
      const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(mt * NC);
      for (int c0 = 0; c0 < NC; c0 += 16) {
        uint32_t v[16];
        if (any) ld_cols<16>(trow + (uint32_t)c0, v);
        else
          for (int i = 0; i < 16; ++i) v[i] = 0u;
        if (m < WA) {
          float* dst = part + (size_t)m * NC + c0;
#pragma unroll
          for (int q = 0; q < 4; ++q)
            *reinterpret_cast<uint4*>(dst + 4 * q) = make_uint4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
      }
    }
    if (!okd) ok = false;
    fence_before();
  }
  if (!ok) set_device_error(P.err, VX_ERR_TIMEOUT);
  __syncthreads();
  if (warp == 0) {
    fence_after();
    dealloc(tmem, tmem_cols);
  }
  (void)done_tiles;
}

// ============================================================================
// Ordered sum of the per-CTA partials into FP32 weight / bias gradients
// ============================================================================
struct ReduceJob {
  const float* part;      // [n_part][WA][NC]
  int n_part;
  int WA, NC;
  int kind;               // 0: hidden / input layer: W[m][n] (n < n_out), b[m] = col WB
                          // 1: output layer: Wh[c][m] = D[m][c] + D[m][c+3] (c < 3)
  int WB;                 // kind 0: the ones column index
  int n_out;              // kind 0: columns written (real input width)
  float* w;               // kind 0: [WA][n_out]; kind 1: [3][WA]
  float* b;               // kind 0: [WA]; kind 1: [3] (from dbh partials)
  const float* bh_part;   // kind 1: [n_bh][4]
  int n_bh;
};

constexpr int MAX_REDUCE_JOBS = 8;
struct ReduceJobs {
  ReduceJob j[MAX_REDUCE_JOBS];
  int n;
};

// Sum over the n_part partials of D[m][col] (col < NC): a block of 256
// threads sums 32 consecutive outputs, warp w taking its contiguous eighth
// of the partials; the eight warp sums are added in warp order (a fixed
// order: the result does not depend on timing).
__device__ __forceinline__ float sum_parts(const float* p, int64_t stride, int n_part, int warp) {
  const int per = (n_part + 7) / 8, k0 = per * warp, k1 = min(n_part, k0 + per);
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
  int k = k0;
  for (; k + 4 <= k1; k += 4) {
    a0 += p[k * stride];
    a1 += p[(k + 1) * stride];
    a2 += p[(k + 2) * stride];
    a3 += p[(k + 3) * stride];
  }
  for (; k < k1; ++k) a0 += p[k * stride];
  return (a0 + a1) + (a2 + a3);
}

__global__ void __launch_bounds__(256) mlp_reduce_kernel(ReduceJobs J) {
  const ReduceJob& R = J.j[blockIdx.y];
  __shared__ float red[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t stride = (int64_t)R.WA * R.NC;
  // outputs: kind 0: WA x (n_out + 1) (weights, then the bias column);
  //          kind 1: 3 x WA weights, then 3 biases (from the dy partials)
  const int64_t total = R.kind == 0 ? (int64_t)R.WA * (R.n_out + 1) : (int64_t)3 * R.WA + 3;
  for (int64_t base = (int64_t)blockIdx.x * 32; base < total; base += (int64_t)gridDim.x * 32) {
    const int64_t i = base + lane;
    float s = 0.f;
    if (i < total) {
      if (R.kind == 0) {
        const int m = (int)(i / (R.n_out + 1)), c = (int)(i % (R.n_out + 1));
        const int col = c < R.n_out ? c : R.WB;
        s = sum_parts(R.part + (int64_t)m * R.NC + col, stride, R.n_part, warp);
      } else if (i < 3 * R.WA) {
        const int c = (int)(i / R.WA), m = (int)(i % R.WA);
        const float* p = R.part + (int64_t)m * R.NC;
        s = sum_parts(p + c, stride, R.n_part, warp) + sum_parts(p + c + 3, stride, R.n_part, warp);
      } else {
        s = sum_parts(R.bh_part + (i - 3 * R.WA), 4, R.n_bh, warp);
      }
    }
    red[warp][lane] = s;
    __syncthreads();
    if (warp == 0 && i < total) {
      float t = 0.f;
      for (int w = 0; w < 8; ++w) t += red[w][lane];
      if (R.kind == 0) {
        const int m = (int)(i / (R.n_out + 1)), c = (int)(i % (R.n_out + 1));
        if (c < R.n_out) R.w[(int64_t)m * R.n_out + c] = t;
        else R.b[m] = t;
      } else if (i < 3 * R.WA) {
        const int c = (int)(i / R.WA), m = (int)(i % R.WA);
        R.w[(int64_t)c * R.WA + m] = t;
      } else {
        R.b[i - 3 * R.WA] = t;
      }
    }
    __syncthreads();
  }
}

// ============================================================================
// Weight packing (one launch for every operand of a step)
// ============================================================================
struct PackJob {
  const float* src;       // row-major FP32, row stride ld
  int64_t ld;
  int N, K;               // mode 0: B[n][k] for n < N, k < K (zero beyond); mode 2: [N][K] copy
  int Np, Kp;             // mode 0/1: packed extents [Kp/8][Np][8]
  int transpose;          // mode 0: 0 -> B[n][k] = src[n][k]; 1 -> B[n][k] = src[k][n]
  int mode;               // 0: BF16 pack; 1: output layer as hi/lo rows (0-2 hi, 3-5 lo, rest 0); 2: FP32 copy;
                          // 3: FP32 [Kp][Np] of Bt[k][n] = src[n][k] (transpose 1) or src[k][n] (0)
  void* dst;
};
constexpr int MAX_PACK_JOBS = 32;
struct PackJobs {
  PackJob j[MAX_PACK_JOBS];
  int n;
};

__global__ void mlp_pack_kernel(PackJobs J) {
  const PackJob& Q = J.j[blockIdx.y];
  if (Q.mode == 2) {
    const int64_t total = (int64_t)Q.N * Q.K;
    float* dst = reinterpret_cast<float*>(Q.dst);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
      dst[i] = Q.src[(i / Q.K) * Q.ld + i % Q.K];
    return;
  }
  if (Q.mode == 3) {
    const int64_t total = (int64_t)Q.Kp * Q.Np;
    float* dst = reinterpret_cast<float*>(Q.dst);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
      const int k = (int)(i / Q.Np), nn = (int)(i % Q.Np);
      float v = 0.f;
      if (nn < Q.N && k < Q.K) v = Q.transpose ? Q.src[(int64_t)nn * Q.ld + k] : Q.src[(int64_t)k * Q.ld + nn];
      dst[i] = v;
    }
    return;
  }
  bf16* dst = reinterpret_cast<bf16*>(Q.dst);
  const int64_t total = (int64_t)Q.Np * Q.Kp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(i & 7), nn = (int)((i >> 3) % Q.Np), kc = (int)(i / (8 * (int64_t)Q.Np));
    const int k = 8 * kc + e;
    float v = 0.f;
    if (Q.mode == 1) {
      if (nn < 6 && k < Q.K) {
        const float x = Q.src[(int64_t)(nn % 3) * Q.ld + k];
        const float hi = __bfloat162float(__float2bfloat16_rn(x));
        v = nn < 3 ? hi : x - hi;
      }
    } else if (nn < Q.N && k < Q.K) {
      v = Q.transpose ? Q.src[(int64_t)k * Q.ld + nn] : Q.src[(int64_t)nn * Q.ld + k];
    }
    dst[i] = __float2bfloat16_rn(v);
  }
}

// ---------------------------------------------------------------------------
template <int W, int L>
size_t fwd_smem(int K0) {
  return (size_t)K0 * W * 2 + (size_t)(L - 1) * W * W * 2 + (size_t)K0 * TM * 2 + 16u * W * 2 + (size_t)L * W * 4 +
         (5 + Geo<W>::STEPS) * 8 + 8;
}
template <int W, int L>
size_t bwd_smem(int K0) {
  return (size_t)(L - 1) * W * W * 2 + (size_t)K0 * W * 2 + 3u * W * 4 + 16 * 4 + (3 + Geo<W>::STEPS) * 8 + 8;
}
inline size_t wgrad_smem(int WA, int WB) { return 2 * wg_a_bytes(WA) + 2 * wg_b_bytes(WB) + 4096 + 6 * 8 + 8; }

template <int W, int L>
int launch_fwd(const FwdParams& P, cudaStream_t st) {
  const size_t smem = fwd_smem<W, L>(P.K0);
  cudaError_t e = cudaFuncSetAttribute(mlp_fwd_kernel<W, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  const int64_t tiles = (P.n_rows + TM - 1) / TM;
  const unsigned grid = (unsigned)(tiles < sm_count() ? tiles : sm_count());
  const uint32_t cols = tmem_cols_for(2 * W + W / 2 + 16);
  mlp_fwd_kernel<W, L><<<grid, THREADS, smem, st>>>(P, cols);
  return launch_status();
}

template <int W, int L>
int launch_bwd(const BwdParams& P, unsigned grid, cudaStream_t st) {
  const size_t smem = bwd_smem<W, L>(P.K0);
  cudaError_t e = cudaFuncSetAttribute(mlp_bwd_kernel<W, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  const int AW = W > P.K0 ? W : P.K0;
  const uint32_t cols = tmem_cols_for(2 * AW + W / 2);
  mlp_bwd_kernel<W, L><<<grid, THREADS, smem, st>>>(P, cols);
  return launch_status();
}

}  // namespace mt
}  // namespace vx

using namespace vx;
using namespace vx::mt;

namespace {

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

int check_shape(int64_t width, int64_t n_hidden, int64_t K0) {
  if (!(width == 32 || width == 64 || width == 128 || width == 192)) return VX_ERR_UNSUPPORTED;
  if (n_hidden < 2 || n_hidden > 3) return VX_ERR_UNSUPPORTED;
  if (K0 < 16 || K0 > MAX_K0 || K0 % 16) return VX_ERR_UNSUPPORTED;
  return VX_OK;
}

template <typename F>
int dispatch(int64_t width, int64_t n_hidden, F&& f) {
#define VX_MT_CASE(W_, L_) \
  if (width == W_ && n_hidden == L_) return f(std::integral_constant<int, W_>{}, std::integral_constant<int, L_>{});
  VX_MT_CASE(192, 3) VX_MT_CASE(192, 2) VX_MT_CASE(128, 3) VX_MT_CASE(128, 2) VX_MT_CASE(64, 3) VX_MT_CASE(64, 2)
  VX_MT_CASE(32, 3) VX_MT_CASE(32, 2)
#undef VX_MT_CASE
  return VX_ERR_UNSUPPORTED;
}

}  // namespace

extern "C" {

size_t vx_mlp_train_tiles(int64_t n_rows) { return (size_t)((n_rows + TM - 1) / TM); }

int vx_mlp_train_pack(const vx_mlp_pack_job* jobs, int n_jobs, void* stream) {
  if (!jobs || n_jobs < 1 || n_jobs > MAX_PACK_JOBS) return VX_ERR_ARG;
  PackJobs J{};
  int64_t most = 0;
  for (int i = 0; i < n_jobs; ++i) {
    const vx_mlp_pack_job& s = jobs[i];
    if (!s.src || !s.dst || s.N < 1 || s.K < 1 || s.ld < 1 || s.mode < 0 || s.mode > 3) return VX_ERR_ARG;
    if ((s.mode == 0 || s.mode == 3) && (s.Np < s.N || s.Kp < s.K || s.Kp % 8)) return VX_ERR_ARG;
    if (s.mode == 1 && (s.N != 3 || s.Np < 6 || s.Kp < s.K || s.Kp % 8)) return VX_ERR_ARG;
    // row stride of the source: [N][K] reads need ld >= K, [K][N] reads ld >= N
    const bool src_kn = (s.mode == 0 && s.transpose) || (s.mode == 3 && !s.transpose);
    if (src_kn ? s.ld < s.N : s.ld < s.K) return VX_ERR_ARG;
    PackJob& d = J.j[i];
    d.src = s.src;
    d.ld = s.ld;
    d.N = (int)s.N;
    d.K = (int)s.K;
    d.Np = (int)s.Np;
    d.Kp = (int)s.Kp;
    d.transpose = s.transpose;
    d.mode = s.mode;
    d.dst = s.dst;
    most = std::max<int64_t>(most, s.mode == 2 ? s.N * s.K : s.Np * s.Kp);
  }
  J.n = n_jobs;
  dim3 grid((unsigned)std::max<int64_t>(1, std::min<int64_t>((most + 255) / 256, 1024)), (unsigned)n_jobs);
  mlp_pack_kernel<<<grid, 256, 0, as_stream(stream)>>>(J);
  return launch_status();
}

int vx_mlp_train_forward(const vx_mlp_train_fwd_args* a, void* stream) {
  if (!a || a->n_rows < 0) return VX_ERR_ARG;
  int s = check_shape(a->width, a->n_hidden, a->K0);
  if (s) return s;
  if (a->n_rows == 0) return VX_OK;
  if (!a->X || !a->W0p || !a->Wp || !a->bias || !a->Whp || !a->bh || !a->out) return VX_ERR_ARG;
  if (a->ldx < a->K0 || a->ldx % 8 || !aligned16(a->X) || !aligned16(a->W0p) || !aligned16(a->Wp) ||
      !aligned16(a->Whp) || !aligned16(a->bias))
    return VX_ERR_ARG;
  const int64_t tiles = (a->n_rows + TM - 1) / TM;
  if ((a->H || a->relu) && (!a->H || !a->relu || a->rows_cap < tiles * TM || !aligned16(a->H) ||
                            reinterpret_cast<uintptr_t>(a->relu) & 3))
    return VX_ERR_ARG;
  FwdParams P{};
  P.X = reinterpret_cast<const bf16*>(a->X);
  P.ldx = a->ldx;
  P.K0 = (int)a->K0;
  P.n_rows = a->n_rows;
  P.n_rows_dev = a->n_rows_dev;
  P.W0p = reinterpret_cast<const bf16*>(a->W0p);
  P.Wp = reinterpret_cast<const bf16*>(a->Wp);
  P.bias = a->bias;
  P.Whp = reinterpret_cast<const bf16*>(a->Whp);
  P.bh = a->bh;
  P.out = a->out;
  P.cols = reinterpret_cast<bf16*>(a->cols);
  P.ld_cols = a->ld_cols;
  P.H = reinterpret_cast<bf16*>(a->H);
  P.relu = reinterpret_cast<uint16_t*>(a->relu);
  P.h_stride = a->rows_cap * a->width;
  P.relu_stride = a->rows_cap * (a->width / 16);
  P.err = device_error_ptr();
  return dispatch(a->width, a->n_hidden, [&](auto Wc, auto Lc) {
    return launch_fwd<decltype(Wc)::value, decltype(Lc)::value>(P, as_stream(stream));
  });
}

int vx_mlp_train_backward(const vx_mlp_train_bwd_args* a, void* stream) {
  if (!a || a->n_rows < 0) return VX_ERR_ARG;
  int s = check_shape(a->width, a->n_hidden, a->K0);
  if (s) return s;
  const int64_t tiles = (a->n_rows + TM - 1) / TM;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(tiles, sm_count()));
  if (!a->dbh_part || a->dbh_part_cap < (int64_t)grid) return VX_ERR_ARG;
  if (a->n_rows == 0) {   // an empty batch: zero output-layer bias partials, nothing else
    cudaError_t e = cudaMemsetAsync(a->dbh_part, 0, sizeof(float) * 4 * grid, as_stream(stream));
    return cuda_status(e);
  }
  if (!a->dY || !a->Wh || !a->relu || !a->WTp || !a->W0Tp || !a->dZ || !a->dYT || !a->dX) return VX_ERR_ARG;
  if (a->rows_cap < tiles * TM || a->ld_dx < a->K0 || !aligned16(a->WTp) || !aligned16(a->W0Tp) ||
      !aligned16(a->Wh) || !aligned16(a->dZ) || !aligned16(a->dYT) || !aligned16(a->dX) ||
      (a->ld_dx * (a->dx_bf16 ? 2 : 4)) % 16 || reinterpret_cast<uintptr_t>(a->relu) & 3)
    return VX_ERR_ARG;
  BwdParams P{};
  P.dY = a->dY;
  P.n_rows = a->n_rows;
  P.n_rows_dev = a->n_rows_dev;
  P.Wh = a->Wh;
  P.relu = reinterpret_cast<const uint16_t*>(a->relu);
  P.relu_stride = a->rows_cap * (a->width / 16);
  P.WTp = reinterpret_cast<const bf16*>(a->WTp);
  P.W0Tp = reinterpret_cast<const bf16*>(a->W0Tp);
  P.K0 = (int)a->K0;
  P.dZ = reinterpret_cast<bf16*>(a->dZ);
  P.dz_stride = a->rows_cap * a->width;
  P.dYT = reinterpret_cast<bf16*>(a->dYT);
  P.dX = a->dX;
  P.ld_dx = a->ld_dx;
  P.dx_bf16 = a->dx_bf16;
  P.dbh_part = a->dbh_part;
  P.err = device_error_ptr();
  return dispatch(a->width, a->n_hidden, [&](auto Wc, auto Lc) {
    return launch_bwd<decltype(Wc)::value, decltype(Lc)::value>(P, grid, as_stream(stream));
  });
}

size_t vx_mlp_wgrad_grid(int64_t n_rows) {
  const int64_t tiles = (n_rows + TM - 1) / TM;
  return (size_t)std::max<int64_t>(1, std::min<int64_t>(tiles, sm_count()));
}

}  // extern "C"

namespace {

// Checks one pass and fills its kernel parameters; ctas = its CTA count.
int wgrad_pass(const vx_mlp_wgrad_args* a, int64_t ctas, vx::mt::WgradParams& P, size_t& smem) {
  using namespace vx::mt;
  if (!a || a->n_rows < 0 || !a->part || ctas < 1) return VX_ERR_ARG;
  if (a->n_rows > 0 && (!a->A || !a->B)) return VX_ERR_ARG;   // an empty batch writes zero partials
  if (a->WA < 16 || a->WA > 256 || a->WA % 16 || a->WB < 16 || a->WB > 240 || a->WB % 16) return VX_ERR_UNSUPPORTED;
  const int MT = (int)((a->WA + TM - 1) / TM);
  const int NC = (int)a->WB + (a->ones ? 16 : 0);
  if (MT * NC > 512) return VX_ERR_UNSUPPORTED;
  // the last M-tile's rows past WA read (MT*128 - WA)/8 core matrices past the A stage
  if ((int64_t)(MT * TM - a->WA) * 16 > (int64_t)WG_TAIL) return VX_ERR_UNSUPPORTED;
  if (a->part_cap < ctas * a->WA * NC) return VX_ERR_ARG;
  if (!aligned16(a->A) || !aligned16(a->B) || !aligned16(a->part)) return VX_ERR_ARG;   // (null is aligned)
  if (a->b_rows && (a->ldb < a->WB || a->ldb % 8)) return VX_ERR_ARG;
  P = WgradParams{};
  P.A = reinterpret_cast<const bf16*>(a->A);
  P.WA = (int)a->WA;
  P.B = reinterpret_cast<const bf16*>(a->B);
  P.WB = (int)a->WB;
  P.ldb = a->ldb;
  P.b_rows = a->b_rows;
  P.ones = a->ones;
  P.n_rows = a->n_rows;
  P.n_rows_dev = a->n_rows_dev;
  P.part = a->part;
  P.err = device_error_ptr();
  smem = std::max(smem, wgrad_smem(P.WA, P.WB));
  return VX_OK;
}

int wgrad_launch(const vx::mt::WgradPasses& PS, size_t smem, void* stream) {
  using namespace vx::mt;
  cudaError_t e = cudaFuncSetAttribute(mlp_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  mlp_wgrad_kernel<<<(unsigned)PS.cta0[PS.n], WG_THREADS, smem, as_stream(stream)>>>(PS);
  return launch_status();
}

}  // namespace

extern "C" {

int vx_mlp_train_wgrad(const vx_mlp_wgrad_args* a, void* stream) {
  if (!a) return VX_ERR_ARG;
  WgradPasses PS{};
  size_t smem = 0;
  const int64_t grid = (int64_t)vx_mlp_wgrad_grid(a->n_rows);
  const int s = wgrad_pass(a, grid, PS.p[0], smem);
  if (s) return s;
  PS.n = 1;
  PS.cta0[0] = 0;
  PS.cta0[1] = (int)grid;
  return wgrad_launch(PS, smem, stream);
}

int vx_mlp_wgrad_split(const vx_mlp_wgrad_args* passes, int n_passes, int32_t* ctas) {
  if (!passes || !ctas || n_passes < 1 || n_passes > MAX_WG_PASSES) return VX_ERR_ARG;
  const int64_t budget = std::max<int64_t>(sm_count(), n_passes);
  double w[MAX_WG_PASSES], tot = 0.0;
  for (int p = 0; p < n_passes; ++p) {
    const vx_mlp_wgrad_args& a = passes[p];
    if (a.WA < 16 || a.WB < 16) return VX_ERR_ARG;
    w[p] = (double)a.WA + (double)a.WB;    // bytes per tile row (both operands)
    tot += w[p];
  }
  // largest remainder over the budget, then at least 1 and at most one CTA per tile
  int64_t given = 0;
  double rem[MAX_WG_PASSES];
  for (int p = 0; p < n_passes; ++p) {
    const double share = (double)budget * w[p] / tot;
    ctas[p] = (int32_t)share;
    rem[p] = share - (double)ctas[p];
    given += ctas[p];
  }
  while (given < budget) {
    int best = 0;
    for (int p = 1; p < n_passes; ++p)
      if (rem[p] > rem[best]) best = p;
    ++ctas[best];
    rem[best] = -1.0;
    ++given;
  }
  for (int p = 0; p < n_passes; ++p) {
    const int64_t cap = (int64_t)vx_mlp_wgrad_grid(passes[p].n_rows);
    ctas[p] = (int32_t)std::max<int64_t>(1, std::min<int64_t>(ctas[p], cap));
  }
  return VX_OK;
}

int vx_mlp_train_wgrad_multi(const vx_mlp_wgrad_args* passes, const int32_t* ctas, int n_passes, void* stream) {
  if (!passes || !ctas || n_passes < 1 || n_passes > MAX_WG_PASSES) return VX_ERR_ARG;
  WgradPasses PS{};
  size_t smem = 0;
  int64_t total = 0;
  PS.cta0[0] = 0;
  for (int p = 0; p < n_passes; ++p) {
    const int s = wgrad_pass(&passes[p], ctas[p], PS.p[p], smem);
    if (s) return s;
    total += ctas[p];
    if (total > 65535) return VX_ERR_ARG;
    PS.cta0[p + 1] = (int)total;
  }
  PS.n = n_passes;
  return wgrad_launch(PS, smem, stream);
}

int vx_mlp_train_reduce(const vx_mlp_reduce_job* jobs, int n_jobs, void* stream) {
  if (!jobs || n_jobs < 1 || n_jobs > MAX_REDUCE_JOBS) return VX_ERR_ARG;
  ReduceJobs J{};
  for (int i = 0; i < n_jobs; ++i) {
    const vx_mlp_reduce_job& s = jobs[i];
    if (!s.part || !s.w || !s.b || s.n_part < 1 || s.WA < 1 || s.NC < 1) return VX_ERR_ARG;
    if (s.kind == 0 && (s.n_out < 1 || s.n_out > s.WB || s.WB >= s.NC)) return VX_ERR_ARG;
    if (s.kind == 1 && (s.NC < 6 || !s.bh_part || s.n_bh < 1)) return VX_ERR_ARG;
    ReduceJob& d = J.j[i];
    d.part = s.part;
    d.n_part = (int)s.n_part;
    d.WA = (int)s.WA;
    d.NC = (int)s.NC;
    d.kind = s.kind;
    d.WB = (int)s.WB;
    d.n_out = (int)s.n_out;
    d.w = s.w;
    d.b = s.b;
    d.bh_part = s.bh_part;
    d.n_bh = (int)s.n_bh;
  }
  J.n = n_jobs;
  int64_t most = 1;
  for (int i = 0; i < n_jobs; ++i)
    most = std::max<int64_t>(most, jobs[i].kind == 0 ? jobs[i].WA * (jobs[i].n_out + 1) : 3 * jobs[i].WA + 3);
  dim3 grid((unsigned)std::min<int64_t>((most + 31) / 32, 2048), (unsigned)n_jobs);
  mlp_reduce_kernel<<<grid, 256, 0, as_stream(stream)>>>(J);
  return launch_status();
}

}  // extern "C"
