// Fused colour-MLP forward on the 5th-generation tensor cores (tcgen05).
//
// One persistent CTA per SM keeps all layers of one colour MLP (rgbnet or
// k_rgbnet, voxurf_fine.py:132-187) resident in shared memory (BF16, 30 +
// 72 + 72 KB hidden, 6 KB output layer) and streams 128-row tiles of its
// input rows through them:
//
//   X tile (128 x K0, BF16, shared) --tcgen05.mma--> TMEM acc (128 x 192 FP32)
//     --tcgen05.ld--> +bias, ReLU, BF16 --tcgen05.st--> TMEM A operand
//     --tcgen05.mma (A from tensor memory)--> acc ... (layers 1, 2)
//   output layer: one more MMA (N = 16) from the TMEM A operand against the
//   FP32 output weights split into BF16 hi + lo rows; logit = hi + lo + b.
//
// Hidden activations never leave tensor memory; HBM traffic per row is the
// input row and 12 bytes of logits.  Shared-memory operands use the canonical K-major layout
// without swizzle: 8 x 16-byte core matrices, chunk c of K (8 elements) of
// all R rows stored contiguously ([K/8][R][8]), so LBO = R * 16 bytes (next
// core matrix along K) and SBO = 128 bytes (next 8 rows).  Weights are
// packed into that layout by the caller (vx_mlp_tc_pack) and copied to
// shared memory once per CTA.
//
// Thread roles: 8 epilogue warps (warps w and w+4 own TMEM lanes / tile rows
// [32(w%4), +32) and split each 64-column step in halves; 16 warps splitting
// it in four measured the same) and one warp
// whose lane 0 issues the MMAs and the commits.  The epilogue hands each
// layer's activations to the next layer in three steps of 64 columns, so
// the next layer's first MMAs overlap the conversion of the last columns
// (layers alternate between two accumulators), and the next tile's first
// layer overlaps the output-layer epilogue.  Weights, biases and the output
// layer arrive by bulk copies on the async proxy (one mbarrier); the next
// input tile is prefetched with 16-byte cp.async (zero fill past the last
// row) as soon as the first layer's MMAs have read the current one.  Tensor
// memory: 512 columns (accumulators 0-191 and 192-383, A operand 384-479,
// output layer 480-495; one CTA per SM).  Every wait on an mbarrier is
// bounded: on expiry the kernel records VX_ERR_TIMEOUT, waits (bounded) for
// its issued MMAs, releases its TMEM and returns.
#include "common.cuh"

namespace vx {

constexpr int TC_M = 128;       // rows per tile (one cta_group::1 MMA)
constexpr int TC_N = 192;       // hidden width
constexpr int TC_KMAX0 = 80;    // largest first-layer K (shared memory: 30 + 144 + 20 + 6 + 2 KB)
constexpr int TC_TMEM_COLS = 512;

struct MlpTcParams {
  const __nv_bfloat16* X;  // [n_rows, ldx] input rows (columns K0.. zero or ignored via zero weights)
  int64_t ldx;
  int K0;                  // first-layer K (multiple of 16, <= TC_KMAX0)
  int64_t n_rows;
  const __nv_bfloat16* W0p;  // packed [K0/8][192][8]
  const __nv_bfloat16* W1p;  // packed [24][192][8]
  const __nv_bfloat16* W2p;
  const float* b0;
  const float* b1;
  const float* b2;
  const __nv_bfloat16* Whp;  // packed [24][16][8] output layer: rows 0-2 hi, 3-5 lo parts
  const float* bh;   // [3]
  const float* add;  // optional [n,3] added to the logits
  float* out;        // [n,3]
  __nv_bfloat16* cols;  // optional: logits also stored (BF16) at cols[row*ld_cols + 0..2]
  int64_t ld_cols;
  int* err;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor, K-major, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);            // bits 0-13: start address >> 4
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;         // bits 16-29: leading byte offset >> 4
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;         // bits 32-45: stride byte offset >> 4
  d |= (uint64_t)1 << 46;                             // bits 46-48: fixed 0b001
  // base offset 0, absolute-LBO mode off, swizzle mode 0 (none)
  return d;
}

// Instruction descriptor: kind::f16, A = B = BF16, D = FP32, both K-major.
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N) {
  return (1u << 4)            // D format F32
         | (1u << 7)          // A format BF16
         | (1u << 10)         // B format BF16
         | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Bounded wait for the phase `parity` of an mbarrier; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < (1u << 26); ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)acc)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane (raw bits; valid
// after tc_wait_ld).
__device__ __forceinline__ void tc_ld32_async(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// This thread's 96 columns [col0, col0 + 96) of its TMEM lane: three loads
// in flight, one wait.
__device__ __forceinline__ void tc_ld96(uint32_t taddr, uint32_t (&r)[3][32]) {
  tc_ld32_async(taddr, r[0]);
  tc_ld32_async(taddr + 32, r[1]);
  tc_ld32_async(taddr + 64, r[2]);
  tc_wait_ld();
  // order every use of the loaded registers after the wait (empty volatile
  // asms stay in program order with the wait and carry the dependency)
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 32; ++i) asm volatile("" : "+r"(r[j][i]));
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// All K/16 MMAs of one layer (issued by one thread) and the commit.
__device__ __forceinline__ void tc_layer(uint32_t tmem, uint32_t a_s, uint32_t b_s, int K, uint64_t* bar) {
  constexpr uint32_t idesc = umma_idesc(TC_M, TC_N);
  for (int ks = 0; ks < K / 16; ++ks) {
    const uint64_t ad = umma_desc(a_s + (uint32_t)(2 * ks) * (TC_M * 16), TC_M * 16, 128);
    const uint64_t bd = umma_desc(b_s + (uint32_t)(2 * ks) * (TC_N * 16), TC_N * 16, 128);
    tc_mma(tmem, ad, bd, idesc, ks > 0);
  }
  tc_commit(bar);
}

// Global -> shared bulk copy (async proxy) completing on an mbarrier.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// 16-byte asynchronous copy with zero fill of the bytes beyond src_bytes.
__device__ __forceinline__ void cp_async16(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Input tile rows [row0, row0+128) -> As chunks [0, K0/8) (zero rows past n).
__device__ __forceinline__ void load_x_tile(const MlpTcParams& P, __nv_bfloat16* As, int64_t row0, int tid,
                                            int nthreads) {
  const int chunks = P.K0 / 8;
  for (int i = tid; i < chunks * TC_M; i += nthreads) {
    const int c = i / TC_M, r = i % TC_M;
    const bool in = row0 + r < P.n_rows;
    const __nv_bfloat16* src = P.X + (in ? (row0 + r) * P.ldx + 8 * c : 0);
    cp_async16(As + ((size_t)c * TC_M + r) * 8, src, in ? 16u : 0u);
  }
  cp_async_commit();
}

// ---- A operand in tensor memory ------------------------------------------
// Hidden activations of layers 1 and 2 and of the output layer stay in
// tensor memory: row m in lane m, K element k in column k/2 (two BF16 per
// 32-bit column, the lower k in the lower half, as pack_bf16 packs them).
__device__ __forceinline__ void tc_mma_ta(uint32_t dtmem, uint32_t atmem, uint64_t bdesc, uint32_t idesc, bool acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(dtmem),
      "r"(atmem), "l"(bdesc), "r"(idesc), "r"((uint32_t)acc)
      : "memory");
}

// All K/16 MMAs of a layer with A in tensor memory (8 columns per K step)
// and B [K/8][N][8] in shared memory, then the commit.
__device__ __forceinline__ void tc_layer_ta(uint32_t dtmem, uint32_t atmem, uint32_t b_s, int N, int K,
                                            uint64_t* bar) {
  const uint32_t idesc = umma_idesc(TC_M, N);
  for (int ks = 0; ks < K / 16; ++ks) {
    const uint64_t bd = umma_desc(b_s + (uint32_t)(2 * ks) * (uint32_t)(N * 16), (uint32_t)(N * 16), 128);
    tc_mma_ta(dtmem, atmem + (uint32_t)(8 * ks), bd, idesc, ks > 0);
  }
  tc_commit(bar);
}

// 16 consecutive 32-bit columns of this thread's TMEM lane <- r.
__device__ __forceinline__ void tc_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
      "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  tc_wait_ld();
#pragma unroll
  for (int i = 0; i < 16; ++i) asm volatile("" : "+r"(r[i]));
}

constexpr int TC_EPI_WARPS = 8;                 // epilogue warps (w, w+4, .. share TMEM lanes 32(w%4)..)
constexpr int TC_THREADS = 32 * (TC_EPI_WARPS + 1);  // + one warp that issues the MMAs
constexpr int TC_NH = 16;        // output-layer tile: rows 0-2 hi, 3-5 lo, rest zero
// tensor-memory columns: two hidden accumulators (layers alternate between
// them), the A operand (192 BF16 = 96 columns), the output-layer accumulator
constexpr uint32_t TM_ACC0 = 0, TM_ACC1 = 192, TM_A = 384, TM_HEAD = 480;
constexpr int TC_STEPS = 3;      // epilogue hand-off steps per layer
constexpr int TC_SW = TC_N / TC_STEPS;          // hidden columns per step (64)
constexpr int TC_KPS = TC_SW / 16;              // MMA K steps per hand-off step
constexpr int TC_PARTS = TC_EPI_WARPS / 4;      // warps sharing one lane quarter
constexpr int TC_CPW = TC_SW / TC_PARTS;        // hidden columns per thread per step
static_assert(TC_CPW == 16 || TC_CPW == 32, "epilogue split");

// 8 consecutive 32-bit columns of this thread's TMEM lane <- r.
__device__ __forceinline__ void tc_st8(uint32_t taddr, const uint32_t (&r)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(r[0]),
               "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
               : "memory");
}

// N consecutive FP32 columns of this thread's TMEM lane (complete on return).
template <int N>
__device__ __forceinline__ void tc_ld_cols(uint32_t taddr, uint32_t (&r)[N]) {
  if constexpr (N == 32) {
    tc_ld32_async(taddr, r);
    tc_wait_ld();
  } else {
    tc_ld16(taddr, r);
  }
}
// N consecutive 32-bit columns of this thread's TMEM lane <- r (N = 16 or 8).
template <int N>
__device__ __forceinline__ void tc_st_cols(uint32_t taddr, const uint32_t (&r)[N]) {
  if constexpr (N == 16)
    tc_st16(taddr, r);
  else
    tc_st8(taddr, r);
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// MMAs of K steps [KPS s, KPS (s + 1)) (K = SW s .. SW (s + 1) - 1) of a
// layer whose A operand is in tensor memory.
__device__ __forceinline__ void tc_layer_ta_step(uint32_t dtmem, uint32_t atmem, uint32_t b_s, int N, int s) {
  const uint32_t idesc = umma_idesc(TC_M, N);
#pragma unroll
  for (int ks = TC_KPS * s; ks < TC_KPS * (s + 1); ++ks) {
    const uint64_t bd = umma_desc(b_s + (uint32_t)(2 * ks) * (uint32_t)(N * 16), (uint32_t)(N * 16), 128);
    tc_mma_ta(dtmem, atmem + (uint32_t)(8 * ks), bd, idesc, ks > 0);
  }
}

// Pipeline of one CTA (one tile of 128 rows at a time):
//   MMA warp:      L0 (A = X tile in shared memory) -> ACC0, commit bar_acc;
//                  then for L1 (-> ACC1), L2 (-> ACC0) and the output layer
//                  (-> HEAD): for each step s, wait bar_a[s] and issue the K
//                  steps of the activations that step made; commit.
//   epilogue warps: for L0, L1, L2: wait bar_acc; in 3 steps, hidden columns
//                  [64s, 64s + 64) (split between the warps of a lane quarter):
//                  tcgen05.ld, +bias, ReLU, BF16, tcgen05.st into the A
//                  operand, arrive on bar_a[s].  After L2 the next X tile is
//                  complete (bar_x); the output layer's logits follow
//                  bar_head.
// So the next layer's first MMAs run while the epilogue still converts the
// last columns of the current one (they write the other accumulator), and
// the next tile's first layer runs during the output-layer epilogue.
// Ordering: an accumulator is rewritten two layers later, after all of its
// reader's steps; the A operand's columns of step s are rewritten only after
// the commit of the layer reading them (every epilogue wait on bar_acc
// follows that commit); each barrier runs at most one phase ahead of its
// waiter (the producer of phase k+1 itself waits on the consumer of phase k).
__global__ void __launch_bounds__(TC_THREADS, 1) mlp_tc_kernel(MlpTcParams P) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int K0 = P.K0;
  __nv_bfloat16* W0s = reinterpret_cast<__nv_bfloat16*>(smem);
  __nv_bfloat16* W1s = W0s + (size_t)K0 * TC_N;
  __nv_bfloat16* W2s = W1s + (size_t)TC_N * TC_N;
  __nv_bfloat16* Xs = W2s + (size_t)TC_N * TC_N;                    // [K0/8][128][8] input tile
  __nv_bfloat16* WHs = Xs + (size_t)K0 * TC_M;                      // [24][16][8] output layer
  float* bias_s = reinterpret_cast<float*>(WHs + (size_t)TC_NH * TC_N);  // [3][192]
  uint64_t* bar_w = reinterpret_cast<uint64_t*>(bias_s + 3 * TC_N);
  uint64_t* bar_acc = bar_w + 1;
  uint64_t* bar_head = bar_w + 2;
  uint64_t* bar_x = bar_w + 3;
  uint64_t* bar_fin = bar_w + 4;
  uint64_t* bar_a = bar_w + 5;  // [TC_STEPS]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_a + TC_STEPS);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool mma_warp = warp == TC_EPI_WARPS;
  const int quarter = warp & 3, part = (warp >> 2) % TC_PARTS;  // TMEM lanes 32*quarter..
  const int epi_threads = 32 * TC_EPI_WARPS;
  const int64_t n_tiles = (P.n_rows + TC_M - 1) / TC_M;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(bar_w, 1);
    mbar_init(bar_acc, 1);
    mbar_init(bar_head, 1);
    mbar_init(bar_x, TC_EPI_WARPS);
    mbar_init(bar_fin, 1);
    for (int s = 0; s < TC_STEPS; ++s) mbar_init(bar_a + s, TC_EPI_WARPS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    // weights and biases: bulk copies on the async proxy
    const uint32_t w0b = (uint32_t)K0 * TC_N * 2, w1b = (uint32_t)TC_N * TC_N * 2, bb = TC_N * 4,
                   whb = (uint32_t)TC_NH * TC_N * 2;
    mbar_expect_tx(bar_w, w0b + 2 * w1b + whb + 3 * bb);
    bulk_g2s(W0s, P.W0p, w0b, bar_w);
    bulk_g2s(W1s, P.W1p, w1b, bar_w);
    bulk_g2s(W2s, P.W2p, w1b, bar_w);
    bulk_g2s(WHs, P.Whp, whb, bar_w);
    bulk_g2s(bias_s, P.b0, bb, bar_w);
    bulk_g2s(bias_s + TC_N, P.b1, bb, bar_w);
    bulk_g2s(bias_s + 2 * TC_N, P.b2, bb, bar_w);
  }
  if (!mma_warp && blockIdx.x < n_tiles) {
    load_x_tile(P, Xs, (int64_t)blockIdx.x * TC_M, tid, epi_threads);
    cp_async_wait_all();
    fence_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(bar_x);
  }
  bool ok = mbar_wait(bar_w, 0);
  const float bh0 = __ldg(P.bh + 0), bh1 = __ldg(P.bh + 1), bh2 = __ldg(P.bh + 2);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t tmem_row = tmem + ((uint32_t)(32 * quarter) << 16);
  const uint32_t x_s = smem_u32(Xs), w_s[3] = {smem_u32(W0s), smem_u32(W1s), smem_u32(W2s)}, wh_s = smem_u32(WHs);

  if (mma_warp) {
    uint32_t ph_x = 0, ph_a = 0;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
      ok = mbar_wait(bar_x, ph_x);
      ph_x ^= 1u;
      tc_fence_after();
      if (!ok) break;
      if (lane == 0) tc_layer(tmem + TM_ACC0, x_s, w_s[0], K0, bar_acc);
      __syncwarp();
#pragma unroll 1
      for (int layer = 1; layer < 4 && ok; ++layer) {
        const uint32_t d = layer == 1 ? TM_ACC1 : layer == 2 ? TM_ACC0 : TM_HEAD;
        const uint32_t b = layer == 1 ? w_s[1] : layer == 2 ? w_s[2] : wh_s;
        const int N = layer < 3 ? TC_N : TC_NH;
#pragma unroll 1
        for (int s = 0; s < TC_STEPS; ++s) {
          ok = mbar_wait(bar_a + s, ph_a);
          tc_fence_after();
          if (!ok) break;
          if (lane == 0) tc_layer_ta_step(tmem + d, tmem + TM_A, b, N, s);
          __syncwarp();
        }
        ph_a ^= 1u;
        if (ok && lane == 0) tc_commit(layer < 3 ? bar_acc : bar_head);
        __syncwarp();
      }
    }
    // nothing of this CTA's may still be in flight when the tensor memory is
    // released
    if (lane == 0) {
      tc_commit(bar_fin);
      if (!mbar_wait(bar_fin, 0)) ok = false;
    }
    __syncwarp();
  } else {
    uint32_t ph_acc = 0, ph_head = 0;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
      const int64_t row = tile * TC_M + 32 * quarter + lane;
#pragma unroll 1
      for (int layer = 0; layer < 3; ++layer) {
        ok = mbar_wait(bar_acc, ph_acc);
        ph_acc ^= 1u;
        tc_fence_after();
        if (!ok) break;
        if (layer == 0) {
          // the input tile is consumed: prefetch the next one
          const int64_t next = tile + gridDim.x;
          if (next < n_tiles) load_x_tile(P, Xs, next * TC_M, tid, epi_threads);
        }
        const uint32_t acc = layer == 1 ? TM_ACC1 : TM_ACC0;
        const float* bl = bias_s + layer * TC_N;
#pragma unroll 1
        for (int s = 0; s < TC_STEPS; ++s) {
          // +bias, ReLU, BF16 -> the A operand: this thread's row, hidden
          // columns [SW s + CPW part, +CPW) -> TMEM columns (the same) / 2
          const int col0 = TC_SW * s + TC_CPW * part;
          uint32_t v[TC_CPW];
          tc_ld_cols<TC_CPW>(tmem_row + acc + (uint32_t)col0, v);
#pragma unroll
          for (int i = 0; i < TC_CPW; ++i) asm volatile("" : "+r"(v[i]));
          uint32_t pk[TC_CPW / 2];
#pragma unroll
          for (int q = 0; q < TC_CPW / 4; ++q) {
            const float4 bq = *reinterpret_cast<const float4*>(bl + col0 + 4 * q);
            const float h0 = fmaxf(__uint_as_float(v[4 * q + 0]) + bq.x, 0.f);
            const float h1 = fmaxf(__uint_as_float(v[4 * q + 1]) + bq.y, 0.f);
            const float h2 = fmaxf(__uint_as_float(v[4 * q + 2]) + bq.z, 0.f);
            const float h3 = fmaxf(__uint_as_float(v[4 * q + 3]) + bq.w, 0.f);
            pk[2 * q] = pack_bf16(h0, h1);
            pk[2 * q + 1] = pack_bf16(h2, h3);
          }
          tc_st_cols<TC_CPW / 2>(tmem_row + TM_A + (uint32_t)(col0 / 2), pk);
          tc_wait_st();
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(bar_a + s);
        }
        if (layer == 2) {
          // the next input tile (if any) is in shared memory
          cp_async_wait_all();
          fence_async_smem();
          __syncwarp();
          if (lane == 0) mbar_arrive(bar_x);
        }
      }
      if (!ok) break;
      if (part == 0) {
        // output layer: hi + lo parts of each logit, + bias (+ residual)
        ok = mbar_wait(bar_head, ph_head);
        tc_fence_after();
        if (!ok) break;
        uint32_t hv[16];
        tc_ld16(tmem_row + TM_HEAD, hv);
        if (row < P.n_rows) {
          float a0 = (__uint_as_float(hv[0]) + __uint_as_float(hv[3])) + bh0;
          float a1 = (__uint_as_float(hv[1]) + __uint_as_float(hv[4])) + bh1;
          float a2 = (__uint_as_float(hv[2]) + __uint_as_float(hv[5])) + bh2;
          if (P.add) {
            a0 += P.add[3 * row + 0];
            a1 += P.add[3 * row + 1];
            a2 += P.add[3 * row + 2];
          }
          P.out[3 * row + 0] = a0;
          P.out[3 * row + 1] = a1;
          P.out[3 * row + 2] = a2;
          if (P.cols) {
            __nv_bfloat16* cp = P.cols + row * P.ld_cols;
            cp[0] = __float2bfloat16_rn(a0);
            cp[1] = __float2bfloat16_rn(a1);
            cp[2] = __float2bfloat16_rn(a2);
          }
        }
        tc_fence_before();
      }
      ph_head ^= 1u;
    }
    cp_async_wait_all();
  }
  if (!ok) set_device_error(P.err, VX_ERR_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

// ---- two tiles in flight ----------------------------------------------------
// mlp_tc2_kernel keeps two 128-row tiles (slots 0 and 1) in flight so that
// the MMAs of one run while the epilogue converts the other's accumulator.
// Tensor memory (512 columns): one accumulator per slot (D0 = 0-191, D1 =
// 192-383), ONE shared A operand (384-479) and an output-layer accumulator
// per slot (480-495, 496-511).  Shared memory: the weights (as above) and an
// input tile per slot (2 x 20 KB at K0 = 80).
//
// MMA order per pair of tiles: L0(0), L0(1) (A = the input tiles), then
// L1(0), L1(1), L2(0), L2(1), H(0), H(1), each from the A operand, which the
// epilogue fills in the same order: E0(0), E0(1), E1(0), E1(1), E2(0),
// E2(1), where E_l(t) converts D_t after L_l(t) (+bias, ReLU, BF16, into
// registers) and stores it into the A operand once the MMA that read the A
// operand last has completed: E0(1) after L1(0), E1(0) after L1(1), E1(1)
// after L2(0), E2(0) after L2(1), E2(1) after H(0), E0(0) after H(1) of the
// previous pair (implied: L0(0) is issued after it and its commit covers
// it).  So while L_l(t) runs, the epilogue converts the other slot's
// accumulator.  The MMAs and the epilogue arithmetic are those of
// mlp_tc_kernel in the same order (bit-identical results).  An odd tile
// count gives the CTA's last pair an empty second tile (zero rows, no
// output).
__device__ __forceinline__ uint32_t tm2_d(int t) { return t ? 192u : 0u; }
__device__ __forceinline__ uint32_t tm2_h(int t) { return t ? 496u : 480u; }
constexpr uint32_t TM2_A = 384;

__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// This thread's hidden columns [96 part, +96) of accumulator `dcol` (its
// TMEM lane): +bias, ReLU, BF16 pairs -> pk (A operand columns [48 part, +48)).
__device__ __forceinline__ void tc2_convert(uint32_t tmem_row, uint32_t dcol, const float* bl, int part,
                                            uint32_t (&pk)[48]) {
  uint32_t v[3][32];
  tc_ld96(tmem_row + dcol + (uint32_t)(96 * part), v);
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 bq = *reinterpret_cast<const float4*>(bl + 96 * part + 32 * j + 4 * q);
      const float h0 = fmaxf(__uint_as_float(v[j][4 * q + 0]) + bq.x, 0.f);
      const float h1 = fmaxf(__uint_as_float(v[j][4 * q + 1]) + bq.y, 0.f);
      const float h2 = fmaxf(__uint_as_float(v[j][4 * q + 2]) + bq.z, 0.f);
      const float h3 = fmaxf(__uint_as_float(v[j][4 * q + 3]) + bq.w, 0.f);
      pk[16 * j + 2 * q] = pack_bf16(h0, h1);
      pk[16 * j + 2 * q + 1] = pack_bf16(h2, h3);
    }
}

// pk -> A operand columns [48 part, +48) of this thread's lane, then the
// hand-off to the MMA warp (one arrival per warp).
__device__ __forceinline__ void tc2_store_a(uint32_t tmem_row, int part, const uint32_t (&pk)[48], uint64_t* bar_a,
                                            int lane) {
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    uint32_t s16[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) s16[i] = pk[16 * j + i];
    tc_st16(tmem_row + TM2_A + (uint32_t)(48 * part + 16 * j), s16);
  }
  tc_wait_st();
  tc_fence_before();
  __syncwarp();
  if (lane == 0) mbar_arrive(bar_a);
}

// Output layer of one tile: hi + lo parts of each logit, + bias (+ residual).
__device__ __forceinline__ void tc2_head(const MlpTcParams& P, uint32_t tmem_row, int t, int64_t row, float bh0,
                                         float bh1, float bh2) {
  uint32_t hv[16];
  tc_ld16(tmem_row + tm2_h(t), hv);
  if (row < P.n_rows) {
    float a0 = (__uint_as_float(hv[0]) + __uint_as_float(hv[3])) + bh0;
    float a1 = (__uint_as_float(hv[1]) + __uint_as_float(hv[4])) + bh1;
    float a2 = (__uint_as_float(hv[2]) + __uint_as_float(hv[5])) + bh2;
    if (P.add) {
      a0 += P.add[3 * row + 0];
      a1 += P.add[3 * row + 1];
      a2 += P.add[3 * row + 2];
    }
    P.out[3 * row + 0] = a0;
    P.out[3 * row + 1] = a1;
    P.out[3 * row + 2] = a2;
    if (P.cols) {
      __nv_bfloat16* cp = P.cols + row * P.ld_cols;
      cp[0] = __float2bfloat16_rn(a0);
      cp[1] = __float2bfloat16_rn(a1);
      cp[2] = __float2bfloat16_rn(a2);
    }
  }
}

__global__ void __launch_bounds__(TC_THREADS, 1) mlp_tc2_kernel(MlpTcParams P) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int K0 = P.K0;
  __nv_bfloat16* W0s = reinterpret_cast<__nv_bfloat16*>(smem);
  __nv_bfloat16* W1s = W0s + (size_t)K0 * TC_N;
  __nv_bfloat16* W2s = W1s + (size_t)TC_N * TC_N;
  __nv_bfloat16* Xs0 = W2s + (size_t)TC_N * TC_N;                   // [K0/8][128][8] slot 0 input tile
  __nv_bfloat16* Xs1 = Xs0 + (size_t)K0 * TC_M;                     // slot 1
  __nv_bfloat16* WHs = Xs1 + (size_t)K0 * TC_M;                     // [24][16][8] output layer
  float* bias_s = reinterpret_cast<float*>(WHs + (size_t)TC_NH * TC_N);  // [3][192]
  uint64_t* bar_w = reinterpret_cast<uint64_t*>(bias_s + 3 * TC_N);
  uint64_t* bar_d = bar_w + 1;    // [2] accumulator of slot t complete
  uint64_t* bar_h = bar_w + 3;    // [2] output layer of slot t complete
  uint64_t* bar_x = bar_w + 5;    // [2] input tile of slot t in shared memory
  uint64_t* bar_a = bar_w + 7;    // A operand filled
  uint64_t* bar_fin = bar_w + 8;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_w + 9);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool mma_warp = warp == TC_EPI_WARPS;
  const int quarter = warp & 3, part = (warp >> 2) & 1;  // TMEM lanes 32*quarter.., column half `part`
  const int epi_threads = 32 * TC_EPI_WARPS;
  const int64_t n_tiles = (P.n_rows + TC_M - 1) / TC_M;
  const int64_t n_j = (int64_t)blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int64_t n_pairs = (n_j + 1) / 2;
  const int64_t g = gridDim.x;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(bar_w, 1);
    for (int t = 0; t < 2; ++t) {
      mbar_init(bar_d + t, 1);
      mbar_init(bar_h + t, 1);
      mbar_init(bar_x + t, TC_EPI_WARPS);
    }
    mbar_init(bar_a, TC_EPI_WARPS);
    mbar_init(bar_fin, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    const uint32_t w0b = (uint32_t)K0 * TC_N * 2, w1b = (uint32_t)TC_N * TC_N * 2, bb = TC_N * 4,
                   whb = (uint32_t)TC_NH * TC_N * 2;
    mbar_expect_tx(bar_w, w0b + 2 * w1b + whb + 3 * bb);
    bulk_g2s(W0s, P.W0p, w0b, bar_w);
    bulk_g2s(W1s, P.W1p, w1b, bar_w);
    bulk_g2s(W2s, P.W2p, w1b, bar_w);
    bulk_g2s(WHs, P.Whp, whb, bar_w);
    bulk_g2s(bias_s, P.b0, bb, bar_w);
    bulk_g2s(bias_s + TC_N, P.b1, bb, bar_w);
    bulk_g2s(bias_s + 2 * TC_N, P.b2, bb, bar_w);
  }
  if (!mma_warp && n_pairs > 0) {
    // the first pair's input tiles (a tile past the last one is all zero rows)
    load_x_tile(P, Xs0, ((int64_t)blockIdx.x) * TC_M, tid, epi_threads);
    load_x_tile(P, Xs1, ((int64_t)blockIdx.x + g) * TC_M, tid, epi_threads);
    cp_async_wait_all();
    fence_async_smem();
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(bar_x);
      mbar_arrive(bar_x + 1);
    }
  }
  bool ok = mbar_wait(bar_w, 0);
  const float bh0 = __ldg(P.bh + 0), bh1 = __ldg(P.bh + 1), bh2 = __ldg(P.bh + 2);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t tmem_row = tmem + ((uint32_t)(32 * quarter) << 16);
  const uint32_t x_s0 = smem_u32(Xs0), x_s1 = smem_u32(Xs1);
  const uint32_t w_s0 = smem_u32(W0s), w_s1 = smem_u32(W1s), w_s2 = smem_u32(W2s), wh_s = smem_u32(WHs);

  if (mma_warp) {
    uint32_t ph_a = 0;
    for (int64_t p = 0; p < n_pairs && ok; ++p) {
      for (int t = 0; t < 2 && ok; ++t) {
        ok = mbar_wait(bar_x + t, (uint32_t)(p & 1));
        tc_fence_after();
        if (!ok) break;
        if (lane == 0) tc_layer(tmem + tm2_d(t), t ? x_s1 : x_s0, w_s0, K0, bar_d + t);
        __syncwarp();
      }
#pragma unroll 1
      for (int step = 0; step < 6 && ok; ++step) {
        const int t = step & 1, layer = 1 + (step >> 1);  // layer 3: the output layer
        ok = mbar_wait(bar_a, ph_a);
        ph_a ^= 1u;
        tc_fence_after();
        if (!ok) break;
        if (lane == 0) {
          if (layer < 3)
            tc_layer_ta(tmem + tm2_d(t), tmem + TM2_A, layer == 1 ? w_s1 : w_s2, TC_N, TC_N, bar_d + t);
          else
            tc_layer_ta(tmem + tm2_h(t), tmem + TM2_A, wh_s, TC_NH, TC_N, bar_h + t);
        }
        __syncwarp();
      }
    }
    // nothing of this CTA's may still be in flight when the tensor memory is
    // released
    if (lane == 0) {
      tc_commit(bar_fin);
      if (!mbar_wait(bar_fin, 0)) ok = false;
    }
    __syncwarp();
  } else {
    uint32_t pk[48];
    for (int64_t p = 0; p < n_pairs && ok; ++p) {
      const bool more = p + 1 < n_pairs;
      const uint32_t d0 = (uint32_t)((3 * p) & 1), d1 = d0 ^ 1u, d2 = d0, hp = (uint32_t)(p & 1);
      // E0(0): L0(0) done -> slot 0's input tile is free: prefetch the next one
      ok = mbar_wait(bar_d, d0);
      tc_fence_after();
      if (!ok) break;
      if (more) load_x_tile(P, Xs0, ((int64_t)blockIdx.x + (2 * p + 2) * g) * TC_M, tid, epi_threads);
      tc2_convert(tmem_row, tm2_d(0), bias_s, part, pk);
      tc2_store_a(tmem_row, part, pk, bar_a, lane);
      // E0(1)
      ok = mbar_wait(bar_d + 1, d0);
      tc_fence_after();
      if (!ok) break;
      if (more) load_x_tile(P, Xs1, ((int64_t)blockIdx.x + (2 * p + 3) * g) * TC_M, tid, epi_threads);
      tc2_convert(tmem_row, tm2_d(1), bias_s, part, pk);
      ok = mbar_wait(bar_d, d1);  // L1(0) done: the A operand is free
      tc_fence_after();
      if (!ok) break;
      tc2_store_a(tmem_row, part, pk, bar_a, lane);
      // E1(0) (L1(0) done)
      tc2_convert(tmem_row, tm2_d(0), bias_s + TC_N, part, pk);
      ok = mbar_wait(bar_d + 1, d1);  // L1(1) done
      tc_fence_after();
      if (!ok) break;
      tc2_store_a(tmem_row, part, pk, bar_a, lane);
      // E1(1) (L1(1) done)
      tc2_convert(tmem_row, tm2_d(1), bias_s + TC_N, part, pk);
      ok = mbar_wait(bar_d, d2);  // L2(0) done
      tc_fence_after();
      if (!ok) break;
      tc2_store_a(tmem_row, part, pk, bar_a, lane);
      // E2(0) (L2(0) done)
      tc2_convert(tmem_row, tm2_d(0), bias_s + 2 * TC_N, part, pk);
      ok = mbar_wait(bar_d + 1, d2);  // L2(1) done
      tc_fence_after();
      if (!ok) break;
      tc2_store_a(tmem_row, part, pk, bar_a, lane);
      if (more) {
        // slot 0's next input tile is in shared memory
        cp_async_wait_one();
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(bar_x);
      }
      // E2(1) (L2(1) done)
      tc2_convert(tmem_row, tm2_d(1), bias_s + 2 * TC_N, part, pk);
      ok = mbar_wait(bar_h, hp);  // H(0) done
      tc_fence_after();
      if (!ok) break;
      tc2_store_a(tmem_row, part, pk, bar_a, lane);
      if (more) {
        cp_async_wait_all();
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(bar_x + 1);
      }
      if (part == 0) {
        const int64_t r0 = ((int64_t)blockIdx.x + 2 * p * g) * TC_M + 32 * quarter + lane;
        tc2_head(P, tmem_row, 0, r0, bh0, bh1, bh2);
        ok = mbar_wait(bar_h + 1, hp);
        tc_fence_after();
        if (!ok) break;
        tc2_head(P, tmem_row, 1, r0 + g * TC_M, bh0, bh1, bh2);
        tc_fence_before();
      }
    }
    cp_async_wait_all();
  }
  if (!ok) set_device_error(P.err, VX_ERR_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

static size_t mlp_tc2_smem_bytes(int K0) {
  return (size_t)K0 * TC_N * 2 + 2 * (size_t)TC_N * TC_N * 2 + 2 * (size_t)K0 * TC_M * 2 +
         (size_t)TC_NH * TC_N * 2 + 3 * TC_N * 4 + 9 * 8 + 8;
}

// [N, K] row-major FP32 weights -> [K/8][N][8] BF16 (K padded with zeros to Kp).
__global__ void mlp_tc_pack_kernel(const float* __restrict__ W, int N, int K, int Kp, __nv_bfloat16* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)N * Kp) return;
  const int e = (int)(i % 8), n = (int)((i / 8) % N), c = (int)(i / (8 * (int64_t)N));
  const int k = 8 * c + e;
  out[i] = __float2bfloat16_rn(k < K ? W[(int64_t)n * K + k] : 0.f);
}

static size_t mlp_tc_smem_bytes(int K0) {
  return (size_t)K0 * TC_N * 2 + 2 * (size_t)TC_N * TC_N * 2 + (size_t)K0 * TC_M * 2 + (size_t)TC_NH * TC_N * 2 +
         3 * TC_N * 4 + (5 + TC_STEPS) * 8 + 8;
}

}  // namespace vx

using namespace vx;

extern "C" {

int vx_mlp_tc_pack(const float* W, int64_t N, int64_t K, int64_t Kp, void* out, void* stream) {
  if (!W || !out || N < 1 || K < 1 || Kp < K || Kp % 8) return VX_ERR_ARG;
  mlp_tc_pack_kernel<<<grid_for(N * Kp), VX_THREADS, 0, as_stream(stream)>>>(W, (int)N, (int)K, (int)Kp,
                                                                          reinterpret_cast<__nv_bfloat16*>(out));
  return launch_status();
}

int vx_mlp_tc_forward(const vx_mlp_tc_args* A, void* stream) {
  if (!A || A->n_rows < 0 || (A->pipeline != 0 && A->pipeline != 1)) return VX_ERR_ARG;
  if (A->n_rows == 0) return VX_OK;
  if (A->width != TC_N || A->K0 < 16 || A->K0 > TC_KMAX0 || A->K0 % 16) return VX_ERR_UNSUPPORTED;
  if (!A->X || !A->W0p || !A->W1p || !A->W2p || !A->b0 || !A->b1 || !A->b2 || !A->Whp || !A->bh || !A->out)
    return VX_ERR_ARG;
  if (A->ldx < A->K0 || (A->ldx % 8) || (reinterpret_cast<uintptr_t>(A->X) & 15)) return VX_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(A->W0p) | reinterpret_cast<uintptr_t>(A->W1p) |
       reinterpret_cast<uintptr_t>(A->W2p) | reinterpret_cast<uintptr_t>(A->Whp) |
       reinterpret_cast<uintptr_t>(A->b0) | reinterpret_cast<uintptr_t>(A->b1) | reinterpret_cast<uintptr_t>(A->b2)) &
      15)
    return VX_ERR_ARG;
  MlpTcParams P{};
  P.X = reinterpret_cast<const __nv_bfloat16*>(A->X);
  P.ldx = A->ldx;
  P.K0 = (int)A->K0;
  P.n_rows = A->n_rows;
  P.W0p = reinterpret_cast<const __nv_bfloat16*>(A->W0p);
  P.W1p = reinterpret_cast<const __nv_bfloat16*>(A->W1p);
  P.W2p = reinterpret_cast<const __nv_bfloat16*>(A->W2p);
  P.b0 = A->b0;
  P.b1 = A->b1;
  P.b2 = A->b2;
  P.Whp = reinterpret_cast<const __nv_bfloat16*>(A->Whp);
  P.bh = A->bh;
  P.add = A->add;
  P.out = A->out;
  P.cols = reinterpret_cast<__nv_bfloat16*>(A->cols);
  P.ld_cols = A->ld_cols;
  P.err = device_error_ptr();
  const int64_t tiles = (A->n_rows + TC_M - 1) / TC_M;
  if (A->pipeline == 1) {
    const size_t smem = mlp_tc2_smem_bytes(P.K0);
    cudaError_t e = cudaFuncSetAttribute(mlp_tc2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e);
    const int64_t pairs = (tiles + 1) / 2;
    const unsigned grid = (unsigned)(pairs < sm_count() ? pairs : sm_count());
    mlp_tc2_kernel<<<grid, TC_THREADS, smem, as_stream(stream)>>>(P);
    return launch_status();
  }
  const size_t smem = mlp_tc_smem_bytes(P.K0);
  cudaError_t e = cudaFuncSetAttribute(mlp_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  const unsigned grid = (unsigned)(tiles < sm_count() ? tiles : sm_count());
  mlp_tc_kernel<<<grid, TC_THREADS, smem, as_stream(stream)>>>(P);
  return launch_status();
}

}  // extern "C"
