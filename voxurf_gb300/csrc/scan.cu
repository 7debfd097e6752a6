// Device-wide exclusive prefix sums over int64/int32 counts.
//
// Used for the per-ray sample offsets of sample_pts_on_rays (which the
// reference gets from `N_steps.cumsum(0)` followed by a host `.item()` sync,
// render_utils_kernel.cu:211-212) and for the per-ray survivor counts of the
// fused march.  Three launches, no host sync: tile reduce -> scan of the tile
// sums (one CTA) -> tile scan with the tile's offset.  out has n+1 entries;
// out[n] is the grand total, so a caller can size outputs from the device.
#include "common.cuh"

namespace vx {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* smem_warp, T* total) {
  // v: per-thread value. Returns exclusive prefix across the CTA.
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T incl = warp_inclusive_sum(v);
  if (lane == 31) smem_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    T w = (lane < SCAN_THREADS / 32) ? smem_warp[lane] : T(0);
    T wi = warp_inclusive_sum(w);
    if (lane < SCAN_THREADS / 32) smem_warp[lane] = wi - w;
    if (lane == SCAN_THREADS / 32 - 1) *total = wi;
  }
  __syncthreads();
  T r = smem_warp[warp] + incl - v;
  __syncthreads();
  return r;
}

template <typename Tin>
__global__ void __launch_bounds__(SCAN_THREADS) tile_reduce_kernel(const Tin* __restrict__ in, int64_t n,
                                                                   int64_t* __restrict__ tile_sums) {
  __shared__ int64_t warp_sums[SCAN_THREADS / 32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int64_t s = 0;
#pragma unroll
  for (int it = 0; it < SCAN_ITEMS; ++it) {
    int64_t i = base + it * SCAN_THREADS + threadIdx.x;
    if (i < n) s += (int64_t)in[i];
  }
  s = warp_sum(s);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warp_sums[warp] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t t = 0;
    for (int w = 0; w < SCAN_THREADS / 32; ++w) t += warp_sums[w];
    tile_sums[blockIdx.x] = t;
  }
}

// One CTA scans the tile sums in place (exclusive); writes the total.
__global__ void __launch_bounds__(SCAN_THREADS) tile_sums_scan_kernel(int64_t* __restrict__ tile_sums, int64_t n_tiles,
                                                                      int64_t* __restrict__ total_out) {
  __shared__ int64_t warp_sums[SCAN_THREADS / 32];
  __shared__ int64_t chunk_total;
  int64_t carry = 0;
  for (int64_t base = 0; base < n_tiles; base += SCAN_THREADS) {
    int64_t i = base + threadIdx.x;
    int64_t v = (i < n_tiles) ? tile_sums[i] : 0;
    int64_t ex = block_exclusive_scan<int64_t>(v, warp_sums, &chunk_total);
    if (i < n_tiles) tile_sums[i] = carry + ex;
    __syncthreads();
    carry += chunk_total;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total_out = carry;
}

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(SCAN_THREADS) tile_scan_kernel(const Tin* __restrict__ in, int64_t n,
                                                                 const int64_t* __restrict__ tile_offsets,
                                                                 Tout* __restrict__ out) {
  __shared__ int64_t warp_sums[SCAN_THREADS / 32];
  __shared__ int64_t total;
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  // Each thread owns SCAN_ITEMS consecutive elements (blocked arrangement).
  int64_t vals[SCAN_ITEMS];
  int64_t local = 0;
#pragma unroll
  for (int it = 0; it < SCAN_ITEMS; ++it) {
    int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + it;
    vals[it] = (i < n) ? (int64_t)in[i] : 0;
    local += vals[it];
  }
  int64_t ex = block_exclusive_scan<int64_t>(local, warp_sums, &total) + tile_offsets[blockIdx.x];
#pragma unroll
  for (int it = 0; it < SCAN_ITEMS; ++it) {
    int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + it;
    if (i < n) out[i] = (Tout)ex;
    ex += vals[it];
  }
}

template <typename Tout>
__global__ void copy_total_kernel(const int64_t* __restrict__ src, Tout* __restrict__ dst) {
  if (threadIdx.x == 0) *dst = (Tout)(*src);
}

int64_t scan_n_tiles(int64_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

template <typename Tin, typename Tout>
int exclusive_scan(const Tin* in, int64_t n, Tout* out, void* scratch, size_t scratch_bytes, cudaStream_t st) {
  if (n < 0 || out == nullptr || (n > 0 && in == nullptr)) return VX_ERR_ARG;
  const int64_t nt = scan_n_tiles(n);
  if (scratch_bytes < (size_t)(nt + 1) * sizeof(int64_t) || (nt > 0 && scratch == nullptr)) return VX_ERR_ARG;
  int64_t* tiles = reinterpret_cast<int64_t*>(scratch);
  if (n == 0) {
    // out[0] = 0
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(Tout), st);
    return cuda_status(e);
  }
  tile_reduce_kernel<Tin><<<(unsigned)nt, SCAN_THREADS, 0, st>>>(in, n, tiles);
  int s = launch_status(); if (s) return s;
  // The grand total lands in tiles[nt] and is then copied to out[n] as Tout.
  tile_sums_scan_kernel<<<1, SCAN_THREADS, 0, st>>>(tiles, nt, tiles + nt);
  s = launch_status(); if (s) return s;
  tile_scan_kernel<Tin, Tout><<<(unsigned)nt, SCAN_THREADS, 0, st>>>(in, n, tiles, out);
  s = launch_status(); if (s) return s;
  copy_total_kernel<Tout><<<1, 32, 0, st>>>(tiles + nt, out + n);
  return launch_status();
}

template int exclusive_scan<int64_t, int64_t>(const int64_t*, int64_t, int64_t*, void*, size_t, cudaStream_t);
template int exclusive_scan<int32_t, int64_t>(const int32_t*, int64_t, int64_t*, void*, size_t, cudaStream_t);

}  // namespace vx

extern "C" {

size_t vx_scan_scratch_bytes(int64_t n) {
  if (n < 0) n = 0;
  return (size_t)(vx::scan_n_tiles(n) + 1) * sizeof(int64_t);
}

int vx_exclusive_scan_i64(const int64_t* in, int64_t n, int64_t* out, void* scratch, size_t scratch_bytes,
                          void* stream) {
  return vx::exclusive_scan<int64_t, int64_t>(in, n, out, scratch, scratch_bytes, vx::as_stream(stream));
}

int vx_exclusive_scan_i32(const int32_t* in, int64_t n, int64_t* out, void* scratch, size_t scratch_bytes,
                          void* stream) {
  return vx::exclusive_scan<int32_t, int64_t>(in, n, out, scratch, scratch_bytes, vx::as_stream(stream));
}

}  // extern "C"
