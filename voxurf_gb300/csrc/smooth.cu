// Gaussian smoothing of the SDF grid and its adjoint.
//
// Replaces nn.Conv3d(1,1,k,padding=k//2,padding_mode='replicate') with the
// normalised Gaussian of Voxurf._gaussian_3dconv (lib/voxurf_fine.py:246-258,
// applied every step at voxurf_fine.py:638; voxurf_coarse.py:180-198, 531).
// exp(-(x^2+y^2+z^2)/(2 s^2)) / sum factorises exactly into three normalised
// 1-D kernels, so the k^3-tap convolution becomes three k-tap passes with
// clamped (replicate) indices.  The backward is the exact adjoint of each
// clamped pass.
//
// One kernel does all three passes in one sweep of the grid.  A CTA owns a
// 32 (y) x 32 (z) column tile and a chunk of x; it streams the chunk's
// x-planes (plus an H-plane halo on each side) through a 4-deep ring of
// shared-memory stages filled by 4-byte cp.async copies (clamped source
// coordinates for the forward, zero fill outside the grid for the adjoint;
// each thread's copy offsets are computed once).  The z pass runs on
// four-output register windows of the staged rows, the y pass on a
// four-output window of the z-passed column of each lane (a warp owns four
// y rows), and the last 2H+1 y-passed values of each of a thread's four
// output columns stay in registers for the x pass; output planes leave as
// 128-byte coalesced rows.  Shared rows have odd padded strides (no bank
// conflicts).  Each input voxel is read from DRAM about once; the x halos
// are mostly L2 hits because the chunks of one tile are neighbouring CTAs.
#include "common.cuh"

namespace vx {

struct Taps {
  float w[9];
  int h;  // half width, ksize = 2h+1 (<= 9)
};

constexpr int SM_T = 32;        // column tile: 32 (y) x 32 (z)
constexpr int SM_THREADS = 256, SM_STAGES = 4;
constexpr int SM_ROWS = SM_T / (SM_THREADS / 32);  // y rows per warp
static_assert(SM_ROWS == 4, "four y rows per warp: one window of pass4");

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// 4-byte asynchronous global->shared copy to a shared-window address;
// src_bytes 0 writes a zero.
__device__ __forceinline__ void cp_async4_s(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit_group() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Adjoint of one clamped 1-D convolution at output position j (0 or n-1) of
// an axis of length n, reading the gradient at position j+d through rel(d)
// for d in [-H, H] (zero outside [0, n)).  Only the two boundary positions
// take this path: they also collect the taps that the forward clamped onto
// them.  The offsets are compile-time after unrolling, so rel may index a
// register array.
template <int H, typename Rel>
__device__ __forceinline__ float adjoint_boundary(const float (&w)[2 * H + 1], int j, int n, Rel rel) {
  float acc = 0.f;
  if (n == 1) {
    float s = 0.f;
#pragma unroll
    for (int tt = -H; tt <= H; ++tt) s += w[tt + H];
    return s * rel(0);
  }
  if (j == 0) {
#pragma unroll
    for (int i = 0; i <= H; ++i) {  // gradient positions i = 0 .. H
      if (i < n) {
        float s = 0.f;
#pragma unroll
        for (int tt = -H; tt <= -i; ++tt) s += w[tt + H];
        acc += s * rel(i);
      }
    }
  } else {  // j == n - 1
#pragma unroll
    for (int d = -H; d <= 0; ++d) {  // gradient positions n-1+d, ascending
      if (n - 1 + d >= 0) {
        float s = 0.f;
#pragma unroll
        for (int tt = -d; tt <= H; ++tt) s += w[tt + H];
        acc += s * rel(d);
      }
    }
  }
  return acc;
}

// Four consecutive outputs j0 .. j0+3 of one 1-D pass along an axis of
// length n, from a register window win[k] = value at position j0 - H + k
// (clamped copies for the forward, zero outside [0, n) for the adjoint).
// The adjoint is the transposed convolution (flipped taps) except at the
// two boundary positions.  Window offsets are compile-time after unrolling.
template <bool ADJOINT, int H>
__device__ __forceinline__ void pass4(const float (&w)[2 * H + 1], const float (&win)[4 + 2 * H], int j0, int n,
                                      float (&out)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int j = j0 + i;
    float acc = 0.f;
    if (ADJOINT) {
      if (j == 0 || j == n - 1) {
        acc = adjoint_boundary<H>(w, j, n, [&](int d) { return win[i + H + d]; });
      } else {
#pragma unroll
        for (int tt = H; tt >= -H; --tt) acc += w[H - tt] * win[i + H + tt];
      }
    } else {
#pragma unroll
      for (int tt = -H; tt <= H; ++tt) acc += w[tt + H] * win[i + H + tt];
    }
    out[i] = acc;
  }
}

template <int H>
struct SmGeom {
  static constexpr int PY = SM_T + 2 * H;          // staged rows (y) incl. halo
  static constexpr int PZ = SM_T + 2 * H;          // staged columns (z) incl. halo
  static constexpr int SPZ = PZ + 1;               // padded row stride: odd, bank-conflict free
  static constexpr int SZQ = SM_T + 1;             // padded row stride of the z-passed rows
  static constexpr int NE = (PY * PZ + SM_THREADS - 1) / SM_THREADS;  // copies per thread and plane
};

template <bool ADJOINT, bool ACCUM, int H>
__global__ void __launch_bounds__(SM_THREADS, 3) smooth_march_kernel(const float* __restrict__ in,
                                                                     float* __restrict__ out, int X, int Y, int Z,
                                                                     int CX, int n_xc, int n_zt, Taps t) {
  using G = SmGeom<H>;
  constexpr int R = 2 * H + 1, PY = G::PY, PZ = G::PZ, SPZ = G::SPZ, SZQ = G::SZQ, NE = G::NE;
  constexpr int W = 4 + 2 * H;  // window of four outputs
  __shared__ __align__(16) float s_in[SM_STAGES][PY][SPZ];
  __shared__ float s_zq[PY][SZQ];
  float w[R];
#pragma unroll
  for (int i = 0; i < R; ++i) w[i] = t.w[i];
  const int xc = blockIdx.x % n_xc, tile = blockIdx.x / n_xc;
  const int y0 = (tile / n_zt) * SM_T, z0 = (tile % n_zt) * SM_T;
  const int x0 = xc * CX, x1 = min(X, x0 + CX);
  const int NP = x1 - x0 + 2 * H;  // input planes x0-H .. x1-1+H
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gz = z0 + lane;
  const int64_t plane = (int64_t)Y * Z;

  // Copy plan of this thread (the same for every plane): halo-tile element
  // e = tid + 256 i -> shared offset soff (-1: none) and in-plane source
  // offset goff (clamped for the forward; -1 outside the grid for the adjoint).
  int soff[NE], goff[NE];
#pragma unroll
  for (int i = 0; i < NE; ++i) {
    const int e = tid + SM_THREADS * i;
    const int b = e / PZ, c = e - b * PZ;
    int gy = y0 + b - H, gzz = z0 + c - H;
    soff[i] = e < PY * PZ ? (b * SPZ + c) * 4 : -1;
    if (!ADJOINT) {
      gy = min(max(gy, 0), Y - 1);
      gzz = min(max(gzz, 0), Z - 1);
      goff[i] = gy * Z + gzz;
    } else {
      goff[i] = (gy >= 0 && gy < Y && gzz >= 0 && gzz < Z) ? gy * Z + gzz : -1;
    }
  }
  const uint32_t sbase = smem_addr(&s_in[0][0][0]);
  auto issue = [&](int q) {  // input plane x0 - H + q -> stage q % SM_STAGES
    const int gx = x0 - H + q;
    const uint32_t st = sbase + (uint32_t)((q % SM_STAGES) * PY * SPZ * 4);
    if (!ADJOINT) {
      const float* base = in + (int64_t)min(max(gx, 0), X - 1) * plane;
#pragma unroll
      for (int i = 0; i < NE; ++i)
        if (soff[i] >= 0) cp_async4_s(st + (uint32_t)soff[i], base + goff[i], 4u);
    } else {
      const bool xin = gx >= 0 && gx < X;
      const float* base = in + (int64_t)(xin ? gx : 0) * plane;
#pragma unroll
      for (int i = 0; i < NE; ++i) {
        if (soff[i] < 0) continue;
        const bool ok = xin && goff[i] >= 0;
        cp_async4_s(st + (uint32_t)soff[i], ok ? base + goff[i] : in, ok ? 4u : 0u);
      }
    }
  };

#pragma unroll
  for (int s = 0; s < SM_STAGES - 1; ++s) {
    if (s < NP) issue(s);
    cp_async_commit_group();
  }
  float ring[SM_ROWS][R];
#pragma unroll
  for (int r = 0; r < SM_ROWS; ++r)
#pragma unroll
    for (int k = 0; k < R; ++k) ring[r][k] = 0.f;

  for (int p = 0; p < NP; ++p) {
    cp_async_wait_group<SM_STAGES - 2>();  // plane p has landed
    __syncthreads();
    {
      const int q = p + SM_STAGES - 1;  // refill the stage plane p-1 used
      if (q < NP) issue(q);
      cp_async_commit_group();
    }
    const float(*sp)[SPZ] = s_in[p % SM_STAGES];
    // z pass: task = four consecutive z outputs of one staged row
    for (int task = tid; task < PY * (SM_T / 4); task += SM_THREADS) {
      const int oct = task / PY, b = task - oct * PY;
      float win[W], o4[4];
#pragma unroll
      for (int k = 0; k < W; ++k) win[k] = sp[b][4 * oct + k];
      pass4<ADJOINT, H>(w, win, z0 + 4 * oct, Z, o4);
#pragma unroll
      for (int i = 0; i < 4; ++i) s_zq[b][4 * oct + i] = o4[i];
    }
    __syncthreads();
    // y pass: this warp's four rows of this lane's column, into the x ring
    {
      float win[W], o4[4];
#pragma unroll
      for (int k = 0; k < W; ++k) win[k] = s_zq[SM_ROWS * warp + k][lane];
      pass4<ADJOINT, H>(w, win, y0 + SM_ROWS * warp, Y, o4);
#pragma unroll
      for (int r = 0; r < SM_ROWS; ++r) {
#pragma unroll
        for (int k = 0; k < R - 1; ++k) ring[r][k] = ring[r][k + 1];
        ring[r][R - 1] = o4[r];
      }
    }
    // x pass: ring[r][k] holds input plane gxo - H + k of output plane gxo
    const int gxo = x0 + p - 2 * H;
    if (gxo < x0 || gz >= Z) continue;
#pragma unroll
    for (int r = 0; r < SM_ROWS; ++r) {
      const int gy = y0 + SM_ROWS * warp + r;
      if (gy >= Y) continue;
      float acc = 0.f;
      if (ADJOINT) {
        if (gxo == 0 || gxo == X - 1) {
          acc = adjoint_boundary<H>(w, gxo, X, [&](int d) { return ring[r][d + H]; });
        } else {
#pragma unroll
          for (int tt = H; tt >= -H; --tt) acc += w[H - tt] * ring[r][tt + H];
        }
      } else {
#pragma unroll
        for (int tt = -H; tt <= H; ++tt) acc += w[tt + H] * ring[r][tt + H];
      }
      const int64_t o = (int64_t)gxo * plane + (int64_t)gy * Z + gz;
      if (ACCUM)
        out[o] += acc;
      else
        out[o] = acc;
    }
  }
  cp_async_wait_group<0>();
}

// x chunking: about two waves of 3 resident CTAs per SM, chunks of >= 8 planes.
template <bool ADJOINT, bool ACCUM, int H>
static void launch_march(const float* in, float* out, int X, int Y, int Z, const Taps& t, cudaStream_t st) {
  const int n_zt = (Z + SM_T - 1) / SM_T, n_yt = (Y + SM_T - 1) / SM_T;
  const int64_t tiles = (int64_t)n_zt * n_yt;
  const int64_t want = (int64_t)sm_count() * 3 * 2;
  int64_t nx = (want + tiles - 1) / tiles;
  const int64_t nx_max = (X + 7) / 8;
  nx = nx < 1 ? 1 : (nx > nx_max ? nx_max : nx);
  int n_xc = (int)nx;
  const int CX = (X + n_xc - 1) / n_xc;
  n_xc = (X + CX - 1) / CX;
  const unsigned blocks = (unsigned)(tiles * n_xc);
  smooth_march_kernel<ADJOINT, ACCUM, H><<<blocks, SM_THREADS, 0, st>>>(in, out, X, Y, Z, CX, n_xc, n_zt, t);
}

template <bool ADJOINT, bool ACCUM>
static void launch_h(const float* in, float* out, int X, int Y, int Z, const Taps& t, cudaStream_t st) {
  switch (t.h) {
    case 0: launch_march<ADJOINT, ACCUM, 0>(in, out, X, Y, Z, t, st); break;
    case 1: launch_march<ADJOINT, ACCUM, 1>(in, out, X, Y, Z, t, st); break;
    case 2: launch_march<ADJOINT, ACCUM, 2>(in, out, X, Y, Z, t, st); break;
    case 3: launch_march<ADJOINT, ACCUM, 3>(in, out, X, Y, Z, t, st); break;
    default: launch_march<ADJOINT, ACCUM, 4>(in, out, X, Y, Z, t, st); break;
  }
}

static int make_taps(const float* taps_host, int ksize, Taps& t) {
  if (ksize < 1 || ksize > 9 || (ksize % 2) == 0) return VX_ERR_ARG;
  t.h = ksize / 2;
  for (int i = 0; i < 9; ++i) t.w[i] = i < ksize ? taps_host[i] : 0.f;
  return VX_OK;
}

}  // namespace vx

using namespace vx;

extern "C" {

int vx_smooth3d(const float* in, float* out, float* tmp1, float* tmp2, int64_t X, int64_t Y, int64_t Z,
                const float* taps_host, int ksize, void* stream) {
  (void)tmp1;
  (void)tmp2;
  if (X <= 0 || Y <= 0 || Z <= 0 || !in || !out || !taps_host) return VX_ERR_ARG;
  if (X * Y * Z > INT32_MAX) return VX_ERR_ARG;
  Taps t;
  const int s = make_taps(taps_host, ksize, t);
  if (s) return s;
  launch_h<false, false>(in, out, (int)X, (int)Y, (int)Z, t, as_stream(stream));
  return launch_status();
}

int vx_smooth3d_adjoint(const float* grad_out, float* grad_in, float* tmp1, float* tmp2, int64_t X, int64_t Y,
                        int64_t Z, const float* taps_host, int ksize, int accumulate, void* stream) {
  (void)tmp1;
  (void)tmp2;
  if (X <= 0 || Y <= 0 || Z <= 0 || !grad_out || !grad_in || !taps_host) return VX_ERR_ARG;
  if (X * Y * Z > INT32_MAX) return VX_ERR_ARG;
  Taps t;
  const int s = make_taps(taps_host, ksize, t);
  if (s) return s;
  cudaStream_t st = as_stream(stream);
  if (accumulate)
    launch_h<true, true>(grad_out, grad_in, (int)X, (int)Y, (int)Z, t, st);
  else
    launch_h<true, false>(grad_out, grad_in, (int)X, (int)Y, (int)Z, t, st);
  return launch_status();
}

}  // extern "C"
