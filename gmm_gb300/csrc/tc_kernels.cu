// Tensor-core (tcgen05) E-step for sm_103a.
//
// The diagonal-covariance log-likelihood is a contraction:
//   s_fm = sum_k Z_fk W_km,  Z_f = [x_f | 1 | 0... | x_f^2 | 0...] (x_d at column d, the
//   constant at D, x_d^2 at K/2 + d), W_m = log2(e) * [mu_m / var_m | c_m | -1 / (2 var_m)],
//   c_m  = log w_m - D/2 log 2pi - 1/2 sum log var_m - 1/2 sum mu_m^2 / var_m
// (log2 units), K = 2D+1 padded to a multiple of 16. Z and W are each held as three bf16 planes
// (v = p1 + p2 + p3, each plane the bf16 rounding of what the previous ones left), and the
// contraction sums the six plane products p_i q_j with i + j <= 2 (0-based) into an FP32 TMEM
// accumulator: every operand is represented to ~2^-24 relative, so the logits carry FP32-level
// error from the accumulation alone.
//
// Operand planes live in HBM as core-matrix tile images: for each plane and each 128-row tile,
// [K/8 column chunks][128 rows][8 bf16], i.e. exactly the no-swizzle UMMA layout, contiguous
// (K x 256 bytes). A tile reaches shared memory in one cp.async.bulk.tensor.2d copy per plane over a
// [rows][128 elements] view (256-byte rows).
//
// A tcgen05.mma with M = 128 and K = 16 costs max(45.5, N / 2) cycles on GB300 (measured), so
// both kernels use N >= 128 for the logits. Two kernels per E-step. Each has one TMA-producer
// warp, MMA-issuing threads in warps on different SM sub-partitions and epilogue warps that each
// own one TMEM lane quadrant (32 rows); the logits MMAs take their A operand from TMEM
// (tcgen05.mma ... [a_tmem], b_desc), so mostly B is read from shared memory. The tensor pipe
// accepts only a few MMAs ahead, and an issuing warp shares its sub-partition with busy epilogue
// warps: two issuers and fully unrolled issue loops (descriptor = per-stage base + constant).
//   ll_kernel  (frame-tile major, persistent): four loader warps fill the 128-frame Z tile in
//              TMEM -- for K <= 80 built from the raw frames on every pass (and written to the
//              plane images on the first), for larger K copied from the plane images --
//              double-buffered where it fits; 128-component W chunks stream through a TMA ring; S[128 frames x 128
//              comps] accumulates in one of two TMEM buffers; the epilogue releases each buffer
//              as soon as it has read it and runs an online log2-sum-exp over all chunks ->
//              per-frame log-likelihood.
//   acc_kernel (component-chunk major, AccCfg: 128-frame tiles, a TMEM plan per K and
//              statistics width): the chunk's W planes are stored into TMEM once (plane 2 in
//              shared memory where TMEM is short); Z tiles stream through a TMA ring. The MMA
//              computes S^T[128 comps x 128 frames]; the epilogue turns it in place into
//              posteriors gamma = 2^(s - ll) (pruned at minGamma, split into bf16 hi + lo) and
//              the statistics MMA uses those TMEM columns as its A operand: D2[comps x N2] +=
//              Gamma^T Z with the five products hi*Z1 + hi*Z2 + hi*Z3 + lo*Z1 + lo*Z2 (x and x^2
//              need all three planes: two leave a 2^-17 relative error that the variance update
//              S/n - mu^2 magnifies), i.e. n, F and S in one product (N2 = K), or only the leading
//              [x | 1] columns when no second-order statistics are wanted. Posteriors never
//              leave TMEM. An accumulator holds one tile's sums: the tensor core's FP32
//              accumulation over many tiles loses low bits steadily, so eight readout warps
//              (apart from the four posterior warps) read it as soon as the tile's MMAs are
//              done (two accumulators where TMEM allows, so the next tile's statistics MMAs queue
//              meanwhile), sum tiles in FP32 registers with round-to-nearest and move them into
//              FP64 partials every 8192 frames; a final kernel reduces the partials over CTAs in
//              a fixed order. Both MMA streams are issued by whole warps (one elected lane):
//              issued from a one-thread branch, the MMAs came slower than the tensor pipe runs
//              them whenever the posterior warps on the same sub-partition were busy.
// Every mbarrier wait is bounded (~2 s); on expiry the kernel raises an error flag, drains its
// own copies and MMAs (bounded), frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <math.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "gmm_internal.cuh"
#include "tc_ptx.cuh"

namespace gmm {

using namespace ptx;

namespace {

constexpr double kLog2e = 1.4426950408889634;
constexpr float kLn2 = 0.69314718055994531f;
constexpr long long kWaitLimit = kDefaultWaitLimit;  // the exit-path drains always use it

// ------------------------------------------------------------------ operand preparation

__device__ __forceinline__ void split3f(float v, uint16_t& a, uint16_t& b, uint16_t& c) {
  __nv_bfloat16 h1 = __float2bfloat16_rn(v);
  float r = v - __bfloat162float(h1);  // exact
  __nv_bfloat16 h2 = __float2bfloat16_rn(r);
  r = r - __bfloat162float(h2);  // exact
  __nv_bfloat16 h3 = __float2bfloat16_rn(r);
  a = __bfloat16_as_ushort(h1);
  b = __bfloat16_as_ushort(h2);
  c = __bfloat16_as_ushort(h3);
}

__device__ __forceinline__ void split3d(double v, uint16_t& a, uint16_t& b, uint16_t& c) {
  __nv_bfloat16 h1 = __float2bfloat16_rn((float)v);
  double r = v - (double)__bfloat162float(h1);
  __nv_bfloat16 h2 = __float2bfloat16_rn((float)r);
  r = r - (double)__bfloat162float(h2);
  __nv_bfloat16 h3 = __float2bfloat16_rn((float)r);
  a = __bfloat16_as_ushort(h1);
  b = __bfloat16_as_ushort(h2);
  c = __bfloat16_as_ushort(h3);
}

// Z planes as tile images: element (row f, column k) of plane p sits at
// ((p * nT + f / 128) * K/8 + k / 8) * 1024 + (f % 128) * 8 + k % 8; row f holds the operand
// columns (x at d, 1 at D, x^2 at K/2 + d) of frame row_frame[f] (identity when row_frame is
// null), zero for padding rows (past N, or row_frame < 0). The logits kernel's loader warps
// build them on their first pass over the frames (features_row_to_tmem), hidden behind the
// MMAs: for K <= 80 straight into the second TMEM Z buffer, for larger K (one Z buffer) one tile
// ahead into the images, copied into TMEM when the MMAs release the buffer.

// W planes as tile images (same layout as Z, rows = active components padded to 128, log2
// units); padded rows carry a constant of -1e30 so they never contribute.
// The model occupies rows [row0, row0 + Mpad) of planes that hold plane_rows rows each (several
// models can share one set of planes, each starting on a 128-row tile).
__global__ void model_kernel(int D, int K, int Mact, int Mpad, long long plane_rows, long long row0,
                             const int* __restrict__ act, const float* __restrict__ w,
                             const float* __restrict__ mu, const float* __restrict__ var,
                             uint16_t* __restrict__ planes, int* __restrict__ comp_of_row,
                             float* __restrict__ cent, const int* __restrict__ mact_dev) {
  if (mact_dev) Mact = *mact_dev;  // active count produced on the device (captured iterations)
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int KC = K / 8;
  if (t >= (long long)Mpad * K) return;
  const int e = (int)(t & 7), rr = (int)((t >> 3) & 127);
  const long long blk = t >> 10;
  const int cchunk = (int)(blk % KC);
  const int r = (int)(blk / KC) * 128 + rr;
  const int k = cchunk * 8 + e;
  if (k == 0) comp_of_row[r] = r < Mact ? act[r] : -1;
  // the centres of the statistics kernel's sums: the row's mean rounded to bf16 (any centre will
  // do; this one the statistics kernel holds in shared memory exactly), zero for padding rows
  if (k < D)
    cent[(size_t)(row0 + r) * D + k] =
        r < Mact ? __bfloat162float(__float2bfloat16_rn(mu[(size_t)act[r] * D + k])) : 0.0f;
  if (k == D) return;  // the constant column: model_const_kernel
  double v = 0.0;
  if (r < Mact) {
    const int m = act[r];
    const float* mm = mu + (size_t)m * D;
    const float* vv = var + (size_t)m * D;
    if (k < D) v = kLog2e * (double)mm[k] / (double)vv[k];
    else if (k >= K / 2 && k < K / 2 + D) v = -0.5 * kLog2e / (double)vv[k - K / 2];
  }
  uint16_t a, b, c;
  split3d(v, a, b, c);
  const size_t plane = (size_t)plane_rows * K;
  const size_t o = (size_t)row0 * K + t;
  planes[o] = a;
  planes[plane + o] = b;
  planes[2 * plane + o] = c;
}

// The constant column (k = D) of the W planes, one warp per row: log w - D/2 log 2pi
// - 1/2 sum log var - 1/2 sum mu^2/var in FP64, the lanes over d and a shuffle reduction (GB300's
// FP64 rate is 1/64 of FP32, so the D logarithms of a row are spread over a warp, and the rows
// over the SMs); padded rows get -1e30 so they never contribute.
__global__ void model_const_kernel(int D, int K, int Mact, int Mpad, long long plane_rows, long long row0,
                                   const int* __restrict__ act, const float* __restrict__ w,
                                   const float* __restrict__ mu, const float* __restrict__ var,
                                   uint16_t* __restrict__ planes, const int* __restrict__ mact_dev) {
  if (mact_dev) Mact = *mact_dev;
  const int r = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= Mpad) return;
  double v = -1e30;
  if (r < Mact) {
    const int m = act[r];
    const float* mm = mu + (size_t)m * D;
    const float* vv = var + (size_t)m * D;
    double sl = 0.0, q = 0.0;
    for (int d = lane; d < D; d += 32) {
      sl += log((double)vv[d]);
      q += (double)mm[d] * (double)mm[d] / (double)vv[d];
    }
    for (int o = 16; o; o >>= 1) {
      sl += __shfl_xor_sync(0xffffffffu, sl, o);
      q += __shfl_xor_sync(0xffffffffu, q, o);
    }
    v = kLog2e * (log((double)w[m]) + kMinusLog2Pi * D / 2.0 - 0.5 * sl - 0.5 * q);
  }
  if (lane != 0) return;
  uint16_t a, b, c;
  split3d(v, a, b, c);
  const int KC = K / 8;
  const size_t t = ((size_t)((r >> 7) * KC + (D >> 3)) << 10) | ((size_t)(r & 127) << 3) | (size_t)(D & 7);
  const size_t plane = (size_t)plane_rows * K;
  const size_t o = (size_t)row0 * K + t;
  planes[o] = a;
  planes[plane + o] = b;
  planes[2 * plane + o] = c;
}

void launch_model(Ctx* c, int D, int K, int Mact, int Mpad, long long plane_rows, long long row0, const int* act,
                  const float* w, const float* mu, const float* var, uint16_t* planes, int* comp_of_row,
                  float* cent, const int* mact_dev) {
  {
    GMM_LAUNCH(c, "tc_model_kernel");
    const long long tot = (long long)Mpad * K;
    model_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(D, K, Mact, Mpad, plane_rows, row0, act, w,
                                                                       mu, var, planes, comp_of_row, cent, mact_dev);
  }
  {
    GMM_LAUNCH(c, "tc_model_const_kernel");
    model_const_kernel<<<(unsigned)((Mpad + 7) / 8), 256, 0, c->stream>>>(D, K, Mact, Mpad, plane_rows, row0, act,
                                                                          w, mu, var, planes, mact_dev);
  }
}

// ------------------------------------------------------------------ shared helpers

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~(uintptr_t)1023);
}

// Wait without the abort short-cut (used to drain in-flight work on the exit path).
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > kWaitLimit) break;
}

// Copy one plane of one 128-row tile image into shared memory: one copy of K x 256 bytes.
__device__ __forceinline__ void load_image(uint8_t* dst, const CUtensorMap* map, int plane, int nT, int K, int tile,
                                           uint64_t* bar) {
  tma_load_2d(dst, map, 0, (plane * nT + tile) * K, bar);
}

__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Plane products (Z plane, W plane) with i + j <= 4 (1-based), small terms first.
// (Z plane, W plane) of product pr: (2,0) (1,1) (0,2) (1,0) (0,1) (0,0).
__host__ __device__ constexpr int prod_z(int pr) { return pr == 0 ? 2 : (pr == 1 || pr == 3) ? 1 : 0; }
__host__ __device__ constexpr int prod_w(int pr) { return pr == 2 ? 2 : (pr == 1 || pr == 4) ? 1 : 0; }

// The MMA issuer shares its SM sub-partition with busy epilogue warps and the tensor pipe
// accepts only a few MMAs ahead, so every cycle between two tcgen05.mma instructions can leave
// the pipe idle. The issue loops below are fully unrolled: each descriptor is a per-stage base
// plus a compile-time offset (the 14-bit address field of a shared-memory descriptor counts
// 16-byte units, and no operand crosses 256 KB), and the accumulate flags are constants.
__device__ __forceinline__ uint64_t desc_add(uint64_t base, uint32_t byte_offset) {
  return base + (uint64_t)(byte_offset >> 4);
}

// Copies row `r` of one 128-row tile image (all three planes) from HBM into TMEM, laid out as
// a tcgen05 A operand: lane = row, each 32-bit column holds two consecutive bf16 of K. Plane p
// occupies columns [col + p K/2, col + (p+1) K/2). Called by a whole warp (lane = row within
// its 32-lane quadrant); `valid` false stores zeros.
__device__ __forceinline__ void image_row_to_tmem(const uint16_t* __restrict__ planes, int nT, int K,
                                                  int tile, int r, uint32_t taddr, bool valid) {
  const int KC = K / 8;
  for (int p = 0; p < 3; ++p) {
    const uint4* src = reinterpret_cast<const uint4*>(planes + ((size_t)(p * nT + tile) * KC) * 1024 + (size_t)r * 8);
    for (int c = 0; c < KC; c += 2) {
      uint4 u0 = make_uint4(0, 0, 0, 0), u1 = make_uint4(0, 0, 0, 0);
      if (valid) {
        u0 = __ldg(src + (size_t)c * 128);
        u1 = __ldg(src + (size_t)(c + 1) * 128);
      }
      const uint32_t w[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
      tmem_st8(taddr + p * (K / 2) + c * 4, w);
    }
  }
}

// image_row_to_tmem for a row that this thread wrote into the images earlier in the same kernel:
// coherent loads (ld.global, ordered after the thread's own stores), not the read-only path.
__device__ __forceinline__ uint4 ld_global_v4(const void* p) {
  uint4 v;
  asm volatile("ld.global.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(reinterpret_cast<uint64_t>(p))
               : "memory");
  return v;
}
template <int K>
__device__ __forceinline__ void own_image_row_to_tmem(const uint16_t* planes, int nT, int tile, int r,
                                                      uint32_t taddr, bool valid) {
  constexpr int KC = K / 8;
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const uint4* src = reinterpret_cast<const uint4*>(planes + ((size_t)(p * nT + tile) * KC) * 1024 + (size_t)r * 8);
#pragma unroll
    for (int c = 0; c < KC; c += 2) {
      uint4 u0 = make_uint4(0, 0, 0, 0), u1 = make_uint4(0, 0, 0, 0);
      if (valid) {
        u0 = ld_global_v4(src + (size_t)c * 128);
        u1 = ld_global_v4(src + (size_t)(c + 1) * 128);
      }
      const uint32_t w[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
      tmem_st8(taddr + p * (K / 2) + c * 4, w);
    }
  }
}

// Row `r` of tile `tile` built from the raw features instead: the operand columns of
// frame f (zeros when f < 0 or !valid), split into three bf16 planes, stored into TMEM (laid out
// as image_row_to_tmem does) and, with TO_IMAGES, into the plane images, which the statistics
// kernel reads next. Building from the 4D bytes of a frame is cheaper than copying its 6K bytes
// of images (at N = 10M, M = 2048, D = 39: 8.65 ms for the logits kernel that builds and writes
// the images, 9.31 ms for one that copies them), so the logits kernel builds from the frames on
// every pass where it has two Z buffers.
// The row's D <= K/2 - 1 features are loaded into registers first (independent loads, one
// latency); the squares sit at the constant column K/2 + d, so every register index is static.
template <int K, bool TO_TMEM = true, bool TO_IMAGES = true>
__device__ __forceinline__ void features_row_to_tmem(const float* __restrict__ X, int D, long long f,
                                                     uint16_t* __restrict__ planes, int nT, int tile, int r,
                                                     uint32_t taddr, bool valid) {
  constexpr int KC = K / 8, DMAX = K / 2 - 1;
  const bool live = valid && f >= 0;
  const float* xr = X + (live ? f : 0) * (long long)D;
  float xv[DMAX];
#pragma unroll
  for (int d = 0; d < DMAX; ++d) xv[d] = (live && d < D) ? __ldg(xr + d) : 0.0f;
#pragma unroll
  for (int c = 0; c < KC; c += 2) {
    uint32_t w[3][8];
#pragma unroll
    for (int e = 0; e < 16; e += 2) {
      uint16_t a[2], b[2], cc[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int k = c * 8 + e + u;  // compile-time
        float v = 0.0f;
        if (k < K / 2) {
          if (k < DMAX && k < D) v = xv[k < DMAX ? k : 0];
          else if (k == D && live) v = 1.0f;
        } else if (k - K / 2 < DMAX) {
          const float x = xv[k - K / 2 < DMAX ? k - K / 2 : 0];
          v = __fmul_rn(x, x);  // zero for d >= D (xv is zero there)
        }
        split3f(v, a[u], b[u], cc[u]);
      }
      w[0][e >> 1] = a[0] | ((uint32_t)a[1] << 16);
      w[1][e >> 1] = b[0] | ((uint32_t)b[1] << 16);
      w[2][e >> 1] = cc[0] | ((uint32_t)cc[1] << 16);
    }
#pragma unroll
    for (int p = 0; p < 3; ++p) {
      if constexpr (TO_TMEM) tmem_st8(taddr + p * (K / 2) + c * 4, w[p]);
      if (TO_IMAGES && valid) {
        uint4* dst = reinterpret_cast<uint4*>(planes + ((size_t)(p * nT + tile) * KC + c) * 1024 + (size_t)r * 8);
        dst[0] = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
        dst[128] = make_uint4(w[p][4], w[p][5], w[p][6], w[p][7]);  // chunk c + 1: 1024 elements on
      }
    }
  }
}

// Sparse tile schedule: the sorted frames' operand planes (built from the raw features as the
// logits kernel builds them), their log2-LSE values, their frame indices, and per sorted tile the
// union of its frames' chunk masks. One CTA per 128-row tile, thread = row.
template <int K>
__global__ void __launch_bounds__(128) sort_rows_kernel(const float* __restrict__ X, int D, long long N,
                                                        const int* __restrict__ perm, const float* __restrict__ ll2,
                                                        const uint32_t* __restrict__ fmask,
                                                        uint16_t* __restrict__ planes, float* __restrict__ sll2,
                                                        long long* __restrict__ srow, uint32_t* __restrict__ tmask,
                                                        int nT) {
  __shared__ uint32_t red[4];
  const int tile = blockIdx.x, r = threadIdx.x;
  const long long row = (long long)tile * 128 + r;
  const int o = perm[row];  // the row's place before the sort (frame index, or padding past N)
  const long long f = o < N ? (long long)o : -1LL;
  features_row_to_tmem<K, false>(X, D, f, planes, nT, tile, r, 0, true);
  sll2[row] = ll2[o];
  srow[row] = f;
  uint32_t m = fmask[o];
  for (int k = 16; k; k >>= 1) m |= __shfl_xor_sync(0xffffffffu, m, k);
  if ((r & 31) == 0) red[r >> 5] = m;
  __syncthreads();
  if (r == 0) tmask[tile] = red[0] | red[1] | red[2] | red[3];
}

// ------------------------------------------------------------------ log-likelihood kernel

// Z tiles (the A operand: 128 frames x K, 3 planes) live in TMEM, double-buffered when it fits;
// W chunks (128 components) stream through an NW-stage shared-memory ring. The MMAs read only W
// from shared memory (A from TMEM), which leaves shared-memory bandwidth for the TMA ring.
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int cmin(int a, int b) { return a < b ? a : b; }
__host__ __device__ constexpr int ll_zb(int K) { return K <= 80 ? 2 : 1; }
// With two Z buffers the loader warps build a tile from the raw features into TMEM (and the
// plane images) while the MMAs run on the previous one. With one, they build the next tile's
// plane images while the MMAs run on the current tile and copy them into TMEM when it is done.
__host__ __device__ constexpr int ll_nw(int K) { return K <= 96 ? 3 : 2; }
// With three W stages the TMA ring holds whole chunks (three planes each). With two, the two
// chunks in flight (one per MMA-issuing thread, their MMAs interleaved in the tensor pipe) end
// together, and a chunk-granular ring would refill both stages at once while the pipe waits. So
// two stages become six plane slots, filled in order of first use and released as soon as a
// plane's last product is issued: the MMAs order the products plane by plane (lo, then mid,
// then hi weight plane), which leaves each plane's slot half a chunk or more to refill.
__host__ __device__ constexpr bool ll_plane_ring(int K) { return ll_nw(K) == 2; }

template <int K>
struct LlCfg {
  static constexpr int ZB = ll_zb(K), NW = ll_nw(K);
  static constexpr int W_PLANE = 128 * K * 2;
  static constexpr int W_STAGE = 3 * W_PLANE;
  static constexpr int ZCOLS = 3 * K / 2;  // TMEM columns of one Z tile
  static constexpr int S_COL = 0;          // 2 accumulator buffers of 128 columns
  static constexpr int Z_COL = 256;        // Z buffers
  static constexpr int OFF_W = 0;
  static constexpr int OFF_BAR = OFF_W + NW * W_STAGE;
  static constexpr int OFF_MISC = OFF_BAR + 24 * 8;
  static constexpr int SMEM = cmax(OFF_MISC + 64 + 1024, 120 * 1024);
  // with frame masks: [chunks][128 rows] chunk maxima of the logits
  static constexpr int OFF_CM = OFF_MISC + 64;
  static constexpr int smem_with_masks(int chunks) { return cmax(SMEM, OFF_CM + chunks * 128 * 4 + 1024); }
  static_assert(Z_COL + ZB * ZCOLS <= 512, "TMEM budget");
};
constexpr int kLlThreads = 352;  // warp 0 TMA, 1 and 10 MMA, 2-5 epilogue, 6-9 Z loaders

template <int K>
__global__ void __launch_bounds__(kLlThreads, 1)
    ll_kernel(const __grid_constant__ CUtensorMap wfull, uint16_t* __restrict__ zplanes,
              long long N, const long long* __restrict__ row_frame, const int* __restrict__ tile_wbase,
              int nTz, int nTw, int tile0, int n_tiles, int n_chunks, float trouble2, float minLL,
              float* __restrict__ ll2_out, float* __restrict__ ll_out, double* __restrict__ llpart,
              int* __restrict__ err, const float* __restrict__ X, int D, int write_images, long long wait_limit,
              uint32_t* __restrict__ fmask, float mask_thr2, int single_comp, const int* __restrict__ mact_dev) {
  // frame tiles tile0 .. tile0 + n_tiles - 1, strided over the CTAs. With X the loaders build
  // the Z tiles from the raw features (and, with write_images, write the plane images for the
  // statistics kernel; with one Z buffer they always do); without, they copy them from the plane
  // images.
  using C = LlCfg<K>;
  constexpr int ZB = C::ZB, NW = C::NW;
  constexpr bool PR = ll_plane_ring(K);
  constexpr int NSLOT = PR ? 3 * NW : NW;  // W ring slots: planes or whole chunks
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
  uint64_t* z_full = bars + 0;   // [ZB <= 2]
  uint64_t* z_empty = bars + 2;  // [ZB]
  uint64_t* w_full = bars + 4;   // [NSLOT <= 6]
  uint64_t* w_empty = bars + 10; // [NSLOT]
  uint64_t* s_full = bars + 16;  // [2]
  uint64_t* s_empty = bars + 18; // [2]
  uint64_t* mma_done = bars + 20;  // [2]: one per MMA-issuing thread
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(smem + C::OFF_MISC);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::OFF_MISC + 8);
  float* cmax_s = reinterpret_cast<float*>(smem + C::OFF_CM);  // with fmask: chunk maxima

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // with an even chunk count two threads issue the MMAs, even chunks (buffer 0) and odd chunks
  // (buffer 1), from different SM sub-partitions: each competes with busy epilogue warps for
  // issue slots, and the tensor pipe accepts only a few MMAs ahead
  const bool two_issuers = (n_chunks % 2) == 0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < ZB; ++i) {
      mbar_init(&z_full[i], 4);
      mbar_init(&z_empty[i], two_issuers ? 2 : 1);
    }
    for (int i = 0; i < NSLOT; ++i) {
      mbar_init(&w_full[i], 1);
      mbar_init(&w_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&s_full[i], 1);
      mbar_init(&s_empty[i], 4);
    }
    mbar_init(&mma_done[0], 1);
    mbar_init(&mma_done[1], 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(tmem_holder, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const int my_tiles = (n_tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
  int w_issued = 0;  // W ring fills issued (loader thread)
  // plane ring: position of fill u (0 = the lo weight plane, 1 = mid, 2 = hi) of chunk j (counted
  // over the CTA's tiles) in the fill order. Two issuers take the chunks of a pair (j even, j + 1)
  // together, so their fills interleave; the slot is position % 6, its use count position / 6.
  auto wpos = [two_issuers](int j, int u) -> int {
    return two_issuers ? 6 * (j >> 1) + 2 * u + (j & 1) : 3 * j + u;
  };

  if (warp == 0) {
    if (lane == 0 && my_tiles > 0) {
      prefetch_tmap(&wfull);
      int j = 0;
      bool ok = true;
      for (int it = 0; it < my_tiles && ok; ++it) {
        // first W chunk of the tile's model (one model unless a per-tile base is given)
        const int wbase = tile_wbase ? tile_wbase[tile0 + (int)blockIdx.x + it * (int)gridDim.x] : 0;
        if constexpr (PR) {
          // fills in position order: a pair of chunks (two issuers) or one chunk at a time
          const int group = two_issuers ? 2 : 1;
          for (int ch = 0; ch < n_chunks && ok; ch += group, j += group) {
            for (int u = 0; u < 3 && ok; ++u) {
              for (int g = 0; g < group; ++g) {
                const int pos = wpos(j + g, u), ws = pos % NSLOT;
                if (!mbar_wait(&w_empty[ws], ((pos / NSLOT) & 1) ^ 1, abort_flag, wait_limit)) { ok = false; break; }
                mbar_arrive_expect_tx(&w_full[ws], C::W_PLANE);
                load_image(smem + C::OFF_W + ws * C::W_PLANE, &wfull, 2 - u, nTw, K, wbase + ch + g, &w_full[ws]);
                w_issued = pos + 1;
              }
            }
          }
        } else {
          for (int ch = 0; ch < n_chunks; ++ch, ++j) {
            const int ws = j % NW;
            if (!mbar_wait(&w_empty[ws], ((j / NW) & 1) ^ 1, abort_flag, wait_limit)) { ok = false; break; }
            mbar_arrive_expect_tx(&w_full[ws], C::W_STAGE);
            uint8_t* dst = smem + C::OFF_W + ws * C::W_STAGE;
            for (int p = 0; p < 3; ++p)
              load_image(dst + p * C::W_PLANE, &wfull, p, nTw, K, wbase + ch, &w_full[ws]);
            w_issued = j + 1;
          }
        }
      }
    }
  } else if (warp == 1 || warp == 10) {
    // one thread issues (here the warp-issued form of the statistics kernel measured slower:
    // 6.0 ms against 3.6 ms at N = 4M, M = 2048, D = 39)
    const int role = warp == 10;  // parity of the chunks this thread issues
    if (lane == 0 && my_tiles > 0 && (two_issuers || role == 0)) {
      const uint32_t idesc = idesc_bf16(128, 128, false, false);
      const uint32_t wb0 = smem_u32(smem + C::OFF_W);
      int j = 0;
      bool ok = true;
      for (int it = 0; it < my_tiles && ok; ++it) {
        const int zb = it % ZB;
        if (!mbar_wait(&z_full[zb], (it / ZB) & 1, abort_flag, wait_limit)) { ok = false; break; }
        const uint32_t za = tmem + C::Z_COL + zb * C::ZCOLS;
        for (int ch = 0; ch < n_chunks && ok; ++ch, ++j) {
          if (two_issuers && (ch & 1) != role) continue;
          const int b = j & 1;
          if (!mbar_wait(&s_empty[b], ((j >> 1) & 1) ^ 1, abort_flag, wait_limit)) { ok = false; break; }
          const uint32_t d = tmem + C::S_COL + b * 128;
          if constexpr (PR) {
            // products plane by plane: (hi, lo) | (mid, mid) (hi, mid) | (lo, hi) (mid, hi) (hi, hi)
            // as (Z plane, W plane); each W plane is waited for before its first product and
            // released after its last
            constexpr int kOrder[6] = {2, 1, 4, 0, 3, 5};
#pragma unroll
            for (int st = 0; st < 6; ++st) {
              const int pr = kOrder[st];
              const int u = 2 - prod_w(pr);  // fill of the chunk that holds the product's W plane
              const int pos = wpos(j, u), ws = pos % NSLOT;
              if (st == 0 || st == 1 || st == 3) {
                if (!mbar_wait(&w_full[ws], (pos / NSLOT) & 1, abort_flag, wait_limit)) { ok = false; break; }
                tc_fence_after();
              }
              const uint64_t wd = smem_desc(wb0 + ws * C::W_PLANE, 128 * 16, 128);
#pragma unroll
              for (int q = 0; q < K / 16; ++q) {
                const uint64_t bd = desc_add(wd, q * 2 * 128 * 16);
                const uint32_t a = za + prod_z(pr) * (K / 2) + q * 8;
                if (st == 0 && q == 0) mma_ts_c<false>(d, a, bd, idesc);
                else mma_ts_c<true>(d, a, bd, idesc);
              }
              if (st == 0 || st == 2 || st == 5) mma_commit(&w_empty[ws]);
            }
            if (!ok) break;
          } else {
            const int ws = j % NW;
            if (!mbar_wait(&w_full[ws], (j / NW) & 1, abort_flag, wait_limit)) { ok = false; break; }
            tc_fence_after();
            const uint64_t wd = smem_desc(wb0 + ws * C::W_STAGE, 128 * 16, 128);
#pragma unroll
            for (int pr = 0; pr < 6; ++pr) {
#pragma unroll
              for (int q = 0; q < K / 16; ++q) {
                const uint64_t bd = desc_add(wd, prod_w(pr) * C::W_PLANE + q * 2 * 128 * 16);
                const uint32_t a = za + prod_z(pr) * (K / 2) + q * 8;
                if (pr == 0 && q == 0) mma_ts_c<false>(d, a, bd, idesc);
                else mma_ts_c<true>(d, a, bd, idesc);
              }
            }
            mma_commit(&w_empty[ws]);
          }
          mma_commit(&s_full[b]);
          if (ch >= n_chunks - (two_issuers ? 2 : 1)) mma_commit(&z_empty[zb]);  // each issuer's last chunk
        }
      }
      mma_commit(&mma_done[role]);
      mbar_drain(&mma_done[role], 0);
    }
  } else if (warp >= 6) {
    // Z loaders: thread = frame row of the tile; fill the next TMEM Z buffer from HBM
    const int q4 = warp & 3;
    const int row = q4 * 32 + lane;
    const uint32_t lane_off = (uint32_t)(q4 * 32) << 16;
    for (int it = 0; it < my_tiles; ++it) {
      const int zb = it % ZB;
      const int tile = tile0 + (int)blockIdx.x + it * (int)gridDim.x;
      if (!mbar_wait_all(&z_empty[zb], ((it / ZB) & 1) ^ 1, abort_flag, wait_limit)) break;
      tc_fence_after();
      const uint32_t zaddr = tmem + lane_off + C::Z_COL + zb * C::ZCOLS;
      auto frame_of = [&](int t) -> long long {
        const long long rr = (long long)t * 128 + row;
        return t < nTz ? (row_frame ? row_frame[rr] : (rr < N ? rr : -1)) : -1;
      };
      if (!X) {
        image_row_to_tmem(zplanes, nTz, K, tile, row, zaddr, tile < nTz);
      } else if constexpr (ZB == 2) {
        if (write_images) features_row_to_tmem<K>(X, D, frame_of(tile), zplanes, nTz, tile, row, zaddr, tile < nTz);
        else features_row_to_tmem<K, true, false>(X, D, frame_of(tile), zplanes, nTz, tile, row, zaddr, tile < nTz);
      } else {
        if (it == 0) features_row_to_tmem<K, false>(X, D, frame_of(tile), zplanes, nTz, tile, row, 0, tile < nTz);
        own_image_row_to_tmem<K>(zplanes, nTz, tile, row, zaddr, tile < nTz);
      }
      tmem_st_wait();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&z_full[zb]);
      if constexpr (ZB == 1) {
        // the next tile's images, while the MMAs run on this one
        const int next = tile + (int)gridDim.x;
        if (X && it + 1 < my_tiles)
          features_row_to_tmem<K, false>(X, D, frame_of(next), zplanes, nTz, next, row, 0, next < nTz);
      }
    }
  } else {
    // epilogue: thread = frame row, one warp per lane quadrant taking all 128 columns of a chunk
    // (two warps per quadrant, each taking a 64-column half and merging the halves at the end of
    // the tile, measured 4.5% slower: more busy warps beside the MMA-issuing threads)
    const int q4 = warp & 3;
    const int row = q4 * 32 + lane;
    const uint32_t lane_off = (uint32_t)(q4 * 32) << 16;
    double llsum = 0.0;
    int j = 0;
    bool ok = true;
    for (int it = 0; it < my_tiles; ++it) {
      const int tile = tile0 + (int)blockIdx.x + it * (int)gridDim.x;
      float m = -INFINITY, sum = 0.0f;
      for (int ch = 0; ch < n_chunks && ok; ++ch, ++j) {
        const int b = j & 1;
        if (!mbar_wait_all(&s_full[b], (j >> 1) & 1, abort_flag, wait_limit)) { ok = false; break; }
        tc_fence_after();
        // read the whole row of the chunk, then hand the accumulator back to the MMA issuer before
        // doing the arithmetic: the issuer waits on this release, so it comes as early as possible
        uint32_t vv[4][32];
#pragma unroll
        for (int sub = 0; sub < 4; ++sub) tmem_ld32(tmem + lane_off + C::S_COL + b * 128 + 32 * sub, vv[sub]);
        tmem_ld_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&s_empty[b]);
        float cm = -INFINITY;
#pragma unroll
        for (int sub = 0; sub < 4; ++sub) {
          const uint32_t* v = vv[sub];
          float mx = __uint_as_float(v[0]);
#pragma unroll
          for (int k = 1; k < 32; ++k) mx = fmaxf(mx, __uint_as_float(v[k]));
          cm = fmaxf(cm, mx);
          const float mn = fmaxf(m, mx);
          if (mn > -INFINITY) {
            float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
            for (int k = 0; k < 32; k += 2) {
              s0 += ex2(__uint_as_float(v[k]) - mn);
              s1 += ex2(__uint_as_float(v[k + 1]) - mn);
            }
            sum = sum * ex2(m - mn) + (s0 + s1);
            m = mn;
          }
        }
        if (fmask) cmax_s[ch * 128 + row] = cm;  // the chunk's largest logit of the row
      }
      if (ok && !*abort_flag) {
        const float M2 = m, S2 = sum;
        // the chunks holding a logit within mask_thr2 of the frame's LSE (one component: every
        // real frame keeps it; trouble frames and padding keep nothing); trouble frames carry
        // +inf (every posterior prunes to 0), padding carries NaN
        const long long f = (long long)tile * 128 + row;  // padded row
        const long long fr = row_frame ? row_frame[f] : (f < N ? f : -1);
        float l2 = M2 + lg2(S2);
        const bool trouble = !(M2 > trouble2) || !isfinite(l2);
        if (fr >= 0) {
          ll2_out[f] = trouble ? INFINITY : l2;
          const float lnat = trouble ? minLL : l2 * kLn2;
          if (ll_out) ll_out[fr] = lnat;
          llsum += (double)lnat;
        } else {
          ll2_out[f] = __int_as_float(0x7fc00000);
        }
        if (fmask) {
          uint32_t msk = 0;
          if (fr >= 0 && !trouble) {
            if (mact_dev ? *mact_dev == 1 : single_comp != 0) {
              msk = 1u;
            } else {
              for (int q = 0; q < n_chunks; ++q)
                if (cmax_s[q * 128 + row] - l2 > mask_thr2) msk |= 1u << q;
            }
          }
          fmask[f] = msk;
        }
      }
      if (__any_sync(0xffffffffu, !ok || *abort_flag != 0)) break;  // the warp leaves together
    }
    llpart[(size_t)blockIdx.x * 128 + row] = llsum;
  }
  __syncthreads();
  if (*abort_flag) {
    // Every role has stopped. The loader's last NSLOT fills may still be in flight (a consumer
    // that gave up never waited for them): let them land before the CTA's shared memory goes.
    // Earlier fills were consumed, so they have landed.
    if (warp == 0 && lane == 0)
      for (int k = max(0, w_issued - NSLOT); k < w_issued; ++k) mbar_drain(&w_full[k % NSLOT], (k / NSLOT) & 1);
    if (threadIdx.x == 0) atomicExch(err, 1);
  }
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// ------------------------------------------------------------------ statistics kernel

// Accumulation periods of one CTA's tile range, identical for the MMA issuer and the epilogue:
// begin(j) must be called for j = 0, 1, 2, ... in order.
struct Periods {
  const int* slot;
  int t0, nt, defslot;
  int run_start = 0, period = -1;
  __device__ Periods(const int* s, int t0_, int nt_, int d) : slot(s), t0(t0_), nt(nt_), defslot(d) {}
  __device__ int slot_of(int j) const { return slot ? slot[t0 + j] : defslot; }
  __device__ bool begin(int j, int flush) {
    if (j == 0 || slot_of(j) != slot_of(j - 1)) run_start = j;
    const bool fresh = ((j - run_start) % flush) == 0;
    if (fresh) ++period;
    return fresh;
  }
  __device__ bool end(int j, int flush) const {
    return j == nt - 1 || slot_of(j + 1) != slot_of(j) || ((j + 1 - run_start) % flush) == 0;
  }
};

// Sparse statistics kernel (second-order statistics for K >= 96, where the dense kernel's split
// accumulators do not fit in TMEM): one CTA per (component chunk, frame range). The chunk's W planes sit in
// TMEM (A operand of the logits MMA); Z tiles and their frame LSE values stream through an
// NZ-stage TMA ring; the logits S^T[128 comps x 128 frames] go into one of NS TMEM buffers.
//
// The epilogue does not multiply dense posteriors. At minGamma = 1e-4 only a few components of
// a frame keep a posterior (7.5 of 2048 on average in UBM EM, N = 10M, M = 2048, D = 39), so it
// finds the kept (frame, component) pairs and accumulates only those:
//   n += g,  F' += g (x - c),  S' += g (x - c)^2        (FP32, round to nearest)
// around a per-component centre c (the component's mean at this E-step; cent[]), with the lanes
// over dimensions (two per lane, one packed FP32x2 instruction for both). Sums around the
// centre carry no cancellation: the variance update S/n - mu^2 no longer magnifies their
// rounding. The readers of the partials add the centre back in FP64 (tc_uncentre_*). x comes
// from the frame's FP32 row in HBM (prefetched into L2 a few tiles ahead, read through L1).
// A second tcgen05 GEMM (Gamma^T Z, five split-bf16 products per tile) did this before: the
// tensor core's FP32 accumulation rounds toward zero, which biased F/n and S/n by -5e-8
// relative, and the variance update magnified that up to 175 times (worst variance 2.1e-5
// relative at N = 1M, M = 2048, D = 39, against 3.9e-6 now).
//
// Sixteen epilogue warps, four per TMEM lane quadrant. Scan: warp p of a quadrant reads frame
// chunk p (32 frames) of the quadrant's 32 component rows (thread = row) and builds, without
// branches, the mask of frames whose logit is within log2(minGamma) of the frame's LSE.
// Accumulate: warp p owns rows 8p .. 8p + 7 of the quadrant; for each masked frame of a row it
// reads that frame's logit column from TMEM (all 32 rows at once, the row's value taken by a
// shuffle), forms g = 2^(s - lse), keeps the pair when g > minGamma, and adds it, lanes over
// dimensions. Sums go to FP64 partials [slot][chunk][K cols][128 rows] (F'_d at column d, n at
// D, S'_d at K/2 + d), zeroed before the launch, by fire-and-forget FP64 reductions (see
// kRowFlushMass for when); each partial has one writer thread, so its additions happen in a
// fixed order. A slot is a speaker piece (tile_slot) or the CTA's frame range.
__host__ __device__ constexpr int acc_ft(int) { return 128; }
// A row's FP32 sums go to the FP64 partials when its posterior mass reaches this (so an FP32 sum
// has at most ~2048 terms of weight 1: relative rounding ~2^-24 sqrt(2048)), at the end of its
// slot, and at the end of the CTA's range; rows without kept pairs are never written.
constexpr float kRowFlushMass = 2048.0f;
constexpr int kNoPeriod = 1 << 30;  // slots end only at slot changes and range ends

template <int K>
struct SparseCfg {
  static constexpr int FT = acc_ft(K);
  static constexpr int DMAX = (K - 1) / 2;  // largest D with this K
  static_assert(DMAX <= 63, "two dimensions per lane, the 64th slot carries the count");
  static constexpr int Z_PLANE = FT * K * 2;
  static constexpr int Z_STAGE = 3 * Z_PLANE;
  static constexpr int LL_STAGE = FT * 4;
  static constexpr int WCOLS = 3 * K / 2;
  static constexpr int NS = cmin(3, (512 - WCOLS) / FT);  // logits buffers
  static constexpr int S_COL = 0;
  static constexpr int W_COL = NS * FT;
  static constexpr int MASK_BYTES = 2 * 128 * 4 * 4;  // [tile parity][row][frame chunk]
  static constexpr int CEN_BYTES = 128 * 64 * 2;      // [row][dimension] centres, bf16
  static constexpr int FIXED = MASK_BYTES + CEN_BYTES + 32 * 8 + 64 + 1024;
  static constexpr int NZ = cmin(3, (227 * 1024 - FIXED) / (Z_STAGE + LL_STAGE));
  static constexpr int OFF_Z = 0;
  static constexpr int OFF_LL = OFF_Z + NZ * Z_STAGE;
  static constexpr int OFF_MASK = OFF_LL + NZ * LL_STAGE;
  static constexpr int OFF_CEN = OFF_MASK + MASK_BYTES;
  static constexpr int OFF_BAR = OFF_CEN + CEN_BYTES;
  static constexpr int OFF_MISC = OFF_BAR + 32 * 8;
  static constexpr int SMEM = OFF_MISC + 64 + 1024;
  static_assert(NS >= 2, "logits buffers");
  static_assert(NZ >= 2, "Z ring");
  static_assert(W_COL + WCOLS <= 512, "TMEM budget");
  static_assert(SMEM <= 227 * 1024, "shared memory budget");
};
constexpr int kAccEpiWarps = 16;
constexpr int kAccThreads = 32 * (2 + kAccEpiWarps);  // warp 0 TMA, warp 1 logits MMA, 2-17 epilogue

// SO: second-order statistics wanted (else n and F only).
template <int K, bool SO>
__global__ void __launch_bounds__(kAccThreads, 1)
    acc_sparse_kernel(const __grid_constant__ CUtensorMap zmap, const uint16_t* __restrict__ wplanes,
               const float* __restrict__ cent, const float* __restrict__ X, long long N,
               const long long* __restrict__ row_frame, int D, int nTz, int nTw, const float* __restrict__ ll2,
               int n_tiles, int n_chunks, int slices, const int* __restrict__ tile_slot,
               const int4* __restrict__ work, float minGamma, int single_comp, const int* __restrict__ mact_dev,
               double* __restrict__ part, int* __restrict__ err, long long wait_limit,
               const int* __restrict__ tile_list, const int* __restrict__ n_work_dev) {
  // with n_work_dev: a fixed grid, of which the first *n_work_dev CTAs have work items
  if (n_work_dev && (int)blockIdx.x >= *n_work_dev) return;
  if (mact_dev) single_comp = *mact_dev == 1;
  using C = SparseCfg<K>;
  constexpr int FT = C::FT, NZ = C::NZ, NS = C::NS, EW = kAccEpiWarps;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
  uint64_t* w_full = bars + 0;
  uint64_t* z_full = bars + 1;    // [NZ <= 3]
  uint64_t* z_empty = bars + 4;   // [NZ]: the logits MMAs and every epilogue warp are done
  uint64_t* s_full = bars + 7;    // [NS <= 3]
  uint64_t* s_free = bars + 10;   // [NS]: every epilogue warp is done with a logits buffer
  uint64_t* mma_done = bars + 13;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(smem + C::OFF_MISC);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::OFF_MISC + 8);
  volatile int* stop_s = reinterpret_cast<volatile int*>(smem + C::OFF_MISC + 16);  // [4]
  float* ll_s = reinterpret_cast<float*>(smem + C::OFF_LL);
  const uint32_t ll_sa = smem_u32(ll_s), mask_sa = smem_u32(smem + C::OFF_MASK);
  const uint32_t cen_sa = smem_u32(smem + C::OFF_CEN);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int chunk = (int)blockIdx.x % n_chunks, slice = (int)blockIdx.x / n_chunks;
  int wchunk = chunk;  // W chunk in the planes (several models may share them)
  int t0, nt;
  if (work) {
    // explicit work item: {W chunk in the planes, chunk within its model, first tile, tiles}
    const int4 wi = work[blockIdx.x];
    wchunk = wi.x;
    chunk = wi.y;
    t0 = wi.z;
    nt = wi.w;
  } else {
    const int per = (n_tiles + slices - 1) / slices;
    t0 = slice * per;
    nt = max(0, min(n_tiles, t0 + per) - t0);
  }
  // Statistics go to "slots": one per speaker piece with tile_slot (work items never split a
  // piece, so each (slot, chunk) has one owner), else one per slice.
  Periods per(tile_slot, t0, nt, slice);

  if (threadIdx.x == 0) {
    mbar_init(w_full, EW);
    for (int i = 0; i < NZ; ++i) {
      mbar_init(&z_full[i], 1);
      mbar_init(&z_empty[i], 1 + EW);
    }
    for (int i = 0; i < NS; ++i) {
      mbar_init(&s_full[i], 1);
      mbar_init(&s_free[i], EW);
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(tmem_holder, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  int issued = 0;  // Z tile copies issued (loader thread)

  if (warp == 0) {
    if (lane == 0 && nt > 0) {
      prefetch_tmap(&zmap);
      // the features' whole 16-byte pieces (the L2 prefetch wants an aligned base)
      const long long xbytes = (N * D * 4) & ~15LL;
      const bool xpf = (reinterpret_cast<uintptr_t>(X) & 15) == 0;
      for (int i = 0; i < nt; ++i) {
        const int s = i % NZ;
        if (!mbar_wait_sleep(&z_empty[s], ((i / NZ) & 1) ^ 1, abort_flag, wait_limit)) break;
        mbar_arrive_expect_tx(&z_full[s], C::Z_STAGE + C::LL_STAGE);
        uint8_t* zs = smem + C::OFF_Z + s * C::Z_STAGE;
        const int t = tile_list ? tile_list[t0 + i] : t0 + i;
        for (int p = 0; p < 3; ++p) load_image(zs + p * C::Z_PLANE, &zmap, p, nTz, K, t, &z_full[s]);
        bulk_load(ll_s + s * FT, ll2 + (size_t)t * FT, FT * 4, &z_full[s]);
        issued = i + 1;
        // the tile's frames into L2 for the epilogue's reads of x, a few tiles ahead of them (a
        // tile's rows are one contiguous run of frames; not so for sorted tiles)
        if (xpf && !tile_list) {
          const long long fb = row_frame ? row_frame[(long long)t * FT] : (long long)t * FT;
          if (fb >= 0 && fb < N) {
            const long long fe = fb + FT < N ? fb + FT : N;
            const long long b0 = (fb * D * 4) & ~15LL, b1 = (fe * D * 4 + 15) & ~15LL;
            const long long e1 = b1 < xbytes ? b1 : xbytes;
            if (e1 > b0) bulk_prefetch_l2(reinterpret_cast<const char*>(X) + b0, (uint32_t)(e1 - b0));
          }
        }
      }
    }
  } else if (warp == 1) {
    // the logits MMAs: S^T[comps x frames] = W Z^T, six split-bf16 plane products
    if (lane == 0 && nt > 0) {
      const uint32_t zb0 = smem_u32(smem + C::OFF_Z);
      const uint32_t idesc_l = idesc_bf16(128, FT, false, false);
      const uint32_t wa = tmem + C::W_COL;
      bool ok = mbar_wait_sleep(w_full, 0, abort_flag, wait_limit);
      for (int i = 0; i < nt && ok; ++i) {
        if (!mbar_wait_sleep(&z_full[i % NZ], (i / NZ) & 1, abort_flag, wait_limit)) break;
        if (i >= NS && !mbar_wait_sleep(&s_free[i % NS], ((i - NS) / NS) & 1, abort_flag, wait_limit)) break;
        tc_fence_after();
        const uint64_t zd = smem_desc(zb0 + (i % NZ) * C::Z_STAGE, FT * 16, 128);
        const uint32_t d = tmem + C::S_COL + (i % NS) * FT;
#pragma unroll
        for (int pr = 0; pr < 6; ++pr) {
#pragma unroll
          for (int q = 0; q < K / 16; ++q) {
            const uint64_t bd = desc_add(zd, prod_z(pr) * C::Z_PLANE + q * 2 * FT * 16);
            const uint32_t a = wa + prod_w(pr) * (K / 2) + q * 8;
            if (pr == 0 && q == 0) mma_ts_c<false>(d, a, bd, idesc_l);
            else mma_ts_c<true>(d, a, bd, idesc_l);
          }
        }
        mma_commit(&s_full[i % NS]);
        mma_commit(&z_empty[i % NZ]);
      }
      mma_commit(mma_done);
      mbar_drain(mma_done, 0);
    }
  } else if (nt > 0) {
    const int q4 = warp & 3;          // TMEM lane quadrant
    const int pw = (warp - 2) >> 2;   // warp of the quadrant: scans chunk pw, owns rows 8 pw ..
    const int row_l = q4 * 32 + lane; // scan: this thread's component row
    const uint32_t lane_off = (uint32_t)(q4 * 32) << 16;
    // the chunk's W planes into TMEM: plane pw by warp pw of the quadrant (0-2)
    if (pw < 3) {
      constexpr int KC = K / 8;
      const uint4* src =
          reinterpret_cast<const uint4*>(wplanes + ((size_t)(pw * nTw + wchunk) * KC) * 1024 + (size_t)row_l * 8);
      for (int c = 0; c < KC; c += 2) {
        const uint4 u0 = __ldg(src + (size_t)c * 128), u1 = __ldg(src + (size_t)(c + 1) * 128);
        const uint32_t w[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
        tmem_st8(tmem + lane_off + C::W_COL + pw * (K / 2) + c * 4, w);
      }
      tmem_st_wait();
    }
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(w_full);
    // lane = dimensions (lane, lane + 32); dimension 63 (lane 31's second one, unused since
    // D <= 63) carries the count: its x is 1 and its centre 0, so F'_63 = n
    const bool d0 = lane < D, d1 = lane + 32 < D, dn = lane == 31;
    const int rowq0 = 8 * pw;                    // first row (within the quadrant) this warp owns
    {
      // this warp's rows' centres into shared memory as bf16 (exact: the centres are bf16 values)
      const float* crow = cent + ((size_t)wchunk * 128 + q4 * 32 + rowq0) * D;
      for (int j = 0; j < 8; ++j) {
        const uint32_t a = cen_sa + (uint32_t)(((q4 * 32 + rowq0 + j) * 64) * 2);
        const float c0 = d0 ? __ldg(crow + (size_t)j * D + lane) : 0.0f;
        const float c1 = d1 ? __ldg(crow + (size_t)j * D + lane + 32) : 0.0f;
        asm volatile("st.shared.u16 [%0], %1;" ::"r"(a + lane * 2), "h"(__bfloat16_as_ushort(__float2bfloat16_rn(c0))) : "memory");
        asm volatile("st.shared.u16 [%0], %1;" ::"r"(a + (lane + 32) * 2), "h"(__bfloat16_as_ushort(__float2bfloat16_rn(c1))) : "memory");
      }
      __syncwarp();
    }
    float2 Fs[8], Ss[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      Fs[j] = make_float2(0.0f, 0.0f);
      Ss[j] = make_float2(0.0f, 0.0f);
    }
    uint32_t dirty = 0;  // rows with sums not yet in the partials
    // row j's sums into the FP64 partials [col][row] of a slot, by reductions (no value comes
    // back, so the warp does not wait); every partial has this one writer thread
    auto flush_row = [&](int j, int slot) {
      double* dst = part + ((size_t)slot * n_chunks + chunk) * K * 128 + q4 * 32 + rowq0 + j;
      if (d0) atomicAdd(dst + (size_t)lane * 128, (double)Fs[j].x);
      if (d1) atomicAdd(dst + (size_t)(lane + 32) * 128, (double)Fs[j].y);
      if (SO && d0) atomicAdd(dst + (size_t)(K / 2 + lane) * 128, (double)Ss[j].x);
      if (SO && d1) atomicAdd(dst + (size_t)(K / 2 + lane + 32) * 128, (double)Ss[j].y);
      if (dn) atomicAdd(dst + (size_t)D * 128, (double)Fs[j].y);
      Fs[j] = make_float2(0.0f, 0.0f);
      Ss[j] = make_float2(0.0f, 0.0f);
    };
    // candidates: posterior above minGamma within a margin (log2 domain), then the exact test
    const float thr = log2f(minGamma) - 0.01f;
    for (int i = 0; i < nt; ++i) {
      const int s = i % NZ, b = i % NS, mb = i & 1;
      per.begin(i, kNoPeriod);
      const bool okw = mbar_wait_sleep_all(&z_full[s], (i / NZ) & 1, abort_flag, wait_limit) &&
                       mbar_wait_sleep_all(&s_full[b], (i / NS) & 1, abort_flag, wait_limit);
      const uint32_t lla = ll_sa + (uint32_t)(s * FT * 4);
      const uint32_t sbuf = tmem + lane_off + C::S_COL + b * FT;
      const long long tile = tile_list ? (long long)tile_list[t0 + i] : (long long)(t0 + i);
      if (okw) {
        // scan frame chunk pw of the quadrant's rows: the candidate mask, without branches
        tc_fence_after();
        uint32_t v[32];
        tmem_ld32(sbuf + 32 * pw, v);
        tmem_ld_wait();
        uint32_t m = 0;
        if (!single_comp) {
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const float4 l = lds_f4(lla + (uint32_t)((32 * pw + 4 * q) * 4));
            // NaN (padding frame) and -inf (a trouble frame's +inf LSE) are never candidates
            if (__uint_as_float(v[4 * q + 0]) - l.x > thr) m |= 1u << (4 * q + 0);
            if (__uint_as_float(v[4 * q + 1]) - l.y > thr) m |= 1u << (4 * q + 1);
            if (__uint_as_float(v[4 * q + 2]) - l.z > thr) m |= 1u << (4 * q + 2);
            if (__uint_as_float(v[4 * q + 3]) - l.w > thr) m |= 1u << (4 * q + 3);
          }
        } else if (row_l == 0) {
          // one component: every real frame has posterior 1
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const float4 l = lds_f4(lla + (uint32_t)((32 * pw + 4 * q) * 4));
            if (!isnan(l.x)) m |= 1u << (4 * q + 0);
            if (!isnan(l.y)) m |= 1u << (4 * q + 1);
            if (!isnan(l.z)) m |= 1u << (4 * q + 2);
            if (!isnan(l.w)) m |= 1u << (4 * q + 3);
          }
        }
        sts_u32(mask_sa + (uint32_t)(((mb * 128 + row_l) * 4 + pw) * 4), m);
      }
      // The quadrant's four warps reach both barriers on every path; the stop decision is one
      // snapshot of the abort flag (raised by any failed wait) taken between them. The masks are
      // double-buffered by tile parity: a warp passes the next tile's first barrier only after
      // all four finished this tile's accumulation.
      named_sync(1 + q4, 128);
      if (pw == 0 && lane == 0) stop_s[q4] = *abort_flag;
      named_sync(1 + q4, 128);
      if (stop_s[q4]) break;
      // the masked frames of this warp's rows
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int rq = rowq0 + j;  // row within the quadrant (= its TMEM lane)
        const uint4 mk = lds_u4(mask_sa + (uint32_t)(((mb * 128 + q4 * 32 + rq) * 4) * 4));
        if ((mk.x | mk.y | mk.z | mk.w) == 0) continue;
        // the row's centre, negated
        float2 wc;
        {
          const uint32_t a = cen_sa + (uint32_t)(((q4 * 32 + rq) * 64) * 2);
          unsigned short h0, h1;
          asm volatile("ld.shared.u16 %0, [%1];" : "=h"(h0) : "r"(a + lane * 2));
          asm volatile("ld.shared.u16 %0, [%1];" : "=h"(h1) : "r"(a + (lane + 32) * 2));
          wc = make_float2(-__uint_as_float((uint32_t)h0 << 16), -__uint_as_float((uint32_t)h1 << 16));
        }
        // frames as one 128-bit set, walked two at a time: both logit columns read from TMEM
        // (the row's value by a shuffle), then both frames' rows loaded, then both sums
        uint64_t lo = ((uint64_t)mk.y << 32) | mk.x, hi = ((uint64_t)mk.w << 32) | mk.z;
        auto next = [&]() -> int {
          if (lo) { const int f = __ffsll((long long)lo) - 1; lo &= lo - 1; return f; }
          if (hi) { const int f = __ffsll((long long)hi) - 1; hi &= hi - 1; return 64 + f; }
          return -1;
        };
        while (lo | hi) {
          const int f0 = next(), f1 = next();
          const uint32_t r0 = tmem_ld1(sbuf + f0);
          const uint32_t r1 = tmem_ld1(sbuf + (f1 >= 0 ? f1 : f0));
          tmem_ld_wait();
          const float s0 = __shfl_sync(0xffffffffu, __uint_as_float(r0), rq);
          const float s1 = __shfl_sync(0xffffffffu, __uint_as_float(r1), rq);
          float g0 = 1.0f, g1 = f1 >= 0 ? 1.0f : 0.0f;
          if (!single_comp) {
            g0 = ex2(s0 - lds_f(lla + (uint32_t)(f0 * 4)));
            g1 = f1 >= 0 ? ex2(s1 - lds_f(lla + (uint32_t)(f1 * 4))) : 0.0f;
          }
          const bool k0 = g0 > minGamma, k1 = g1 > minGamma;
          float2 x0 = make_float2(0.0f, 0.0f), x1 = make_float2(0.0f, 0.0f);
          if (k0) {
            const float* xr = X + (row_frame ? row_frame[tile * 128 + f0] : tile * 128 + f0) * D;
            x0 = make_float2(d0 ? __ldg(xr + lane) : 0.0f, d1 ? __ldg(xr + lane + 32) : (dn ? 1.0f : 0.0f));
          }
          if (k1) {
            const float* xr = X + (row_frame ? row_frame[tile * 128 + f1] : tile * 128 + f1) * D;
            x1 = make_float2(d0 ? __ldg(xr + lane) : 0.0f, d1 ? __ldg(xr + lane + 32) : (dn ? 1.0f : 0.0f));
          }
          if (k0) {
            const float2 dx = __fadd2_rn(x0, wc);
            const float2 t = __fmul2_rn(make_float2(g0, g0), dx);
            Fs[j] = __fadd2_rn(Fs[j], t);
            if (SO) Ss[j] = __ffma2_rn(t, dx, Ss[j]);
          }
          if (k1) {
            const float2 dx = __fadd2_rn(x1, wc);
            const float2 t = __fmul2_rn(make_float2(g1, g1), dx);
            Fs[j] = __fadd2_rn(Fs[j], t);
            if (SO) Ss[j] = __ffma2_rn(t, dx, Ss[j]);
          }
        }
        // a row whose FP32 sums hold kRowFlushMass of posterior mass goes to FP64 now
        dirty |= 1u << j;
        if (__shfl_sync(0xffffffffu, Fs[j].y, 31) >= kRowFlushMass) {
          flush_row(j, per.slot_of(i));
          dirty &= ~(1u << j);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&s_free[b]);
        mbar_arrive(&z_empty[s]);
      }
      if (dirty && per.end(i, kNoPeriod)) {
        // the slot ends here (a speaker piece, or this CTA's frame range)
        const int slot = per.slot_of(i);
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (dirty & (1u << j)) flush_row(j, slot);
        dirty = 0;
      }
    }
  }
  __syncthreads();
  if (*abort_flag) {
    // Every role has stopped. The loader's last NZ copies may still be in flight (a consumer
    // that gave up never waited for them): let them land before the CTA's shared memory goes.
    // Earlier copies were consumed, so they have landed.
    if (warp == 0 && lane == 0)
      for (int i = max(0, issued - NZ); i < issued; ++i) mbar_drain(&z_full[i % NZ], (i / NZ) & 1);
    if (threadIdx.x == 0) atomicExch(err, 1);
  }
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// Statistics MMAs issued by a whole warp (one elected lane) or by one thread; the forms below
// pick one at compile time.
template <int K>
constexpr bool kWarpIssue = K <= 80;

template <bool WARPED>
__device__ __forceinline__ bool mbar_wait_x(uint64_t* bar, uint32_t parity, volatile int* abort_flag, long long limit) {
  if constexpr (WARPED) return mbar_wait_warp(bar, parity, abort_flag, limit);
  else return mbar_wait(bar, parity, abort_flag, limit);
}

template <bool WARPED, bool ACC>
__device__ __forceinline__ void mma_ts_x(uint32_t d, uint32_t a, uint64_t b, uint32_t idesc) {
  if constexpr (WARPED) mma_ts_e<ACC>(d, a, b, idesc);
  else mma_ts_c<ACC>(d, a, b, idesc);
}

template <bool WARPED>
__device__ __forceinline__ void mma_commit_x(uint64_t* bar) {
  if constexpr (WARPED) mma_commit_e(bar);
  else mma_commit(bar);
}

// dense kernel: warp 0 TMA, warp 1 logits MMA, warps 2-5 posteriors (one per TMEM lane
// quadrant), warp 6 statistics MMA, warps 7-14 statistics readout
constexpr int kAccStatsWarp = 6;
constexpr int kAccReadWarp0 = 7;
constexpr int kThreads = 32 * (kAccReadWarp0 + 8);

// Dense statistics kernel. The component chunk's W planes are stored into TMEM once (A operand of
// the logits MMA); Z tiles stream through an NZ-stage shared-memory ring; posteriors go from the
// logits accumulator into TMEM in place and feed the statistics MMA, flushed to FP64 partials
// every FLUSH tiles.
//
// With second-order statistics (SPLIT) the statistics MMA writes two accumulators: A takes the
// hi x Z1 product alone and B the four smaller ones (lo x Z2, hi x Z3, lo x Z1, hi x Z2). The
// tensor core's FP32 accumulation rounds toward zero; a bf16 x bf16 product has 16 significant
// bits, so a component's A sum over a tile is exact as long as its frames' products lie within
// 8 binades of each other (always so for one frame), and B's rounding is 2^-8 smaller again.
// With one accumulator the truncation of every frame's five-product sum biased F/n and S/n by
// -5e-8 relative, which the variance update S/n - mu^2 magnified up to 175 times (worst variance
// 2.1e-5 relative at N = 1M, M = 2048, D = 39). The epilogue adds A + B per tile in FP32 with
// round-to-nearest and moves the sums into FP64 every FLUSH = 16 tiles.

// Statistics columns without second-order statistics: the [x | 1] columns rounded up to the MMA
// granularity. For every D with this K (K = 2D + 1 rounded up to 16) that is the same number.
__host__ __device__ constexpr int acc_mean_cols(int K) { return ((K - 1) / 2 + 1 + 15) / 16 * 16; }

// Resources of the statistics kernel for K and SO (second-order statistics wanted). Tiles are
// FT = 128 frames: a tcgen05.mma with M = 128 and K = 16 costs max(45.5, N / 2) cycles on GB300
// (measured), so the logits MMA (N = frames) reaches the full rate only from N = 96 on; 64-frame
// tiles would cost the logits 42% more. TMEM holds two 128-column posterior buffers, the W planes
// (K/2 columns each) and ND statistics accumulators of N2 columns. Two accumulators let the
// statistics MMAs of tile j + 1 queue behind those of tile j before the epilogue has read tile j
// out; W plane 2 (one of the six logits products) moves to shared memory, where that product
// reads both operands, when that makes room. Plans in order of preference: (3 W planes in TMEM,
// 2 accumulators), (2, 2), (3, 1), (2, 1). The Z ring takes as many stages (2 or 3) as the
// shared memory left holds.
template <int K, bool SO>
struct AccCfg {
  static constexpr int FT = acc_ft(K);
  static_assert(FT == 128, "a posterior warp converts four 32-frame chunks, signalled in two halves");
  static constexpr int N2 = SO ? K : acc_mean_cols(K);
  static constexpr bool SPLIT = SO && K <= 80;    // A and B accumulators (see above)
  static constexpr int NSET = SPLIT ? 2 : 1;       // accumulators of N2 columns per tile
  static constexpr int Z_PLANE = FT * K * 2;
  static constexpr int Z_STAGE = 3 * Z_PLANE;
  static constexpr int LL_STAGE = FT * 4;
  static constexpr int WC3 = (3 * K / 2 + 15) / 16 * 16, WC2 = (K + 15) / 16 * 16;
  static constexpr bool P1 = 2 * FT + WC3 + 2 * NSET * N2 <= 512;
  static constexpr bool P2 = !P1 && 2 * FT + WC2 + 2 * NSET * N2 <= 512;
  static constexpr bool P3 = !P1 && !P2 && 2 * FT + WC3 + NSET * N2 <= 512;
  static constexpr int WT = (P1 || P3) ? 3 : 2;   // W planes in TMEM
  static constexpr int ND = (P1 || P2) ? 2 : 1;   // statistics accumulators
  static constexpr int NS = 2;                    // posterior buffers
  static constexpr int S_COL = 0;
  static constexpr int W_COL = NS * FT;
  static constexpr int D_COL = (W_COL + WT * K / 2 + 15) / 16 * 16;
  static constexpr int W2_BYTES = WT == 2 ? K * 256 : 0;  // W plane 2 image in shared memory
  static constexpr int FIXED = W2_BYTES + 32 * 8 + 64 + 1024;
  static constexpr int NZ = cmin(3, (227 * 1024 - FIXED) / (Z_STAGE + LL_STAGE));
  static constexpr int OFF_Z = 0;
  static constexpr int OFF_W2 = OFF_Z + NZ * Z_STAGE;
  static constexpr int OFF_LL = OFF_W2 + W2_BYTES;
  static constexpr int OFF_BAR = OFF_LL + NZ * LL_STAGE;
  static constexpr int OFF_MISC = OFF_BAR + 32 * 8;
  static constexpr int SMEM = cmax(OFF_MISC + 64 + 1024, 120 * 1024);
  static constexpr int FLUSH = SPLIT ? 16 : 64 * 128 / FT;  // tiles per FP64 flush
  static constexpr int PIECE = 64 * 128 / FT;                // tiles per speaker piece (batched calls)
  static_assert(NZ >= 2 && NZ <= 4, "Z ring");
  static_assert(D_COL + ND * NSET * N2 <= 512, "TMEM budget");
  static_assert(SMEM <= 227 * 1024, "shared memory budget");
};

// SO: second-order statistics wanted. The statistics MMA multiplies and the epilogue reads N2
// columns: all K, or the leading [x | 1] ones.
template <int K, bool SO>
__global__ void __launch_bounds__(kThreads, 1)
    acc_dense_kernel(const __grid_constant__ CUtensorMap zmap, const uint16_t* __restrict__ wplanes,
               int nTz, int nTw, const float* __restrict__ ll2, int n_tiles, int n_chunks, int slices,
               const int* __restrict__ tile_slot, const int4* __restrict__ work, float minGamma,
               int single_comp, const int* __restrict__ mact_dev,
               double* __restrict__ part, int* __restrict__ err, long long wait_limit,
               const int* __restrict__ tile_list, const int* __restrict__ n_work_dev) {
  // with n_work_dev: a fixed grid, of which the first *n_work_dev CTAs have work items
  if (n_work_dev && (int)blockIdx.x >= *n_work_dev) return;
  if (mact_dev) single_comp = *mact_dev == 1;
  using C = AccCfg<K, SO>;
  constexpr int FT = C::FT, NZ = C::NZ, NS = C::NS, ND = C::ND, N2 = C::N2, FLUSH = C::FLUSH;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
  uint64_t* w_full = bars + 0;
  uint64_t* z_full = bars + 1;   // [NZ <= 4]
  uint64_t* z_empty = bars + 5;  // [NZ]
  uint64_t* s_full = bars + 9;   // [NS <= 4]
  uint64_t* g_full = bars + 13;  // [NS buffers][2 frame halves]
  uint64_t* d_full = bars + 21;     // [ND]
  uint64_t* d_empty = bars + 23;    // [ND]
  uint64_t* mma_done = bars + 25;   // [2]: one per MMA-issuing thread
  uint64_t* s_free = bars + 27;     // [NS]: the statistics MMAs are done with a posterior buffer
  uint64_t* w2_full = bars + 31;    // W plane 2 in shared memory (WT == 2)
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(smem + C::OFF_MISC);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + C::OFF_MISC + 8);
  float* ll_s = reinterpret_cast<float*>(smem + C::OFF_LL);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int chunk = (int)blockIdx.x % n_chunks, slice = (int)blockIdx.x / n_chunks;
  int wchunk = chunk;  // W chunk in the planes (several models may share them)
  int t0, nt;
  if (work) {
    // explicit work item: {W chunk in the planes, chunk within its model, first tile, tiles}
    const int4 wi = work[blockIdx.x];
    wchunk = wi.x;
    chunk = wi.y;
    t0 = wi.z;
    nt = wi.w;
  } else {
    const int per = (n_tiles + slices - 1) / slices;
    t0 = slice * per;
    nt = max(0, min(n_tiles, t0 + per) - t0);
  }
  // Statistics go to "slots": one per speaker with tile_slot (slices never split a speaker, so
  // each (slot, chunk) has one owner), else one per slice. An accumulation period ends at a
  // slot change or after FLUSH tiles of the same slot.
  Periods per(tile_slot, t0, nt, slice);

  if (threadIdx.x == 0) {
    mbar_init(w_full, 4);
    for (int i = 0; i < NZ; ++i) {
      mbar_init(&z_full[i], 1);
      mbar_init(&z_empty[i], 1);
    }
    for (int i = 0; i < NS; ++i) {
      mbar_init(&s_full[i], 1);
      mbar_init(&g_full[2 * i], 4);
      mbar_init(&g_full[2 * i + 1], 4);
      mbar_init(&s_free[i], 1);
    }
    for (int i = 0; i < ND; ++i) {
      mbar_init(&d_full[i], 1);
      mbar_init(&d_empty[i], 8);
    }
    mbar_init(w2_full, 1);
    mbar_init(&mma_done[0], 1);
    mbar_init(&mma_done[1], 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(tmem_holder, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  int issued = 0;  // Z tile copies issued (loader thread)

  if (warp == 0) {
    if (lane == 0 && nt > 0) {
      prefetch_tmap(&zmap);
      if (C::WT == 2) {  // W plane 2: its image is already the operand layout, one bulk copy
        mbar_arrive_expect_tx(w2_full, C::W2_BYTES);
        bulk_load(smem + C::OFF_W2, wplanes + (size_t)(2 * nTw + wchunk) * (K / 8) * 1024, C::W2_BYTES, w2_full);
      }
      for (int i = 0; i < nt; ++i) {
        const int s = i % NZ;
        if (!mbar_wait(&z_empty[s], ((i / NZ) & 1) ^ 1, abort_flag, wait_limit)) break;
        mbar_arrive_expect_tx(&z_full[s], C::Z_STAGE + C::LL_STAGE);
        uint8_t* zs = smem + C::OFF_Z + s * C::Z_STAGE;
        const int t = tile_list ? tile_list[t0 + i] : t0 + i;
        for (int p = 0; p < 3; ++p) load_image(zs + p * C::Z_PLANE, &zmap, p, nTz, K, t, &z_full[s]);
        bulk_load(ll_s + s * FT, ll2 + (size_t)t * FT, FT * 4, &z_full[s]);
        issued = i + 1;
      }
    }
  } else if (warp == 1 || warp == kAccStatsWarp) {
    // Two MMA-issuing roles on different SM sub-partitions: the logits (warp 1) and the
    // statistics (warp 6). Each shares its sub-partition with a posterior warp and two readout
    // warps. The logits come from one thread; the statistics for K <= 80 from a whole converged
    // warp with one elected lane issuing (kWarpIssue), which keeps their issue rate up while the
    // posterior warp is busy (measured: 8.15 against 8.50 ms at N = 4M, M = 2048, D = 39). The
    // warp-issued forms measured slower for the logits stream (8.41 ms there) and for K = 128
    // (batched MAP, D = 60: 10.7 against 6.8 ms). A posterior buffer is reused by the logits of
    // tile i + NS only after the statistics of tile i released it (s_free).
    constexpr bool WARPED = kWarpIssue<K>;
    if (nt > 0 && (warp == kAccStatsWarp ? (WARPED || lane == 0) : lane == 0)) {
      const uint32_t zb0 = smem_u32(smem + C::OFF_Z);
      bool ok = true;
      if (warp == 1) {
        const uint32_t idesc_l = idesc_bf16(128, FT, false, false);
        const uint32_t wa = tmem + C::W_COL;
        ok = mbar_wait(w_full, 0, abort_flag, wait_limit);
        if (ok && C::WT == 2) ok = mbar_wait(w2_full, 0, abort_flag, wait_limit);
        const uint64_t w2d = smem_desc(smem_u32(smem + C::OFF_W2), 128 * 16, 128);
        for (int i = 0; i < nt && ok; ++i) {
          if (!mbar_wait(&z_full[i % NZ], (i / NZ) & 1, abort_flag, wait_limit)) break;
          if (i >= NS && !mbar_wait(&s_free[i % NS], ((i - NS) / NS) & 1, abort_flag, wait_limit)) break;
          tc_fence_after();
          const uint64_t zd = smem_desc(zb0 + (i % NZ) * C::Z_STAGE, FT * 16, 128);
          const uint32_t d = tmem + C::S_COL + (i % NS) * FT;
#pragma unroll
          for (int pr = 0; pr < 6; ++pr) {
#pragma unroll
            for (int q = 0; q < K / 16; ++q) {
              const uint64_t bd = desc_add(zd, prod_z(pr) * C::Z_PLANE + q * 2 * FT * 16);
              const uint32_t a = wa + prod_w(pr) * (K / 2) + q * 8;
              if (prod_w(pr) >= C::WT) mma_ss_c<true>(d, desc_add(w2d, q * 2 * 128 * 16), bd, idesc_l);
              else if (pr == 0 && q == 0) mma_ts_c<false>(d, a, bd, idesc_l);
              else mma_ts_c<true>(d, a, bd, idesc_l);
            }
          }
          mma_commit(&s_full[i % NS]);
        }
        mma_commit(&mma_done[0]);
        mbar_drain(&mma_done[0], 0);
      } else {
        const uint32_t idesc_s = idesc_bf16(128, N2, false, true);
        const uint32_t idesc_s2 = idesc_bf16(128, C::SPLIT ? 2 * N2 : N2, false, true);  // [A | B]
        for (int j = 0; j < nt && ok; ++j) {
          const int b = j % NS;
          const uint32_t dcol = tmem + C::D_COL + (j % ND) * (C::NSET * N2);
          const uint32_t dsmall = C::SPLIT ? dcol + N2 : dcol;  // B (the small products)
          // the tile's operands are in its stage; an accumulator holds one tile: wait until the
          // readout of tile j - ND
          if (!mbar_wait_x<WARPED>(&z_full[j % NZ], (j / NZ) & 1, abort_flag, wait_limit)) break;
          if (j >= ND && !mbar_wait_x<WARPED>(&d_empty[j % ND], ((j - ND) / ND) & 1, abort_flag, wait_limit)) break;
          const uint32_t gb = tmem + C::S_COL + b * FT;
          // B = Z as [N = K columns] x [K' = frames], MN-major: LBO along frames, SBO along columns
          const uint64_t zd = smem_desc(zb0 + (j % NZ) * C::Z_STAGE, 128, FT * 16);
#pragma unroll
          for (int q = 0; q < FT / 16; ++q) {
            // the posteriors of each half of the tile's frames are signalled separately, so the
            // statistics of the first half run while the epilogue converts the second
            if (q % (FT / 32) == 0) {
              if (!mbar_wait_x<WARPED>(&g_full[2 * b + q / (FT / 32)], (j / NS) & 1, abort_flag, wait_limit)) {
                ok = false;
                break;
              }
              tc_fence_after();
            }
            const uint32_t hi = gb + 32 * (q >> 1) + 8 * (q & 1);
            const uint32_t lo = hi + 16;
            const uint64_t z1 = desc_add(zd, 0 * C::Z_PLANE + q * 2 * 128);
            const uint64_t z2 = desc_add(zd, 1 * C::Z_PLANE + q * 2 * 128);
            const uint64_t z3 = desc_add(zd, 2 * C::Z_PLANE + q * 2 * 128);
            // gamma (hi + lo) x Z (z1 + z2 + z3): the five products above 2^-18
            if constexpr (C::SPLIT) {
              // hi x Z1 into accumulator A, the four smaller products into B (right after A).
              // Planes Z1 and Z2 are adjacent column groups of one MN-major operand and B
              // follows A in TMEM, so one MMA of N = 2 N2 computes hi x [Z1 | Z2] into [A | B].
              if (q == 0) {
                mma_ts_x<WARPED, false>(dcol, hi, z1, idesc_s2);
                mma_ts_x<WARPED, true>(dsmall, lo, z2, idesc_s);
                mma_ts_x<WARPED, true>(dsmall, hi, z3, idesc_s);
                mma_ts_x<WARPED, true>(dsmall, lo, z1, idesc_s);
              } else {
                mma_ts_x<WARPED, true>(dsmall, lo, z2, idesc_s);
                mma_ts_x<WARPED, true>(dsmall, hi, z3, idesc_s);
                mma_ts_x<WARPED, true>(dsmall, lo, z1, idesc_s);
                mma_ts_x<WARPED, true>(dcol, hi, z1, idesc_s2);
              }
            } else {
              // one accumulator, smallest products first
              if (q == 0) mma_ts_x<WARPED, false>(dcol, lo, z2, idesc_s);
              else mma_ts_x<WARPED, true>(dcol, lo, z2, idesc_s);
              mma_ts_x<WARPED, true>(dcol, hi, z3, idesc_s);
              mma_ts_x<WARPED, true>(dcol, lo, z1, idesc_s);
              mma_ts_x<WARPED, true>(dcol, hi, z2, idesc_s);
              mma_ts_x<WARPED, true>(dcol, hi, z1, idesc_s);
            }
          }
          if (!ok) break;
          mma_commit_x<WARPED>(&z_empty[j % NZ]);
          mma_commit_x<WARPED>(&d_full[j % ND]);
          mma_commit_x<WARPED>(&s_free[b]);
        }
        mma_commit_x<WARPED>(&mma_done[1]);
        if (lane == 0) mbar_drain(&mma_done[1], 0);
      }
    }
  } else if (warp >= 2 && warp < kAccStatsWarp && nt > 0) {
    // posteriors: thread = component row, one warp per TMEM lane quadrant (measured 1.7% faster
    // than two warps per quadrant: fewer busy warps beside the MMA-issuing ones)
    const int q4 = warp & 3;
    const int row = q4 * 32 + lane;
    const uint32_t lane_off = (uint32_t)(q4 * 32) << 16;
    // the chunk's W planes into TMEM (A operand of the logits MMA)
    {
      const int KC = K / 8;
      for (int p = 0; p < C::WT; ++p) {
        const uint4* src = reinterpret_cast<const uint4*>(wplanes + ((size_t)(p * nTw + wchunk) * KC) * 1024 + (size_t)row * 8);
        for (int c = 0; c < KC; c += 2) {
          const uint4 u0 = __ldg(src + (size_t)c * 128), u1 = __ldg(src + (size_t)(c + 1) * 128);
          const uint32_t w[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
          tmem_st8(tmem + lane_off + C::W_COL + p * (K / 2) + c * 4, w);
        }
      }
      tmem_st_wait();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(w_full);
    }
    constexpr int NCH = FT / 32;  // 32-frame chunks per warp (4)
    for (int i = 0; i < nt; ++i) {
      const int b = i % NS;
      if (!mbar_wait_all(&z_full[i % NZ], (i / NZ) & 1, abort_flag, wait_limit)) break;
      if (!mbar_wait_all(&s_full[b], (i / NS) & 1, abort_flag, wait_limit)) break;
      tc_fence_after();
      const float* lls = ll_s + (i % NZ) * FT;
      // pass c converts 32-frame chunk c; the first half of the tile's frames is signalled
      // before the second is converted
#pragma unroll 1
      for (int c = 0; c < NCH; ++c) {
        const uint32_t col = tmem + lane_off + C::S_COL + b * FT + 32 * c;
        uint32_t v[32];
        tmem_ld32(col, v);
        tmem_ld_wait();
        uint32_t hi[16], lo[16];
        if (!single_comp) {
#pragma unroll
          for (int k = 0; k < 32; k += 4) {
            const float4 l4 = *reinterpret_cast<const float4*>(lls + 32 * c + k);
            float g0 = ex2(__uint_as_float(v[k + 0]) - l4.x);
            float g1 = ex2(__uint_as_float(v[k + 1]) - l4.y);
            float g2 = ex2(__uint_as_float(v[k + 2]) - l4.z);
            float g3 = ex2(__uint_as_float(v[k + 3]) - l4.w);
            g0 = g0 > minGamma ? g0 : 0.0f;  // NaN (padding) and 0 (trouble: +inf LSE) prune
            g1 = g1 > minGamma ? g1 : 0.0f;
            g2 = g2 > minGamma ? g2 : 0.0f;
            g3 = g3 > minGamma ? g3 : 0.0f;
            const uint32_t h01 = pack_bf16(g0, g1), h23 = pack_bf16(g2, g3);
            hi[k >> 1] = h01;
            hi[(k >> 1) + 1] = h23;
            lo[k >> 1] = pack_bf16(g0 - __uint_as_float(h01 << 16), g1 - __uint_as_float(h01 & 0xffff0000u));
            lo[(k >> 1) + 1] = pack_bf16(g2 - __uint_as_float(h23 << 16), g3 - __uint_as_float(h23 & 0xffff0000u));
          }
        } else {
          // one component: every real frame has posterior 1 (padding 0)
#pragma unroll
          for (int k = 0; k < 32; k += 2) {
            const float g0 = isnan(lls[32 * c + k]) ? 0.0f : 1.0f;
            const float g1 = isnan(lls[32 * c + k + 1]) ? 0.0f : 1.0f;
            hi[k >> 1] = pack_bf16(g0, g1);
            lo[k >> 1] = 0u;
          }
        }
        tmem_st16(col, hi);
        tmem_st16(col + 16, lo);
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0 && (c & 1)) mbar_arrive(&g_full[2 * b + (c >> 1)]);
      }
    }
  } else if (warp >= kAccReadWarp0 && nt > 0) {
    // statistics readout: thread = component row; the two warps of a lane quadrant split the
    // columns
    const int q4 = warp & 3;
    const int hf = (warp - kAccReadWarp0) >> 2;
    const int row = q4 * 32 + lane;
    const uint32_t lane_off = (uint32_t)(q4 * 32) << 16;
    constexpr int KCH = N2 / 16;         // 16-column chunks of the statistics
    constexpr int KH = (KCH + 1) / 2;    // chunks per warp of a pair
    const int kc0 = hf ? KH : 0, kc1 = hf ? KCH : KH;
    // The statistics MMA leaves one tile's sums in the accumulator. These warps read them as
    // soon as the MMA is done, add them into FP32 registers with round-to-nearest and move the
    // registers into the FP64 partials at the end of each accumulation period (FLUSH tiles of one
    // slot). Being separate from the warps that form the posteriors, the readout of tile j never
    // waits behind the conversion of tile j + 1, and the statistics MMAs of tile j + 1 (one
    // accumulator set: they wait for that readout) start as soon as their posteriors are there.
    float dacc[KH * 16];
#pragma unroll
    for (int k = 0; k < KH * 16; ++k) dacc[k] = 0.0f;
    auto readout = [&](int t, bool flush, int slot) -> bool {
      if (!mbar_wait_all(&d_full[t % ND], (t / ND) & 1, abort_flag, wait_limit)) return false;
      tc_fence_after();
      const uint32_t dbase = tmem + lane_off + C::D_COL + (t % ND) * (C::NSET * N2);
      if constexpr (C::SPLIT) {
        // A + B per column, then into the running sums (both in FP32, round to nearest)
#pragma unroll
        for (int g = 0; g < KH; ++g) {
          if (kc0 + g < kc1) {
            uint32_t ra[16], rb[16];
            tmem_ld16(dbase + 16 * (kc0 + g), ra);
            tmem_ld16(dbase + N2 + 16 * (kc0 + g), rb);
            tmem_ld_wait();
#pragma unroll
            for (int k = 0; k < 16; ++k)
              dacc[g * 16 + k] += __uint_as_float(ra[k]) + __uint_as_float(rb[k]);
          }
        }
      } else {
        constexpr int RB = KH <= 3 ? KH : 2;  // loads in flight before each wait
#pragma unroll
        for (int g = 0; g < KH; g += RB) {
          uint32_t r[RB][16];
#pragma unroll
          for (int u = 0; u < RB; ++u)
            if (g + u < KH && kc0 + g + u < kc1) tmem_ld16(dbase + 16 * (kc0 + g + u), r[u]);
          tmem_ld_wait();
#pragma unroll
          for (int u = 0; u < RB; ++u) {
            if (g + u < KH && kc0 + g + u < kc1) {
#pragma unroll
              for (int k = 0; k < 16; ++k) dacc[(g + u) * 16 + k] += __uint_as_float(r[u][k]);
            }
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&d_empty[t % ND]);
      if (flush) {
        // into the zeroed FP64 partials [col][row] by reductions: no value comes back, so the
        // warp does not wait; each partial has this one writer thread (a fixed order of additions)
        double* mypart = part + ((size_t)slot * n_chunks + chunk) * K * 128 + row;
#pragma unroll
        for (int cc = 0; cc < KH; ++cc) {
          if (kc0 + cc < kc1) {
#pragma unroll
            for (int k = 0; k < 16; ++k) {
              atomicAdd(mypart + (size_t)(16 * (kc0 + cc) + k) * 128, (double)dacc[cc * 16 + k]);
              dacc[cc * 16 + k] = 0.0f;
            }
          }
        }
      }
      return true;
    };
    for (int t = 0; t < nt; ++t) {
      per.begin(t, FLUSH);
      if (!readout(t, per.end(t, FLUSH), per.slot_of(t))) break;
    }
  }
  __syncthreads();
  if (*abort_flag) {
    // Every role has stopped. The loader's last NZ copies (and the W plane 2 copy) may still be
    // in flight (a consumer that gave up never waited for them): let them land before the CTA's
    // shared memory goes. Earlier copies were consumed, so they have landed.
    if (warp == 0 && lane == 0 && nt > 0) {
      for (int i = max(0, issued - NZ); i < issued; ++i) mbar_drain(&z_full[i % NZ], (i / NZ) & 1);
      if (C::WT == 2) mbar_drain(w2_full, 0);
    }
    if (threadIdx.x == 0) atomicExch(err, 1);
  }
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// part [slice][chunk][K][128] -> stats (caller order): thread = (chunk, d, row) sums n, F_d and
// S_d over the slices in order; with cent (the sparse kernel's centred sums) it adds the centre
// back.
__global__ void reduce_kernel(int M, int D, int K, int Mact, int n_chunks, int slices, int n_tiles,
                              const int* __restrict__ comp_of_row, const float* __restrict__ cent,
                              const double* __restrict__ part, int flags, double* __restrict__ stats) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n_chunks * D * 128) return;
  const int rr = (int)(t & 127), d = (int)((t >> 7) % D), ch = (int)(t / (128LL * D));
  const int r = ch * 128 + rr;
  if (r >= Mact) return;
  const int m = comp_of_row[r];
  if (m < 0) return;  // padding row
  const int per = (n_tiles + slices - 1) / slices;
  const bool sv = (flags & GMM_ACC_VAR) != 0;
  double n = 0.0, Fc = 0.0, Sc = 0.0;
  for (int sl = 0; sl < slices; ++sl) {
    if (sl * per >= n_tiles) break;
    const double* p = part + ((size_t)sl * n_chunks + ch) * K * 128 + rr;
    n += p[(size_t)D * 128];
    Fc += p[(size_t)d * 128];
    if (sv) Sc += p[(size_t)(K / 2 + d) * 128];
  }
  const double c = cent ? (double)cent[(size_t)r * D + d] : 0.0;
  if (d == 0) stats[m] += n;
  if (flags & GMM_ACC_MEAN) stats[(size_t)M + (size_t)m * D + d] += tc_uncentre_F(Fc, n, c);
  if (sv) stats[(size_t)M + (size_t)M * D + (size_t)m * D + d] += tc_uncentre_S(Sc, Fc, n, c);
}

__global__ void ll_total_kernel(int n, const double* __restrict__ llpart, double* __restrict__ tot) {
  __shared__ double red[32];
  double v = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) v += llpart[k];
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    *tot += s;
  }
}

// ------------------------------------------------------------------ batched MAP support

// row_of_comp[m] = row of component m in the padded active list, -1 when m is inactive.
__global__ void row_of_comp_kernel(int M, int Mpad, const int* __restrict__ comp_of_row,
                                   int* __restrict__ row_of_comp) {
  for (int m = threadIdx.x; m < M; m += blockDim.x) row_of_comp[m] = -1;
  __syncthreads();
  for (int r = threadIdx.x; r < Mpad; r += blockDim.x)
    if (comp_of_row[r] >= 0) row_of_comp[comp_of_row[r]] = r;
}

// Per-speaker total log-likelihood: FP64 sum of the speaker's frame log-likelihoods (strided
// per thread, then a fixed warp and block tree).
// Padded row r of a speaker batch -> its frame (-1 for the padding rows at a speaker's end):
// speaker s owns rows [pad[s], pad[s+1]) and frames [offs[s], offs[s+1]).
__global__ void row_frame_kernel(int S, const long long* __restrict__ pad, const long long* __restrict__ offs,
                                 long long Rpad, long long* __restrict__ rf) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= Rpad) return;
  int lo = 0, hi = S;  // the last s with pad[s] <= r
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (pad[mid] <= r) lo = mid;
    else hi = mid;
  }
  const long long f = S > 0 ? offs[lo] + (r - pad[lo]) : -1;
  rf[r] = (S > 0 && f < offs[lo + 1]) ? f : -1;
}

__global__ void seg_sum_kernel(const long long* __restrict__ offs, const float* __restrict__ ll,
                               double* __restrict__ out) {
  __shared__ double red[32];
  const int s = blockIdx.x;
  double v = 0.0;
  for (long long f = offs[s] + threadIdx.x; f < offs[s + 1]; f += blockDim.x) v += (double)ll[f];
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    out[s] = t;
  }
}

// ------------------------------------------------------------------ host side

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 2-D map over the plane images viewed as [rows][128 bf16] (256-byte rows): a box of
// 128 x box_rows lands box_rows * 256 contiguous bytes in shared memory.
int make_map(Ctx* c, CUtensorMap* map, const uint16_t* base, long long total_elems, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return fail(c, GMM_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  cuuint64_t dims[2] = {128, (cuuint64_t)(total_elems / 128)};
  cuuint64_t strides[1] = {256};
  cuuint32_t box[2] = {128, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(c, GMM_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return GMM_OK;
}

// build_planes: the logits kernel writes the feature planes of its tiles, built from c->X on the
// way (with two Z buffers, K <= 80, it builds its Z tiles from c->X on every pass)
// Largest dynamic shared memory of the logits kernel: room for the chunk maxima of 32 chunks
// where that fits (the frame masks of the sparse tile schedule), else the plain layout.
template <int K>
constexpr int ll_smem_max() {
  return LlCfg<K>::smem_with_masks(kSchedChunksMax) <= 227 * 1024 ? LlCfg<K>::smem_with_masks(kSchedChunksMax)
                                                                   : LlCfg<K>::SMEM;
}

// masks: also write the frame chunk masks of the sparse tile schedule (c->sched.fmask)
template <int K>
int launch_ll_part(Ctx* c, int tile0, int n_tiles_ll, float* ll_out_dev, bool want_total, bool build_planes,
                   bool masks) {
  using LC = LlCfg<K>;
  const long long Npad = c->tcx.Npad;
  const int nTz = (int)(Npad / 128), nTw = c->tcm.Mpad / 128;
  const int n_chunks = nTw;
  int grid_ll = std::min(n_tiles_ll, c->sms);
  if (grid_ll < 1) grid_ll = 1;
  size_t need = (size_t)grid_ll * 128;
  if (need > c->tc_llpart_cap) {
    dfree(c, c->tc_llpart, c->tc_llpart_cap * sizeof(double));
    c->tc_llpart = nullptr;
    int rc = dalloc(c, (void**)&c->tc_llpart, need * sizeof(double), "tc llpart");
    if (rc) return rc;
    c->tc_llpart_cap = need;
  }
  static bool attr_set_ll = false;
  if (!attr_set_ll) {
    cudaFuncSetAttribute(ll_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, ll_smem_max<K>());
    attr_set_ll = true;
  }
  const float trouble2 = (float)(c->minLL * kLog2e);
  const int smem = masks ? LC::smem_with_masks(n_chunks) : LC::SMEM;
  if (smem > ll_smem_max<K>()) return fail(c, GMM_ERR_STATE, "frame masks do not fit the logits kernel");
  {
    GMM_LAUNCH(c, "tc_ll_kernel");
    ll_kernel<K><<<grid_ll, kLlThreads, smem, c->stream>>>(
        c->tm_wfull, c->tcx.planes, c->N, nullptr, nullptr, nTz, nTw, tile0, n_tiles_ll, n_chunks, trouble2,
        c->minLL, c->tcm.ll2, ll_out_dev, c->tc_llpart, c->tc_err,
        (build_planes || LC::ZB == 2) ? c->X : nullptr, c->D, build_planes ? 1 : 0, c->wait_limit,
        masks ? c->sched.fmask : nullptr,
        (float)(log2((double)c->minGamma) - kSchedMargin2), c->Mact == 1,
        c->static_shapes ? c->flag + 4 : nullptr);
  }
  if (!want_total) return GMM_OK;
  {
    GMM_LAUNCH(c, "tc_ll_total_kernel");
    ll_total_kernel<<<1, 1024, 0, c->stream>>>(grid_ll * 128, c->tc_llpart,
                                                c->stats + (size_t)c->M * (1 + 2 * c->D));
  }
  return GMM_OK;
}

template <int K>
int launch_acc_part(Ctx* c, int flags);

template <int K>
int launch_acc_sched(Ctx* c, int flags);

template <int K>
int launch_estep(Ctx* c, int flags, bool want_stats, float* ll_out_dev, bool build_planes) {
  const bool sched = want_stats && c->sched_active;
  const int rc = launch_ll_part<K>(c, 0, (int)(c->tcx.Npad / 128), ll_out_dev, want_stats, build_planes, sched);
  if (rc || !want_stats) return rc;
  return sched ? launch_acc_sched<K>(c, flags) : launch_acc_part<K>(c, flags);
}

// The statistics over the sparse tile schedule (tc_schedule.cu): sort the frames by their chunk
// masks, write the sorted operand planes, list each chunk's active tiles, run the statistics
// kernel over work items on a fixed grid, add the items' partials per chunk.
template <int K>
int launch_acc_sched(Ctx* c, int flags) {
  using DA = AccCfg<K, true>;
  using DM = AccCfg<K, false>;
  TileSched& s = c->sched;
  const long long Npad = c->tcx.Npad;
  const int nT = (int)(Npad / 128), chunks = c->tcm.Mpad / 128;
  const bool so = (flags & GMM_ACC_VAR) != 0;
  const int grid = std::min(kSchedGridMax, 2 * c->sms);
  const size_t pneed = (size_t)grid * K * 128 * sizeof(double);
  if (pneed > c->tcpart_cap) {
    dfree(c, c->tcpart, c->tcpart_cap);
    c->tcpart = nullptr;
    c->tcpart_cap = 0;
    int rc = dalloc(c, (void**)&c->tcpart, pneed, "tc partial statistics");
    if (rc) return rc;
    c->tcpart_cap = pneed;
  }
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(acc_dense_kernel<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, DA::SMEM);
    cudaFuncSetAttribute(acc_dense_kernel<K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, DM::SMEM);
    attr_set = true;
  }
  sched_sort(c, Npad, chunks);
  {
    GMM_LAUNCH(c, "tc_sort_rows_kernel");
    sort_rows_kernel<K><<<nT, 128, 0, c->stream>>>(c->X, c->D, c->N, s.perm, c->tcm.ll2, s.fmask, s.planes, s.ll2,
                                                   s.srow, s.tmask, nT);
  }
  int rc = make_map(c, &s.zmap, s.planes, 3 * Npad * K, K);
  if (rc) return rc;
  sched_lists(c, Npad, chunks, grid);
  cudaMemsetAsync(c->tcpart, 0, pneed, c->stream);  // the kernel adds into its item's partials
  const int* mact_dev = c->static_shapes ? c->flag + 4 : nullptr;
  {
    GMM_LAUNCH(c, "tc_acc_kernel");
    auto kern = so ? acc_dense_kernel<K, true> : acc_dense_kernel<K, false>;
    kern<<<grid, kThreads, so ? DA::SMEM : DM::SMEM, c->stream>>>(
        s.zmap, c->tcm.planes, nT, chunks, s.ll2, nT, 1, 1, nullptr, s.work, c->minGamma, c->Mact == 1, mact_dev,
        c->tcpart, c->tc_err, c->wait_limit, s.lists, s.item_off + chunks);
  }
  sched_reduce(c, K, c->static_shapes ? c->tcm.Mpad : c->Mact, chunks, c->tcm.comp_of_row, nullptr, c->tcpart,
               flags);
  return GMM_OK;
}

template <int K>
int launch_acc_part(Ctx* c, int flags) {
  using DA = AccCfg<K, true>;
  using DM = AccCfg<K, false>;
  using SC = SparseCfg<K>;
  const long long Npad = c->tcx.Npad;
  const int nTz = (int)(Npad / 128), nTw = c->tcm.Mpad / 128;
  const int n_chunks = nTw;
  static bool attr_set_acc = false;
  const int n_tiles = (int)(Npad / DA::FT);
  const bool so = (flags & GMM_ACC_VAR) != 0;  // second-order statistics
  const bool sparse = tc_stats_centred(K, so);
  // CTAs = component chunks x frame slices, one CTA per SM at a time: `waves` full waves of the
  // SMs (more waves = finer slices, which fill the SMs that a single wave leaves idle, at the
  // cost of more CTA start-ups). The autotuner measures 1-3 waves once per shape.
  auto slices_for = [&](int waves) { return std::max(1, std::min(n_tiles, waves * c->sms / n_chunks)); };
  const size_t pneed = (size_t)n_chunks * slices_for(3) * 128 * K * sizeof(double);
  if (pneed > c->tcpart_cap) {
    dfree(c, c->tcpart, c->tcpart_cap);
    c->tcpart = nullptr;
    c->tcpart_cap = 0;
    int rc = dalloc(c, (void**)&c->tcpart, pneed, "tc partial statistics");
    if (rc) return rc;
    c->tcpart_cap = pneed;
  }
  if (!attr_set_acc) {
    cudaFuncSetAttribute(acc_dense_kernel<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, DA::SMEM);
    cudaFuncSetAttribute(acc_dense_kernel<K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, DM::SMEM);
    cudaFuncSetAttribute(acc_sparse_kernel<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SC::SMEM);
    attr_set_acc = true;
  }
  const CUtensorMap& zm = c->tm_zfull;
  const int* mact_dev = c->static_shapes ? c->flag + 4 : nullptr;
  auto launch_acc = [&](int sl) {
    // both kernels add into their partials
    cudaMemsetAsync(c->tcpart, 0, (size_t)n_chunks * sl * 128 * K * sizeof(double), c->stream);
    if (sparse) {
      acc_sparse_kernel<K, true><<<n_chunks * sl, kAccThreads, SC::SMEM, c->stream>>>(
          zm, c->tcm.planes, c->tcm.cent, c->X, c->N, nullptr, c->D, nTz, nTw, c->tcm.ll2, n_tiles, n_chunks, sl,
          nullptr, nullptr, c->minGamma, c->Mact == 1, mact_dev, c->tcpart, c->tc_err, c->wait_limit, nullptr,
          nullptr);
    } else {
      auto kern = so ? acc_dense_kernel<K, true> : acc_dense_kernel<K, false>;
      kern<<<n_chunks * sl, kThreads, so ? DA::SMEM : DM::SMEM, c->stream>>>(
          zm, c->tcm.planes, nTz, nTw, c->tcm.ll2, n_tiles, n_chunks, sl, nullptr, nullptr, c->minGamma,
          c->Mact == 1, mact_dev, c->tcpart, c->tc_err, c->wait_limit, nullptr, nullptr);
    }
  };
  int waves = 1;
  {
    int tb = 0;
    while ((1LL << (tb + 1)) <= n_tiles) ++tb;  // frame-tile bucket: power of two
    const long long key = ((long long)so << 62) | ((long long)K << 40) | ((long long)n_chunks << 20) | tb;
    auto it = c->tuned_waves.find(key);
    if (it != c->tuned_waves.end()) {
      waves = it->second;
    } else if (c->autotune && !c->profile && c->wait_limit == kDefaultWaitLimit) {
      // each candidate launch rewrites the partials it uses, so the timed runs are harmless
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      float best = 1e30f;
      for (int w = 1; w <= 3; ++w) {
        if (w > 1 && slices_for(w) == slices_for(w - 1)) break;
        cudaEventRecord(e0, c->stream);
        launch_acc(slices_for(w));
        cudaEventRecord(e1, c->stream);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) { best = ms; waves = w; }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      c->tuned_waves[key] = waves;
    }
  }
  const int slices = slices_for(waves);
  {
    GMM_LAUNCH(c, "tc_acc_kernel");
    launch_acc(slices);
  }
  {
    GMM_LAUNCH(c, "tc_reduce_kernel");
    long long tot = (long long)n_chunks * c->D * 128;
    reduce_kernel<<<(int)((tot + 255) / 256), 256, 0, c->stream>>>(
        c->M, c->D, K, c->static_shapes ? c->tcm.Mpad : c->Mact, n_chunks, slices, n_tiles, c->tcm.comp_of_row,
        sparse ? c->tcm.cent : nullptr, c->tcpart, flags, c->stats);
  }
  return GMM_OK;
}

}  // namespace

int tc_supported(int D) { return D >= 1 && D <= 63; }

static int tc_K(int D) { return (2 * D + 1 + 15) / 16 * 16; }

int tc_prepare_features(Ctx* c) {
  const int K = tc_K(c->D);
  const long long Npad = (c->N + 127) / 128 * 128;
  const size_t bytes = (size_t)3 * Npad * K * sizeof(uint16_t);
  if (c->tcx.planes == nullptr || c->tcx.Npad != Npad || c->tcx.K != K) {
    dfree(c, c->tcx.planes, (size_t)3 * c->tcx.Npad * c->tcx.K * sizeof(uint16_t));
    dfree(c, c->tcm.ll2, sizeof(float) * (size_t)c->tcx.Npad);
    c->tcx.planes = nullptr;
    c->tcm.ll2 = nullptr;
    c->tcx.Npad = 0;
    int rc = dalloc(c, (void**)&c->tcx.planes, bytes, "tensor-core feature planes");
    if (!rc) rc = dalloc(c, (void**)&c->tcm.ll2, sizeof(float) * (size_t)Npad, "tensor-core frame LSE");
    if (rc) return rc;
    c->tcx.Npad = Npad;
    c->tcx.K = K;
  }
  // the logits kernel fills the planes from the features on its first pass over them
  int rc = make_map(c, &c->tm_zfull, c->tcx.planes, 3 * Npad * K, K);
  return rc;
}

// sched_ok: the caller runs the E-step of the resident features (tc_estep, tc_estep_streamed),
// which may use the sparse tile schedule
int tc_prepare_model(Ctx* c, bool sched_ok) {
  const int K = tc_K(c->D);
  // fixed shapes: every component gets a row (dead ones are padding rows)
  const int Mpad = ((c->static_shapes ? c->M : c->Mact) + 127) / 128 * 128;
  if (c->tcm.planes == nullptr || c->tcm.Mpad != Mpad || c->tcm.K != K || c->tcm.D != c->D) {
    dfree(c, c->tcm.planes, (size_t)3 * c->tcm.Mpad * c->tcm.K * sizeof(uint16_t));
    dfree(c, c->tcm.comp_of_row, sizeof(int) * (size_t)c->tcm.Mpad);
    dfree(c, c->tcm.cent, sizeof(float) * (size_t)c->tcm.Mpad * c->tcm.D);
    c->tcm.planes = nullptr;
    c->tcm.comp_of_row = nullptr;
    c->tcm.cent = nullptr;
    int rc = dalloc(c, (void**)&c->tcm.planes, (size_t)3 * Mpad * K * sizeof(uint16_t), "tensor-core model planes");
    if (!rc) rc = dalloc(c, (void**)&c->tcm.comp_of_row, sizeof(int) * Mpad, "row map");
    if (!rc) rc = dalloc(c, (void**)&c->tcm.cent, sizeof(float) * (size_t)Mpad * c->D, "statistics centres");
    if (rc) return rc;
    c->tcm.Mpad = Mpad;
    c->tcm.K = K;
    c->tcm.D = c->D;
  }
  // the sparse tile schedule of the statistics (K <= 80: the dense statistics kernel) wants the
  // components grouped into spatially coherent chunks; the row order is free otherwise
  const int* mact_dev = c->static_shapes ? c->flag + 4 : nullptr;
  const int chunks = Mpad / 128;
  c->sched_active = sched_ok && K <= 80 && c->tcx.Npad > 0 &&
                    (c->sched.mode == 2 || (c->sched.mode == 1 && c->tcx.Npad / 128 >= kSchedMinTiles)) &&
                    sched_supported(chunks, c->static_shapes ? c->M : c->Mact);
  if (c->sched_active) {
    int rc = sched_prepare(c, c->tcx.Npad, K, chunks);
    if (rc) return rc;
    sched_group(c, c->act, c->Mact, mact_dev, chunks, c->D, c->mu);
  }
  launch_model(c, c->D, K, c->Mact, Mpad, Mpad, 0, c->sched_active ? c->sched.gact : c->act, c->w, c->mu, c->var,
               c->tcm.planes, c->tcm.comp_of_row, c->tcm.cent, mact_dev);
  int rc = make_map(c, &c->tm_wfull, c->tcm.planes, 3LL * Mpad * K, K);
  return rc;
}

// E-step whose features arrive from the host while it runs: the frames go up in chunks of
// whole 128-frame tiles on a copy stream, and each chunk's feature planes and log-likelihood
// tiles start as soon as its copy lands, so the transfer hides behind the logits kernels; the
// statistics kernel then runs over all tiles. c->X must be the handle's own device buffer of
// c->N x c->D floats; Xh is the host block (page-locked for the copies to overlap).
int ensure_copy_stream(Ctx* c, int n_events) {
  if (!c->copy_stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamCreate(copy)");
  }
  while ((int)c->copy_events.size() < n_events) {
    cudaEvent_t ev;
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaEventCreate");
    c->copy_events.push_back(ev);
  }
  return GMM_OK;
}

int tc_estep_streamed(Ctx* c, const float* Xh, int flags, int nchunks) {
  if (!tc_supported(c->D)) return fail(c, GMM_ERR_UNSUPPORTED, "tensor-core path supports 1 <= D <= 63");
  if (c->N == 0) return GMM_OK;
  if (!c->tc_err) {
    int rc = dalloc(c, (void**)&c->tc_err, sizeof(int), "tc error flag");
    if (rc) return rc;
    cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
    int dev;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const int K = tc_K(c->D);
  const long long Npad = (c->N + 127) / 128 * 128;
  if (c->tcx.planes == nullptr || c->tcx.Npad != Npad || c->tcx.K != K) {
    dfree(c, c->tcx.planes, (size_t)3 * c->tcx.Npad * c->tcx.K * sizeof(uint16_t));
    dfree(c, c->tcm.ll2, sizeof(float) * (size_t)c->tcx.Npad);
    c->tcx.planes = nullptr;
    c->tcm.ll2 = nullptr;
    c->tcx.Npad = 0;
    int rc = dalloc(c, (void**)&c->tcx.planes, (size_t)3 * Npad * K * sizeof(uint16_t), "tensor-core feature planes");
    if (!rc) rc = dalloc(c, (void**)&c->tcm.ll2, sizeof(float) * (size_t)Npad, "tensor-core frame LSE");
    if (rc) return rc;
    c->tcx.Npad = Npad;
    c->tcx.K = K;
  }
  int rc = make_map(c, &c->tm_zfull, c->tcx.planes, 3 * Npad * K, K);
  if (!rc) rc = tc_prepare_model(c, true);
  if (rc) return rc;
  if (!c->copy_stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamCreate(copy)");
  }
  // Chunks of whole 128-frame tiles: the first ones grow geometrically from 1/8 of the steady
  // chunk (nT / nchunks) so that little of the transfer is exposed before the first kernels run;
  // the copies outpace the logits kernels from then on.
  const int nT = (int)(Npad / 128);
  const int per = (nT + nchunks - 1) / nchunks;
  std::vector<int> bounds{0};
  for (int sz = std::max(1, per / 8); bounds.back() < nT; sz = std::min(per, 2 * sz))
    bounds.push_back(std::min(nT, bounds.back() + sz));
  const int nck = (int)bounds.size() - 1;
  while ((int)c->copy_events.size() < nck) {
    cudaEvent_t ev;
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaEventCreate");
    c->copy_events.push_back(ev);
  }
  // the copies must not overwrite frames a previous E-step on the compute stream still reads
  cudaEventRecord(c->copy_events[0], c->stream);
  cudaStreamWaitEvent(c->copy_stream, c->copy_events[0], 0);
  float* X = const_cast<float*>(c->X);
  for (int k = 0; k < nck; ++k) {
    const int ta = bounds[k], tb = bounds[k + 1];
    if (ta >= tb) break;
    const long long fa = (long long)ta * 128, fb = std::min(c->N, (long long)tb * 128);
    if (fb > fa) {
      cudaError_t e = cudaMemcpyAsync(X + fa * c->D, Xh + fa * c->D, sizeof(float) * (size_t)(fb - fa) * c->D,
                                      cudaMemcpyHostToDevice, c->copy_stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpyAsync(feature chunk)");
    }
    cudaEventRecord(c->copy_events[k], c->copy_stream);
    cudaStreamWaitEvent(c->stream, c->copy_events[k], 0);
    // the logits kernel builds the chunk's feature planes as it reads the frames
    switch (K) {
      case 16: rc = launch_ll_part<16>(c, ta, tb - ta, nullptr, true, true, c->sched_active); break;
      case 32: rc = launch_ll_part<32>(c, ta, tb - ta, nullptr, true, true, c->sched_active); break;
      case 48: rc = launch_ll_part<48>(c, ta, tb - ta, nullptr, true, true, c->sched_active); break;
      case 64: rc = launch_ll_part<64>(c, ta, tb - ta, nullptr, true, true, c->sched_active); break;
      case 80: rc = launch_ll_part<80>(c, ta, tb - ta, nullptr, true, true, c->sched_active); break;
      case 96: rc = launch_ll_part<96>(c, ta, tb - ta, nullptr, true, true, c->sched_active); break;
      case 112: rc = launch_ll_part<112>(c, ta, tb - ta, nullptr, true, true, c->sched_active); break;
      default: rc = launch_ll_part<128>(c, ta, tb - ta, nullptr, true, true, c->sched_active); break;
    }
    if (rc) return rc;
  }
  c->tcx_valid = true;
  if (c->sched_active) {
    switch (K) {
      case 16: rc = launch_acc_sched<16>(c, flags); break;
      case 32: rc = launch_acc_sched<32>(c, flags); break;
      case 48: rc = launch_acc_sched<48>(c, flags); break;
      case 64: rc = launch_acc_sched<64>(c, flags); break;
      default: rc = launch_acc_sched<80>(c, flags); break;
    }
  } else {
    switch (K) {
      case 16: rc = launch_acc_part<16>(c, flags); break;
      case 32: rc = launch_acc_part<32>(c, flags); break;
      case 48: rc = launch_acc_part<48>(c, flags); break;
      case 64: rc = launch_acc_part<64>(c, flags); break;
      case 80: rc = launch_acc_part<80>(c, flags); break;
      case 96: rc = launch_acc_part<96>(c, flags); break;
      case 112: rc = launch_acc_part<112>(c, flags); break;
      default: rc = launch_acc_part<128>(c, flags); break;
    }
  }
  if (rc) return rc;
  int herr = 0;
  cudaMemcpyAsync(&herr, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  rc = sync(c, "tensor-core E-step");
  if (rc) return rc;
  if (herr) {
    // kernels that gave up may have left the feature planes half built
    c->tcx_valid = false;
    cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
    return fail(c, GMM_ERR_TIMEOUT, "tensor-core E-step: a bounded device wait expired");
  }
  return GMM_OK;
}

int tc_estep(Ctx* c, int flags, bool want_stats, float* ll_out_dev) {
  if (!tc_supported(c->D)) return fail(c, GMM_ERR_UNSUPPORTED, "tensor-core path supports 1 <= D <= 63");
  if (c->N == 0) return GMM_OK;
  if (!c->tc_err) {
    int rc = dalloc(c, (void**)&c->tc_err, sizeof(int), "tc error flag");
    if (rc) return rc;
    cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
    int dev;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev);
  }
  int rc;
  const bool build = !c->tcx_valid || c->tcx.planes == nullptr;
  if (build) {
    rc = tc_prepare_features(c);
    if (rc) return rc;
  }
  rc = tc_prepare_model(c, true);  // model may change every iteration
  if (rc) return rc;
  switch (c->tcm.K) {
    case 16: rc = launch_estep<16>(c, flags, want_stats, ll_out_dev, build); break;
    case 32: rc = launch_estep<32>(c, flags, want_stats, ll_out_dev, build); break;
    case 48: rc = launch_estep<48>(c, flags, want_stats, ll_out_dev, build); break;
    case 64: rc = launch_estep<64>(c, flags, want_stats, ll_out_dev, build); break;
    case 80: rc = launch_estep<80>(c, flags, want_stats, ll_out_dev, build); break;
    case 96: rc = launch_estep<96>(c, flags, want_stats, ll_out_dev, build); break;
    case 112: rc = launch_estep<112>(c, flags, want_stats, ll_out_dev, build); break;
    case 128: rc = launch_estep<128>(c, flags, want_stats, ll_out_dev, build); break;
    default: return fail(c, GMM_ERR_UNSUPPORTED, "tensor-core path: unsupported K");
  }
  if (rc) return rc;
  c->tcx_valid = true;
  if (c->static_shapes) return GMM_OK;  // checked by the caller after the captured iterations
  // surface a bounded-wait expiry as an error status (the context stays usable)
  int herr = 0;
  cudaMemcpyAsync(&herr, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  rc = sync(c, "tensor-core E-step");
  if (rc) return rc;
  if (herr) {
    // kernels that gave up may have left the feature planes half built
    c->tcx_valid = false;
    cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
    return fail(c, GMM_ERR_TIMEOUT, "tensor-core E-step: a bounded device wait expired");
  }
  return GMM_OK;
}


// Per-speaker statistics of S speakers in one fused E-step over the resident features (speaker s
// owns frames [offs[s], offs[s+1])). Every speaker starts on a 128-row tile of a padded row
// layout; its frames are cut into pieces of one FP64 flush period (8192 frames), each piece with
// its own FP64 slot, and the statistics kernel runs over work items (component chunk x range of
// whole pieces) of about equal size. A speaker's sums are the piece slots added in piece order.
namespace {
// A speaker batch between its host preparation and its launches.
struct SpeakerBatch {
  TcBatch t;
  long long* d_pad = nullptr;     // padded speaker offsets (device)
  std::vector<long long> pad;     // the same on the host
};

// Host side of a speaker batch: the padded row layout, pieces and work items, the scratch
// buffers, every host-to-device copy of the batch, and the row map (row_frame_kernel, launched
// between the copies: issued after all of them, it cost the host-frames path its overlap of
// frame copies and logits kernels -- batched MAP end to end 16.4 -> 21-29 ms).
int speaker_prepare(Ctx* c, int S, const long long* offs, const long long* d_offs, bool second_order,
                    SpeakerStats* ss, SpeakerBatch* sb) {
  *ss = SpeakerStats();
  if (!tc_supported(c->D)) return fail(c, GMM_ERR_UNSUPPORTED, "tensor-core path supports 1 <= D <= 63");
  if (!d_offs) return fail(c, GMM_ERR_ARG, "per-speaker statistics: device speaker offsets missing");
  if (!c->tc_err) {
    int rc = dalloc(c, (void**)&c->tc_err, sizeof(int), "tc error flag");
    if (rc) return rc;
    cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
    int dev;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const int M = c->M, D = c->D, K = tc_K(D);
  int rc = tc_prepare_model(c, false);
  if (rc) return rc;
  const int FT = acc_ft(K), FLUSH = 64 * 128 / FT;
  const int n_chunks = c->tcm.Mpad / 128;
  // padded row layout (the row map itself is built on the device) and pieces
  std::vector<long long>& pad = sb->pad;
  pad.assign((size_t)S + 1, 0);
  for (int s = 0; s < S; ++s) pad[s + 1] = pad[s] + (offs[s + 1] - offs[s] + 127) / 128 * 128;
  const long long Rpad = pad[S] > 0 ? pad[S] : 128;
  const long long ntiles = Rpad / FT;
  std::vector<int> tile_slot((size_t)ntiles, 0), piece0((size_t)S, 0), npieces((size_t)S, 0);
  int pieces = 0;
  for (int s = 0; s < S; ++s) {
    const long long t0 = pad[s] / FT, t1 = pad[s + 1] / FT;
    piece0[s] = pieces;
    npieces[s] = (int)((t1 - t0 + FLUSH - 1) / FLUSH);
    for (long long t = t0; t < t1; ++t) tile_slot[(size_t)t] = pieces + (int)((t - t0) / FLUSH);
    pieces += npieces[s];
  }
  // work items: ranges of whole pieces of about equal tile counts, one CTA per (range, chunk)
  std::vector<int4> work;
  {
    const long long target = std::max<long long>(FLUSH / 4, ntiles * n_chunks / std::max(1, c->sms));
    long long t0 = 0, acc = 0, cur = 0;
    for (int s = 0; s < S; ++s) {
      const long long rt = (pad[s + 1] - pad[s]) / FT;
      for (int p = 0; p < npieces[s]; ++p) {
        const long long pt = std::min<long long>(FLUSH, rt - (long long)p * FLUSH);
        acc += pt;
        cur += pt;
        if (acc >= target) {
          for (int ch = 0; ch < n_chunks; ++ch) work.push_back(make_int4(ch, ch, (int)t0, (int)(cur - t0)));
          t0 = cur;
          acc = 0;
        }
      }
    }
    if (cur > t0)
      for (int ch = 0; ch < n_chunks; ++ch) work.push_back(make_int4(ch, ch, (int)t0, (int)(cur - t0)));
  }
  const size_t rf_bytes = sizeof(long long) * (size_t)Rpad, ts_bytes = sizeof(int) * (size_t)ntiles;
  const size_t wk_bytes = sizeof(int4) * std::max<size_t>(1, work.size());
  const size_t pad_bytes = sizeof(long long) * ((size_t)S + 1);
  long long* d_rf = nullptr;
  long long*& d_pad = sb->d_pad;
  int* d_ts = nullptr;
  int4* d_wk = nullptr;
  ss->S = S;
  ss->cent = tc_stats_centred(K, second_order) ? c->tcm.cent : nullptr;
  ss->n_chunks = n_chunks;
  ss->K = K;
  ss->pieces = pieces;
  ss->part_bytes = (size_t)std::max(pieces, 1) * n_chunks * K * 128 * sizeof(double);
  // all from the handle's grow-only scratch: nothing is allocated once the largest batch was seen
  rc = scratch(c, SC_ROWMAP, rf_bytes, "row map", (void**)&d_rf);
  if (!rc) rc = scratch(c, SC_PAD, pad_bytes, "padded speaker offsets", (void**)&d_pad);
  if (!rc) rc = scratch(c, SC_TILESLOT, ts_bytes, "tile slots", (void**)&d_ts);
  if (!rc) rc = scratch(c, SC_WORK, wk_bytes, "work items", (void**)&d_wk);
  if (!rc) rc = scratch(c, SC_PART, ss->part_bytes, "per-speaker statistics", (void**)&ss->part);
  if (!rc) rc = scratch(c, SC_PIECE0, sizeof(int) * std::max(S, 1), "speaker pieces", (void**)&ss->piece0);
  if (!rc) rc = scratch(c, SC_NPIECES, sizeof(int) * std::max(S, 1), "speaker pieces", (void**)&ss->npieces);
  if (!rc) rc = scratch(c, SC_ROWCOMP, sizeof(int) * M, "component rows", (void**)&ss->row_of_comp);
  if (!rc) {
    // operand planes in the padded layout; the next regular E-step rebuilds its own
    const size_t pbytes = (size_t)3 * Rpad * K * sizeof(uint16_t);
    if (c->tcx.planes == nullptr || c->tcx.Npad != Rpad || c->tcx.K != K) {
      dfree(c, c->tcx.planes, (size_t)3 * c->tcx.Npad * c->tcx.K * sizeof(uint16_t));
      dfree(c, c->tcm.ll2, sizeof(float) * (size_t)c->tcx.Npad);
      c->tcx.planes = nullptr;
      c->tcm.ll2 = nullptr;
      c->tcx.Npad = 0;
      rc = dalloc(c, (void**)&c->tcx.planes, pbytes, "tensor-core feature planes");
      if (!rc) rc = dalloc(c, (void**)&c->tcm.ll2, sizeof(float) * (size_t)Rpad, "tensor-core frame LSE");
      if (!rc) {
        c->tcx.Npad = Rpad;
        c->tcx.K = K;
      }
    }
    c->tcx_valid = false;
  }
  const size_t need = (size_t)std::max(1, c->sms) * 128;
  if (!rc && need > c->tc_llpart_cap) {
    dfree(c, c->tc_llpart, c->tc_llpart_cap * sizeof(double));
    c->tc_llpart = nullptr;
    c->tc_llpart_cap = 0;
    rc = dalloc(c, (void**)&c->tc_llpart, need * sizeof(double), "tc llpart");
    if (!rc) c->tc_llpart_cap = need;
  }
  if (!rc) {
    cudaMemcpyAsync(d_pad, pad.data(), pad_bytes, cudaMemcpyHostToDevice, c->stream);
    {
      GMM_LAUNCH(c, "row_frame_kernel");
      row_frame_kernel<<<(unsigned)((Rpad + 255) / 256), 256, 0, c->stream>>>(S, d_pad, d_offs, Rpad, d_rf);
    }
    cudaMemcpyAsync(d_ts, tile_slot.data(), ts_bytes, cudaMemcpyHostToDevice, c->stream);
    if (!work.empty()) cudaMemcpyAsync(d_wk, work.data(), work.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream);
    if (S > 0) {
      cudaMemcpyAsync(ss->piece0, piece0.data(), sizeof(int) * S, cudaMemcpyHostToDevice, c->stream);
      cudaMemcpyAsync(ss->npieces, npieces.data(), sizeof(int) * S, cudaMemcpyHostToDevice, c->stream);
    }
    TcBatch& t = sb->t;
    t = TcBatch();
    t.D = D;
    t.K = K;
    t.n_chunks = n_chunks;
    t.w_chunks_total = n_chunks;
    t.wplanes = c->tcm.planes;
    t.cent = c->tcm.cent;
    t.wmap = &c->tm_wfull;
    t.X = c->X;
    t.N = c->N;
    t.Rpad = Rpad;
    t.row_frame = d_rf;
    t.tile_wbase = nullptr;
    t.zplanes = c->tcx.planes;
    t.ll2 = c->tcm.ll2;
    t.ll = c->ll;
    t.llpart = c->tc_llpart;
    t.n_work = (int)work.size();
    t.work = d_wk;
    t.tile_slot = d_ts;
    t.part = ss->part;
    t.part_bytes = ss->part_bytes;
    t.single_comp = c->Mact == 1;
    t.second_order = second_order;
  }
  return rc;
}

// The launches of a prepared speaker batch: the logits and statistics kernels (over the
// resident frames, or over Xh copied in chunks of speakers on the copy stream), the component
// rows and the per-speaker log-likelihoods. Over resident frames these are stream operations
// only (a CUDA graph can capture them).
int speaker_launch(Ctx* c, int S, const long long* offs, const long long* d_offs, double* d_ll, const float* Xh,
                   SpeakerBatch* sb, SpeakerStats* ss) {
  const TcBatch& t = sb->t;
  const std::vector<long long>& pad = sb->pad;
  const long long Rpad = t.Rpad;
  int rc = GMM_OK;
  if (!Xh) {
    rc = tc_run_batch(c, t);
  } else {
    // Frames from host memory: copied in chunks of whole speakers on the copy stream (the first
    // chunks growing geometrically from 1/64 of the frames, then 1/8), each chunk's rows going
    // through the logits kernel as soon as its frames land; then the statistics in one launch
    // (statistics launches per chunk measured slower: a partial wave per chunk).
    const long long f_all = offs[S] - offs[0];
    const long long steady = std::max(1LL, (f_all + 7) / 8);
    std::vector<int> cuts{0};  // chunk boundaries (speaker indices)
    for (long long target = std::max(1LL, steady / 8); cuts.back() < S; target = std::min(steady, 2 * target)) {
      int next = cuts.back() + 1;
      while (next < S && offs[next] - offs[cuts.back()] < target) ++next;
      cuts.push_back(next);
    }
    rc = ensure_copy_stream(c, (int)cuts.size());
    int k = 0;
    if (!rc) {
      cudaEventRecord(c->copy_events[k], c->stream);  // frames a previous call may still read
      cudaStreamWaitEvent(c->copy_stream, c->copy_events[k], 0);
      ++k;
    }
    for (size_t ci = 0; !rc && ci + 1 < cuts.size(); ++ci) {
      const int sa = cuts[ci], se = cuts[ci + 1];  // speakers [sa, se)
      const long long fa = offs[sa], fb = offs[se];
      if (fb > fa) {
        cudaError_t e = cudaMemcpyAsync(const_cast<float*>(c->X) + fa * c->D, Xh + fa * c->D,
                                        sizeof(float) * (size_t)(fb - fa) * c->D, cudaMemcpyHostToDevice,
                                        c->copy_stream);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "cudaMemcpyAsync(speaker frames)");
      }
      if (!rc) {
        cudaEventRecord(c->copy_events[k], c->copy_stream);
        cudaStreamWaitEvent(c->stream, c->copy_events[k], 0);
        ++k;
        const int ta = (int)(pad[sa] / 128), tb = (int)(pad[se] / 128);
        if (tb > ta) rc = tc_run_batch_part(c, t, ta, tb - ta, 1);
      }
    }
    if (!rc) rc = tc_run_batch_part(c, t, 0, (int)(Rpad / 128), 2);
  }
  if (!rc) {
    {
      GMM_LAUNCH(c, "row_of_comp_kernel");
      row_of_comp_kernel<<<1, 1024, 0, c->stream>>>(c->M, c->tcm.Mpad, c->tcm.comp_of_row, ss->row_of_comp);
    }
    if (S > 0 && d_ll) {
      GMM_LAUNCH(c, "seg_sum_kernel");
      seg_sum_kernel<<<S, 256, 0, c->stream>>>(d_offs, c->ll, d_ll);
    }
  }
  return rc;
}

// After the launches: a bounded wait that gave up shows in the error flag.
int speaker_finish(Ctx* c, const char* what, int rc) {
  if (!rc) {
    int herr = 0;
    cudaMemcpyAsync(&herr, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    rc = sync(c, what);
    if (!rc && herr) {
      c->tcx_valid = false;
      cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
      rc = fail(c, GMM_ERR_TIMEOUT, std::string(what) + ": a bounded device wait expired");
    }
  }
  cudaStreamSynchronize(c->stream);
  return rc;
}
}  // namespace

int tc_speaker_stats(Ctx* c, int S, const long long* offs, const long long* d_offs, double* d_ll,
                     bool second_order, const float* Xh, SpeakerStats* ss) {
  SpeakerBatch sb;
  int rc = speaker_prepare(c, S, offs, d_offs, second_order, ss, &sb);
  if (!rc) rc = speaker_launch(c, S, offs, d_offs, d_ll, Xh, &sb, ss);
  rc = speaker_finish(c, "per-speaker statistics (tensor-core path)", rc);
  if (rc) tc_free_speaker_stats(c, ss);
  return rc;
}

// The buffers belong to the handle's scratch (reused by the next batch).
void tc_free_speaker_stats(Ctx*, SpeakerStats* ss) { *ss = SpeakerStats(); }

// Batched MAP. Over the resident frames the kernels of a call after the row map (logits,
// statistics, component rows, speaker log-likelihoods, the MAP update) are captured into a CUDA
// graph after an eager run of a batch layout seen on the previous call too, and a later call
// with the same batch layout and the same buffers replays it; its host-to-device copies (offsets, pieces, work items) and the row map stay
// outside the graph and are issued every call, so a replay sees the call's own speaker offsets.
// With per-kernel profiling on, calls run eagerly (a graph has no per-kernel timing events).
int tc_map_batch(Ctx* c, const MapBatch& b) {
  SpeakerStats ss;
  SpeakerBatch sb;
  int rc = speaker_prepare(c, b.S, b.offs, b.d_offs, b.upV != 0, &ss, &sb);
  if (rc) return rc;
  auto run = [&]() -> int {
    int r = speaker_launch(c, b.S, b.offs, b.d_offs, b.ll, b.Xh, &sb, &ss);
    if (!r) r = mstep_map_batch(c, b, nullptr, &ss);
    return r;
  };
  if (b.Xh || c->profile) {
    rc = run();
  } else {
    const TcBatch& t = sb.t;
    auto bits = [](float v) { uint32_t u; std::memcpy(&u, &v, 4); return (long long)u; };
    const long long key[] = {b.S, t.Rpad, t.n_work, c->N, c->M, c->D, t.K, t.n_chunks, c->tcm.Mpad, c->Mact,
                             b.tau, b.upW | b.upM << 1 | b.upV << 2 | (t.second_order ? 8 : 0),
                             bits(c->minGamma), bits((float)c->minLL), bits(c->min_var), c->wait_limit,
                             (long long)(size_t)b.d_offs, (long long)(size_t)b.w, (long long)(size_t)b.mu,
                             (long long)(size_t)b.var, (long long)(size_t)b.aw, (long long)(size_t)b.ll,
                             (long long)(size_t)sb.d_pad, (long long)(size_t)t.row_frame,
                             (long long)(size_t)t.tile_slot, (long long)(size_t)t.work, (long long)(size_t)t.part,
                             (long long)(size_t)ss.piece0, (long long)(size_t)ss.npieces,
                             (long long)(size_t)ss.row_of_comp, (long long)(size_t)ss.cent,
                             (long long)(size_t)t.zplanes, (long long)(size_t)t.ll2, (long long)(size_t)t.ll,
                             (long long)(size_t)t.llpart, (long long)(size_t)t.wplanes, (long long)(size_t)c->X,
                             (long long)(size_t)c->w, (long long)(size_t)c->mu, (long long)(size_t)c->var,
                             (long long)(size_t)c->tc_err, (long long)(size_t)c->tcm.comp_of_row, 0, 0, 0, 0, 0, 0};
    static_assert(sizeof(key) == sizeof(c->map_graph_key), "graph key size");
    if (c->map_graph && std::memcmp(key, c->map_graph_key, sizeof(key)) == 0) {
      cudaError_t e = cudaGraphLaunch(c->map_graph, c->stream);
      if (e != cudaSuccess) rc = cuda_fail(c, e, "cudaGraphLaunch(batched MAP)");
      c->launches += c->map_graph_launches;
    } else {
      // a layout is captured the second time in a row it comes (calls whose layouts keep
      // changing run eagerly and pay no capture)
      const bool repeat = std::memcmp(key, c->map_last_key, sizeof(key)) == 0;
      std::memcpy(c->map_last_key, key, sizeof(key));
      rc = run();  // eager (also sets the kernels' attributes before any capture)
      if (!rc && repeat) {
        if (c->map_graph) cudaGraphExecDestroy(c->map_graph);
        c->map_graph = nullptr;
        const bool prof = c->profile;
        const long long l0 = c->launches;
        c->profile = false;  // no timing events inside the graph
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
          const int r = run();
          e = cudaStreamEndCapture(c->stream, &g);
          if (!r && e == cudaSuccess) e = cudaGraphInstantiate(&c->map_graph, g, 0);
          if (r && e == cudaSuccess) e = cudaErrorUnknown;
          if (g) cudaGraphDestroy(g);
        }
        c->map_graph_launches = (int)(c->launches - l0);
        c->launches = l0;
        c->profile = prof;
        if (e != cudaSuccess) {
          // no graph this time: the eager run stands, the next call tries again
          if (c->map_graph) cudaGraphExecDestroy(c->map_graph);
          c->map_graph = nullptr;
          cudaGetLastError();
        } else {
          std::memcpy(c->map_graph_key, key, sizeof(key));
        }
      }
    }
  }
  rc = speaker_finish(c, "batched MAP update", rc);
  tc_free_speaker_stats(c, &ss);
  return rc;
}

// ------------------------------------------------------------------ request batches

int tc_stats_ft(int K) { return acc_ft(K); }
int tc_flush_tiles(int K) { return 64 * 128 / acc_ft(K); }
bool tc_stats_centred(int K, bool second_order) { return second_order && K > 80; }
int tc_k(int D) { return tc_K(D); }

int tc_make_wmap(Ctx* c, CUtensorMap* map, const uint16_t* planes, long long rows, int K) {
  return make_map(c, map, planes, 3 * rows * K, K);
}

int tc_build_model(Ctx* c, int D, int K, int Mact, int Mpad, long long plane_rows, long long row0,
                   const int* act, const float* w, const float* mu, const float* var,
                   uint16_t* planes, int* comp_of_row, float* cent) {
  launch_model(c, D, K, Mact, Mpad, plane_rows, row0, act, w, mu, var, planes, comp_of_row, cent, nullptr);
  return GMM_OK;
}

namespace {
template <int K>
// stages: 1 = feature planes and logits of the row tiles [tile0, tile0 + ntl), 2 = statistics of
// the whole batch
void run_batch_k(Ctx* c, const TcBatch& b, const CUtensorMap& zfull, int tile0, int ntl, int stages) {
  using LC = LlCfg<K>;
  using DA = AccCfg<K, true>;
  using DM = AccCfg<K, false>;
  using SC = SparseCfg<K>;
  const int nTz = (int)(b.Rpad / 128);
  const int grid_ll = std::max(1, std::min(ntl, c->sms));
  // the same limits as the resident-feature launches set (the largest shared memory the kernel
  // is launched with anywhere): a smaller limit here would fail their later launches
  cudaFuncSetAttribute(ll_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, ll_smem_max<K>());
  cudaFuncSetAttribute(acc_dense_kernel<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, DA::SMEM);
  cudaFuncSetAttribute(acc_dense_kernel<K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, DM::SMEM);
  cudaFuncSetAttribute(acc_sparse_kernel<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SC::SMEM);
  if ((stages & 1) && ntl > 0) {
    GMM_LAUNCH(c, "tc_ll_kernel");
    ll_kernel<K><<<grid_ll, kLlThreads, LC::SMEM, c->stream>>>(
        *b.wmap, b.zplanes, b.N, b.row_frame, b.tile_wbase, nTz, b.w_chunks_total, tile0, ntl, b.n_chunks,
        (float)(c->minLL * kLog2e), c->minLL, b.ll2, b.ll, b.llpart, c->tc_err,
        b.X, b.D, 1, c->wait_limit, nullptr, 0.0f, 0, nullptr);
  }
  if ((stages & 2) && b.n_work > 0) {
    GMM_LAUNCH(c, "tc_acc_kernel");
    const CUtensorMap& zm = zfull;
    if (b.part_bytes) cudaMemsetAsync(b.part, 0, b.part_bytes, c->stream);  // the kernels add into it
    if (tc_stats_centred(K, b.second_order)) {
      acc_sparse_kernel<K, true><<<b.n_work, kAccThreads, SC::SMEM, c->stream>>>(
          zm, b.wplanes, b.cent, b.X, b.N, b.row_frame, b.D, nTz, b.w_chunks_total, b.ll2, (int)(b.Rpad / SC::FT),
          b.n_chunks, 1, b.tile_slot, b.work, c->minGamma, b.single_comp, nullptr, b.part, c->tc_err,
          c->wait_limit, nullptr, nullptr);
    } else {
      auto kern = b.second_order ? acc_dense_kernel<K, true> : acc_dense_kernel<K, false>;
      kern<<<b.n_work, kThreads, b.second_order ? DA::SMEM : DM::SMEM, c->stream>>>(
          zm, b.wplanes, nTz, b.w_chunks_total, b.ll2, (int)(b.Rpad / DA::FT), b.n_chunks, 1, b.tile_slot,
          b.work, c->minGamma, b.single_comp, nullptr, b.part, c->tc_err, c->wait_limit, nullptr, nullptr);
    }
  }
}
}  // namespace

int tc_run_batch_part(Ctx* c, const TcBatch& b, int tile0, int ntl, int stages) {
  if (b.Rpad <= 0) return GMM_OK;
  // the logits kernel builds the feature planes (row map applied) from b.X as it goes
  CUtensorMap zfull;
  int rc = make_map(c, &zfull, b.zplanes, 3 * b.Rpad * b.K, b.K);
  if (rc) return rc;
  switch (b.K) {
    case 16: run_batch_k<16>(c, b, zfull, tile0, ntl, stages); break;
    case 32: run_batch_k<32>(c, b, zfull, tile0, ntl, stages); break;
    case 48: run_batch_k<48>(c, b, zfull, tile0, ntl, stages); break;
    case 64: run_batch_k<64>(c, b, zfull, tile0, ntl, stages); break;
    case 80: run_batch_k<80>(c, b, zfull, tile0, ntl, stages); break;
    case 96: run_batch_k<96>(c, b, zfull, tile0, ntl, stages); break;
    case 112: run_batch_k<112>(c, b, zfull, tile0, ntl, stages); break;
    case 128: run_batch_k<128>(c, b, zfull, tile0, ntl, stages); break;
    default: return fail(c, GMM_ERR_UNSUPPORTED, "tensor-core path: unsupported K");
  }
  return GMM_OK;
}

int tc_run_batch(Ctx* c, const TcBatch& b) { return tc_run_batch_part(c, b, 0, (int)(b.Rpad / 128), 3); }

}  // namespace gmm
