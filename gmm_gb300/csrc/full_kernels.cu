// Full-covariance GMMs: model precompute, E-step and EM / MAP updates on the device.
//
// Semantics followed (GMM/lib_bmssr):
//   insertModel, full branch   trainer/OL_GMMStatsEstimator.cpp:298-305: inverse and log-det of
//                              each covariance (getCovInverse / getLogDet, :155-229, Cholesky
//                              through single-precision LAPACK), logGconst = -D/2 log 2pi -
//                              logdet/2, logW = log w; a factorisation failure throws
//   computeMixLogLikeFullCov   :593-620: ll = logGconst - 0.5 (x-mu)^T cov^-1 (x-mu); non-finite
//                              -> minLogLike; then the same LSE / posterior / pruning rules as
//                              the diagonal path (getLikeAndGammas, compGammas)
//   accumulateStats, _fFullVar :1334-1378: n += g, F_k += g x_k, S_k,kk += (g x_k) x_kk for
//                              kk >= k (packed upper triangle, row order), float products
//   UpdateModelEM / UpdateModelMAP, full branches: trainer/OL_ModelAdapt.cpp:905-917, 1074-1083
//
// Arithmetic (our design): the covariance is factored in FP64 on the device (cov = L L^T), and
// the quadratic form is |U (x - mu)|^2 with U = L^-1 stored in float, evaluated by forward
// products with fused multiply-adds: D(D+1)/2 + D FMAs per frame x component instead of the
// reference's 3 D^2 float operations with an explicit inverse, and closer to the exact value
// (the reference's inverse and its D^2-term float sum carry the larger rounding). The
// statistics keep the reference's float products and accumulate them in double-float
// (two-float TwoSum) registers: about 2^-44 relative, versus FP64 sums that run on GB300's
// narrow FP64 pipe at a sixth of the rate.
//
// Layout in HBM: w [M], mu [M][D], cov [M][D][D] (caller order, row-major), U [M][UP] with row i
// of U stored at rowoff(i) padded with zeros to a multiple of 4 floats (UP = rowoff(DP), DP = D
// rounded up to a kernel width), statistics [n (M) | F (M x D) | S (M x P) | totLL | pad] with
// P = D(D+1)/2.
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <cstring>
#include <new>

#include "gmm_internal.cuh"
#include "tc_ptx.cuh"

namespace gmm {

struct FullModel {
  int M = 0, D = 0, DP = 0, UP = 0, P = 0, Mact = 0;
  float *w = nullptr, *mu = nullptr, *cov = nullptr, *U = nullptr, *logG = nullptr, *logW = nullptr;
  float* aw = nullptr;  // MAP adapted-weight scratch [M]
  int* act = nullptr;
  float *pw = nullptr, *pmu = nullptr, *pcov = nullptr;
  bool have_prior = false;
  double* stats = nullptr;
  bool stats_valid = false;
  int acc_flags = 0;
  long long tot_frames = 0;
  bool dirty = true;
  double* aux = nullptr;  // --robust auxiliary statistics [M x D | M | M]
  size_t aux_cap = 0;
  bool aux_valid = false;
  uint16_t* tcB = nullptr;  // tensor-core operand images of [U | -U mu], per component group
  size_t tcB_cap = 0;
  float2* tcC = nullptr;    // (log Gconst, log w) of the active components in order [M]
  int tc_ng = 0;            // component groups (0: the FP32 kernel is used)
  size_t stats_count() const { return (size_t)M * (1 + D + P) + 2; }
};

namespace {

constexpr int kFullMaxDim = 64;

// Row i of U holds i + 1 values padded to row_len4(i); it starts at rowoff(i) = sum of the
// previous rows' lengths = 4 (a + 1)(2a + b) for i = 4a + b.
__host__ __device__ __forceinline__ constexpr int row_len4(int i) { return (i / 4 + 1) * 4; }
__host__ __device__ __forceinline__ constexpr int rowoff(int i) { return 4 * (i / 4 + 1) * (2 * (i / 4) + i % 4); }

int dp_for(int D) {
  if (D <= 8) return 8;
  if (D <= 16) return 16;
  if (D <= 24) return 24;
  if (D <= 32) return 32;
  if (D <= 40) return 40;
  if (D <= 48) return 48;
  return 64;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// h + l += t (Knuth's TwoSum into a double-float accumulator).
__device__ __forceinline__ void two_sum(float& h, float& l, float t) {
  const float s = __fadd_rn(h, t);
  const float bb = __fsub_rn(s, h);
  const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(t, bb));
  h = s;
  l = __fadd_rn(l, err);
}

__device__ __forceinline__ void add_log(float& p1, float p2) {
  if (__fsub_rn(p1, 15.0f) > p2) return;
  if (p1 > p2) p1 = __fadd_rn(p1, logf(__fadd_rn(1.0f, expf(__fsub_rn(p2, p1)))));
  else p1 = __fadd_rn(p2, logf(__fadd_rn(1.0f, expf(__fsub_rn(p1, p2)))));
}

// ------------------------------------------------------------------ tensor-core log-likelihood
//
// y = U (x - mu) for every frame and component as one tcgen05 GEMM per group of GC components:
// A = the 128-frame tile [x | 1 | 0...] (KX = D + 1 rounded up to 16 columns), B = the group's
// rows [U_m | -U_m mu_m | 0...] (KX rows per component, N = GC KX), D[128 frames x N] in TMEM.
// Both operands are split into three bf16 planes and the six plane products with i + j <= 2 are
// summed (FP32-level products); -U mu is formed in FP64 and rounded to float. The epilogue
// (thread = frame) sums y_i^2 over the D rows of each component in four interleaved FMA chains,
// then applies the FP32 kernel's rules (non-finite -> minLogLike, log weight, sequential addLog
// over the active components in order).
constexpr int kFtThreads = 192;  // warp 0 copies, warp 1 MMA, warps 2-5 epilogue (one per lane quadrant)
constexpr long long kFtWait = 4000000000LL;
__host__ __device__ constexpr int ft_gc(int KX) { return KX == 16 ? 15 : KX == 32 ? 7 : KX == 48 ? 4 : 3; }
__host__ __device__ constexpr int ft_min(int a, int b) { return a < b ? a : b; }

template <int KX>
struct FtCfg {
  static constexpr int GC = ft_gc(KX), N = GC * KX;
  static constexpr int A_COL = 2 * N;            // two accumulators at 0 and N, then the X tile
  static constexpr int B_PLANE = N * KX * 2;     // bytes of one plane of a group image
  static constexpr int B_STAGE = 3 * B_PLANE;
  static constexpr int NB = ft_min(3, (227 * 1024 - 2048) / B_STAGE);
  static constexpr int OFF_BAR = NB * B_STAGE;
  static constexpr int SMEM = OFF_BAR + 256 + 1024;
  static_assert(N <= 256 && A_COL + 3 * KX / 2 <= 512 && NB >= 2, "tensor-core full LL budget");
};

__device__ __forceinline__ void ft_split3(float v, uint16_t& a, uint16_t& b, uint16_t& c) {
  const __nv_bfloat16 h1 = __float2bfloat16_rn(v);
  float r = v - __bfloat162float(h1);
  const __nv_bfloat16 h2 = __float2bfloat16_rn(r);
  r = r - __bfloat162float(h2);
  const __nv_bfloat16 h3 = __float2bfloat16_rn(r);
  a = __bfloat16_as_ushort(h1);
  b = __bfloat16_as_ushort(h2);
  c = __bfloat16_as_ushort(h3);
}

// Group images: element (row, k) of plane p of group g at
// ((g * 3 + p) * KX/8 + k / 8) * N * 8 + row * 8 + k % 8, row = j * KX + i for component slot j
// and row i of U. One thread per element of a plane, in image order.
__global__ void full_tc_b_kernel(int Mact, int D, int UP, int KX, int GC, int ng, const int* __restrict__ act,
                                 const float* __restrict__ mu, const float* __restrict__ U,
                                 const float* __restrict__ logG, const float* __restrict__ logW,
                                 uint16_t* __restrict__ B, float2* __restrict__ cpair) {
  const int N = GC * KX;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < Mact) cpair[t] = make_float2(logG[act[t]], logW[act[t]]);
  if (t >= (long long)ng * N * KX) return;
  const int g = (int)(t / ((long long)N * KX));
  const int e = (int)(t - (long long)g * N * KX);
  const int kc = e / (N * 8), row = (e / 8) % N, k = kc * 8 + (e & 7);
  const int j = row / KX, i = row - j * KX, a = g * GC + j;
  float v = 0.0f;
  if (a < Mact && i < D) {
    const int m = act[a];
    const float* Ur = U + (size_t)m * UP + rowoff(i);
    if (k <= i) {
      v = Ur[k];
    } else if (k == D) {
      double sum = 0.0;
      for (int kk = 0; kk <= i; ++kk) sum += (double)Ur[kk] * (double)mu[(size_t)m * D + kk];
      v = (float)(-sum);
    }
  }
  uint16_t p1, p2, p3;
  ft_split3(v, p1, p2, p3);
  uint16_t* base = B + (size_t)g * 3 * N * KX + e;
  base[0] = p1;
  base[(size_t)N * KX] = p2;
  base[2 * (size_t)N * KX] = p3;
}

__device__ __forceinline__ int ft_pa(int pr) { return pr == 0 ? 2 : (pr == 1 || pr == 3) ? 1 : 0; }
__device__ __forceinline__ int ft_pb(int pr) { return pr == 2 ? 2 : (pr == 1 || pr == 4) ? 1 : 0; }

// One component's KX accumulator columns of this thread's row (all loads in flight at once).
template <int KX>
__device__ __forceinline__ void ft_ld(uint32_t taddr, uint32_t (&y)[KX / 16][16]) {
#pragma unroll
  for (int q = 0; q < KX / 16; ++q) ptx::tmem_ld16(taddr + 16 * q, y[q]);
  ptx::tmem_ld_wait();
}

template <int KX>
__global__ void __launch_bounds__(kFtThreads, 1)
    full_tc_ll_kernel(const float* __restrict__ X, long long f0, long long nf, int D, int Mact,
                      const float2* __restrict__ cpair, const uint16_t* __restrict__ Bimg, int ng, float minLL,
                      float* __restrict__ G, long long ldg, float* __restrict__ ll, double* __restrict__ llpart,
                      int* __restrict__ flag, int* __restrict__ err) {
  using namespace ptx;
  using C = FtCfg<KX>;
  constexpr int GC = C::GC, N = C::N, NB = C::NB;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
  uint64_t* b_full = bars;           // [NB <= 3]
  uint64_t* b_empty = bars + 3;      // [NB]
  uint64_t* d_full = bars + 6;       // [2]
  uint64_t* d_empty = bars + 8;      // [2]
  uint64_t* a_full = bars + 10;
  uint64_t* mma_done = bars + 11;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 12);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 13);
  double* s_red = reinterpret_cast<double*>(bars + 14);  // [4]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long n_tiles = (nf + 127) / 128;
  const int my_tiles = blockIdx.x < n_tiles ? (int)((n_tiles - 1 - blockIdx.x) / gridDim.x) + 1 : 0;
  const int steps = my_tiles * ng;

  if (threadIdx.x == 0) {
    for (int i = 0; i < NB; ++i) {
      mbar_init(&b_full[i], 1);
      mbar_init(&b_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&d_full[i], 1);
      mbar_init(&d_empty[i], 4);
    }
    mbar_init(a_full, 4);
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
  int issued = 0;  // B stage copies issued (loader thread)

  if (warp == 0) {
    if (lane == 0) {
      for (int sidx = 0; sidx < steps; ++sidx) {
        const int st = sidx % NB, g = sidx % ng;
        if (!mbar_wait(&b_empty[st], ((sidx / NB) & 1) ^ 1, abort_flag, kFtWait)) break;
        mbar_arrive_expect_tx(&b_full[st], C::B_STAGE);
        bulk_load(smem + st * C::B_STAGE, Bimg + (size_t)g * 3 * N * KX, C::B_STAGE, &b_full[st]);
        issued = sidx + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16(128, N, false, false);
      const uint32_t sb = smem_u32(smem);
      bool ok = true;
      for (int it = 0; it < my_tiles && ok; ++it) {
        if (!mbar_wait(a_full, it & 1, abort_flag, kFtWait)) break;
        tc_fence_after();
        for (int g = 0; g < ng; ++g) {
          const int sidx = it * ng + g, st = sidx % NB, b = sidx & 1;
          if (!mbar_wait(&b_full[st], (sidx / NB) & 1, abort_flag, kFtWait)) { ok = false; break; }
          if (sidx >= 2 && !mbar_wait(&d_empty[b], ((sidx - 2) >> 1) & 1, abort_flag, kFtWait)) { ok = false; break; }
          tc_fence_after();
          const uint32_t d = tmem + (uint32_t)(b * N);
#pragma unroll
          for (int q = 0; q < KX / 16; ++q) {
#pragma unroll
            for (int pr = 0; pr < 6; ++pr) {
              const uint32_t a = tmem + C::A_COL + ft_pa(pr) * (KX / 2) + q * 8;
              const uint64_t bd = smem_desc(sb + st * C::B_STAGE + ft_pb(pr) * C::B_PLANE + q * 2 * N * 16, N * 16, 128);
              mma_ts(d, a, bd, idesc, (q > 0 || pr > 0) ? 1u : 0u);
            }
          }
          mma_commit(&b_empty[st]);
          mma_commit(&d_full[b]);
        }
      }
      mma_commit(mma_done);
      const long long t0 = clock64();
      while (!mbar_try_wait(mma_done, 0))
        if (clock64() - t0 > kFtWait) break;
    }
  } else {
    // epilogue: thread = frame row of the tile
    const int q4 = warp & 3, row = q4 * 32 + lane;
    const uint32_t lane_off = (uint32_t)(q4 * 32) << 16;
    double v = 0.0;
    bool ok = true;
    for (int it = 0; it < my_tiles && ok; ++it) {
      const long long fi = ((long long)blockIdx.x + (long long)it * gridDim.x) * 128 + row;
      const bool valid = fi < nf;
      // the X tile into TMEM (the previous tile's MMAs are complete: their last accumulator
      // was read below)
      {
        const float* xr = X + (size_t)(f0 + (valid ? fi : 0)) * D;
        for (int c = 0; c < KX / 8; c += 2) {
          uint32_t w[3][8];
#pragma unroll
          for (int e = 0; e < 16; e += 2) {
            uint16_t a[2], b[2], cc[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
              const int k = c * 8 + e + u;
              const float val = !valid ? 0.0f : k < D ? __ldg(xr + k) : (k == D ? 1.0f : 0.0f);
              ft_split3(val, a[u], b[u], cc[u]);
            }
            w[0][e >> 1] = a[0] | ((uint32_t)a[1] << 16);
            w[1][e >> 1] = b[0] | ((uint32_t)b[1] << 16);
            w[2][e >> 1] = cc[0] | ((uint32_t)cc[1] << 16);
          }
#pragma unroll
          for (int p = 0; p < 3; ++p) tmem_st8(tmem + lane_off + C::A_COL + p * (KX / 2) + c * 4, w[p]);
        }
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(a_full);
      }
      float maxLL = minLL, sumLL = minLL;
      for (int g = 0; g < ng && ok; ++g) {
        const int sidx = it * ng + g, b = sidx & 1;
        if (!mbar_wait_all(&d_full[b], (sidx >> 1) & 1, abort_flag, kFtWait)) { ok = false; break; }
        tc_fence_after();
        const int nt = min(GC, Mact - g * GC);
        float2 cp[GC];  // the group's constants, loaded before the accumulator
#pragma unroll
        for (int j = 0; j < GC; ++j) cp[j] = j < nt ? __ldg(cpair + g * GC + j) : make_float2(0.0f, 0.0f);
        // one component's columns in flight while the previous one is summed
        uint32_t ya[KX / 16][16], yb[KX / 16][16];
#pragma unroll
        for (int q = 0; q < KX / 16; ++q) tmem_ld16(tmem + lane_off + (uint32_t)(b * N + 16 * q), ya[q]);
#pragma unroll
        for (int j = 0; j < GC; ++j) {
          if (j < nt) {
            tmem_ld_wait();
            uint32_t (&y)[KX / 16][16] = (j & 1) ? yb : ya;
            uint32_t (&yn)[KX / 16][16] = (j & 1) ? ya : yb;
            if (j + 1 < nt) {
#pragma unroll
              for (int q = 0; q < KX / 16; ++q)
                tmem_ld16(tmem + lane_off + (uint32_t)(b * N + (j + 1) * KX + 16 * q), yn[q]);
            }
            // four interleaved FMA chains (rows i mod 4), then their sum
            float e4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int i = 0; i < KX; ++i)
              if (i < D) {
                const float yi = __uint_as_float(y[i / 16][i % 16]);
                e4[i & 3] = __fmaf_rn(yi, yi, e4[i & 3]);
              }
            const float e = __fadd_rn(__fadd_rn(e4[0], e4[1]), __fadd_rn(e4[2], e4[3]));
            const int a = g * GC + j;
            float s = __fsub_rn(cp[j].x, __fmul_rn(0.5f, e));
            if (!isfinite(s)) s = minLL;
            const float gv = __fadd_rn(s, cp[j].y);
            if (G != nullptr && valid) G[(size_t)a * ldg + fi] = gv;
            if (maxLL < gv) maxLL = gv;
            add_log(sumLL, gv);
          }
        }
        tmem_ld_wait();  // nothing left in flight before the buffer is released
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&d_empty[b]);
      }
      if (ok && valid) {
        const float l = (maxLL == minLL) ? minLL : sumLL;
        if (maxLL == minLL) flag[1] = 1;
        ll[f0 + fi] = l;
        v += (double)l;
      }
    }
    v = warp_sum(v);
    if (lane == 0) s_red[q4] = v;
  }
  __syncthreads();
  if (*abort_flag && warp == 0 && lane == 0) {
    // Every role has stopped. The loader's last NB copies may still be in flight (a consumer
    // that gave up never waited for them): let them land before the CTA's shared memory goes.
    for (int sidx = max(0, issued - NB); sidx < issued; ++sidx) {
      const long long t0 = clock64();
      while (!mbar_try_wait(&b_full[sidx % NB], (sidx / NB) & 1))
        if (clock64() - t0 > kFtWait) break;
    }
  }
  if (threadIdx.x == 0) {
    if (*abort_flag) atomicExch(err, 1);
    llpart[blockIdx.x] = s_red[0] + s_red[1] + s_red[2] + s_red[3];
  }
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// (k, kk) of packed entry e of the upper triangle in row order, kk >= k.
__device__ __forceinline__ void unpack(int e, int D, int& k, int& kk) {
  k = 0;
  int rem = e;
  while (rem >= D - k) {
    rem -= D - k;
    ++k;
  }
  kk = k + rem;
}

__global__ void full_active_kernel(int M, const float* __restrict__ w, int* __restrict__ act,
                                   int* __restrict__ count) {
  int lane = threadIdx.x;
  int base = 0;
  for (int s = 0; s < M; s += 32) {
    int m = s + lane;
    bool on = m < M && w[m] > 0.0f;
    unsigned b = __ballot_sync(0xffffffffu, on);
    if (on) act[base + __popc(b & ((1u << lane) - 1u))] = m;
    base += __popc(b);
  }
  if (lane == 0) *count = base;
}

// insertModel for one component per block (64 threads): FP64 Cholesky, log-det, U = L^-1 in
// the padded row layout. flag[7] <- 1 when a covariance is not positive definite.
__global__ void __launch_bounds__(64) full_prepare_kernel(int M, int D, int DP, int UP,
                                                          const float* __restrict__ w,
                                                          const float* __restrict__ cov, float minLL,
                                                          float* __restrict__ U, float* __restrict__ logG,
                                                          float* __restrict__ logW, int* __restrict__ flag) {
  extern __shared__ double sm[];
  const int LD = D + 1;
  double* A = sm;             // D x LD: covariance, then L in the lower triangle
  double* V = sm + D * LD;    // D x LD: L^-1 (lower)
  __shared__ int s_fail;
  const int m = blockIdx.x, t = threadIdx.x;
  const float wm = w[m];
  if (t == 0) {
    logW[m] = (wm > 0.0f) ? (float)log((double)wm) : minLL;
    s_fail = 0;
  }
  if (!(wm > 0.0f)) {
    if (t == 0) logG[m] = 0.0f;
    return;
  }
  const float* C = cov + (size_t)m * D * D;
  for (int e = t; e < D * D; e += blockDim.x) {
    const int i = e / D, j = e - i * D;
    A[i * LD + j] = (double)C[e];
  }
  __syncthreads();
  for (int k = 0; k < D; ++k) {
    if (t == 0) {
      const double p = A[k * LD + k];
      if (!(p > 0.0)) s_fail = 1;
      else A[k * LD + k] = sqrt(p);
    }
    __syncthreads();
    if (s_fail) break;
    const double lkk = A[k * LD + k];
    for (int i = k + 1 + t; i < D; i += blockDim.x) A[i * LD + k] = A[i * LD + k] / lkk;
    __syncthreads();
    for (int i = k + 1 + t; i < D; i += blockDim.x) {
      const double lik = A[i * LD + k];
      for (int j = k + 1; j <= i; ++j) A[i * LD + j] -= lik * A[j * LD + k];
    }
    __syncthreads();
  }
  if (s_fail) {
    if (t == 0) {
      atomicExch(&flag[7], 1);
      logG[m] = 0.0f;
    }
    return;
  }
  for (int c = t; c < D; c += blockDim.x) {
    V[c * LD + c] = 1.0 / A[c * LD + c];
    for (int i = c + 1; i < D; ++i) {
      double s = 0.0;
      for (int k = c; k < i; ++k) s += A[i * LD + k] * V[k * LD + c];
      V[i * LD + c] = -s / A[i * LD + i];
    }
  }
  __syncthreads();
  if (t == 0) {
    // getLogDet returns a float; logGconst = (float)(MINUS_LOG_2PI * dim/2 - logdet/2)
    double ld = 0.0;
    for (int i = 0; i < D; ++i) ld += log(A[i * LD + i]);
    const float lf = (float)(2.0 * ld);
    logG[m] = (float)(kMinusLog2Pi * D / 2 - (double)__fdiv_rn(lf, 2.0f));
  }
  float* Um = U + (size_t)m * UP;
  int off = 0;
  for (int i = 0; i < DP; ++i) {
    const int len = row_len4(i);
    for (int j = t; j < len; j += blockDim.x)
      Um[off + j] = (i < D && j <= i) ? (float)V[i * LD + j] : 0.0f;
    off += len;
  }
}

template <int DP>
struct FullTile {
  static constexpr int UP = rowoff(DP);
  static constexpr int TC = DP <= 40 ? 8 : 4;  // components per shared-memory tile
};

// FPT frames per thread (each U row loaded from shared memory serves all of them): log joint
// g = logGconst - 0.5 |U (x - mu)|^2 + logW per active component, raw values written
// component-major [Mact][chunk], frame LL by sequential addLog. Block = 128 threads covering
// 128 * FPT frames; frame i of the block's range is thread i % 128, slot i / 128.
template <int DP, int FPT>
__global__ void __launch_bounds__(128) full_ll_kernel(
    const float* __restrict__ X, long long f0, long long nf, int D, int Mact,
    const int* __restrict__ act, const float* __restrict__ mu, const float* __restrict__ U,
    const float* __restrict__ logG, const float* __restrict__ logW, float minLL,
    float* __restrict__ G, long long ldg, float* __restrict__ ll, double* __restrict__ llpart,
    int* __restrict__ flag) {
  constexpr int UP = FullTile<DP>::UP, TC = FullTile<DP>::TC;
  __shared__ __align__(16) float s_u[TC][UP];
  __shared__ __align__(16) float s_mu[TC][DP];
  __shared__ float s_c[TC], s_lw[TC];
  __shared__ double s_red[4];
  long long fi[FPT];
  bool valid[FPT];
  float x[FPT][DP];
#pragma unroll
  for (int p = 0; p < FPT; ++p) {
    fi[p] = (long long)blockIdx.x * (128 * FPT) + p * 128 + threadIdx.x;
    valid[p] = fi[p] < nf;
#pragma unroll
    for (int d = 0; d < DP; ++d) x[p][d] = (valid[p] && d < D) ? X[(size_t)(f0 + fi[p]) * D + d] : 0.0f;
  }
  float maxLL[FPT], sumLL[FPT];
#pragma unroll
  for (int p = 0; p < FPT; ++p) maxLL[p] = sumLL[p] = minLL;
  for (int t0 = 0; t0 < Mact; t0 += TC) {
    const int nt = min(TC, Mact - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < nt * (UP / 4); e += blockDim.x) {
      const int j = e / (UP / 4), q = e - j * (UP / 4);
      reinterpret_cast<float4*>(&s_u[j][0])[q] =
          reinterpret_cast<const float4*>(U + (size_t)act[t0 + j] * UP)[q];
    }
    for (int e = threadIdx.x; e < nt * DP; e += blockDim.x) {
      const int j = e / DP, d = e - j * DP;
      s_mu[j][d] = d < D ? mu[(size_t)act[t0 + j] * D + d] : 0.0f;
    }
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
      const int m = act[t0 + j];
      s_c[j] = logG[m];
      s_lw[j] = logW[m];
    }
    __syncthreads();
    for (int j = 0; j < nt; ++j) {
      float a[FPT][DP];
#pragma unroll
      for (int d = 0; d < DP; ++d) {
        const float m = s_mu[j][d];
#pragma unroll
        for (int p = 0; p < FPT; ++p) a[p][d] = __fsub_rn(x[p][d], m);
      }
      const float4* u4 = reinterpret_cast<const float4*>(&s_u[j][0]);
      float e[FPT];
#pragma unroll
      for (int p = 0; p < FPT; ++p) e[p] = 0.0f;
#pragma unroll
      for (int r = 0; r < DP; ++r) {
        float acc[FPT];
#pragma unroll
        for (int p = 0; p < FPT; ++p) acc[p] = 0.0f;
#pragma unroll
        for (int q = 0; q < row_len4(r) / 4; ++q) {
          const float4 u = u4[rowoff(r) / 4 + q];
#pragma unroll
          for (int p = 0; p < FPT; ++p) {
            acc[p] = __fmaf_rn(u.x, a[p][4 * q + 0], acc[p]);
            acc[p] = __fmaf_rn(u.y, a[p][4 * q + 1], acc[p]);
            acc[p] = __fmaf_rn(u.z, a[p][4 * q + 2], acc[p]);
            acc[p] = __fmaf_rn(u.w, a[p][4 * q + 3], acc[p]);
          }
        }
#pragma unroll
        for (int p = 0; p < FPT; ++p) e[p] = __fmaf_rn(acc[p], acc[p], e[p]);
      }
#pragma unroll
      for (int p = 0; p < FPT; ++p) {
        float s = __fsub_rn(s_c[j], __fmul_rn(0.5f, e[p]));
        if (!isfinite(s)) s = minLL;
        const float g = __fadd_rn(s, s_lw[j]);
        if (G != nullptr && valid[p]) G[(size_t)(t0 + j) * ldg + fi[p]] = g;
        if (maxLL[p] < g) maxLL[p] = g;
        add_log(sumLL[p], g);
      }
    }
  }
  double v = 0.0;
#pragma unroll
  for (int p = 0; p < FPT; ++p) {
    const float l = (maxLL[p] == minLL) ? minLL : sumLL[p];
    if (valid[p]) {
      if (maxLL[p] == minLL) flag[1] = 1;
      ll[f0 + fi[p]] = l;
      v += (double)l;
    }
  }
  v = warp_sum(v);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += s_red[k];
    llpart[blockIdx.x] = t;
  }
}

// Lanes hold at most kMaxEntries packed entries each; wider triangles are split over
// gridDim.z entry groups, each re-deriving the posteriors (group 0 also sums n and F).
constexpr int kMaxEntries = 34;
__host__ __device__ constexpr int lane_rows(int DP) { return (DP * (DP + 1) / 2 + 31) / 32; }
__host__ __device__ constexpr int entry_groups(int DP) { return (lane_rows(DP) + kMaxEntries - 1) / kMaxEntries; }
__host__ __device__ constexpr int entries_per_lane(int DP) {
  return (lane_rows(DP) + entry_groups(DP) - 1) / entry_groups(DP);
}

template <int DP>
__global__ void __launch_bounds__(128) full_stats_kernel(
    const float* __restrict__ X, long long f0, long long nf, int D, int Mact,
    const float* __restrict__ G, long long ldg, const float* __restrict__ ll, float minLL,
    float minGamma, int single_comp, int flags, int slices, long long slice_len,
    double* __restrict__ part) {
  constexpr int PP = DP * (DP + 1) / 2, R = entries_per_lane(DP);
  __shared__ unsigned short s_pair[PP];
  __shared__ float s_x[4][DP];
  const int P = D * (D + 1) / 2;
  for (int e = threadIdx.x; e < P; e += blockDim.x) {
    int k, kk;
    unpack(e, D, k, kk);
    s_pair[e] = (unsigned short)(k << 8 | kk);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x;
  const int s = blockIdx.y * (blockDim.x >> 5) + warp;
  if (s >= slices) return;
  const int grp = blockIdx.z, e0 = grp * R * 32;
  const bool fm = (flags & GMM_ACC_MEAN) != 0 && grp == 0, fv = (flags & GMM_ACC_VAR) != 0;
  const bool probs_only = (flags & GMM_ACC_PROBS_ONLY) != 0;
  const long long a = (long long)s * slice_len;
  const long long b = min(nf, a + slice_len);
  float nh = 0.0f, nl = 0.0f, Fh[2] = {0.0f, 0.0f}, Fl[2] = {0.0f, 0.0f}, Sh[R], Sl[R];
#pragma unroll
  for (int r = 0; r < R; ++r) Sh[r] = Sl[r] = 0.0f;
  const float* Gj = G + (size_t)j * ldg;
  float* xs = s_x[warp];
  for (long long f = a; f < b; f += 32) {
    const long long fi = f + lane;
    float gam = 0.0f;
    bool kept = false;
    if (fi < b) {
      const float g = Gj[fi];
      const float l = ll[f0 + fi];
      if (single_comp) gam = 1.0f;
      else if (l == minLL) gam = minGamma;
      else gam = (float)(g > minLL) * expf(__fsub_rn(g, l));
      kept = gam > minGamma;
    }
    unsigned mask = __ballot_sync(0xffffffffu, kept);
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1u;
      const float gb = __shfl_sync(0xffffffffu, gam, src);
      if (lane == 0) two_sum(nh, nl, gb);
      if (probs_only) continue;
      const float* xr = X + (size_t)(f0 + f + src) * D;
      __syncwarp();
      if (lane < D) xs[lane] = xr[lane];
      if (lane + 32 < D) xs[lane + 32] = xr[lane + 32];
      __syncwarp();
      if (fm) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int d = lane + 32 * q;
          if (d < D) two_sum(Fh[q], Fl[q], __fmul_rn(gb, xs[d]));
        }
      }
      if (fv) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int e = e0 + lane + 32 * r;
          if (e < P) {
            const unsigned pr = s_pair[e];
            two_sum(Sh[r], Sl[r], __fmul_rn(__fmul_rn(gb, xs[pr >> 8]), xs[pr & 255u]));
          }
        }
      }
    }
  }
  const int E = 1 + D + P;
  double* out = part + ((size_t)s * Mact + j) * (size_t)E;
  if (grp == 0) {
    if (lane == 0) out[0] = (double)nh + (double)nl;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int d = lane + 32 * q;
      if (d < D) out[1 + d] = (double)Fh[q] + (double)Fl[q];
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int e = e0 + lane + 32 * r;
    if (e < P) out[1 + D + e] = (double)Sh[r] + (double)Sl[r];
  }
}

// stats[n | F | S] (caller order) += sum over slices of part (fixed order).
__global__ void full_reduce_kernel(int M, int D, int P, int Mact, const int* __restrict__ act,
                                   int slices, const double* __restrict__ part,
                                   double* __restrict__ stats) {
  const int E = 1 + D + P;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)Mact * E) return;
  const int j = (int)(t / E), e = (int)(t - (long long)j * E);
  double s = 0.0;
  for (int k = 0; k < slices; ++k) s += part[((size_t)k * Mact + j) * E + e];
  const int m = act[j];
  size_t dst;
  if (e == 0) dst = (size_t)m;
  else if (e <= D) dst = (size_t)M + (size_t)m * D + (e - 1);
  else dst = (size_t)M + (size_t)M * D + (size_t)m * P + (e - 1 - D);
  stats[dst] += s;
}

__global__ void full_ll_total_kernel(int nblocks, const double* __restrict__ llpart,
                                     double* __restrict__ tot) {
  __shared__ double s_red[32];
  double v = 0.0;
  for (int k = threadIdx.x; k < nblocks; k += blockDim.x) v += llpart[k];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += s_red[k];
    *tot += t;
  }
}

// UpdateModelEM, full branch, one block per component. flag[5] <- weights changed,
// flag[6] <- components that had zero weight before the update.
__global__ void full_em_kernel(int M, int D, int P, float* __restrict__ w, float* __restrict__ mu,
                               float* __restrict__ cov, const double* __restrict__ stats,
                               unsigned int tot, int upW, int upM, int upV, const double* __restrict__ nind,
                               int* __restrict__ flag) {
  __shared__ float s_mean[kFullMaxDim];
  const int j = blockIdx.x, t = threadIdx.x;
  const double* n = stats;
  const double* F = stats + M;
  const double* Sp = stats + M + (size_t)M * D;
  if (w[j] == 0.0f) {
    if (t == 0) atomicAdd(&flag[6], 1);
    return;
  }
  const double mp = n[j];
  float* mj = mu + (size_t)j * D;
  float* C = cov + (size_t)j * D * D;
  if ((nind ? nind[j] : mp) < 2.0) {  // _MIN_IND_SAMPLES_ (robust: on nind): Reset -> mean 0, identity
    for (int e = t; e < D * D; e += blockDim.x) C[e] = (e / D == e % D) ? 1.0f : 0.0f;
    for (int k = t; k < D; k += blockDim.x) mj[k] = 0.0f;
    if (t == 0) {
      w[j] = 0.0f;
      atomicExch(&flag[5], 1);
    }
    return;
  }
  if (upW && t == 0) {
    w[j] = (float)__ddiv_rn(mp, (double)tot);
    atomicExch(&flag[5], 1);
  }
  if (!(upM || upV)) return;
  for (int k = t; k < D; k += blockDim.x) s_mean[k] = (float)__ddiv_rn(F[(size_t)j * D + k], mp);
  __syncthreads();
  if (upV) {
    for (int e = t; e < P; e += blockDim.x) {
      int k, kk;
      unpack(e, D, k, kk);
      const float mm = __fmul_rn(s_mean[k], s_mean[kk]);
      const float v = (float)__dsub_rn(__ddiv_rn(Sp[(size_t)j * P + e], mp), (double)mm);
      C[(size_t)k * D + kk] = v;
      C[(size_t)kk * D + k] = v;
    }
  }
  if (upM)
    for (int k = t; k < D; k += blockDim.x) mj[k] = s_mean[k];
}

__global__ void full_em_norm_kernel(int M, float* __restrict__ w, int* __restrict__ flag) {
  __shared__ double s_corr;
  if (threadIdx.x == 0) {
    double corr = 0.0;
    for (int j = 0; j < M; ++j) corr = __dadd_rn(corr, (double)w[j]);
    s_corr = corr;
    flag[2] = M - flag[6];
  }
  __syncthreads();
  const double corr = s_corr;
  if (flag[5] && corr > 0.0)
    for (int j = threadIdx.x; j < M; j += blockDim.x) w[j] = (float)__ddiv_rn((double)w[j], corr);
}

// UpdateModelMAP with tau > 0, full branch, one block per component.
__global__ void full_map_kernel(int M, int D, int P, float* __restrict__ w, float* __restrict__ mu,
                                float* __restrict__ cov, const float* __restrict__ uw,
                                const float* __restrict__ umu, const float* __restrict__ ucov,
                                const double* __restrict__ stats, unsigned int tot, int tau, int upW,
                                int upM, int upV, float* __restrict__ adapted_w) {
  __shared__ float s_am[kFullMaxDim];
  const int j = blockIdx.x, t = threadIdx.x;
  if (t == 0) adapted_w[j] = 0.0f;
  if (uw[j] == 0.0f) return;
  const double* n = stats;
  const double* F = stats + M;
  const double* Sp = stats + M + (size_t)M * D;
  const double mp = n[j];
  if (!(mp > 0.0)) return;
  const double alfa = __ddiv_rn(mp, __dadd_rn(mp, (double)tau));
  const double one_m = __dsub_rn(1.0, alfa);
  if (upW && tot > 0 && t == 0) {
    const double t1 = __dmul_rn(alfa, __ddiv_rn(mp, (double)tot));
    const float aw = (float)__dadd_rn(t1, __dmul_rn(one_m, (double)uw[j]));
    w[j] = aw;
    adapted_w[j] = aw;
  }
  if (!(upM || upV)) return;
  const float* um = umu + (size_t)j * D;
  const float* uc = ucov + (size_t)j * D * D;
  for (int k = t; k < D; k += blockDim.x) {
    const double a1 = __ddiv_rn(__dmul_rn(alfa, F[(size_t)j * D + k]), mp);
    s_am[k] = (float)__dadd_rn(a1, __dmul_rn(one_m, (double)um[k]));
  }
  __syncthreads();
  if (upV) {
    float* C = cov + (size_t)j * D * D;
    for (int e = t; e < P; e += blockDim.x) {
      int k, kk;
      unpack(e, D, k, kk);
      const float second = __fadd_rn(uc[(size_t)k * D + kk], __fmul_rn(um[k], um[kk]));
      const float msq = __fmul_rn(s_am[k], s_am[kk]);
      const double b1 = __ddiv_rn(__dmul_rn(alfa, Sp[(size_t)j * P + e]), mp);
      const double b2 = __dadd_rn(b1, __dmul_rn(one_m, (double)second));
      const float v = (float)__dsub_rn(b2, (double)msq);
      C[(size_t)k * D + kk] = v;
      C[(size_t)kk * D + k] = v;
    }
  }
  for (int k = t; k < D; k += blockDim.x) mu[(size_t)j * D + k] = s_am[k];
}

__global__ void full_map_norm_kernel(int M, float* __restrict__ w, const float* __restrict__ adapted_w,
                                     const float* __restrict__ uw, const double* __restrict__ stats,
                                     int upW, unsigned int tot) {
  __shared__ double s_corr;
  if (!upW) return;
  if (threadIdx.x == 0) {
    double corr = 0.0;
    for (int j = 0; j < M; ++j)
      if (uw[j] != 0.0f && stats[j] > 0.0 && tot > 0) corr = __dadd_rn(corr, (double)adapted_w[j]);
    s_corr = corr;
  }
  __syncthreads();
  if (s_corr != 0.0) {
    const float fc = (float)s_corr;
    for (int j = threadIdx.x; j < M; j += blockDim.x) w[j] = __fdiv_rn(w[j], fc);
  }
}

// Diagonal of each covariance (GMModel::GetMixtureVarDiag): out [M][D].
__global__ void full_diag_kernel(int M, int D, const float* __restrict__ cov, float* __restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)M * D) return;
  const int m = (int)(t / D), d = (int)(t - (long long)m * D);
  out[t] = cov[((size_t)m * D + d) * D + d];
}

// ------------------------------------------------------------------ host side

void free_full(Ctx* c) {
  FullModel* f = c->full;
  if (!f) return;
  const size_t m1 = sizeof(float) * (size_t)f->M, md = m1 * f->D, mdd = md * f->D;
  dfree(c, f->w, m1); dfree(c, f->mu, md); dfree(c, f->cov, mdd);
  dfree(c, f->U, sizeof(float) * (size_t)f->M * f->UP);
  dfree(c, f->logG, m1); dfree(c, f->logW, m1); dfree(c, f->aw, m1);
  dfree(c, f->act, sizeof(int) * (size_t)f->M);
  dfree(c, f->pw, m1); dfree(c, f->pmu, md); dfree(c, f->pcov, mdd);
  dfree(c, f->stats, sizeof(double) * f->stats_count());
  dfree(c, f->aux, f->aux_cap);
  dfree(c, f->tcB, f->tcB_cap);
  dfree(c, f->tcC, sizeof(float2) * (size_t)f->M);
  *f = FullModel();
}

int ensure_full(Ctx* c, int M, int D) {
  if (!c->full) {
    c->full = new (std::nothrow) FullModel();
    if (!c->full) return fail(c, GMM_ERR_NOMEM, "out of host memory");
  }
  FullModel* f = c->full;
  if (f->w && f->M == M && f->D == D) return GMM_OK;
  free_full(c);
  f->M = M;
  f->D = D;
  f->DP = dp_for(D);
  f->UP = rowoff(f->DP);
  f->P = D * (D + 1) / 2;
  const size_t m1 = sizeof(float) * (size_t)M, md = m1 * D, mdd = md * D;
  int rc = dalloc(c, (void**)&f->w, m1, "full model weights");
  if (!rc) rc = dalloc(c, (void**)&f->mu, md, "full model means");
  if (!rc) rc = dalloc(c, (void**)&f->cov, mdd, "full model covariances");
  if (!rc) rc = dalloc(c, (void**)&f->U, sizeof(float) * (size_t)M * f->UP, "inverse Cholesky factors");
  if (!rc) rc = dalloc(c, (void**)&f->logG, m1, "log constants");
  if (!rc) rc = dalloc(c, (void**)&f->logW, m1, "log weights");
  if (!rc) rc = dalloc(c, (void**)&f->aw, m1, "adapted weights");
  if (!rc) rc = dalloc(c, (void**)&f->act, sizeof(int) * (size_t)M, "active list");
  if (!rc) rc = dalloc(c, (void**)&f->stats, sizeof(double) * f->stats_count(), "full statistics");
  if (rc) {
    free_full(c);
    return rc;
  }
  return GMM_OK;
}

int full_precompute(Ctx* c) {
  FullModel* f = c->full;
  {
    GMM_LAUNCH(c, "full_active_kernel");
    full_active_kernel<<<1, 32, 0, c->stream>>>(f->M, f->w, f->act, c->flag + 4);
  }
  cudaMemsetAsync(c->flag + 7, 0, sizeof(int), c->stream);
  {
    GMM_LAUNCH(c, "full_prepare_kernel");
    const size_t smem = sizeof(double) * 2 * (size_t)f->D * (f->D + 1);
    cudaFuncSetAttribute(full_prepare_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    full_prepare_kernel<<<f->M, 64, smem, c->stream>>>(f->M, f->D, f->DP, f->UP, f->w, f->cov, c->minLL,
                                                       f->U, f->logG, f->logW, c->flag);
  }
  cudaError_t e = cudaMemcpyAsync(c->hflag, c->flag, 8 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpyAsync(flags)");
  int rc = sync(c, "full-covariance model precompute");
  if (rc) return rc;
  f->Mact = c->hflag[4];
  if (c->hflag[7]) {
    cudaMemsetAsync(c->flag + 7, 0, sizeof(int), c->stream);
    return fail(c, GMM_ERR_MODEL, "getCovInverse(): cholesky factorization failed!");
  }
  // operand images of the tensor-core log-likelihood kernel (D <= 63)
  f->tc_ng = 0;
  if (f->D <= 63 && f->Mact > 0) {
    const int KX = (f->D + 1 + 15) / 16 * 16, GC = ft_gc(KX), N = GC * KX;
    const int ng = (f->Mact + GC - 1) / GC;
    const size_t need = sizeof(uint16_t) * (size_t)ng * 3 * N * KX;
    if (need > f->tcB_cap) {
      dfree(c, f->tcB, f->tcB_cap);
      f->tcB = nullptr;
      f->tcB_cap = 0;
      const int rc2 = dalloc(c, (void**)&f->tcB, need, "full-covariance operand images");
      if (rc2) return rc2;
      f->tcB_cap = need;
    }
    if (!c->tc_err) {
      const int rc2 = dalloc(c, (void**)&c->tc_err, sizeof(int), "tc error flag");
      if (rc2) return rc2;
      cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
    }
    if (!f->tcC) {
      const int rc2 = dalloc(c, (void**)&f->tcC, sizeof(float2) * (size_t)f->M, "full-covariance log constants");
      if (rc2) return rc2;
    }
    if (c->sms == 0) {
      int dev;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev);
    }
    GMM_LAUNCH(c, "full_tc_b_kernel");
    const long long tot = (long long)ng * N * KX;
    full_tc_b_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(
        f->Mact, f->D, f->UP, KX, GC, ng, f->act, f->mu, f->U, f->logG, f->logW, f->tcB, f->tcC);
    f->tc_ng = ng;
  }
  f->dirty = false;
  return GMM_OK;
}

// frames per thread of the log-likelihood kernel (register budget: FPT x 2 x DP floats)
constexpr int ll_fpt(int DP) { return DP <= 40 ? 2 : 1; }

template <int DP>
void launch_full_ll(Ctx* c, long long f0, long long nf, float* G, long long ldg, float* llout) {
  FullModel* f = c->full;
  constexpr int FPT = ll_fpt(DP);
  const int blocks = (int)((nf + 128 * FPT - 1) / (128 * FPT));
  GMM_LAUNCH(c, "full_ll_kernel");
  full_ll_kernel<DP, FPT><<<blocks, 128, 0, c->stream>>>(c->X, f0, nf, f->D, f->Mact, f->act, f->mu, f->U,
                                                         f->logG, f->logW, c->minLL, G, ldg, llout,
                                                         c->llpart, c->flag);
}

// Statistics of frames [f0, f0 + nf) from the log joints in c->logits and the LLs in c->ll, for a
// model with D dimensions and Mact active components (full or diagonal).
template <int DP>
void launch_full_stats(Ctx* c, int D, int Mact, long long f0, long long nf, long long ldg, int flags,
                       int slices, long long slice_len) {
  GMM_LAUNCH(c, "full_stats_kernel");
  constexpr int R = entries_per_lane(DP);
  const int P = D * (D + 1) / 2;
  const int groups = (P + 32 * R - 1) / (32 * R);
  dim3 grid(Mact, (slices + 3) / 4, groups);
  full_stats_kernel<DP><<<grid, 128, 0, c->stream>>>(c->X, f0, nf, D, Mact, c->logits, ldg, c->ll, c->minLL,
                                                     c->minGamma, Mact == 1, flags, slices, slice_len, c->part);
}

template <int KX>
int launch_full_tc_ll(Ctx* c, long long f0, long long nf, float* G, long long ldg, float* llout) {
  FullModel* f = c->full;
  using C = FtCfg<KX>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(full_tc_ll_kernel<KX>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    attr = true;
  }
  const long long n_tiles = (nf + 127) / 128;
  const int grid = (int)std::max(1LL, std::min<long long>(n_tiles, c->sms));
  GMM_LAUNCH(c, "full_tc_ll_kernel");
  full_tc_ll_kernel<KX><<<grid, kFtThreads, C::SMEM, c->stream>>>(
      c->X, f0, nf, f->D, f->Mact, f->tcC, f->tcB, f->tc_ng, c->minLL, G, ldg, llout,
      c->llpart, c->flag, c->tc_err);
  return grid;
}

// Launches the log-likelihood kernel for D's width (the tensor-core one for D <= 63); returns its
// block count.
int dispatch_ll(Ctx* c, long long f0, long long nf, float* G, long long ldg, float* llout) {
  if (c->full->tc_ng > 0) {
    switch ((c->full->D + 1 + 15) / 16 * 16) {
      case 16: return launch_full_tc_ll<16>(c, f0, nf, G, ldg, llout);
      case 32: return launch_full_tc_ll<32>(c, f0, nf, G, ldg, llout);
      case 48: return launch_full_tc_ll<48>(c, f0, nf, G, ldg, llout);
      default: return launch_full_tc_ll<64>(c, f0, nf, G, ldg, llout);
    }
  }
  const int DP = c->full->DP;
  switch (DP) {
    case 8: launch_full_ll<8>(c, f0, nf, G, ldg, llout); break;
    case 16: launch_full_ll<16>(c, f0, nf, G, ldg, llout); break;
    case 24: launch_full_ll<24>(c, f0, nf, G, ldg, llout); break;
    case 32: launch_full_ll<32>(c, f0, nf, G, ldg, llout); break;
    case 40: launch_full_ll<40>(c, f0, nf, G, ldg, llout); break;
    case 48: launch_full_ll<48>(c, f0, nf, G, ldg, llout); break;
    default: launch_full_ll<64>(c, f0, nf, G, ldg, llout); break;
  }
  const int fpt = DP <= 40 ? 2 : 1;
  return (int)((nf + 128 * fpt - 1) / (128 * fpt));
}

void dispatch_stats(Ctx* c, int DP, int D, int Mact, long long f0, long long nf, long long ldg, int flags,
                    int slices, long long slice_len) {
  switch (DP) {
    case 8: launch_full_stats<8>(c, D, Mact, f0, nf, ldg, flags, slices, slice_len); break;
    case 16: launch_full_stats<16>(c, D, Mact, f0, nf, ldg, flags, slices, slice_len); break;
    case 24: launch_full_stats<24>(c, D, Mact, f0, nf, ldg, flags, slices, slice_len); break;
    case 32: launch_full_stats<32>(c, D, Mact, f0, nf, ldg, flags, slices, slice_len); break;
    case 40: launch_full_stats<40>(c, D, Mact, f0, nf, ldg, flags, slices, slice_len); break;
    case 48: launch_full_stats<48>(c, D, Mact, f0, nf, ldg, flags, slices, slice_len); break;
    default: launch_full_stats<64>(c, D, Mact, f0, nf, ldg, flags, slices, slice_len); break;
  }
}

// Frame slices of a statistics launch (about 64 warps per SM in total) and the FP64 partials
// buffer they need.
int plan_slices(Ctx* c, int Mact, int E, long long nf, long long* slices_out, long long* slice_len_out) {
  long long slices = 152LL * 64 / Mact;
  if (slices < 1) slices = 1;
  if (slices > nf / 128) slices = nf / 128;
  if (slices < 1) slices = 1;
  slices = (slices + 3) / 4 * 4;
  long long slice_len = (nf + slices - 1) / slices;
  slice_len = (slice_len + 31) / 32 * 32;
  const size_t need = (size_t)slices * Mact * E * sizeof(double);
  if (need > c->part_cap) {
    dfree(c, c->part, c->part_cap);
    c->part = nullptr;
    c->part_cap = 0;
    const int rc = dalloc(c, (void**)&c->part, need, "partial statistics");
    if (rc) return rc;
    c->part_cap = need;
  }
  *slices_out = slices;
  *slice_len_out = slice_len;
  return GMM_OK;
}

// The log-posterior buffer for `chunk` frames of Mact components.
int ensure_logits(Ctx* c, int Mact, long long chunk) {
  const size_t need = (size_t)Mact * (size_t)chunk * sizeof(float);
  if (need <= c->logits_cap) return GMM_OK;
  dfree(c, c->logits, c->logits_cap);
  c->logits = nullptr;
  c->logits_cap = 0;
  const int rc = dalloc(c, (void**)&c->logits, need, "log-posterior buffer");
  if (rc) return rc;
  c->logits_cap = need;
  return GMM_OK;
}

// One E-step over the resident features with the full-covariance model.
int full_estep(Ctx* c, int flags, bool want_stats, float* ll_out_dev) {
  FullModel* f = c->full;
  if (!f || !f->w) return fail(c, GMM_ERR_STATE, "no full-covariance model uploaded");
  if (!c->X) return fail(c, GMM_ERR_STATE, "no features uploaded");
  if (c->Dx != f->D) return fail(c, GMM_ERR_ARG, "Inconsistent model & feature vector - different dimensions");
  if (f->dirty) {
    const int rc = full_precompute(c);
    if (rc) return rc;
  }
  if (f->Mact <= 0) return fail(c, GMM_ERR_STATE, "no component with non-zero weight");
  const long long N = c->N;
  const int D = f->D, E = 1 + D + f->P;
  const size_t budget = (size_t)4 << 30;
  long long chunk = want_stats ? (long long)(budget / ((size_t)f->Mact * sizeof(float))) : N;
  chunk = chunk / 256 * 256;
  if (chunk < 256) chunk = 256;
  if (chunk > N) chunk = N;
  if (want_stats) {
    const int rc = ensure_logits(c, f->Mact, chunk);
    if (rc) return rc;
  }
  float* llbuf = ll_out_dev ? ll_out_dev : c->ll;
  // per-block LL partials: this kernel runs 128-frame blocks (the buffer is sized for 256)
  const size_t need_part = (size_t)((chunk + 127) / 128) + 1;
  if (need_part > c->llpart_cap) {
    const int rc0 = sync(c, "full-covariance E-step");
    if (rc0) return rc0;
    dfree(c, c->llpart, c->llpart_cap * sizeof(double));
    c->llpart = nullptr;
    c->llpart_cap = 0;
    const int rc = dalloc(c, (void**)&c->llpart, need_part * sizeof(double), "log-likelihood partial sums");
    if (rc) return rc;
    c->llpart_cap = need_part;
  }
  for (long long f0 = 0; f0 < N; f0 += chunk) {
    const long long nf = (N - f0 < chunk) ? N - f0 : chunk;
    if ((size_t)((nf + 127) / 128) > c->llpart_cap) return fail(c, GMM_ERR_STATE, "llpart too small");
    const int blocks = dispatch_ll(c, f0, nf, want_stats ? c->logits : nullptr, chunk, llbuf);
    if (!want_stats) continue;
    {
      GMM_LAUNCH(c, "full_ll_total_kernel");
      full_ll_total_kernel<<<1, 1024, 0, c->stream>>>(blocks, c->llpart, f->stats + (size_t)f->M * E);
    }
    long long slices = 0, slice_len = 0;
    const int rc = plan_slices(c, f->Mact, E, nf, &slices, &slice_len);
    if (rc) return rc;
    dispatch_stats(c, f->DP, D, f->Mact, f0, nf, chunk, flags, (int)slices, slice_len);
    {
      GMM_LAUNCH(c, "full_reduce_kernel");
      const long long tot = (long long)f->Mact * E;
      full_reduce_kernel<<<(int)((tot + 255) / 256), 256, 0, c->stream>>>(f->M, D, f->P, f->Mact, f->act,
                                                                          (int)slices, c->part, f->stats);
    }
    if (c->robust && f->aux) {
      const int rc2 = robust_chunk(c, f->M, D, f->Mact, f->act, f0, nf, chunk, f->aux);
      if (rc2) return rc2;
    }
  }
  if (f->tc_ng > 0) {  // surface a bounded-wait expiry of the tensor-core kernel
    int herr = 0;
    cudaMemcpyAsync(&herr, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    const int rc = sync(c, "full-covariance E-step");
    if (rc) return rc;
    if (herr) {
      cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
      return fail(c, GMM_ERR_TIMEOUT, "full-covariance E-step: a bounded device wait expired");
    }
  }
  return GMM_OK;
}

int full_accumulate_device(Ctx* c, int flags) {
  FullModel* f = c->full;
  if (!f || !f->w) return fail(c, GMM_ERR_STATE, "no full-covariance model uploaded");
  cudaError_t e = cudaMemsetAsync(f->stats, 0, sizeof(double) * f->stats_count(), c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemsetAsync(full statistics)");
  f->stats_valid = false;
  f->aux_valid = false;
  if (c->robust) {
    const int rc0 = ensure_aux(c, &f->aux, &f->aux_cap, f->M, f->D);
    if (rc0) return rc0;
  }
  int rc = full_estep(c, flags, true, nullptr);
  if (rc) return rc;
  f->tot_frames = c->N;
  f->acc_flags = flags;
  f->stats_valid = true;
  f->aux_valid = c->robust;
  return sync(c, "full-covariance E-step");
}

int full_read_stats(Ctx* c, double* n, double* F, double* Sp, double* tl, long long* tn) {
  FullModel* f = c->full;
  if (!f || !f->stats_valid) return fail(c, GMM_ERR_STATE, "no statistics accumulated");
  const size_t M = f->M, MD = M * f->D, MP = M * f->P;
  std::vector<double> h(M + MD + MP + 1);
  cudaError_t e = cudaMemcpyAsync(h.data(), f->stats, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpyAsync(full statistics)");
  int rc = sync(c, "read full statistics");
  if (rc) return rc;
  if (n) memcpy(n, h.data(), M * sizeof(double));
  if (F) memcpy(F, h.data() + M, MD * sizeof(double));
  if (Sp) memcpy(Sp, h.data() + M + MD, MP * sizeof(double));
  if (tl) *tl = h[M + MD + MP];
  if (tn) *tn = f->tot_frames;
  return GMM_OK;
}

}  // namespace

int diag_fullstats_estep(Ctx* c, double* stats) {
  if (!c->w) return fail(c, GMM_ERR_STATE, "no model uploaded");
  if (!c->X) return fail(c, GMM_ERR_STATE, "no features uploaded");
  if (c->Dx != c->D) return fail(c, GMM_ERR_ARG, "Inconsistent model & feature vector - different dimensions");
  if (c->D > kFullMaxDim) return fail(c, GMM_ERR_UNSUPPORTED, "full second-order statistics support D <= 64");
  if (c->model_dirty) {
    const int rc = plain_precompute(c);
    if (rc) return rc;
  }
  if (c->Mact <= 0) return fail(c, GMM_ERR_STATE, "no component with non-zero weight");
  const int M = c->M, D = c->D, P = D * (D + 1) / 2, E = 1 + D + P;
  cudaError_t e = cudaMemsetAsync(stats, 0, sizeof(double) * ((size_t)M * E + 2), c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemsetAsync(statistics)");
  const long long N = c->N;
  long long chunk = (long long)(((size_t)4 << 30) / ((size_t)c->Mact * sizeof(float)));
  chunk = chunk / 256 * 256;
  if (chunk < 256) chunk = 256;
  if (chunk > N) chunk = N;
  int rc = ensure_logits(c, c->Mact, chunk);
  if (rc) return rc;
  for (long long f0 = 0; f0 < N; f0 += chunk) {
    const long long nf = (N - f0 < chunk) ? N - f0 : chunk;
    if ((size_t)((nf + 255) / 256) > c->llpart_cap) return fail(c, GMM_ERR_STATE, "llpart too small");
    const int blocks = plain_ll_chunk(c, f0, nf, c->logits, chunk, c->ll);
    {
      GMM_LAUNCH(c, "full_ll_total_kernel");
      full_ll_total_kernel<<<1, 1024, 0, c->stream>>>(blocks, c->llpart, stats + (size_t)M * E);
    }
    long long slices = 0, slice_len = 0;
    rc = plan_slices(c, c->Mact, E, nf, &slices, &slice_len);
    if (rc) return rc;
    dispatch_stats(c, dp_for(D), D, c->Mact, f0, nf, chunk, GMM_ACC_MEAN | GMM_ACC_VAR, (int)slices, slice_len);
    {
      GMM_LAUNCH(c, "full_reduce_kernel");
      const long long tot = (long long)c->Mact * E;
      full_reduce_kernel<<<(int)((tot + 255) / 256), 256, 0, c->stream>>>(M, D, P, c->Mact, c->act, (int)slices,
                                                                          c->part, stats);
    }
  }
  return GMM_OK;
}

int full_fmllr_inputs(Ctx* c, const double** stats, const float** mu, float** diag, int* M, int* D,
                      long long* frames) {
  FullModel* f = c->full;
  if (!f || !f->stats_valid) return fail(c, GMM_ERR_STATE, "no statistics accumulated");
  if (f->M < 1) return fail(c, GMM_ERR_STATE, "no full-covariance model uploaded");
  const int rc = dalloc(c, (void**)diag, sizeof(float) * (size_t)f->M * f->D, "covariance diagonals");
  if (rc) return rc;
  const long long tot = (long long)f->M * f->D;
  full_diag_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(f->M, f->D, f->cov, *diag);
  *stats = f->stats;
  *mu = f->mu;
  *M = f->M;
  *D = f->D;
  *frames = f->tot_frames;
  return GMM_OK;
}

bool full_aux(Ctx* c, const double** aux, int* M, int* D) {
  FullModel* f = c->full;
  if (!f || !f->aux_valid) return false;
  *aux = f->aux;
  *M = f->M;
  *D = f->D;
  return true;
}

void full_destroy(Ctx* c) {
  if (!c->full) return;
  free_full(c);
  delete c->full;
  c->full = nullptr;
}

}  // namespace gmm

using namespace gmm;

extern "C" {

int gmm_upload_model_full(gmm_handle h, int M, int D, const float* w, const float* mu, const float* cov) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!w || !mu || !cov) return fail(c, GMM_ERR_ARG, "gmm_upload_model_full: null array");
  if (M < 1 || M > kMaxMix) return fail(c, GMM_ERR_ARG, "gmm_upload_model_full: M must be in [1, 32767]");
  if (D < 1 || D > kFullMaxDim)
    return fail(c, GMM_ERR_UNSUPPORTED, "gmm_upload_model_full: full covariances support 1 <= D <= 64");
  cudaSetDevice(c->device);
  int rc = ensure_full(c, M, D);
  if (rc) return rc;
  FullModel* f = c->full;
  const size_t md = sizeof(float) * (size_t)M * D;
  cudaMemcpyAsync(f->w, w, sizeof(float) * M, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(f->mu, mu, md, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(f->cov, cov, md * D, cudaMemcpyHostToDevice, c->stream);
  f->stats_valid = false;
  f->dirty = true;
  return full_precompute(c);
}

int gmm_set_prior_full(gmm_handle h, const float* w, const float* mu, const float* cov) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  FullModel* f = c->full;
  if (!f || !f->w) return fail(c, GMM_ERR_STATE, "upload a full-covariance model before its prior");
  const size_t m1 = sizeof(float) * (size_t)f->M, md = m1 * f->D;
  if (!f->pw) {
    int rc = dalloc(c, (void**)&f->pw, m1, "prior weights");
    if (!rc) rc = dalloc(c, (void**)&f->pmu, md, "prior means");
    if (!rc) rc = dalloc(c, (void**)&f->pcov, md * f->D, "prior covariances");
    if (rc) return rc;
  }
  const cudaMemcpyKind k = (w && mu && cov) ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  cudaMemcpyAsync(f->pw, w && mu && cov ? w : f->w, m1, k, c->stream);
  cudaMemcpyAsync(f->pmu, w && mu && cov ? mu : f->mu, md, k, c->stream);
  cudaMemcpyAsync(f->pcov, w && mu && cov ? cov : f->cov, md * f->D, k, c->stream);
  f->have_prior = true;
  return sync(c, "gmm_set_prior_full");
}

int gmm_read_model_full(gmm_handle h, float* w, float* mu, float* cov) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  FullModel* f = c->full;
  if (!f || !f->w) return fail(c, GMM_ERR_STATE, "no full-covariance model uploaded");
  const size_t md = sizeof(float) * (size_t)f->M * f->D;
  if (w) cudaMemcpyAsync(w, f->w, sizeof(float) * f->M, cudaMemcpyDeviceToHost, c->stream);
  if (mu) cudaMemcpyAsync(mu, f->mu, md, cudaMemcpyDeviceToHost, c->stream);
  if (cov) cudaMemcpyAsync(cov, f->cov, md * f->D, cudaMemcpyDeviceToHost, c->stream);
  return sync(c, "gmm_read_model_full");
}

int gmm_accumulate_full_device(gmm_handle h, int flags) {
  if (!h) return GMM_ERR_ARG;
  cudaSetDevice(h->device);
  return full_accumulate_device(h, flags);
}

int gmm_read_stats_full(gmm_handle h, double* n, double* F, double* Sp, double* tl, long long* tn) {
  if (!h) return GMM_ERR_ARG;
  return full_read_stats(h, n, F, Sp, tl, tn);
}

int gmm_accumulate_full(gmm_handle h, int flags, double* n, double* F, double* Sp, double* tl,
                        long long* tn) {
  if (!h) return GMM_ERR_ARG;
  cudaSetDevice(h->device);
  int rc = full_accumulate_device(h, flags);
  if (rc) return rc;
  return full_read_stats(h, n, F, Sp, tl, tn);
}

int gmm_loglikes_full(gmm_handle h, float* out) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!out && c->N > 0) return fail(c, GMM_ERR_ARG, "gmm_loglikes_full: null output");
  cudaSetDevice(c->device);
  int rc = full_estep(c, 0, false, c->ll);
  if (rc) return rc;
  if (c->N > 0) {
    cudaError_t e = cudaMemcpyAsync(out, c->ll, sizeof(float) * (size_t)c->N, cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpyAsync(loglikes)");
  }
  return sync(c, "gmm_loglikes_full");
}

int gmm_em_update_full(gmm_handle h, int upW, int upM, int upV, int* alive) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  FullModel* f = c->full;
  if (!f || !f->stats_valid) return fail(c, GMM_ERR_STATE, "no statistics accumulated");
  cudaSetDevice(c->device);
  double* nind = nullptr;
  if (c->robust && f->aux_valid) {  // UpdateModelEM with _robustCov: MakeRobustStats first
    const int rc0 = robust_make(c, f->M, f->D, 1, f->stats, f->aux, &nind);
    if (rc0) return rc0;
    f->aux_valid = false;
  }
  cudaMemsetAsync(c->flag + 5, 0, 2 * sizeof(int), c->stream);
  const unsigned int tot = (unsigned int)f->tot_frames;
  {
    GMM_LAUNCH(c, "full_em_kernel");
    full_em_kernel<<<f->M, 128, 0, c->stream>>>(f->M, f->D, f->P, f->w, f->mu, f->cov, f->stats, tot, upW,
                                                upM, upV, nind, c->flag);
  }
  {
    GMM_LAUNCH(c, "full_em_norm_kernel");
    full_em_norm_kernel<<<1, 1024, 0, c->stream>>>(f->M, f->w, c->flag);
  }
  f->dirty = true;
  cudaError_t e = cudaMemcpyAsync(c->hflag, c->flag, 8 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpyAsync(flags)");
  int rc = sync(c, "full-covariance EM update");
  if (rc) return rc;
  if (alive) *alive = c->hflag[2];
  return GMM_OK;
}

// MLLR of a full-covariance model: the reference's ComputeKiGi_MLLR / prepareKiGiInitMatrices
// read GetMixtureVarDiag, so the diagonal model's MLLR routines run on the full model's
// occupancies, first-order statistics, means and covariance diagonals (the statistics layout
// [n | F | ...] is the same).
namespace {
struct DiagView {  // the diagonal-model fields of the context, saved while they point at the full model
  int M, D;
  float *mu, *var, *pmu, *pvar;
  bool have_prior, stats_valid, model_dirty;
  double* stats;
  int acc_flags;
  long long tot_frames;
};
DiagView save_view(Ctx* c) {
  return {c->M, c->D, c->mu, c->var, c->pmu, c->pvar, c->have_prior, c->stats_valid, c->model_dirty,
          c->stats, c->acc_flags, c->tot_frames};
}
void restore_view(Ctx* c, const DiagView& v) {
  c->M = v.M; c->D = v.D; c->mu = v.mu; c->var = v.var; c->pmu = v.pmu; c->pvar = v.pvar;
  c->have_prior = v.have_prior; c->stats_valid = v.stats_valid; c->model_dirty = v.model_dirty;
  c->stats = v.stats; c->acc_flags = v.acc_flags; c->tot_frames = v.tot_frames;
}
}  // namespace

int gmm_mllr_estimate_full(gmm_handle h, int ubm_init, double* W) {
  if (!h || !W) return GMM_ERR_ARG;
  Ctx* c = h;
  FullModel* f = c->full;
  if (!f || !f->stats_valid) return fail(c, GMM_ERR_STATE, "no statistics accumulated");
  cudaSetDevice(c->device);
  const size_t md = sizeof(float) * (size_t)f->M * f->D;
  float* dv = nullptr;
  float* dpv = nullptr;
  int rc = dalloc(c, (void**)&dv, md, "covariance diagonals");
  if (!rc && f->have_prior) rc = dalloc(c, (void**)&dpv, md, "prior covariance diagonals");
  if (rc) {
    dfree(c, dv, md);
    return rc;
  }
  const long long tot = (long long)f->M * f->D;
  full_diag_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(f->M, f->D, f->cov, dv);
  if (dpv) full_diag_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(f->M, f->D, f->pcov, dpv);
  const DiagView saved = save_view(c);
  c->M = f->M; c->D = f->D; c->mu = f->mu; c->var = dv; c->pmu = f->pmu; c->pvar = dpv;
  c->have_prior = f->have_prior; c->stats = f->stats; c->stats_valid = true; c->acc_flags = f->acc_flags;
  c->tot_frames = f->tot_frames;
  rc = mstep_mllr(c, ubm_init, W);
  restore_view(c, saved);
  cudaStreamSynchronize(c->stream);
  dfree(c, dv, md);
  dfree(c, dpv, md);
  return rc;
}

int gmm_mllr_apply_full(gmm_handle h, const double* W) {
  if (!h || !W) return GMM_ERR_ARG;
  Ctx* c = h;
  FullModel* f = c->full;
  if (!f || !f->w) return fail(c, GMM_ERR_STATE, "no full-covariance model uploaded");
  cudaSetDevice(c->device);
  const DiagView saved = save_view(c);
  c->M = f->M; c->D = f->D; c->mu = f->mu;
  const int rc = mstep_mllr_apply(c, W);
  restore_view(c, saved);
  f->dirty = true;
  return rc;
}

int gmm_map_update_full(gmm_handle h, int tau, int upW, int upM, int upV) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (tau < 0) return fail(c, GMM_ERR_ARG, "tau must be >= 0");
  if (tau == 0) return gmm_em_update_full(h, upW, upM, upV, nullptr);
  FullModel* f = c->full;
  if (!f || !f->stats_valid) return fail(c, GMM_ERR_STATE, "no statistics accumulated");
  if (!f->have_prior) return fail(c, GMM_ERR_STATE, "MAP needs a prior model (gmm_set_prior_full)");
  cudaSetDevice(c->device);
  if (c->robust && f->aux_valid) {  // UpdateModelMAP with _robustCov: MakeRobustStats first
    double* nind = nullptr;
    const int rc0 = robust_make(c, f->M, f->D, 1, f->stats, f->aux, &nind);
    if (rc0) return rc0;
    f->aux_valid = false;
  }
  const unsigned int tot = (unsigned int)f->tot_frames;
  {
    GMM_LAUNCH(c, "full_map_kernel");
    full_map_kernel<<<f->M, 128, 0, c->stream>>>(f->M, f->D, f->P, f->w, f->mu, f->cov, f->pw, f->pmu, f->pcov,
                                                 f->stats, tot, tau, upW, upM, upV, f->aw);
  }
  {
    GMM_LAUNCH(c, "full_map_norm_kernel");
    full_map_norm_kernel<<<1, 1024, 0, c->stream>>>(f->M, f->w, f->aw, f->pw, f->stats, upW, tot);
  }
  f->dirty = true;
  return sync(c, "full-covariance MAP update");
}

}  // extern "C"
