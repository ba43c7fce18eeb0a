// Tensor-core (tcgen05) form of the G data term of batched global MLLR for sm_103a.
//
// The data terms of ComputeKiGi_MLLR (OL_ModelAdapt.cpp:1525-1581) for every speaker s and row i:
//   G[s][i][t] = sum_m a_i[s][m] * B[m][t],  a_i[s][m] = fl(n[s][m] * fl(1 / var[m][i])),
//   B[m][t] = fl(xi_a * xi_b), t = upper-triangle pair (a, b) of xi_m = [mu_m; 1].
// For each row i this is a GEMM over the components, [S x M] x [M x T]: D of them share B.
// Both FP32 operands are held as three bf16 planes (v = p1 + p2 + p3, each the bf16 rounding of
// what the previous ones left) and the six plane products with i + j <= 2 go to the tensor core,
// so the products carry FP32-level error. The tensor core accumulates 128 components at a time
// in FP32 (TMEM); the epilogue adds those partial sums in FP32 registers with round-to-nearest
// and writes G in FP64 for the solve.
//
// Operand images, K-major without swizzle (the canonical tcgen05 layout): element (row r,
// component m) of a [rows x Mpad] plane sits at ((m / 8) * rows + r) * 8 + m % 8, so the
// components [32 j, 32 j + 32) of a plane are one contiguous block of 4 * rows * 16 bytes and a
// pipeline stage is six cp.async.bulk copies (three planes of the speakers' a_i tile, three of
// the columns' B tile).
//
// mllr_g_kernel: one CTA per (column tile, speaker tile, row i); warp 0 issues the copies into a
// 3-stage ring, warp 1 the MMAs (M = 128 speakers, N = the column tile, K = 16 components, both
// operands from shared memory) into one of two TMEM accumulators per 128 components, warps 2-9
// read the accumulators out (two warps per lane quadrant, each half of the columns). All
// mbarrier waits are bounded; on expiry the kernel raises the error flag, drains its own copies
// and MMAs and frees TMEM.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "gmm_internal.cuh"
#include "tc_ptx.cuh"

namespace gmm {

using namespace ptx;

namespace {

constexpr long long kWait = 4000000000LL;  // clock cycles (~2 s)
constexpr int kKS = 32;                    // components per pipeline stage
constexpr int kStages = 3;
constexpr int kChunkStages = 4;            // stages per accumulator readout (128 components)
constexpr int kThreadsG = 320;             // warp 0 copies, warp 1 MMA, warps 2-9 epilogue
constexpr int kMaxNT = 256;                // column tile (MMA N) at most
constexpr int kEpiChunks = kMaxNT / 16 / 2;  // 16-column chunks per epilogue warp, at most

__device__ __forceinline__ void split3(float v, uint16_t& a, uint16_t& b, uint16_t& c) {
  const __nv_bfloat16 h1 = __float2bfloat16_rn(v);
  float r = v - __bfloat162float(h1);  // exact
  const __nv_bfloat16 h2 = __float2bfloat16_rn(r);
  r = r - __bfloat162float(h2);  // exact
  const __nv_bfloat16 h3 = __float2bfloat16_rn(r);
  a = __bfloat16_as_ushort(h1);
  b = __bfloat16_as_ushort(h2);
  c = __bfloat16_as_ushort(h3);
}

__device__ __forceinline__ void mbar_drain_g(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > kWait) break;
}

// 1 / var as floats, [M][D] (the same rounding as the FP32 GEMM: fl(1 / var)).
__global__ void mllr_rvar_kernel(int M, int D, const float* __restrict__ var, float* __restrict__ rvar) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long long)M * D) rvar[t] = __frcp_rn(var[t]);
}

// a_i planes for every row i and speaker tile: thread = one image element (speaker row r of tile
// st, component m), in image order; it converts n once and writes all D rows' planes.
// A[((i * nS + st) * 3 + p) * Mpad * 128 + image offset].
__global__ void mllr_a_planes_kernel(int S, int M, int Mpad, int D, int nS, const double* __restrict__ n,
                                     const float* __restrict__ rvar, uint16_t* __restrict__ A) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per_tile = (long long)Mpad * 128;
  if (t >= per_tile * nS) return;
  const int st = (int)(t / per_tile);
  const long long e = t - st * per_tile;  // image offset within the plane
  const int m = (int)((e >> 10) * 8 + (e & 7)), r = (int)((e >> 3) & 127);
  const int s = st * 128 + r;
  const bool live = s < S && m < M;
  const float nf = live ? __double2float_rn(n[(size_t)s * M + m]) : 0.0f;
  for (int i = 0; i < D; ++i) {
    uint16_t a, b, c;
    split3(live ? __fmul_rn(nf, rvar[(size_t)m * D + i]) : 0.0f, a, b, c);
    uint16_t* base = A + (size_t)((long long)i * nS + st) * 3 * per_tile + e;
    base[0] = a;
    base[per_tile] = b;
    base[2 * per_tile] = c;
  }
}

// B planes per column tile: B[(tt * 3 + p) * Mpad * NT + image offset], t = tt NT + row.
__global__ void mllr_b_planes_kernel(int M, int Mpad, int D, int T, int NT, int nT, const float* __restrict__ mu,
                                     uint16_t* __restrict__ B) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per_tile = (long long)Mpad * NT;
  if (t >= per_tile * nT) return;
  const int tt = (int)(t / per_tile);
  const long long e = t - tt * per_tile;
  const long long kc = e / (8LL * NT);
  const int r = (int)((e / 8) % NT), m = (int)(kc * 8 + (e & 7));
  const int col = tt * NT + r;
  float v = 0.0f;
  if (m < M && col < T) {
    const int E = D + 1;
    int x = col, a = 0;
    while (x >= E - a) {
      x -= E - a;
      ++a;
    }
    const int b = a + x;
    const float xa = a < D ? mu[(size_t)m * D + a] : 1.0f, xb = b < D ? mu[(size_t)m * D + b] : 1.0f;
    v = (float)((double)xa * (double)xb);
  }
  uint16_t p1, p2, p3;
  split3(v, p1, p2, p3);
  uint16_t* base = B + (size_t)tt * 3 * per_tile + e;
  base[0] = p1;
  base[per_tile] = p2;
  base[2 * per_tile] = p3;
}

// Plane products (a plane, B plane) with i + j <= 2, small terms first.
__device__ __forceinline__ int g_pa(int pr) { return pr == 0 ? 2 : (pr == 1 || pr == 3) ? 1 : 0; }
__device__ __forceinline__ int g_pb(int pr) { return pr == 2 ? 2 : (pr == 1 || pr == 4) ? 1 : 0; }

__global__ void __launch_bounds__(kThreadsG, 1)
    mllr_g_kernel(int S, int D, int T, int Mpad, int nS, int NT, const uint16_t* __restrict__ Aimg,
                  const uint16_t* __restrict__ Bimg, double* __restrict__ G, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int A_P = kKS / 8 * 128 * 16, B_P = kKS / 8 * NT * 16;  // bytes of one plane per stage
  const int STAGE = 3 * (A_P + B_P);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * STAGE);
  uint64_t* z_full = bars;                // [kStages]
  uint64_t* z_empty = bars + kStages;     // [kStages]
  uint64_t* d_full = bars + 2 * kStages;  // [2]
  uint64_t* d_empty = d_full + 2;         // [2]
  uint64_t* mma_done = d_empty + 2;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(mma_done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 2);

  const int tt = blockIdx.x, st = blockIdx.y, i = blockIdx.z;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nst = Mpad / kKS, nch = (nst + kChunkStages - 1) / kChunkStages;
  const long long a_plane = (long long)Mpad * 128, b_plane = (long long)Mpad * NT;
  const uint16_t* a_img = Aimg + (size_t)((long long)i * nS + st) * 3 * a_plane;
  const uint16_t* b_img = Bimg + (size_t)tt * 3 * b_plane;

  if (threadIdx.x == 0) {
    for (int j = 0; j < kStages; ++j) {
      mbar_init(&z_full[j], 1);
      mbar_init(&z_empty[j], 1);
    }
    for (int j = 0; j < 2; ++j) {
      mbar_init(&d_full[j], 1);
      mbar_init(&d_empty[j], 8);
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
  int issued = 0;  // stage copies issued (loader thread)

  if (warp == 0) {
    if (lane == 0) {
      for (int j = 0; j < nst; ++j) {
        const int sg = j % kStages;
        if (!mbar_wait(&z_empty[sg], ((j / kStages) & 1) ^ 1, abort_flag, kWait)) break;
        mbar_arrive_expect_tx(&z_full[sg], STAGE);
        uint8_t* dst = smem + sg * STAGE;
        const size_t off_a = (size_t)j * (kKS / 8) * 128 * 8, off_b = (size_t)j * (kKS / 8) * NT * 8;
        for (int p = 0; p < 3; ++p) bulk_load(dst + p * A_P, a_img + p * a_plane + off_a, A_P, &z_full[sg]);
        for (int p = 0; p < 3; ++p) bulk_load(dst + 3 * A_P + p * B_P, b_img + p * b_plane + off_b, B_P, &z_full[sg]);
        issued = j + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16(128, NT, false, false);
      const uint32_t sb = smem_u32(smem);
      bool ok = true;
      for (int c = 0; c < nch && ok; ++c) {
        const int b = c & 1;
        if (c >= 2 && !mbar_wait(&d_empty[b], ((c - 2) >> 1) & 1, abort_flag, kWait)) break;
        const uint32_t d = tmem + (uint32_t)(b * NT);
        const int j1 = min(nst, (c + 1) * kChunkStages);
        for (int j = c * kChunkStages; j < j1; ++j) {
          const int sg = j % kStages;
          if (!mbar_wait(&z_full[sg], (j / kStages) & 1, abort_flag, kWait)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t base = sb + sg * STAGE;
#pragma unroll
          for (int q = 0; q < kKS / 16; ++q) {
#pragma unroll
            for (int pr = 0; pr < 6; ++pr) {
              const uint64_t ad = smem_desc(base + g_pa(pr) * A_P + q * 2 * 128 * 16, 128 * 16, 128);
              const uint64_t bd = smem_desc(base + 3 * A_P + g_pb(pr) * B_P + q * 2 * NT * 16, NT * 16, 128);
              mma_ss(d, ad, bd, idesc, (j > c * kChunkStages || q > 0 || pr > 0) ? 1u : 0u);
            }
          }
          mma_commit(&z_empty[sg]);
        }
        if (ok) mma_commit(&d_full[b]);
      }
      mma_commit(mma_done);
      mbar_drain_g(mma_done, 0);
    }
  } else {
    // epilogue: thread = speaker row; the two warps of a lane quadrant split the column chunks
    const int q4 = warp & 3, hf = (warp - 2) >> 2;
    const int row = q4 * 32 + lane;
    const uint32_t lane_off = (uint32_t)(q4 * 32) << 16;
    const int nc16 = NT / 16, half = (nc16 + 1) / 2;
    const int c0 = hf ? half : 0, c1 = hf ? nc16 : half;
    float acc[kEpiChunks * 16];
#pragma unroll
    for (int k = 0; k < kEpiChunks * 16; ++k) acc[k] = 0.0f;
    bool ok = true;
    for (int c = 0; c < nch; ++c) {
      const int b = c & 1;
      if (!mbar_wait(&d_full[b], (c >> 1) & 1, abort_flag, kWait)) {
        ok = false;
        break;
      }
      tc_fence_after();
#pragma unroll
      for (int g = 0; g < kEpiChunks; ++g) {
        if (c0 + g < c1) {
          uint32_t r[16];
          tmem_ld16(tmem + lane_off + (uint32_t)(b * NT + 16 * (c0 + g)), r);
          tmem_ld_wait();
#pragma unroll
          for (int k = 0; k < 16; ++k) acc[g * 16 + k] = __fadd_rn(acc[g * 16 + k], __uint_as_float(r[k]));
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&d_empty[b]);
    }
    const int s = st * 128 + row;
    if (ok && !*abort_flag && s < S) {
      double* out = G + ((size_t)s * D + i) * T;
#pragma unroll
      for (int cc = 0; cc < kEpiChunks; ++cc)
        if (c0 + cc < c1) {
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int t = tt * NT + 16 * (c0 + cc) + k;  // column of G
            if (t < T) out[t] = (double)acc[cc * 16 + k];
          }
        }
    }
  }
  __syncthreads();
  if (*abort_flag) {
    // Every role has stopped. The loader's last kStages copies may still be in flight (a
    // consumer that gave up never waited for them): let them land before the CTA's shared
    // memory goes.
    if (warp == 0 && lane == 0)
      for (int j = max(0, issued - kStages); j < issued; ++j) mbar_drain_g(&z_full[j % kStages], (j / kStages) & 1);
    if (threadIdx.x == 0) atomicExch(err, 1);
  }
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

}  // namespace

// Column tiling of the T = (D+1)(D+2)/2 upper-triangle pairs: nT tiles of NT (a multiple of 16,
// at most 256) columns.
static void g_tiling(int D, int* nT, int* NT) {
  const int E = D + 1, T = E * (E + 1) / 2;
  *nT = (T + kMaxNT - 1) / kMaxNT;
  *NT = ((T + *nT - 1) / *nT + 15) / 16 * 16;
}

int tc_mllr_g(Ctx* c, int S, const double* d_n, double* d_G) {
  const int M = c->M, D = c->D, E = D + 1, T = E * (E + 1) / 2;
  const int Mpad = (M + kKS - 1) / kKS * kKS, nS = (S + 127) / 128;
  int nT, NT;
  g_tiling(D, &nT, &NT);
  if (!c->tc_err) {
    int rc = dalloc(c, (void**)&c->tc_err, sizeof(int), "tc error flag");
    if (rc) return rc;
    cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
  }
  const size_t a_bytes = sizeof(uint16_t) * (size_t)D * nS * 3 * Mpad * 128;
  const size_t b_bytes = sizeof(uint16_t) * (size_t)nT * 3 * Mpad * NT;
  uint16_t *A = nullptr, *B = nullptr;
  float* rvar = nullptr;
  int rc = scratch(c, SC_MLLR_AIMG, a_bytes, "MLLR a planes", (void**)&A);
  if (!rc) rc = scratch(c, SC_MLLR_BIMG, b_bytes, "MLLR B planes", (void**)&B);
  if (!rc) rc = scratch(c, SC_MLLR_RVAR, sizeof(float) * (size_t)M * D, "MLLR 1/var", (void**)&rvar);
  if (rc) return rc;
  {
    GMM_LAUNCH(c, "mllr_rvar_kernel");
    mllr_rvar_kernel<<<(unsigned)(((long long)M * D + 255) / 256), 256, 0, c->stream>>>(M, D, c->var, rvar);
  }
  {
    GMM_LAUNCH(c, "mllr_a_planes_kernel");
    const long long tot = (long long)nS * 128 * Mpad;
    mllr_a_planes_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(S, M, Mpad, D, nS, d_n, rvar, A);
  }
  {
    GMM_LAUNCH(c, "mllr_b_planes_kernel");
    const long long tot = (long long)nT * Mpad * NT;
    mllr_b_planes_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(M, Mpad, D, T, NT, nT, c->mu, B);
  }
  const int stage = 3 * (kKS / 8 * 128 * 16 + kKS / 8 * NT * 16);
  const int smem = kStages * stage + 16 * 8 + 64 + 1024;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(mllr_g_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    attr_set = true;
  }
  {
    GMM_LAUNCH(c, "mllr_g_kernel");
    mllr_g_kernel<<<dim3(nT, nS, D), kThreadsG, smem, c->stream>>>(S, D, T, Mpad, nS, NT, A, B, d_G, c->tc_err);
  }
  return GMM_OK;
}

}  // namespace gmm
