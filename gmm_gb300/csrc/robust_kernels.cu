// --robust statistics on the device: the auxiliary statistics of consecutive frames and the
// MakeRobustStats correction of the second-order statistics before an EM / MAP update.
//
// Semantics (GMM/lib_bmssr):
//   accumulateAuxStats, no-pruning branch   trainer/OL_GMMStatsEstimator.cpp:1253-1286, called
//       for every frame i >= 1 of the block (:1175-1188, one thread): with the float posteriors p
//       of frames i and i-1, gs = 1 / (float sum over active m of p_i,m p_i-1,m where > minGamma);
//       aux2_m += sqrt(p_i,m) when p_i,m > minGamma; for g = (gs p_i,m) p_i-1,m > minGamma:
//       aux_m[k] += g |x_i,k - x_i-1,k| (float products, double sums) and aux3_m += g
//   GetNIndFrames / MakeRobustStats           trainer/OL_ModelAdapt.cpp:468-588: global mean and
//       standard deviation from the statistics, the per-component count of independent frames
//       nind = 1 + (aux2 Nglob / sum aux2 - 1) (mean_d(aux_d / aux3 / std_d) / 1.12)^3, and the
//       second-order statistics pulled toward the squared means with float multipliers
//       dc(nind) (diagonal) and odc(nind) (off-diagonal); UpdateModelEM kills on nind < 2
//
// The posteriors come from the raw log joints [Mact][chunk] and frame LLs of the plain E-step
// (diagonal or full-covariance), so robust E-steps always run on the plain kernels. Pairs that
// straddle two chunks of an E-step use the previous chunk's last posteriors (carried in
// c->gprev); the first frame of the resident block has no predecessor.
#include <math.h>

#include "gmm_internal.cuh"

namespace gmm {
namespace {

__device__ __forceinline__ float posterior(float g, float l, float minLL, float minGamma, int single) {
  if (single) return 1.0f;
  if (l == minLL) return minGamma;
  return (float)(g > minLL) * expf(__fsub_rn(g, l));
}

// gs of every frame of the chunk (thread per frame, sequential float sum in component order).
__global__ void robust_gs_kernel(long long f0, long long nf, int Mact, const float* __restrict__ G, long long ldg,
                                 const float* __restrict__ ll, const float* __restrict__ gprev, float minLL,
                                 float minGamma, int single, float* __restrict__ gs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nf) return;
  if (f0 + i == 0) {
    gs[i] = 0.0f;
    return;
  }
  const float lc = ll[f0 + i];
  const float lp = i > 0 ? ll[f0 + i - 1] : 0.0f;
  float s = 0.0f;
  for (int j = 0; j < Mact; ++j) {
    const float pc = posterior(G[(size_t)j * ldg + i], lc, minLL, minGamma, single);
    const float pp = i > 0 ? posterior(G[(size_t)j * ldg + i - 1], lp, minLL, minGamma, single) : gprev[j];
    const float g = __fmul_rn(pc, pp);
    if (g > minGamma) s = __fadd_rn(s, g);
  }
  gs[i] = s > 0.0f ? __fdiv_rn(1.0f, s) : s;
}

// One warp per (active component j, frame slice s): aux [D], aux2, aux3 partial sums in FP64.
template <int DW>
__global__ void __launch_bounds__(128) robust_aux_kernel(
    const float* __restrict__ X, long long f0, long long nf, int D, int Mact, const float* __restrict__ G,
    long long ldg, const float* __restrict__ ll, const float* __restrict__ gprev, const float* __restrict__ gs,
    float minLL, float minGamma, int single, int slices, long long slice_len, double* __restrict__ part) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x;
  const int s = blockIdx.y * (blockDim.x >> 5) + warp;
  if (s >= slices) return;
  const long long a = (long long)s * slice_len;
  const long long b = min(nf, a + slice_len);
  double aux[DW], a2 = 0.0, a3 = 0.0;
#pragma unroll
  for (int q = 0; q < DW; ++q) aux[q] = 0.0;
  const float* Gj = G + (size_t)j * ldg;
  for (long long f = a; f < b; f += 32) {
    const long long fi = f + lane;
    float g = 0.0f;
    bool kept = false;
    if (fi < b && f0 + fi > 0) {
      const float pc = posterior(Gj[fi], ll[f0 + fi], minLL, minGamma, single);
      const float pp = fi > 0 ? posterior(Gj[fi - 1], ll[f0 + fi - 1], minLL, minGamma, single) : gprev[j];
      if (pc > minGamma) a2 += sqrt((double)pc);
      g = __fmul_rn(__fmul_rn(gs[fi], pc), pp);
      kept = g > minGamma;
      if (kept) a3 += (double)g;
    }
    unsigned mask = __ballot_sync(0xffffffffu, kept);
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1u;
      const float gb = __shfl_sync(0xffffffffu, g, src);
      const float* xc = X + (size_t)(f0 + f + src) * D;
      const float* xp = xc - D;
#pragma unroll
      for (int q = 0; q < DW; ++q) {
        const int d = lane + 32 * q;
        if (d < D) aux[q] += (double)__fmul_rn(gb, fabsf(__fsub_rn(xc[d], xp[d])));
      }
    }
  }
  for (int o = 16; o; o >>= 1) {
    a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    a3 += __shfl_xor_sync(0xffffffffu, a3, o);
  }
  double* out = part + ((size_t)s * Mact + j) * (size_t)(D + 2);
#pragma unroll
  for (int q = 0; q < DW; ++q) {
    const int d = lane + 32 * q;
    if (d < D) out[d] = aux[q];
  }
  if (lane == 0) {
    out[D] = a2;
    out[D + 1] = a3;
  }
}

// aux (caller order: aux [M][D] | aux2 [M] | aux3 [M]) += sum over slices of part.
__global__ void robust_reduce_kernel(int M, int D, int Mact, const int* __restrict__ act, int slices,
                                     const double* __restrict__ part, double* __restrict__ aux) {
  const int E = D + 2;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)Mact * E) return;
  const int j = (int)(t / E), e = (int)(t - (long long)j * E);
  double s = 0.0;
  for (int k = 0; k < slices; ++k) s += part[((size_t)k * Mact + j) * E + e];
  const int m = act[j];
  if (e < D) aux[(size_t)m * D + e] += s;
  else if (e == D) aux[(size_t)M * D + m] += s;
  else aux[(size_t)M * D + M + m] += s;
}

// Posteriors of the chunk's last frame, for the first pair of the next chunk.
__global__ void robust_carry_kernel(long long f0, long long nf, int Mact, const float* __restrict__ G, long long ldg,
                                    const float* __restrict__ ll, float minLL, float minGamma, int single,
                                    float* __restrict__ gprev) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= Mact || nf <= 0) return;
  gprev[j] = posterior(G[(size_t)j * ldg + nf - 1], ll[f0 + nf - 1], minLL, minGamma, single);
}

__device__ __forceinline__ float diag_mult(double nind) {
  if (nind < 2) return (float)pow(pow((1.0 + (1.0 / (2.0 - 1.25))), 3.5), (3 - nind));
  return (float)pow((1.0 + (1.0 / (nind - 1.25))), 3.5);
}

__device__ __forceinline__ float offdiag_mult(double nind, int D) {
  if (nind < 2) return 0.0f;
  return (float)(1 - pow(((double)D / (D - 1 + nind)), 1.4));
}

// GetNIndFrames + MakeRobustStats (one block): stats = [n (M) | F (M x D) | S (M x V)], V = D
// (diagonal) or D(D+1)/2 (full, packed). S is modified in place; nind out; *status = 1 when a
// global standard deviation is zero.
__global__ void robust_make_kernel(int M, int D, int full, double* __restrict__ stats, const double* __restrict__ aux,
                                   double* __restrict__ nind, int* __restrict__ status) {
  extern __shared__ double sh[];
  double* gmean = sh;      // D
  double* gstd = sh + D;   // D
  __shared__ double s_gmp, s_sumNg;
  __shared__ int s_bad;
  const int V = full ? D * (D + 1) / 2 : D;
  const double* n = stats;
  const double* F = stats + M;
  double* S = stats + M + (size_t)M * D;
  const double* a1 = aux;
  const double* a2 = aux + (size_t)M * D;
  const double* a3 = a2 + M;
  const int t = threadIdx.x;
  if (t == 0) {
    double gmp = 0.0, sng = 0.0;
    for (int m = 0; m < M; ++m) {
      gmp = __dadd_rn(gmp, n[m]);
      sng = __dadd_rn(sng, a2[m]);
    }
    s_gmp = gmp;
    s_sumNg = sng;
    s_bad = 0;
  }
  for (int d = t; d < D; d += blockDim.x) {
    double gm = 0.0, gs = 0.0;
    const int dd = full ? d * D + d - d * (d + 1) / 2 : d;  // the packed diagonal entry
    for (int m = 0; m < M; ++m) {
      gm = __dadd_rn(gm, F[(size_t)m * D + d]);
      gs = __dadd_rn(gs, S[(size_t)m * V + dd]);
    }
    gmean[d] = gm;
    gstd[d] = gs;
  }
  __syncthreads();
  const double gmp = s_gmp;
  for (int d = t; d < D; d += blockDim.x) {
    gmean[d] = __ddiv_rn(gmean[d], gmp);
    gstd[d] = sqrt(__dsub_rn(__ddiv_rn(gstd[d], gmp), __dmul_rn(gmean[d], gmean[d])));
    if (gstd[d] == 0.0) s_bad = 1;
  }
  __syncthreads();
  if (s_bad) {
    if (t == 0) *status = 1;
    return;
  }
  for (int m = t; m < M; m += blockDim.x) {
    double v = 0.0;
    if (!(n[m] == 0.0 || a3[m] == 0.0)) {
      for (int d = 0; d < D; ++d) v = __dadd_rn(v, __ddiv_rn(__ddiv_rn(a1[(size_t)m * D + d], a3[m]), gstd[d]));
      v = __ddiv_rn(v, (double)D);
      v = pow(__ddiv_rn(v, 1.12), 3.0);
      v = __dadd_rn(1.0, __dmul_rn(__dsub_rn(__ddiv_rn(__dmul_rn(a2[m], gmp), s_sumNg), 1.0), v));
    }
    nind[m] = v;
  }
  __syncthreads();
  for (long long e = t; e < (long long)M * V; e += blockDim.x) {
    const int m = (int)(e / V), q = (int)(e - (long long)m * V);
    float dc = diag_mult(nind[m]);
    dc = (float)((double)dc * __ddiv_rn(nind[m], __dsub_rn(nind[m], 1.0)));
    const double* Fm = F + (size_t)m * D;
    double& x = S[(size_t)m * V + q];
    const double nm = n[m];
    if (!full) {
      x = __dadd_rn(__dmul_rn((double)dc, x), __ddiv_rn(__dmul_rn((double)(1.0f - dc), pow(Fm[q], 2.0)), nm));
    } else {
      int k = 0, rem = q;
      while (rem >= D - k) {
        rem -= D - k;
        ++k;
      }
      const int kk = k + rem;
      if (k == kk) {
        x = __dadd_rn(__dmul_rn((double)dc, x), __ddiv_rn(__dmul_rn((double)(1.0f - dc), pow(Fm[k], 2.0)), nm));
      } else {
        const float odc = offdiag_mult(nind[m], D);
        x = __dadd_rn(__dmul_rn((double)odc, x),
                      __ddiv_rn(__dmul_rn(__dmul_rn((double)(1.0f - odc), Fm[k]), Fm[kk]), nm));
      }
    }
  }
}

}  // namespace

int robust_chunk(Ctx* c, int M, int D, int Mact, const int* act, long long f0, long long nf, long long ldg,
                 double* aux) {
  if (nf <= 0) return GMM_OK;
  if ((size_t)nf > c->gs_cap) {
    dfree(c, c->gs, c->gs_cap * sizeof(float));
    c->gs = nullptr;
    c->gs_cap = 0;
    const int rc = dalloc(c, (void**)&c->gs, sizeof(float) * (size_t)nf, "robust gs");
    if (rc) return rc;
    c->gs_cap = (size_t)nf;
  }
  if ((size_t)Mact > c->gprev_cap) {
    dfree(c, c->gprev, c->gprev_cap * sizeof(float));
    c->gprev = nullptr;
    c->gprev_cap = 0;
    const int rc = dalloc(c, (void**)&c->gprev, sizeof(float) * (size_t)Mact, "robust previous posteriors");
    if (rc) return rc;
    c->gprev_cap = (size_t)Mact;
  }
  const int single = Mact == 1;
  {
    GMM_LAUNCH(c, "robust_gs_kernel");
    robust_gs_kernel<<<(unsigned)((nf + 127) / 128), 128, 0, c->stream>>>(f0, nf, Mact, c->logits, ldg, c->ll,
                                                                        c->gprev, c->minLL, c->minGamma, single,
                                                                        c->gs);
  }
  long long slices = 152LL * 64 / Mact;
  if (slices > nf / 256) slices = nf / 256;
  if (slices < 1) slices = 1;
  slices = (slices + 3) / 4 * 4;
  long long slice_len = (nf + slices - 1) / slices;
  slice_len = (slice_len + 31) / 32 * 32;
  const size_t need = (size_t)slices * Mact * (D + 2) * sizeof(double);
  if (need > c->part_cap) {
    dfree(c, c->part, c->part_cap);
    c->part = nullptr;
    c->part_cap = 0;
    const int rc = dalloc(c, (void**)&c->part, need, "partial statistics");
    if (rc) return rc;
    c->part_cap = need;
  }
  {
    GMM_LAUNCH(c, "robust_aux_kernel");
    dim3 grid(Mact, (unsigned)((slices + 3) / 4));
    const int DW = (D + 31) / 32;
#define GMM_ROBUST_AUX(W)                                                                                    \
  robust_aux_kernel<W><<<grid, 128, 0, c->stream>>>(c->X, f0, nf, D, Mact, c->logits, ldg, c->ll, c->gprev, \
                                                    c->gs, c->minLL, c->minGamma, single, (int)slices,      \
                                                    slice_len, c->part)
    if (DW <= 1) GMM_ROBUST_AUX(1);
    else if (DW <= 2) GMM_ROBUST_AUX(2);
    else if (DW <= 4) GMM_ROBUST_AUX(4);
    else if (DW <= 8) GMM_ROBUST_AUX(8);
    else if (DW <= 16) GMM_ROBUST_AUX(16);
    else GMM_ROBUST_AUX(32);
#undef GMM_ROBUST_AUX
  }
  {
    GMM_LAUNCH(c, "robust_reduce_kernel");
    const long long tot = (long long)Mact * (D + 2);
    robust_reduce_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(M, D, Mact, act, (int)slices, c->part,
                                                                              aux);
  }
  {
    GMM_LAUNCH(c, "robust_carry_kernel");
    robust_carry_kernel<<<(Mact + 127) / 128, 128, 0, c->stream>>>(f0, nf, Mact, c->logits, ldg, c->ll, c->minLL,
                                                                   c->minGamma, single, c->gprev);
  }
  return GMM_OK;
}

// The auxiliary-statistics buffer [M x D | M | M], zeroed.
int ensure_aux(Ctx* c, double** aux, size_t* cap, int M, int D) {
  const size_t need = sizeof(double) * (size_t)M * (D + 2);
  if (need > *cap) {
    dfree(c, *aux, *cap);
    *aux = nullptr;
    *cap = 0;
    const int rc = dalloc(c, (void**)aux, need, "auxiliary statistics");
    if (rc) return rc;
    *cap = need;
  }
  const cudaError_t e = cudaMemsetAsync(*aux, 0, need, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemsetAsync(auxiliary statistics)");
  return GMM_OK;
}

int robust_make(Ctx* c, int M, int D, int full, double* stats, const double* aux, double** nind) {
  if ((size_t)M > c->nind_cap) {
    dfree(c, c->nind, c->nind_cap * sizeof(double));
    c->nind = nullptr;
    c->nind_cap = 0;
    const int rc = dalloc(c, (void**)&c->nind, sizeof(double) * (size_t)M, "independent frame counts");
    if (rc) return rc;
    c->nind_cap = (size_t)M;
  }
  cudaMemsetAsync(c->flag + 9, 0, sizeof(int), c->stream);
  {
    GMM_LAUNCH(c, "robust_make_kernel");
    robust_make_kernel<<<1, 256, sizeof(double) * 2 * D, c->stream>>>(M, D, full, stats, aux, c->nind, c->flag + 9);
  }
  int bad = 0;
  cudaMemcpyAsync(&bad, c->flag + 9, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  const int rc = sync(c, "robust statistics");
  if (rc) return rc;
  if (bad) return fail(c, GMM_ERR_STATE, "GetNIndFrames(): global variance equal zero!");
  *nind = c->nind;
  return GMM_OK;
}

}  // namespace gmm

extern "C" int gmm_set_robust(gmm_handle h, int on) {
  if (!h) return GMM_ERR_ARG;
  h->robust = on != 0;
  h->aux_valid = false;
  return GMM_OK;
}
