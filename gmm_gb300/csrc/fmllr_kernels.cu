// fMLLR (feature-space MLLR, one regression class) of the resident diagonal model on the device.
//
// Semantics (GMM/lib_bmssr/trainer/OL_ModelAdapt.cpp):
//   ComputeW_fMLLR     :1614-1719  E-step with full second-order statistics of the diagonal
//                                  model (AccumulateStats(..., varFull)), CheckInvertibility, per
//                                  row i G_i and k_i, G_i^-1 (MATRIX::Invert, pivot-free
//                                  Gauss-Jordan), then _iter_fMLLR passes over the rows from
//                                  A = I, b = 0 with the cofactors of A taken at the start of a pass
//   ComputeKiGi_fMLLR  :1794-1848  G_i = sum_m (1/var_mi) [S_m F_m; F_m^T n_m],
//                                  k_i = sum_m (mu_mi/var_mi) [F_m; n_m] (float quotients, double
//                                  sums in component order)
//   EstimateAb_fmllr   :1721-1792  row update: the quadratic beta f^2 - (c G^-1 k) f - c G^-1 c = 0
//                                  (c = the row's cofactors, beta = the frame count as a float),
//                                  w = G^-1 (c / f + k) for both roots, the root with the larger
//                                  w (k - G w / 2) wins
// Every FP64 operation is written with an explicit round-to-nearest intrinsic (no fused
// multiply-add), in the reference's loop orders, so the transform from given statistics is
// bit-identical to the reference's (tested against the oracle port of these routines).
//
// Kernels: the E-step is the plain diagonal log-likelihood kernel + the packed full-statistics
// kernel (full_kernels.cu); fmllr_gk_kernel (one thread per G / k entry, a loop over components),
// fmllr_ginv_kernel (one block per row, Gauss-Jordan in shared memory), fmllr_rows_kernel (one
// block, the passes over the rows; statuses through a device word).
#include <math.h>

#include <vector>

#include "gmm_internal.cuh"

namespace gmm {
namespace {

// In-place pivot-free Gauss-Jordan inverse of the n x n row-major matrix a (shared memory), by
// the whole block; each pivot step updates the other entries, then the pivot row and column,
// then the pivot (the reference's MATRIX::_Invert_Gen order, element by element).
__device__ void gj_invert_block(double* a, int n) {
  for (int k = 0; k < n; ++k) {
    const double akk = a[k * n + k];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e / n, j = e - i * n;
      if (i != k && j != k) a[e] = __dsub_rn(a[e], __ddiv_rn(__dmul_rn(a[k * n + j], a[i * n + k]), akk));
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      if (t != k) {
        a[k * n + t] = __ddiv_rn(-a[k * n + t], akk);
        a[t * n + k] = __ddiv_rn(a[t * n + k], akk);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) a[k * n + k] = __ddiv_rn(1.0, akk);
    __syncthreads();
  }
}

// G_i (E x E, both halves) and k_i (E) for every row i; one thread per (i, entry). Entries
// 0 .. E(E+1)/2 - 1 are the upper triangle of G_i in row order, then E entries of k_i.
__global__ void fmllr_gk_kernel(int M, int D, const float* __restrict__ mu, const float* __restrict__ var,
                                const double* __restrict__ stats, double* __restrict__ G, double* __restrict__ K) {
  const int E = D + 1, PU = E * (E + 1) / 2, P = D * (D + 1) / 2;
  const int i = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= PU + E) return;
  const double* n = stats;
  const double* F = stats + M;
  const double* S = stats + M + (size_t)M * D;
  int a = 0, b = 0, kidx = -1;
  if (t < PU) {
    int rem = t;
    while (rem >= E - a) {
      rem -= E - a;
      ++a;
    }
    b = a + rem;
  } else {
    kidx = t - PU;
  }
  const int sidx = (a < D && b < D) ? a * D + b - a * (a + 1) / 2 : 0;
  double acc = 0.0;
  for (int m = 0; m < M; ++m) {
    const double mp = n[m];
    if (!(mp > 0.0)) continue;
    const float vm = var[(size_t)m * D + i];
    if (kidx < 0) {
      const double cv = (double)__fdiv_rn(1.0f, vm);
      double x;
      if (b < D) x = S[(size_t)m * P + sidx];
      else if (a < D) x = F[(size_t)m * D + a];
      else x = mp;
      acc = __dadd_rn(acc, __dmul_rn(cv, x));
    } else {
      const double cm = (double)__fdiv_rn(mu[(size_t)m * D + i], vm);
      const double x = kidx < D ? F[(size_t)m * D + kidx] : mp;
      acc = __dadd_rn(acc, __dmul_rn(cm, x));
    }
  }
  if (kidx < 0) {
    double* g = G + (size_t)i * E * E;
    g[a * E + b] = acc;
    g[b * E + a] = acc;
  } else {
    K[(size_t)i * E + kidx] = acc;
  }
}

__global__ void fmllr_ginv_kernel(int E, const double* __restrict__ G, double* __restrict__ Ginv) {
  extern __shared__ double sa[];
  const int i = blockIdx.x;
  for (int e = threadIdx.x; e < E * E; e += blockDim.x) sa[e] = G[(size_t)i * E * E + e];
  __syncthreads();
  gj_invert_block(sa, E);
  for (int e = threadIdx.x; e < E * E; e += blockDim.x) Ginv[(size_t)i * E * E + e] = sa[e];
}

// The passes over the rows (one block). status: 0 ok, 5 negative discriminant or zero root.
__global__ void fmllr_rows_kernel(int D, int iters, double beta, const double* __restrict__ G,
                                  const double* __restrict__ Ginv, const double* __restrict__ K,
                                  double* __restrict__ W, int* __restrict__ status) {
  extern __shared__ double sm[];
  const int E = D + 1;
  double* A = sm;                 // D x D
  double* cof = A + D * D;        // D x D: inv(A) det(A) of the pass
  double* tmp = cof + D * D;      // D x D: elimination copy for the determinant
  double* b = tmp + D * D;        // D
  double* c = b + D;              // E: the row's cofactors, 0 at position D
  double* foo = c + E;            // E
  double* wv = foo + E;           // 2 x E
  double* w2 = wv + 2 * E;        // 2 x E
  double* gw = w2 + 2 * E;        // 2 x E
  __shared__ double s_det, s_f[2], s_q[2];
  __shared__ int s_bad, s_piv;
  const int t = threadIdx.x;
  for (int e = t; e < D * D; e += blockDim.x) A[e] = (e / D == e % D) ? 1.0 : 0.0;
  for (int e = t; e < D; e += blockDim.x) b[e] = 0.0;
  if (t == 0) s_bad = 0;
  __syncthreads();
  for (int it = 0; it < iters; ++it) {
    for (int e = t; e < D * D; e += blockDim.x) {
      cof[e] = A[e];
      tmp[e] = A[e];
    }
    if (t == 0) s_det = 1.0;
    __syncthreads();
    gj_invert_block(cof, D);
    // determinant by elimination with partial pivoting (MATRIX::_Det_Gen / pivot)
    for (int k = 0; k < D; ++k) {
      if (t == 0) {
        int p = k;
        double amax = -1.0;
        for (int r = k; r < D; ++r) {
          const double v = fabs(tmp[r * D + k]);
          if (v > amax && v != 0.0) {
            amax = v;
            p = r;
          }
        }
        s_piv = (tmp[p * D + k] == 0.0) ? -1 : p;
      }
      __syncthreads();
      const int p = s_piv;
      if (p < 0) {  // singular: det = 0
        if (t == 0) s_det = 0.0;
        break;
      }
      if (p != k) {
        for (int j = t; j < D; j += blockDim.x) {
          const double x = tmp[p * D + j];
          tmp[p * D + j] = tmp[k * D + j];
          tmp[k * D + j] = x;
        }
      }
      __syncthreads();
      if (t == 0) s_det = __dmul_rn(p != k ? -s_det : s_det, tmp[k * D + k]);
      for (int e = t; e < (D - k - 1) * (D - k - 1); e += blockDim.x) {
        const int r = k + 1 + e / (D - k - 1), j = k + 1 + e % (D - k - 1);
        const double piv = __ddiv_rn(tmp[r * D + k], tmp[k * D + k]);
        tmp[r * D + j] = __dsub_rn(tmp[r * D + j], __dmul_rn(piv, tmp[k * D + j]));
      }
      __syncthreads();
    }
    __syncthreads();
    const double det = s_det;
    for (int e = t; e < D * D; e += blockDim.x) cof[e] = __dmul_rn(cof[e], det);
    __syncthreads();
    for (int i = 0; i < D; ++i) {
      const double* g = G + (size_t)i * E * E;
      const double* gi = Ginv + (size_t)i * E * E;
      const double* k = K + (size_t)i * E;
      for (int a = t; a < E; a += blockDim.x) c[a] = a < D ? cof[a * D + i] : 0.0;
      __syncthreads();
      for (int q = t; q < E; q += blockDim.x) {  // foo = c^T G_i^-1
        double s = 0.0;
        for (int p = 0; p < E; ++p) s = __dadd_rn(s, __dmul_rn(c[p], gi[p * E + q]));
        foo[q] = s;
      }
      __syncthreads();
      if (t == 0) {
        double bb = 0.0, cc = 0.0;
        for (int q = 0; q < E; ++q) bb = __dadd_rn(bb, __dmul_rn(foo[q], k[q]));
        for (int q = 0; q < E; ++q) cc = __dadd_rn(cc, __dmul_rn(foo[q], c[q]));
        bb = -bb;
        cc = -cc;
        const double disc = __dsub_rn(__dmul_rn(bb, bb), __dmul_rn(__dmul_rn(4.0, beta), cc));
        const double sq = __dsqrt_rn(disc);
        const double den = __dmul_rn(2.0, beta);
        s_f[0] = __ddiv_rn(__dadd_rn(-bb, sq), den);
        s_f[1] = __ddiv_rn(__dsub_rn(-bb, sq), den);
        if (sq < 0 || isnan(sq) || s_f[0] == 0.0 || s_f[1] == 0.0) s_bad = 1;
      }
      __syncthreads();
      if (s_bad) break;
      for (int e = t; e < 2 * E; e += blockDim.x) {
        const int j = e / E, a = e - j * E;
        wv[e] = __dadd_rn(__ddiv_rn(c[a], s_f[j]), k[a]);
      }
      __syncthreads();
      for (int e = t; e < 2 * E; e += blockDim.x) {  // w = wv^T G_i^-1
        const int j = e / E, q = e - j * E;
        double s = 0.0;
        for (int p = 0; p < E; ++p) s = __dadd_rn(s, __dmul_rn(wv[j * E + p], gi[p * E + q]));
        w2[e] = s;
      }
      __syncthreads();
      for (int e = t; e < 2 * E; e += blockDim.x) {  // G_i w
        const int j = e / E, a = e - j * E;
        double s = 0.0;
        for (int q = 0; q < E; ++q) s = __dadd_rn(s, __dmul_rn(g[a * E + q], w2[j * E + q]));
        gw[e] = s;
      }
      __syncthreads();
      if (t < 2) {
        double Q = 0.0;
        for (int a = 0; a < E; ++a)
          Q = __dadd_rn(Q, __dmul_rn(w2[t * E + a], __dsub_rn(k[a], __dmul_rn(0.5, gw[t * E + a]))));
        s_q[t] = Q;
      }
      __syncthreads();
      const int best = s_q[0] > s_q[1] ? 0 : 1;
      for (int a = t; a < D; a += blockDim.x) A[i * D + a] = w2[best * E + a];
      if (t == 0) b[i] = w2[best * E + D];
      __syncthreads();
    }
    if (s_bad) break;
  }
  if (t == 0) *status = s_bad ? 5 : 0;
  if (!s_bad)
    for (int e = t; e < D * E; e += blockDim.x) {
      const int i = e / E, j = e - i * E;
      W[e] = j < D ? A[i * D + j] : b[i];
    }
}

// x' = A x + b over the resident frames (A: D x D, b: D, from W = [A | b]).
__global__ void fmllr_apply_kernel(long long N, int D, const double* __restrict__ W, float* __restrict__ X) {
  extern __shared__ double sw[];
  for (int e = threadIdx.x; e < D * (D + 1); e += blockDim.x) sw[e] = W[e];
  __syncthreads();
  const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= N) return;
  float* x = X + (size_t)f * D;
  float in[64];
  for (int d = 0; d < D; ++d) in[d] = x[d];
  for (int r = 0; r < D; ++r) {
    double s = sw[r * (D + 1) + D];
    for (int d = 0; d < D; ++d) s += sw[r * (D + 1) + d] * (double)in[d];
    x[r] = (float)s;
  }
}

}  // namespace
}  // namespace gmm

using namespace gmm;

namespace gmm {
// From the E-step statistics on the device ([n | F | S packed | ...], M components of dimension
// D) and the model's means and variances (diagonals for a full model): CheckInvertibility, G and
// k, the inverses and the row passes; W to the host. beta = the frame count.
static int fmllr_from_stats(Ctx* c, int M, int D, const float* mu, const float* var, const double* d_stats,
                            long long frames, int iters, double* W) {
  const int E = D + 1;
  double *dG = nullptr, *dGi = nullptr, *dK = nullptr, *dW = nullptr;
  int* dstatus = nullptr;
  int rc = dalloc(c, (void**)&dG, sizeof(double) * (size_t)D * E * E, "fMLLR G");
  if (!rc) rc = dalloc(c, (void**)&dGi, sizeof(double) * (size_t)D * E * E, "fMLLR G inverse");
  if (!rc) rc = dalloc(c, (void**)&dK, sizeof(double) * (size_t)D * E, "fMLLR k");
  if (!rc) rc = dalloc(c, (void**)&dW, sizeof(double) * (size_t)D * E, "fMLLR transform");
  if (!rc) rc = dalloc(c, (void**)&dstatus, sizeof(int), "fMLLR status");
  // CheckInvertibility (OL_ModelAdapt.cpp:1851-1878) on the occupancies
  std::vector<double> n((size_t)M);
  if (!rc) {
    cudaMemcpyAsync(n.data(), d_stats, sizeof(double) * M, cudaMemcpyDeviceToHost, c->stream);
    rc = sync(c, "fMLLR statistics");
  }
  if (!rc) {
    int active = 0;
    double occ = 0.0;
    for (int m = 0; m < M; ++m)
      if (n[(size_t)m] > 0) {
        ++active;
        occ += n[(size_t)m];
      }
    if (M < E || active < E || occ * D < (double)D * E)
      rc = fail(c, GMM_ERR_MLLR, "CheckInvertibility(): not enough components or data for a D x (D+1) fMLLR transform");
  }
  if (!rc) {
    GMM_LAUNCH(c, "fmllr_gk_kernel");
    const int entries = E * (E + 1) / 2 + E;
    dim3 grid((entries + 127) / 128, D);
    fmllr_gk_kernel<<<grid, 128, 0, c->stream>>>(M, D, mu, var, d_stats, dG, dK);
  }
  if (!rc) {
    GMM_LAUNCH(c, "fmllr_ginv_kernel");
    fmllr_ginv_kernel<<<D, 256, sizeof(double) * E * E, c->stream>>>(E, dG, dGi);
  }
  if (!rc) {
    const size_t smem = sizeof(double) * (3 * (size_t)D * D + D + 8 * (size_t)E);
    cudaFuncSetAttribute(fmllr_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    GMM_LAUNCH(c, "fmllr_rows_kernel");
    // beta: the frame count as the reference passes it, (float) getTotAccSamples()
    const double beta = (double)(float)frames;
    fmllr_rows_kernel<<<1, 256, smem, c->stream>>>(D, iters, beta, dG, dGi, dK, dW, dstatus);
  }
  int status = 0;
  if (!rc) {
    cudaMemcpyAsync(&status, dstatus, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(W, dW, sizeof(double) * (size_t)D * E, cudaMemcpyDeviceToHost, c->stream);
    rc = sync(c, "fMLLR transform");
  }
  if (!rc && status) rc = fail(c, GMM_ERR_MLLR, "EstimateAb_fmllr(): Discriminant < 0 or a zero root!");
  cudaStreamSynchronize(c->stream);
  dfree(c, dG, sizeof(double) * (size_t)D * E * E);
  dfree(c, dGi, sizeof(double) * (size_t)D * E * E);
  dfree(c, dK, sizeof(double) * (size_t)D * E);
  dfree(c, dW, sizeof(double) * (size_t)D * E);
  dfree(c, dstatus, sizeof(int));
  return rc;
}
}  // namespace gmm

extern "C" {

int gmm_fmllr_estimate(gmm_handle h, int iters, double* W) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!W) return fail(c, GMM_ERR_ARG, "gmm_fmllr_estimate: null output");
  if (iters < 1) return fail(c, GMM_ERR_ARG, "gmm_fmllr_estimate: iters must be >= 1");
  if (!c->w) return fail(c, GMM_ERR_STATE, "no model uploaded");
  cudaSetDevice(c->device);
  const int M = c->M, D = c->D, P = D * (D + 1) / 2;
  if (D > 64) return fail(c, GMM_ERR_UNSUPPORTED, "fMLLR supports D <= 64");
  const size_t nst = (size_t)M * (1 + D + P) + 2;
  double* d_stats = nullptr;
  int rc = dalloc(c, (void**)&d_stats, nst * sizeof(double), "fMLLR statistics");
  if (!rc) rc = diag_fullstats_estep(c, d_stats);
  if (!rc) rc = fmllr_from_stats(c, M, D, c->mu, c->var, d_stats, c->N, iters, W);
  cudaStreamSynchronize(c->stream);
  dfree(c, d_stats, nst * sizeof(double));
  return rc;
}

int gmm_fmllr_estimate_full(gmm_handle h, int iters, double* W) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!W) return fail(c, GMM_ERR_ARG, "gmm_fmllr_estimate_full: null output");
  if (iters < 1) return fail(c, GMM_ERR_ARG, "gmm_fmllr_estimate_full: iters must be >= 1");
  cudaSetDevice(c->device);
  // the full model's E-step with full second-order statistics, then its covariance diagonals
  int rc = gmm_accumulate_full_device(h, GMM_ACC_MEAN | GMM_ACC_VAR);
  if (rc) return rc;
  const double* stats = nullptr;
  const float *mu = nullptr, *dvar = nullptr;
  int M = 0, D = 0;
  long long frames = 0;
  float* diag = nullptr;
  rc = full_fmllr_inputs(c, &stats, &mu, &diag, &M, &D, &frames);
  if (!rc) {
    dvar = diag;
    rc = fmllr_from_stats(c, M, D, mu, dvar, stats, frames, iters, W);
  }
  cudaStreamSynchronize(c->stream);
  dfree(c, diag, sizeof(float) * (size_t)M * D);
  return rc;
}

int gmm_fmllr_apply(gmm_handle h, const double* W) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!W) return fail(c, GMM_ERR_ARG, "gmm_fmllr_apply: null transform");
  if (!c->Xown || c->X != c->Xown)
    return fail(c, GMM_ERR_STATE, "gmm_fmllr_apply transforms features uploaded with gmm_upload_features only");
  const int D = c->Dx;
  if (D > 64) return fail(c, GMM_ERR_UNSUPPORTED, "fMLLR supports D <= 64");
  cudaSetDevice(c->device);
  double* dW = nullptr;
  int rc = dalloc(c, (void**)&dW, sizeof(double) * (size_t)D * (D + 1), "fMLLR transform");
  if (rc) return rc;
  cudaMemcpyAsync(dW, W, sizeof(double) * (size_t)D * (D + 1), cudaMemcpyHostToDevice, c->stream);
  if (c->N > 0) {
    GMM_LAUNCH(c, "fmllr_apply_kernel");
    fmllr_apply_kernel<<<(unsigned)((c->N + 127) / 128), 128, sizeof(double) * D * (D + 1), c->stream>>>(
        c->N, D, dW, c->Xown);
  }
  c->tcx_valid = false;  // operand planes of the old frames
  c->stats_valid = false;
  rc = sync(c, "gmm_fmllr_apply");
  dfree(c, dW, sizeof(double) * (size_t)D * (D + 1));
  return rc;
}

}  // extern "C"
