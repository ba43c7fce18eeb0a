// M-step on the device: EM, MAP and global-MLLR re-estimation from the FP64 statistics.
//
// The model stays device-resident between E-steps; nothing goes through the host per EM
// iteration. Arithmetic follows the reference's CModelAdapt (GMM/lib_bmssr/trainer/
// OL_ModelAdapt.cpp) expression by expression -- FP64 math, float stores, the same
// sequential sums for the weight normalisers -- and uses explicit round-to-nearest intrinsics
// so no multiply-add is fused. Given the same statistics the updates are bit-identical to the
// reference's.
#include <math.h>

#include "gmm_internal.cuh"

namespace gmm {

namespace {

// FP64 -> FP32, round to nearest even, on the integer pipes. GB300 runs the conversion
// instruction on its FP64 pipe (1/64 of the FP32 rate), where it was most of the batched MAP
// update's FP64 work. This is the IEEE 754 rounding of the 52-bit significand to 23 bits for
// results in the normal FP32 range; zero, subnormal, overflowing and non-finite inputs take the
// conversion instruction. A round-up carry out of the significand increments the exponent (up to
// infinity), which is the correctly rounded result.
__device__ __forceinline__ float f64_to_f32_rn(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned int hi = (unsigned int)(b >> 32), lo = (unsigned int)b;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023;  // unbiased exponent
  if (e < -126 || e > 127) return __double2float_rn(d);
  const unsigned int keep = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 significand bits
  const unsigned int rest = lo & 0x1fffffffu;                     // the 29 bits rounded away
  unsigned int f = (hi & 0x80000000u) | ((unsigned int)(e + 127) << 23) | keep;
  if (rest > 0x10000000u || (rest == 0x10000000u && (keep & 1u))) f += 1u;
  return __uint_as_float(f);
}

__device__ __forceinline__ float reset_var_value() {
  // GMMMixture::Reset (OL_GMModel.cpp:73-83) fills diagonal variances with memset(.., 1, ..)
  return __int_as_float(0x01010101);
}

// UpdateModelEM per component (OL_ModelAdapt.cpp:858-921). flag[5] <- weights changed,
// flag[6] <- number of components that had zero weight before the update.
// var64: the variance as S/n - (F/n)^2 in FP64 throughout (the tensor-core path's update); the
// reference squares the float-rounded mean, which alone moves a variance by up to ~1e-5 relative
// when mu^2 >> var. Without var64 the update is the reference's, bit for bit.
__global__ void em_comp_kernel(int M, int D, float* __restrict__ w, float* __restrict__ mu,
                               float* __restrict__ var, const double* __restrict__ stats,
                               unsigned int tot, int upW, int upM, int upV, float min_var,
                               const double* __restrict__ nind, int* __restrict__ flag, int var64) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const double* n = stats;
  const double* F = stats + M;
  const double* S = stats + M + (size_t)M * D;
  if (w[j] == 0.0f) { atomicAdd(&flag[6], 1); return; }
  double mp = n[j];
  float* mj = mu + (size_t)j * D;
  float* vj = var + (size_t)j * D;
  if ((nind ? nind[j] : mp) < 2.0) {  // _MIN_IND_SAMPLES_ (OL_ModelAdapt.h:54); robust: on nind
    for (int k = 0; k < D; ++k) { mj[k] = 0.0f; vj[k] = reset_var_value(); }
    w[j] = 0.0f;
    atomicExch(&flag[5], 1);
    return;
  }
  if (upW) {
    w[j] = (float)__ddiv_rn(mp, (double)tot);
    atomicExch(&flag[5], 1);
  }
  if (upM || upV) {
    for (int k = 0; k < D; ++k) {
      const double mean_d = __ddiv_rn(F[(size_t)j * D + k], mp);
      float mean = (float)mean_d;
      if (upV) {
        const double mv = var64 ? mean_d : (double)mean;
        double m2 = __dmul_rn(mv, mv);
        float v = (float)__dsub_rn(__ddiv_rn(S[(size_t)j * D + k], mp), m2);
        if (v < min_var) v = min_var;
        vj[k] = v;
      }
      if (upM) mj[k] = mean;
    }
  }
}

// Weight renormalisation (OL_ModelAdapt.cpp:928-931): the normaliser is the sequential FP64
// sum in component order (one thread, as the reference adds them); the divisions are
// independent and run across the block.
// The weights are staged in shared memory by all threads first, so the serial sum waits on
// additions only, not on global loads.
constexpr int kNormStage = 4096;
__global__ void em_norm_kernel(int M, float* __restrict__ w, int* __restrict__ flag) {
  __shared__ double s_corr;
  __shared__ float s_w[kNormStage];
  for (int j = threadIdx.x; j < M && j < kNormStage; j += blockDim.x) s_w[j] = w[j];
  __syncthreads();
  if (threadIdx.x == 0) {
    double corr = 0.0;
    for (int j = 0; j < M; ++j) corr = __dadd_rn(corr, (double)(j < kNormStage ? s_w[j] : w[j]));
    s_corr = corr;
    flag[2] = M - flag[6];
  }
  __syncthreads();
  const double corr = s_corr;
  if (flag[5] && corr > 0.0)
    for (int j = threadIdx.x; j < M; j += blockDim.x) w[j] = (float)__ddiv_rn((double)w[j], corr);
}

// UpdateModelMAP, tau > 0 (OL_ModelAdapt.cpp:1024-1099), one thread per component. var64: the
// variance update in FP64 throughout (see em_comp_kernel).
__global__ void map_comp_kernel(int M, int D, float* __restrict__ w, float* __restrict__ mu,
                                float* __restrict__ var, const float* __restrict__ uw,
                                const float* __restrict__ umu, const float* __restrict__ uvar,
                                const double* __restrict__ stats, unsigned int tot, int tau,
                                int upW, int upM, int upV, float min_var,
                                float* __restrict__ adapted_w, int var64) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  adapted_w[j] = 0.0f;
  if (uw[j] == 0.0f) return;
  const double* n = stats;
  const double* F = stats + M;
  const double* S = stats + M + (size_t)M * D;
  double mp = n[j];
  if (!(mp > 0.0)) return;
  double alfa = __ddiv_rn(mp, __dadd_rn(mp, (double)tau));
  double one_m = __dsub_rn(1.0, alfa);
  if (upW && tot > 0) {
    double t1 = __dmul_rn(alfa, __ddiv_rn(mp, (double)tot));
    float aw = (float)__dadd_rn(t1, __dmul_rn(one_m, (double)uw[j]));
    w[j] = aw;
    adapted_w[j] = aw;
  }
  if (upM || upV) {
    const float* um = umu + (size_t)j * D;
    const float* uv = uvar + (size_t)j * D;
    for (int k = 0; k < D; ++k) {
      double a1 = __ddiv_rn(__dmul_rn(alfa, F[(size_t)j * D + k]), mp);
      const double amd = __dadd_rn(a1, __dmul_rn(one_m, (double)um[k]));
      float am = (float)amd;
      if (upV) {
        float second = __fadd_rn(uv[k], __fmul_rn(um[k], um[k]));
        float msq = __fmul_rn(am, am);
        double b1 = __ddiv_rn(__dmul_rn(alfa, S[(size_t)j * D + k]), mp);
        const double second_d =
            var64 ? __dadd_rn((double)uv[k], __dmul_rn((double)um[k], (double)um[k])) : (double)second;
        double b2 = __dadd_rn(b1, __dmul_rn(one_m, second_d));
        float av = (float)__dsub_rn(b2, var64 ? __dmul_rn(amd, amd) : (double)msq);
        if (av < min_var) av = min_var;
        var[(size_t)j * D + k] = av;
      }
      mu[(size_t)j * D + k] = am;
    }
  }
}

__global__ void map_norm_kernel(int M, float* __restrict__ w, const float* __restrict__ adapted_w,
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

// GMModel::RearrangeMixtures (OL_GMModel.cpp:857-885), single block: non-zero-weight
// components keep their order, the k-th zero-weight one goes to slot M-1-k.
__global__ void rearrange_kernel(int M, int D, float* __restrict__ w, float* __restrict__ mu,
                                 float* __restrict__ var, float* __restrict__ tw,
                                 float* __restrict__ tmu, float* __restrict__ tvar,
                                 int* __restrict__ order) {
  __shared__ int s_nz;
  if (threadIdx.x == 0) {
    int nz = 0, z = 1;
    for (int m = 0; m < M; ++m) {
      if (w[m] > 0.0f) order[nz++] = m;
      else order[M - z++] = m;
    }
    s_nz = nz;
  }
  __syncthreads();
  for (size_t e = threadIdx.x; e < (size_t)M * D; e += blockDim.x) {
    tmu[e] = mu[e];
    tvar[e] = var[e];
  }
  for (int m = threadIdx.x; m < M; m += blockDim.x) tw[m] = w[m];
  __syncthreads();
  for (size_t e = threadIdx.x; e < (size_t)M * D; e += blockDim.x) {
    int k = (int)(e / D), d = (int)(e - (size_t)k * D);
    mu[e] = tmu[(size_t)order[k] * D + d];
    var[e] = tvar[(size_t)order[k] * D + d];
  }
  for (int m = threadIdx.x; m < M; m += blockDim.x) w[m] = tw[order[m]];
}

// CheckInvertibility sums (OL_ModelAdapt.cpp:1857-1866): sequential, component order.
__global__ void mllr_check_kernel(int M, const double* __restrict__ n, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int act = 0;
  double occ = 0.0;
  for (int m = 0; m < M; ++m)
    if (n[m] > 0.0) { ++act; occ = __dadd_rn(occ, n[m]); }
  out[0] = act;
  out[1] = occ;
}

// One block per transform row i: G_i, k_i (ComputeKiGi_MLLR :1525-1581, with the
// prepareKiGiInitMatrices prior :1484-1523), pivot-free Gauss-Jordan inverse
// (MATRIX::_Invert_Gen, Matrix4_LMa.cpp:2232-2300), w_i = G_i^-1 k_i (MATRIX::Mult).
// Shared memory: (D+1)^2 + (D+1) doubles.
__global__ void mllr_row_kernel(int M, int D, const float* __restrict__ mu,
                                const float* __restrict__ var, const float* __restrict__ umu,
                                const float* __restrict__ uvar, const double* __restrict__ stats,
                                int ubm_init, float min_var, double* __restrict__ W) {
  extern __shared__ double sm[];
  const int E = D + 1;
  const int i = blockIdx.x;
  double* G = sm;
  double* kv = sm + E * E;
  const double* n = stats;
  const double* F = stats + M;
  // each thread owns entries (a, b) of the upper triangle incl. the last column, plus k[a]
  for (int e = threadIdx.x; e < E * E; e += blockDim.x) {
    int a = e / E, b = e - a * E;
    if (a > b) continue;
    double g = 0.0;
    if (ubm_init) {
      // prior terms over all UBM components, accumulated in the reference's order
      for (int m = 0; m < M; ++m) {
        const float* v = uvar + (size_t)m * D;
        const float* me = umu + (size_t)m * D;
        double cG = (v[i] < min_var) ? (double)__fdiv_rn(1.0f, min_var) : (double)__fdiv_rn(1.0f, v[i]);
        if (a < D && b < D) {
          g = __dadd_rn(g, __dmul_rn(__dmul_rn(cG, (double)me[a]), (double)me[b]));
          if (a == b) g = __dadd_rn(g, __dmul_rn(cG, (double)v[a]));
        } else if (a < D) {
          g = __dadd_rn(g, __dmul_rn(cG, (double)me[a]));
        } else {
          g = __dadd_rn(g, cG);
        }
      }
    }
    for (int m = 0; m < M; ++m) {
      double mp = n[m];
      if (!(mp > 0.0)) continue;
      const float* mm = mu + (size_t)m * D;
      double cv = __ddiv_rn(mp, (double)var[(size_t)m * D + i]);
      if (a < D && b < D) g = __dadd_rn(g, __dmul_rn(__dmul_rn(cv, (double)mm[a]), (double)mm[b]));
      else if (a < D) g = __dadd_rn(g, __dmul_rn(cv, (double)mm[a]));
      else g = __dadd_rn(g, cv);
    }
    G[a * E + b] = g;
  }
  for (int a = threadIdx.x; a < E; a += blockDim.x) {
    double k = 0.0;
    if (ubm_init) {
      for (int m = 0; m < M; ++m) {
        const float* v = uvar + (size_t)m * D;
        const float* me = umu + (size_t)m * D;
        double cG = (v[i] < min_var) ? (double)__fdiv_rn(1.0f, min_var) : (double)__fdiv_rn(1.0f, v[i]);
        double ck = __dmul_rn((double)me[i], cG);
        k = __dadd_rn(k, a < D ? __dmul_rn(ck, (double)me[a]) : ck);
      }
    }
    for (int m = 0; m < M; ++m) {
      double mp = n[m];
      if (!(mp > 0.0)) continue;
      double cm = __ddiv_rn(F[(size_t)m * D + i], (double)var[(size_t)m * D + i]);
      k = __dadd_rn(k, a < D ? __dmul_rn(cm, (double)mu[(size_t)m * D + a]) : cm);
    }
    kv[a] = k;
  }
  __syncthreads();
  // the reference mirrors the upper triangle into the lower one as it accumulates
  for (int e = threadIdx.x; e < E * E; e += blockDim.x) {
    int a = e / E, b = e - a * E;
    if (a > b) G[a * E + b] = G[b * E + a];
  }
  __syncthreads();
  for (int k = 0; k < E; ++k) {
    const double piv = G[k * E + k];
    for (int e = threadIdx.x; e < E * E; e += blockDim.x) {
      int a = e / E, b = e - a * E;
      if (a != k && b != k)
        G[e] = __dsub_rn(G[e], __ddiv_rn(__dmul_rn(G[k * E + b], G[a * E + k]), piv));
    }
    __syncthreads();
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
      if (e != k) {
        G[k * E + e] = __ddiv_rn(-G[k * E + e], piv);
        G[e * E + k] = __ddiv_rn(G[e * E + k], piv);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) G[k * E + k] = __ddiv_rn(1.0, piv);
    __syncthreads();
  }
  for (int a = threadIdx.x; a < E; a += blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < E; ++b) s = __dadd_rn(s, __dmul_rn(G[a * E + b], kv[b]));
    W[(size_t)i * E + a] = s;
  }
}

// AdaptModelMLLR (OL_ModelAdapt.cpp:1597-1608): one block per component.
__global__ void mllr_apply_kernel(int M, int D, float* __restrict__ mu, const double* __restrict__ W) {
  extern __shared__ float row[];
  const int m = blockIdx.x;
  const int E = D + 1;
  for (int k = threadIdx.x; k < D; k += blockDim.x) row[k] = mu[(size_t)m * D + k];
  __syncthreads();
  for (int k = threadIdx.x; k < D; k += blockDim.x) {
    double v = 0.0;
    for (int kk = 0; kk < D; ++kk) v = __dadd_rn(v, __dmul_rn(W[(size_t)k * E + kk], (double)row[kk]));
    mu[(size_t)m * D + k] = (float)__dadd_rn(v, W[(size_t)k * E + D]);
  }
}

// CModelAdapt::UpdateModelMAP (OL_ModelAdapt.cpp:1024-1099) for every (speaker, component),
// with the resident model as both the starting point and the prior: AdaptModelMAP copies the UBM
// (:1259-1260) and the first MAP iteration adapts that copy towards the statistics. Same
// expression order as map_comp_kernel. A block takes kMapPairs (speaker, component) pairs: first
// one thread per pair forms the pair's scalars (occupation, alpha, 1 - alpha, 1 / occupation)
// and its weight; then the block's threads take the (pair, dimension) elements, pairs fastest
// (consecutive components are consecutive rows of the partials: coalesced reads), so that the
// FP64 work of the D dimensions runs in parallel instead of in one thread per pair (1.47 ms for
// C3's 1000 x 1024 pairs with one thread per pair). Means and variances are staged in shared
// memory ([pair][D + 1], an odd stride) and written out as one contiguous range.
// Statistics come in one of two layouts (kStatsSlots / kStatsPlain); in the plain layout the
// speaker's total log-likelihood is copied out as well.
constexpr int kMapPairs = 32;     // (speaker, component) pairs per block
constexpr int kMapThreads = 256;
__global__ void __launch_bounds__(kMapThreads, 5) map_batch_kernel(
    int S, int M, int D, const double* __restrict__ plain, const double* __restrict__ part, int K, int n_chunks,
    const int* __restrict__ piece0, const int* __restrict__ npieces, const int* __restrict__ row_of_comp,
    const float* __restrict__ cent, const long long* __restrict__ offs, const float* __restrict__ uw, const float* __restrict__ umu,
    const float* __restrict__ uvar, int tau, int upW, int upM, int upV, float min_var, float* __restrict__ ow,
    float* __restrict__ omu, float* __restrict__ ovar, float* __restrict__ adapted_w, double* __restrict__ ll) {
  extern __shared__ float s_out[];
  __shared__ double s_mp[kMapPairs], s_alfa[kMapPairs], s_one[kMapPairs], s_rmp[kMapPairs];
  __shared__ float s_alfa_f[kMapPairs], s_one_f[kMapPairs], s_rmp_f[kMapPairs];  // FP32 copies
  __shared__ int s_adapt[kMapPairs], s_spk[kMapPairs], s_comp[kMapPairs];
  const int SD = D + 1;
  float* s_mu = s_out;
  float* s_var = s_out + kMapPairs * SD;
  const long long tot_pairs = (long long)S * M;
  const long long t0 = (long long)blockIdx.x * kMapPairs;
  const int n_here = (int)(tot_pairs - t0 < kMapPairs ? tot_pairs - t0 : kMapPairs);
  // statistic e (n / F / S order; operand-layout columns of the tensor-core partials) of
  // component m for speaker s
  auto stat = [&](int s, int m, int e) -> double {  // e in [0, 2D]: F_k = e < D, S_k = D + k, n = 2D
    if (plain) {
      const double* pst = plain + (size_t)s * ((size_t)M * (1 + 2 * D) + 2);
      if (e == 2 * D) return pst[m];
      if (e < D) return pst[M + (size_t)m * D + e];
      return pst[M + (size_t)M * D + (size_t)m * D + (e - D)];
    }
    const int row = row_of_comp[m];
    if (row < 0) return 0.0;  // inactive components were never accumulated
    const int np = npieces[s], p0 = piece0[s];
    double v = 0.0;
    const int col = tc_stat_col(D, K, e);
    for (int p = 0; p < np; ++p) {
      const double x = part[((size_t)(p0 + p) * n_chunks + row / 128) * K * 128 + (size_t)col * 128 + (row % 128)];
      v = p == 0 ? x : __dadd_rn(v, x);
    }
    return v;
  };
  if (threadIdx.x < n_here) {
    const long long t = t0 + threadIdx.x;
    const int s = (int)(t / M), m = (int)(t - (long long)s * M);
    if (plain && m == 0) ll[s] = plain[(size_t)s * ((size_t)M * (1 + 2 * D) + 2) + (size_t)M * (1 + 2 * D)];
    const double mp = stat(s, m, 2 * D);
    const bool adapt = uw[m] != 0.0f && mp > 0.0;
    const unsigned int tot = (unsigned int)(offs[s + 1] - offs[s]);
    const double alfa = adapt ? __ddiv_rn(mp, __dadd_rn(mp, (double)tau)) : 0.0;
    const double one_m = __dsub_rn(1.0, alfa);
    float aw = 0.0f;
    const bool wset = adapt && upW && tot > 0;
    if (wset) {
      const double t1 = __dmul_rn(alfa, __ddiv_rn(mp, (double)tot));
      aw = (float)__dadd_rn(t1, __dmul_rn(one_m, (double)uw[m]));
    }
    ow[t] = wset ? aw : uw[m];
    adapted_w[t] = aw;
    s_mp[threadIdx.x] = mp;
    s_alfa[threadIdx.x] = alfa;
    s_one[threadIdx.x] = one_m;
    s_rmp[threadIdx.x] = adapt ? __drcp_rn(mp) : 0.0;  // the D quotients share the divisor mp
    s_alfa_f[threadIdx.x] = (float)alfa;
    s_one_f[threadIdx.x] = (float)one_m;
    s_rmp_f[threadIdx.x] = (float)s_rmp[threadIdx.x];
    s_adapt[threadIdx.x] = adapt ? 1 : 0;
    s_spk[threadIdx.x] = s;
    s_comp[threadIdx.x] = m;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kMapPairs * D; i += kMapThreads) {
    const int j = i % kMapPairs, k = i / kMapPairs;
    if (j >= n_here) continue;
    const int s = s_spk[j], m = s_comp[j];  // (one 64-bit division per pair, in the first phase)
    const float* um = umu + (size_t)m * D;
    const float* uv = uvar + (size_t)m * D;
    const bool adapt = s_adapt[j] != 0;
    const double mp = s_mp[j], alfa = s_alfa[j], one_m = s_one[j], rmp = s_rmp[j];
    // the sparse statistics kernel's partials are centred on the component's mean (cr): tc_uncentre
    const int row = plain ? 0 : row_of_comp[m];
    const float* cr = (plain || !cent) ? nullptr : cent + (size_t)(row >= 0 ? row : 0) * D;
    float am = um[k], av = uv[k];
    if (adapt && !plain && upM && !upV) {
      // tensor-core path, means only: FP32 arithmetic (GB300's FP64 rate -- conversions
      // included -- is 1/64 of FP32); the statistics already carry ~1e-6 relative error, FP32
      // adds ~1e-7 of the mean. FP64 stays for the variance update.
      const double Fd = stat(s, m, k);
      const float Ff = f64_to_f32_rn(cr ? tc_uncentre_F(Fd, mp, (double)cr[k]) : Fd);
      am = __fmaf_rn(s_alfa_f[j], __fmul_rn(Ff, s_rmp_f[j]), __fmul_rn(s_one_f[j], um[k]));
    } else if (adapt && (upM || upV)) {
      const double Fk = stat(s, m, k);
      const double c = cr ? (double)cr[k] : 0.0;
      const double a1 = div_by_rcp(__dmul_rn(alfa, plain ? Fk : tc_uncentre_F(Fk, mp, c)), mp, rmp);
      const double amd = __dadd_rn(a1, __dmul_rn(one_m, (double)um[k]));
      am = (float)amd;
      if (upV && plain) {
        // the reference's expression: second moment and squared mean in float
        const float second = __fadd_rn(uv[k], __fmul_rn(um[k], um[k]));
        const float msq = __fmul_rn(am, am);
        const double b1 = div_by_rcp(__dmul_rn(alfa, stat(s, m, D + k)), mp, rmp);
        const double b2 = __dadd_rn(b1, __dmul_rn(one_m, (double)second));
        av = (float)__dsub_rn(b2, (double)msq);
        if (av < min_var) av = min_var;
      } else if (upV) {
        // tensor-core path: the variance in FP64 throughout
        const double second = __dadd_rn((double)uv[k], __dmul_rn((double)um[k], (double)um[k]));
        const double b1 = div_by_rcp(__dmul_rn(alfa, tc_uncentre_S(stat(s, m, D + k), Fk, mp, c)), mp, rmp);
        const double b2 = __dadd_rn(b1, __dmul_rn(one_m, second));
        av = (float)__dsub_rn(b2, __dmul_rn(amd, amd));
        if (av < min_var) av = min_var;
      }
    }
    s_mu[j * SD + k] = am;
    s_var[j * SD + k] = av;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n_here * D; i += kMapThreads) {
    const int j = i / D, k = i - j * D;
    if (omu) omu[(size_t)t0 * D + i] = s_mu[j * SD + k];
    if (ovar) ovar[(size_t)t0 * D + i] = s_var[j * SD + k];
  }
}

// Weight renormalisation per speaker (OL_ModelAdapt.cpp:1100-1104): one warp per speaker, the
// FP64 sum taken sequentially in component order by lane 0 (entries of components that were not
// adapted are +0.0 and leave it unchanged, as in map_norm_kernel), the divisions by all lanes.
__global__ void map_batch_norm_kernel(int S, int M, const float* __restrict__ adapted_w,
                                      float* __restrict__ ow) {
  const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (s >= S) return;
  double corr = 0.0;
  if (lane == 0)
    for (int m = 0; m < M; ++m) corr = __dadd_rn(corr, (double)adapted_w[(size_t)s * M + m]);
  corr = __shfl_sync(0xffffffffu, corr, 0);
  if (corr != 0.0) {
    const float fc = (float)corr;
    for (int m = lane; m < M; m += 32) ow[(size_t)s * M + m] = __fdiv_rn(ow[(size_t)s * M + m], fc);
  }
}

// ------------------------------------------------------------------ batched MLLR

__host__ __device__ inline int tri_index(int a, int b, int E) { return a * E - a * (a - 1) / 2 + (b - a); }

// Dense per-speaker mean statistics of MLLR (n [S][M], F [S][M][D], FP64) from either the plain
// layout or the tensor-core pieces. One thread per (speaker, component): the pieces of
// consecutive components are consecutive rows (coalesced reads); a block's F rows are staged in
// shared memory ([pair][D | 1]) and written out as one contiguous range.
constexpr int kGatherThreads = 64;
__global__ void __launch_bounds__(kGatherThreads) mllr_gather_kernel(
    int S, int M, int D, const double* __restrict__ plain, const double* __restrict__ part, int K, int n_chunks,
    const int* __restrict__ piece0, const int* __restrict__ npieces, const int* __restrict__ row_of_comp,
    const float* __restrict__ cent, double* __restrict__ n_out, double* __restrict__ F_out, double* __restrict__ ll_out) {
  extern __shared__ double s_F[];
  const int SD = D | 1;  // odd stride: the lanes' rows start in distinct banks
  const long long tot = (long long)S * M;
  const long long t0 = (long long)blockIdx.x * kGatherThreads, t = t0 + threadIdx.x;
  if (t < tot) {
    const int s = (int)(t / M), m = (int)(t - (long long)s * M);
    const int row = plain ? 0 : row_of_comp[m];
    const double* pst = plain ? plain + (size_t)s * ((size_t)M * (1 + 2 * D) + 2) : nullptr;
    const int np = plain ? 0 : npieces[s], p0 = plain ? 0 : piece0[s];
    auto stat = [&](int e) -> double {
      if (plain) return e == 2 * D ? pst[m] : pst[M + (size_t)m * D + e];
      if (row < 0) return 0.0;
      double v = 0.0;
      const int col = tc_stat_col(D, K, e);
      for (int p = 0; p < np; ++p) {
        const double x = part[((size_t)(p0 + p) * n_chunks + row / 128) * K * 128 + (size_t)col * 128 + (row % 128)];
        v = p == 0 ? x : __dadd_rn(v, x);
      }
      return v;
    };
    const double nn = stat(2 * D);
    n_out[t] = nn;
    if (plain && ll_out && m == 0) ll_out[s] = pst[(size_t)M * (1 + 2 * D)];
    if (plain) {
      for (int k = 0; k < D; ++k) s_F[threadIdx.x * SD + k] = stat(k);
    } else if (row < 0) {
      for (int k = 0; k < D; ++k) s_F[threadIdx.x * SD + k] = 0.0;
    } else {
      // the sparse statistics kernel's partials are centred on the component's mean: tc_uncentre
      const float* cr = cent ? cent + (size_t)row * D : nullptr;
      if (np == 1) {
        // one piece (the common case): independent loads, eight in flight at a time
        const double* src = part + ((size_t)p0 * n_chunks + row / 128) * K * 128 + (row % 128);
#pragma unroll 8
        for (int k = 0; k < D; ++k)
          s_F[threadIdx.x * SD + k] =
              tc_uncentre_F(src[(size_t)tc_stat_col(D, K, k) * 128], nn, cr ? (double)cr[k] : 0.0);
      } else {
        for (int k = 0; k < D; ++k) s_F[threadIdx.x * SD + k] = tc_uncentre_F(stat(k), nn, cr ? (double)cr[k] : 0.0);
      }
    }
  }
  __syncthreads();
  const long long n_here = tot - t0 < kGatherThreads ? tot - t0 : kGatherThreads;
  for (int i = threadIdx.x; i < n_here * D; i += kGatherThreads) {
    const int j = i / D, k = i - j * D;
    F_out[(size_t)t0 * D + i] = s_F[j * SD + k];
  }
}

// CheckInvertibility (OL_ModelAdapt.cpp:1851-1878) per speaker: enough components and data for a
// D x (D+1) transform. One warp per speaker.
__global__ void mllr_batch_check_kernel(int S, int M, int D, const double* __restrict__ n,
                                        int* __restrict__ status) {
  const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (s >= S) return;
  int act = 0;
  double occ = 0.0;
  for (int m = lane; m < M; m += 32) {
    const double v = n[(size_t)s * M + m];
    if (v > 0.0) { ++act; occ += v; }
  }
  for (int o = 16; o; o >>= 1) {
    act += __shfl_xor_sync(0xffffffffu, act, o);
    occ += __shfl_xor_sync(0xffffffffu, occ, o);
  }
  if (lane == 0) {
    const int E = D + 1;
    status[s] = (M < E || act < E || occ * D < (double)D * E) ? GMM_ERR_MLLR : GMM_OK;
  }
}

// xi_m xi_m^T over the upper triangle (incl. diagonal), xi_m = [mu_m; 1]: B[m][tri(a, b)] (float).
__global__ void mllr_outer_kernel(int M, int D, const float* __restrict__ mu, float* __restrict__ B) {
  const int E = D + 1, T = E * (E + 1) / 2;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)M * T) return;
  const int m = (int)(t / T);
  int e = (int)(t - (long long)m * T), a = 0;
  while (e >= E - a) { e -= E - a; ++a; }
  const int b = a + e;
  const float xa = a < D ? mu[(size_t)m * D + a] : 1.0f, xb = b < D ? mu[(size_t)m * D + b] : 1.0f;
  B[t] = (float)((double)xa * (double)xb);
}

// xi_m = [mu_m; 1] as floats: X[m][a].
__global__ void mllr_xi_kernel(int M, int D, const float* __restrict__ mu, float* __restrict__ X) {
  const int E = D + 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)M * E) return;
  const int m = (int)(t / E), a = (int)(t - (long long)m * E);
  X[t] = a < D ? mu[(size_t)m * D + a] : 1.0f;
}

// The data terms of ComputeKiGi_MLLR (OL_ModelAdapt.cpp:1525-1581) for all speakers and rows as
// GEMMs over the components: out[s][i][c] = sum_m (coef(s, m) / var[m][i]) * B[m][c], with
// coef = n (G, c = upper-triangle pair) or coef = F[.][.][i] (k, c = a, B = xi). FP32 operands
// (coef * 1/var rounded to float) and products in 128 x 64 tiles, FP32 sums over 128 components
// at a time, added into FP64.
__global__ void __launch_bounds__(256) mllr_gemm_kernel(int S, int M, int D, int C, const double* __restrict__ coef,
                                                         long long cs_s, long long cs_m, int coef_i_stride,
                                                         const float* __restrict__ var,
                                                         const float* __restrict__ B, int ldb,
                                                         double* __restrict__ out) {
  // 128 speakers x 64 columns per block, 8 x 4 outputs per thread
  __shared__ float As[32][129];
  __shared__ float Bs[32][64];
  const int i = blockIdx.z;
  const int s0 = blockIdx.y * 128, c0 = blockIdx.x * 64;
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  float acc[8][4];
  double dacc[8][4];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) { acc[u][v] = 0.0f; dacc[u][v] = 0.0; }
  for (int m0 = 0; m0 < M; m0 += 32) {
    for (int e = tid; e < 32 * 128; e += 256) {
      const int mm = e >> 7, ss = e & 127;
      const int m = m0 + mm, s = s0 + ss;
      float a = 0.0f;
      if (m < M && s < S)
        a = __fmul_rn((float)coef[(size_t)s * cs_s + (size_t)m * cs_m + (size_t)i * coef_i_stride],
                      __frcp_rn(var[(size_t)m * D + i]));
      As[mm][ss] = a;
    }
    for (int e = tid; e < 32 * 64; e += 256) {
      const int mm = e >> 6, cc = e & 63;
      const int m = m0 + mm, c = c0 + cc;
      Bs[mm][cc] = (m < M && c < C) ? B[(size_t)m * ldb + c] : 0.0f;
    }
    __syncthreads();
#pragma unroll 4
    for (int mm = 0; mm < 32; ++mm) {
      float av[8], bv[4];
#pragma unroll
      for (int u = 0; u < 8; ++u) av[u] = As[mm][ty * 8 + u];
#pragma unroll
      for (int v = 0; v < 4; ++v) bv[v] = Bs[mm][tx * 4 + v];
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
    }
    __syncthreads();
    if (((m0 + 32) & 127) == 0 || m0 + 32 >= M) {
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) { dacc[u][v] += (double)acc[u][v]; acc[u][v] = 0.0f; }
    }
  }
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int s = s0 + ty * 8 + u;
    if (s >= S) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = c0 + tx * 4 + v;
      if (c < C) out[((size_t)s * D + i) * C + c] = dacc[u][v];
    }
  }
}

// The k data term of ComputeKiGi_MLLR (OL_ModelAdapt.cpp:1525-1581) for all speakers:
// k[s][i][a] = sum_m (F[s][m][i] / var[m][i]) xi[m][a], with the operands and sums of
// mllr_gemm_kernel (coef * 1/var rounded to float, FP32 fused multiply-adds over 128 components
// in order, added into FP64), so the result is bit-identical to it. One block per speaker: the
// speaker's F rows are read once, contiguously, in chunks of 32 components, each chunk's loads
// issued before the multiply-adds of the previous one (a block is alone on its SM at C4 sizes,
// so nothing else hides the memory latency); a thread owns a 4 x 4 tile of (i, a).
constexpr int kMllrKChunk = 32, kMllrKPf = 10;  // components per chunk, loads per thread per chunk
__host__ inline int mllr_k_threads(int D) {
  const int E = D + 1, owners = ((D + 3) / 4) * ((E + 3) / 4);
  const int loads = (kMllrKChunk * ((E + 3) / 4) * 4 + kMllrKPf - 1) / kMllrKPf;
  const int t = owners > loads ? owners : loads;
  return t > 64 ? (t + 31) / 32 * 32 : 64;
}
__global__ void mllr_k_kernel(int S, int M, int D, const double* __restrict__ F, const float* __restrict__ var,
                              const float* __restrict__ Xi, double* __restrict__ kd) {
  extern __shared__ __align__(16) float sm_k[];
  const int E = D + 1, TI = (D + 3) / 4, TA = (E + 3) / 4, D4 = TI * 4, E4 = TA * 4;
  const int ny = kMllrKChunk * D4, nx = kMllrKChunk * E4;
  float* Ys = sm_k;       // [32][D4]
  float* Xs = sm_k + ny;  // [32][E4]
  const int s = blockIdx.x;
  const int t = threadIdx.x, ti = t / TA, ta = t - ti * TA;
  const bool owner = t < TI * TA;
  const double* Fs = F + (size_t)s * M * D;
  double fy[kMllrKPf];
  float vy[kMllrKPf], xx[kMllrKPf];
  auto fetch = [&](int m0) {
#pragma unroll
    for (int j = 0; j < kMllrKPf; ++j) {
      const int e = t + j * (int)blockDim.x;
      fy[j] = 0.0;
      vy[j] = 1.0f;
      xx[j] = 0.0f;
      if (e < ny) {
        const int mm = e / D4, i = e - mm * D4, m = m0 + mm;
        if (m < M && i < D) {
          fy[j] = Fs[(size_t)m * D + i];
          vy[j] = var[(size_t)m * D + i];
        }
      }
      if (e < nx) {
        const int mm = e / E4, a = e - mm * E4, m = m0 + mm;
        if (m < M && a < E) xx[j] = Xi[(size_t)m * E + a];
      }
    }
  };
  float acc[4][4];
  double dacc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) { acc[u][v] = 0.0f; dacc[u][v] = 0.0; }
  fetch(0);
  for (int m0 = 0; m0 < M; m0 += kMllrKChunk) {
#pragma unroll
    for (int j = 0; j < kMllrKPf; ++j) {
      const int e = t + j * (int)blockDim.x;
      if (e < ny) Ys[e] = __fmul_rn((float)fy[j], __frcp_rn(vy[j]));  // padding: 0 * 1 = 0
      if (e < nx) Xs[e] = xx[j];
    }
    __syncthreads();
    if (m0 + kMllrKChunk < M) fetch(m0 + kMllrKChunk);
    if (owner) {
#pragma unroll 4
      for (int mm = 0; mm < kMllrKChunk; ++mm) {
        const float4 y = *reinterpret_cast<const float4*>(Ys + mm * D4 + ti * 4);
        const float4 x = *reinterpret_cast<const float4*>(Xs + mm * E4 + ta * 4);
        const float yv[4] = {y.x, y.y, y.z, y.w}, xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(yv[u], xv[v], acc[u][v]);
      }
    }
    __syncthreads();
    if (((m0 + kMllrKChunk) & 127) == 0 || m0 + kMllrKChunk >= M) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) { dacc[u][v] += (double)acc[u][v]; acc[u][v] = 0.0f; }
    }
  }
  if (!owner) return;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = ti * 4 + u;
    if (i >= D) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int a = ta * 4 + v;
      if (a < E) kd[((size_t)s * D + i) * E + a] = dacc[u][v];
    }
  }
}

// The prior terms of prepareKiGiInitMatrices (OL_ModelAdapt.cpp:1484-1523), the same for every
// speaker: Gp[i][tri(a, b)], kp[i][a], accumulated over the UBM components in order. One block
// per row i.
__global__ void mllr_prior_kernel(int M, int D, const float* __restrict__ umu, const float* __restrict__ uvar,
                                  float min_var, double* __restrict__ Gp, double* __restrict__ kp) {
  const int E = D + 1, T = E * (E + 1) / 2;
  const int i = blockIdx.x;
  for (int e = threadIdx.x; e < T + E; e += blockDim.x) {
    double g = 0.0;
    if (e < T) {
      int r = e, a = 0;
      while (r >= E - a) { r -= E - a; ++a; }
      const int b = a + r;
      for (int m = 0; m < M; ++m) {
        const float* v = uvar + (size_t)m * D;
        const float* me = umu + (size_t)m * D;
        const double cG = (v[i] < min_var) ? (double)__fdiv_rn(1.0f, min_var) : (double)__fdiv_rn(1.0f, v[i]);
        if (a < D && b < D) {
          g = __dadd_rn(g, __dmul_rn(__dmul_rn(cG, (double)me[a]), (double)me[b]));
          if (a == b) g = __dadd_rn(g, __dmul_rn(cG, (double)v[a]));
        } else if (a < D) {
          g = __dadd_rn(g, __dmul_rn(cG, (double)me[a]));
        } else {
          g = __dadd_rn(g, cG);
        }
      }
      Gp[(size_t)i * T + e] = g;
    } else {
      const int a = e - T;
      for (int m = 0; m < M; ++m) {
        const float* v = uvar + (size_t)m * D;
        const float* me = umu + (size_t)m * D;
        const double cG = (v[i] < min_var) ? (double)__fdiv_rn(1.0f, min_var) : (double)__fdiv_rn(1.0f, v[i]);
        const double ck = __dmul_rn((double)me[i], cG);
        g = __dadd_rn(g, a < D ? __dmul_rn(ck, (double)me[a]) : ck);
      }
      kp[(size_t)i * E + a] = g;
    }
  }
}

// w_i = G_i^-1 k_i per (speaker, row): Gaussian elimination without pivoting on the augmented
// system [G_i | k_i] and a column-oriented back substitution -- the pivots in the order of the
// reference's pivot-free Gauss-Jordan inverse (MATRIX::_Invert_Gen, Matrix4_LMa.cpp:2232-2300)
// followed by the product with k, without forming the inverse. G_i is symmetric and so is every
// trailing block of the elimination, so only the upper triangle and k are updated (a sixth of
// E^3 multiply-adds instead of a half for Gauss-Jordan): at pivot p the multipliers
// l_r = a_pr / a_pp go into the unused lower column p, then the lanes walk the entries (r, c),
// r > p, c >= r, of the trailing block as one flat list. The list holds the rows from the last
// to the first, so the entries of every trailing block are a prefix of it; it is built once per
// block in shared memory. One warp per (row i, speaker s), four systems per block. Row stride LD
// is odd so that the lanes' 8-byte accesses to one column hit distinct banks. FP64 throughout,
// the updates a - l b as fused multiply-adds (one rounding). GB300 runs FP64 at 1/64 of its FP32
// rate, so the lanes must stay busy: the full-matrix form with a lane per row took 2.1 ms for the
// 19,500 systems at C4, and 5.3 ms with separate multiply and subtract and a one-lane back
// substitution.
constexpr int kSolveWarps = 4;
__host__ __device__ inline int solve_ld(int E) { return (E + 1) | 1; }
// entries (r, c) with 0 <= r < E, r <= c <= E (c = E is k)
__host__ __device__ inline int solve_list_len(int E) { return E * (E + 1) / 2 + E; }
__host__ inline size_t solve_smem(int E) {
  return sizeof(double) * (size_t)kSolveWarps * E * solve_ld(E) + sizeof(unsigned short) * solve_list_len(E);
}
__global__ void mllr_solve_kernel(int S, int D, const double* __restrict__ Gd, const double* __restrict__ kd,
                                  const double* __restrict__ Gp, const double* __restrict__ kp,
                                  const int* __restrict__ status, double* __restrict__ W) {
  extern __shared__ __align__(16) unsigned char sm_solve[];
  const int E = D + 1, T = E * (E + 1) / 2, LD = solve_ld(E);  // E columns + k
  const int L = solve_list_len(E);
  unsigned short* list = reinterpret_cast<unsigned short*>(sm_solve + sizeof(double) * (size_t)kSolveWarps * E * LD);
  for (int r = threadIdx.x; r < E; r += blockDim.x) {
    // rows E-1, E-2, ..., 0; row r holds the E + 1 - r entries c = r .. E after the n = E-1-r
    // rows below it: n (E + 1) - (n (r + E)) / 2 entries
    const int n = E - 1 - r;
    unsigned short* dst = list + n * (E + 1) - n * (r + E) / 2;
    for (int c = r; c <= E; ++c) dst[c - r] = (unsigned short)(r << 8 | c);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long sys = (long long)blockIdx.x * kSolveWarps + warp;
  if (sys >= (long long)S * D) return;
  const int s = (int)(sys / D), i = (int)(sys - (long long)s * D);
  double* A = reinterpret_cast<double*>(sm_solve) + (size_t)warp * E * LD;
  double* Wr = W + ((size_t)s * D + i) * E;
  if (status[s] != GMM_OK) {
    for (int a = lane; a < E; a += 32) Wr[a] = 0.0;
    return;
  }
  for (int a = 0; a < E; ++a) {  // upper triangle, row by row
    for (int b = a + lane; b < E; b += 32) {
      const int ti = tri_index(a, b, E);
      double g = Gd[((size_t)s * D + i) * T + ti];
      if (Gp) g = __dadd_rn(Gp[(size_t)i * T + ti], g);
      A[a * LD + b] = g;
    }
  }
  for (int a = lane; a < E; a += 32) {
    double k = kd[((size_t)s * D + i) * E + a];
    if (kp) k = __dadd_rn(kp[(size_t)i * E + a], k);
    A[a * LD + E] = k;
  }
  __syncwarp();
  int P = L - (E + 1);  // entries of rows 1 .. E-1
  for (int p = 0; p < E - 1; ++p) {
    const double ipiv = __drcp_rn(A[p * LD + p]);
    for (int r = p + 1 + lane; r < E; r += 32) A[r * LD + p] = __dmul_rn(A[p * LD + r], ipiv);
    __syncwarp();
    for (int e = lane; e < P; e += 32) {
      const unsigned v = list[e];
      const int r = (int)(v >> 8), c = (int)(v & 0xffu);
      A[r * LD + c] = __fma_rn(-A[r * LD + p], A[p * LD + c], A[r * LD + c]);
    }
    __syncwarp();
    P -= E - p;  // drop row p + 1
  }
  for (int r = E - 1; r >= 0; --r) {
    if (lane == 0) A[r * LD + E] = __ddiv_rn(A[r * LD + E], A[r * LD + r]);
    __syncwarp();
    const double x = A[r * LD + E];
    for (int q = lane; q < r; q += 32) A[q * LD + E] = __fma_rn(-A[q * LD + r], x, A[q * LD + E]);
    __syncwarp();
  }
  for (int a = lane; a < E; a += 32) Wr[a] = A[a * LD + E];
}

// AdaptModelMLLR (OL_ModelAdapt.cpp:1597-1608) for every (speaker, component): mu' = A mu + b.
// One warp per (speaker, component); speakers whose transform failed keep the UBM means.
__global__ void mllr_batch_apply_kernel(int S, int M, int D, const float* __restrict__ mu,
                                        const double* __restrict__ W, const int* __restrict__ status,
                                        float* __restrict__ out) {
  const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= (long long)S * M) return;
  const int s = (int)(t / M), m = (int)(t - (long long)s * M);
  const int E = D + 1;
  const float* row = mu + (size_t)m * D;
  for (int k = lane; k < D; k += 32) {
    float r = row[k];
    if (status[s] == GMM_OK) {
      const double* Wk = W + ((size_t)s * D + k) * E;
      double v = 0.0;
      for (int kk = 0; kk < D; ++kk) v = __dadd_rn(v, __dmul_rn(Wk[kk], (double)row[kk]));
      r = (float)__dadd_rn(v, Wk[D]);
    }
    out[(size_t)t * D + k] = r;
  }
}

// IterEM keeps a copy of the model and UpdateModelMAP restores it when no component survives
// (OL_ModelAdapt.cpp:1276-1296): the device-side form for a captured iteration.
__global__ void em_restore_kernel(int M, int D, const int* __restrict__ flag, float* __restrict__ w,
                                  float* __restrict__ mu, float* __restrict__ var,
                                  const float* __restrict__ bw, const float* __restrict__ bmu,
                                  const float* __restrict__ bvar) {
  if (flag[2] != 0) return;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < M) w[t] = bw[t];
  if (t < (long long)M * D) {
    mu[t] = bmu[t];
    var[t] = bvar[t];
  }
}

// hist[counter] = total LL of the statistics; ++counter (the counter is the last element).
__global__ void ll_record_kernel(const double* __restrict__ tot, double* __restrict__ hist, int cap) {
  const int k = (int)hist[cap];
  if (k < cap) hist[k] = *tot;
  hist[cap] = (double)(k + 1);
}

}  // namespace

int mstep_em(Ctx* c, int upW, int upM, int upV, int* alive) {
  if (!c->stats_valid) return fail(c, GMM_ERR_STATE, "no statistics accumulated");
  double* nind = nullptr;
  if (c->robust && c->aux_valid) {  // UpdateModelEM with _robustCov: MakeRobustStats first
    const int rc = robust_make(c, c->M, c->D, 0, c->stats, c->aux, &nind);
    if (rc) return rc;
    c->aux_valid = false;
  }
  cudaMemsetAsync(c->flag + 5, 0, 2 * sizeof(int), c->stream);
  unsigned int tot = (unsigned int)c->tot_frames;
  {
    GMM_LAUNCH(c, "em_comp_kernel");
    em_comp_kernel<<<(c->M + 127) / 128, 128, 0, c->stream>>>(
        c->M, c->D, c->w, c->mu, c->var, c->stats, tot, upW, upM, upV, c->min_var, nind, c->flag,
        c->precision == GMM_PREC_TC);
  }
  {
    GMM_LAUNCH(c, "em_norm_kernel");
    em_norm_kernel<<<1, 1024, 0, c->stream>>>(c->M, c->w, c->flag);
  }
  c->model_dirty = true;
  c->tcx_valid = c->tcx_valid;  // features unaffected
  if (alive) {
    cudaError_t e = cudaMemcpyAsync(c->hflag, c->flag, 8 * sizeof(int), cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpyAsync(flags)");
    int rc = sync(c, "EM update");
    if (rc) return rc;
    *alive = c->hflag[2];
  }
  return GMM_OK;
}

int mstep_map(Ctx* c, int tau, int upW, int upM, int upV) {
  if (!c->stats_valid) return fail(c, GMM_ERR_STATE, "no statistics accumulated");
  if (!c->have_prior) return fail(c, GMM_ERR_STATE, "MAP needs a prior model (gmm_set_prior)");
  if (c->robust && c->aux_valid) {  // UpdateModelMAP with _robustCov: MakeRobustStats first
    double* nind = nullptr;
    const int rc = robust_make(c, c->M, c->D, 0, c->stats, c->aux, &nind);
    if (rc) return rc;
    c->aux_valid = false;
  }
  unsigned int tot = (unsigned int)c->tot_frames;
  // adapted weights scratch: reuse the logW buffer (recomputed by the next precompute)
  {
    GMM_LAUNCH(c, "map_comp_kernel");
    map_comp_kernel<<<(c->M + 127) / 128, 128, 0, c->stream>>>(
        c->M, c->D, c->w, c->mu, c->var, c->pw, c->pmu, c->pvar, c->stats, tot, tau, upW, upM,
        upV, c->min_var, c->logW, c->precision == GMM_PREC_TC);
  }
  {
    GMM_LAUNCH(c, "map_norm_kernel");
    map_norm_kernel<<<1, 1024, 0, c->stream>>>(c->M, c->w, c->logW, c->pw, c->stats, upW, tot);
  }
  c->model_dirty = true;
  return GMM_OK;
}

int mstep_rearrange(Ctx* c) {
  GMM_LAUNCH(c, "rearrange_kernel");
  rearrange_kernel<<<1, 1024, 0, c->stream>>>(c->M, c->D, c->w, c->mu, c->var, c->bw, c->bmu,
                                               c->bvar, c->act);
  c->model_dirty = true;
  return GMM_OK;
}

int mstep_mllr(Ctx* c, int ubm_init, double* W_host) {
  if (!c->stats_valid) return fail(c, GMM_ERR_STATE, "no statistics accumulated");
  if (!(c->acc_flags & GMM_ACC_MEAN)) return fail(c, GMM_ERR_STATE, "MLLR needs mean statistics");
  const int D = c->D, M = c->M, E = D + 1;
  if (ubm_init && !c->have_prior) return fail(c, GMM_ERR_STATE, "MLLR UBM init needs a prior model");
  double* dW = nullptr;
  int rc = dalloc(c, (void**)&dW, sizeof(double) * ((size_t)D * E + 2), "MLLR transform");
  if (rc) return rc;
  {
    GMM_LAUNCH(c, "mllr_check_kernel");
    mllr_check_kernel<<<1, 32, 0, c->stream>>>(M, c->stats, dW + (size_t)D * E);
  }
  double chk[2];
  cudaMemcpyAsync(chk, dW + (size_t)D * E, sizeof(chk), cudaMemcpyDeviceToHost, c->stream);
  rc = sync(c, "MLLR check");
  if (rc) { dfree(c, dW, sizeof(double) * ((size_t)D * E + 2)); return rc; }
  if (M < E || chk[0] < E || chk[1] * D < (double)D * E) {
    dfree(c, dW, sizeof(double) * ((size_t)D * E + 2));
    return fail(c, GMM_ERR_MLLR, "CheckInvertibility(): not enough components or data for a D x (D+1) MLLR transform");
  }
  size_t smem = sizeof(double) * ((size_t)E * E + E);
  if (smem > 200 * 1024) {
    dfree(c, dW, sizeof(double) * ((size_t)D * E + 2));
    return fail(c, GMM_ERR_UNSUPPORTED, "MLLR: D too large for the shared-memory solve");
  }
  cudaFuncSetAttribute(mllr_row_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  {
    GMM_LAUNCH(c, "mllr_row_kernel");
    const float* umu = c->have_prior ? c->pmu : c->mu;
    const float* uvar = c->have_prior ? c->pvar : c->var;
    mllr_row_kernel<<<D, 256, smem, c->stream>>>(M, D, c->mu, c->var, umu, uvar, c->stats,
                                                 ubm_init, c->min_var, dW);
  }
  cudaError_t e = cudaMemcpyAsync(W_host, dW, sizeof(double) * (size_t)D * E,
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) { dfree(c, dW, 0); return cuda_fail(c, e, "cudaMemcpyAsync(W)"); }
  rc = sync(c, "MLLR solve");
  dfree(c, dW, sizeof(double) * ((size_t)D * E + 2));
  return rc;
}

int mstep_mllr_apply(Ctx* c, const double* W_host) {
  const int D = c->D, E = D + 1;
  double* dW = nullptr;
  int rc = dalloc(c, (void**)&dW, sizeof(double) * (size_t)D * E, "MLLR transform");
  if (rc) return rc;
  cudaMemcpyAsync(dW, W_host, sizeof(double) * (size_t)D * E, cudaMemcpyHostToDevice, c->stream);
  {
    GMM_LAUNCH(c, "mllr_apply_kernel");
    mllr_apply_kernel<<<c->M, 64, sizeof(float) * D, c->stream>>>(c->M, D, c->mu, dW);
  }
  rc = sync(c, "MLLR apply");
  dfree(c, dW, sizeof(double) * (size_t)D * E);
  c->model_dirty = true;
  return rc;
}

int mstep_map_batch(Ctx* c, const MapBatch& b, const double* plain, const SpeakerStats* ss) {
  const long long tot = (long long)b.S * c->M;
  if (tot == 0) return GMM_OK;
  {
    GMM_LAUNCH(c, "map_batch_kernel");
    const size_t smem = sizeof(float) * 2 * kMapPairs * (size_t)(c->D + 1);
    cudaFuncSetAttribute(map_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    map_batch_kernel<<<(unsigned)((tot + kMapPairs - 1) / kMapPairs), kMapThreads, smem, c->stream>>>(
        b.S, c->M, c->D, plain, ss ? ss->part : nullptr, ss ? ss->K : 0, ss ? ss->n_chunks : 0,
        ss ? ss->piece0 : nullptr, ss ? ss->npieces : nullptr, ss ? ss->row_of_comp : nullptr,
        ss ? ss->cent : nullptr, b.d_offs, c->w, c->mu, c->var, b.tau, b.upW, b.upM, b.upV, c->min_var, b.w, b.mu, b.var, b.aw, b.ll);
  }
  if (b.upW) {
    GMM_LAUNCH(c, "map_batch_norm_kernel");
    map_batch_norm_kernel<<<(b.S + 7) / 8, 256, 0, c->stream>>>(b.S, c->M, b.aw, b.w);
  }
  return GMM_OK;
}

// Batched global MLLR: per-speaker statistics (plain layout or tensor-core pieces) -> dense n, F
// -> invertibility check -> G and k data terms as FP32-product GEMMs with FP64 sums (+ the UBM
// prior terms when ubm_init) -> FP64 Gauss-Jordan solves -> optional adapted means. The resident
// model is the UBM. dW [S][D][D+1], dstatus [S], dmu_out [S][M][D] or null.
int mstep_mllr_batch(Ctx* c, int S, const double* plain, const SpeakerStats* ss, int ubm_init, double* dW,
                     int* dstatus, float* dmu_out, double* dll) {
  const int M = c->M, D = c->D, E = D + 1, T = E * (E + 1) / 2;
  if (S == 0) return GMM_OK;
  const float* umu = c->mu;
  const float* uvar = c->var;
  double *n = nullptr, *F = nullptr, *Gd = nullptr, *kd = nullptr, *Gp = nullptr, *kp = nullptr;
  float *B = nullptr, *Xi = nullptr;
  const size_t bn = sizeof(double) * (size_t)S * M, bF = bn * D, bG = sizeof(double) * (size_t)S * D * T;
  const size_t bk = sizeof(double) * (size_t)S * D * E, bB = sizeof(float) * (size_t)M * T;
  const size_t bXi = sizeof(float) * (size_t)M * E;
  const size_t bGp = sizeof(double) * (size_t)D * T, bkp = sizeof(double) * (size_t)D * E;
  int rc = scratch(c, SC_MLLR_N, bn, "MLLR n", (void**)&n);
  if (!rc) rc = scratch(c, SC_MLLR_F, bF, "MLLR F", (void**)&F);
  if (!rc) rc = scratch(c, SC_MLLR_G, bG, "MLLR G", (void**)&Gd);
  if (!rc) rc = scratch(c, SC_MLLR_K, bk, "MLLR k", (void**)&kd);
  if (!rc) rc = scratch(c, SC_MLLR_B, bB, "MLLR outer products", (void**)&B);
  if (!rc) rc = scratch(c, SC_MLLR_XI, bXi, "MLLR extended means", (void**)&Xi);
  if (!rc && ubm_init) rc = scratch(c, SC_MLLR_GP, bGp, "MLLR prior G", (void**)&Gp);
  if (!rc && ubm_init) rc = scratch(c, SC_MLLR_KP, bkp, "MLLR prior k", (void**)&kp);
  const size_t smem = solve_smem(E);
  if (!rc && smem > 200 * 1024) rc = fail(c, GMM_ERR_UNSUPPORTED, "MLLR: D too large for the shared-memory solve");
  const long long tot = (long long)S * M;
  if (!rc) {
    {
      GMM_LAUNCH(c, "mllr_gather_kernel");
      mllr_gather_kernel<<<(unsigned)((tot + kGatherThreads - 1) / kGatherThreads), kGatherThreads,
                           sizeof(double) * kGatherThreads * (D | 1), c->stream>>>(
          S, M, D, plain, ss ? ss->part : nullptr, ss ? ss->K : 0, ss ? ss->n_chunks : 0, ss ? ss->piece0 : nullptr,
          ss ? ss->npieces : nullptr, ss ? ss->row_of_comp : nullptr, ss ? ss->cent : nullptr, n, F, dll);
    }
    {
      GMM_LAUNCH(c, "mllr_batch_check_kernel");
      mllr_batch_check_kernel<<<(S + 7) / 8, 256, 0, c->stream>>>(S, M, D, n, dstatus);
    }
    if (c->precision != GMM_PREC_TC) {
      GMM_LAUNCH(c, "mllr_outer_kernel");
      mllr_outer_kernel<<<(unsigned)(((long long)M * T + 255) / 256), 256, 0, c->stream>>>(M, D, umu, B);
    }
    {
      GMM_LAUNCH(c, "mllr_xi_kernel");
      mllr_xi_kernel<<<(unsigned)(((long long)M * E + 255) / 256), 256, 0, c->stream>>>(M, D, umu, Xi);
    }
    if (c->precision == GMM_PREC_TC) {
      // G data term on the tensor cores (split-bf16 operands, FP32 products)
      rc = tc_mllr_g(c, S, n, Gd);
    } else {
      // G data term: coef = n[s][m]
      GMM_LAUNCH(c, "mllr_gemm_kernel");
      dim3 grid((T + 63) / 64, (S + 127) / 128, D);
      mllr_gemm_kernel<<<grid, 256, 0, c->stream>>>(S, M, D, T, n, (long long)M, 1, 0, uvar, B, T, Gd);
    }
  }
  if (!rc) {
    {
      // k data term: coef = F[s][m][i]
      GMM_LAUNCH(c, "mllr_k_kernel");
      const int threads = mllr_k_threads(D);
      const size_t ksmem = sizeof(float) * kMllrKChunk * (size_t)(((D + 3) / 4) * 4 + ((E + 3) / 4) * 4);
      mllr_k_kernel<<<S, threads, ksmem, c->stream>>>(S, M, D, F, uvar, Xi, kd);
    }
    if (ubm_init) {
      GMM_LAUNCH(c, "mllr_prior_kernel");
      mllr_prior_kernel<<<D, 256, 0, c->stream>>>(M, D, umu, uvar, c->min_var, Gp, kp);
    }
    cudaFuncSetAttribute(mllr_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    {
      GMM_LAUNCH(c, "mllr_solve_kernel");
      const long long nsys = (long long)S * D;
      mllr_solve_kernel<<<(unsigned)((nsys + kSolveWarps - 1) / kSolveWarps), 32 * kSolveWarps, smem, c->stream>>>(
          S, D, Gd, kd, Gp, kp, dstatus, dW);
    }
    if (dmu_out) {
      GMM_LAUNCH(c, "mllr_batch_apply_kernel");
      mllr_batch_apply_kernel<<<(unsigned)((tot + 7) / 8), 256, 0, c->stream>>>(S, M, D, umu, dW, dstatus, dmu_out);
    }
    rc = sync(c, "batched MLLR");
    if (!rc && c->precision == GMM_PREC_TC && c->tc_err) {
      int herr = 0;
      cudaMemcpy(&herr, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost);
      if (herr) {
        cudaMemset(c->tc_err, 0, sizeof(int));
        rc = fail(c, GMM_ERR_TIMEOUT, "batched MLLR: a bounded device wait expired");
      }
    }
  }
  return rc;
}

int mstep_em_restore(Ctx* c) {
  GMM_LAUNCH(c, "em_restore_kernel");
  const long long tot = (long long)c->M * c->D;
  em_restore_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(c->M, c->D, c->flag, c->w, c->mu,
                                                                          c->var, c->bw, c->bmu, c->bvar);
  return GMM_OK;
}

int record_iteration_ll(Ctx* c) {
  GMM_LAUNCH(c, "ll_record_kernel");
  ll_record_kernel<<<1, 1, 0, c->stream>>>(c->stats + (size_t)c->M * (1 + 2 * c->D), c->ll_hist, c->ll_hist_cap);
  return GMM_OK;
}

}  // namespace gmm
