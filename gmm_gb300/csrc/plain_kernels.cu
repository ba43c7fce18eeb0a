// Plain FP32 E-step: a replica of the reference CPU estimator's float arithmetic on SIMT cores.
//
// Semantics followed (GMM/lib_bmssr/trainer/OL_GMMStatsEstimator.cpp):
//   insertModel :234-313        icov = 1/var, logGconst = -D/2 log(2 pi) - 1/2 sum log var
//                               (float sum), logW = log w
//   computeMixLogLike :563-588  e = sum_d ((x-mu)*(x-mu))*icov in float, sequential over d;
//                               ll = logGconst - 0.5f*e; non-finite -> minLogLike
//   getLikeAndGammas :444-510   g = ll + logW; frame LL by sequential addLog (:1449-1458,
//                               15-nat cutoff) in component order; all at minLogLike ->
//                               stability trouble, LL = minLogLike
//   compGammas :515-558         gamma = (g > minLL) * exp(g - LL); one component -> 1;
//                               stability trouble -> minGamma
//   accumulateStats(vec) :1334-1378  gamma <= minGamma skipped; n += gamma, F += gamma*x,
//                               S += (gamma*x)*x: float products, double sums
// Every float operation is written with an explicit round-to-nearest intrinsic so the compiler
// cannot fuse a multiply and an add: the results round exactly as the x86-64 reference build
// does. The remaining difference from the reference is the last-ulp behaviour of expf/logf.
//
// Design (GB300, one GPU): kernel ll_kernel runs one thread per frame with the frame in
// registers and the component parameters broadcast from shared memory; it writes the raw log
// posteriors of a frame chunk component-major [Mact][chunk] and the frame LL. Kernel
// stats_kernel runs one warp per (component, frame slice): lanes evaluate 32 posteriors at
// once, a ballot picks the kept ones, and the warp accumulates their FP64 statistics over the
// feature row (lanes split the dimensions). Per-slice FP64 partials are summed in a fixed
// order by reduce_kernel, so results do not depend on scheduling.
#include <math.h>

#include "gmm_internal.cuh"

namespace gmm {

namespace {

constexpr int kCompTile = 32;

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Ordered list of components with w > 0 (one warp; M <= 32767).
__global__ void active_list_kernel(int M, const float* __restrict__ w, int* __restrict__ act,
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

// insertModel numerics, one thread per component.
__global__ void precompute_kernel(int M, int D, const float* __restrict__ w,
                                  const float* __restrict__ var, float min_var, float minLL,
                                  float* __restrict__ icov, float* __restrict__ logG,
                                  float* __restrict__ logW, int* __restrict__ flag) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  float wm = w[m];
  logW[m] = (wm > 0.0f) ? (float)log((double)wm) : minLL;
  if (!(wm > 0.0f)) { logG[m] = 0.0f; return; }
  float acc = 0.0f;
  for (int d = 0; d < D; ++d) {
    float v = var[(size_t)m * D + d];
    if (v < min_var) atomicExch(&flag[0], 1);
    icov[(size_t)m * D + d] = __fdiv_rn(1.0f, v);
    acc = __fadd_rn(acc, (float)log((double)v));
  }
  logG[m] = (float)(kMinusLog2Pi * D / 2 - (double)__fdiv_rn(acc, 2.0f));
}

__device__ __forceinline__ void add_log(float& p1, float p2) {
  if (__fsub_rn(p1, 15.0f) > p2) return;
  if (p1 > p2) p1 = __fadd_rn(p1, logf(__fadd_rn(1.0f, expf(__fsub_rn(p2, p1)))));
  else p1 = __fadd_rn(p2, logf(__fadd_rn(1.0f, expf(__fsub_rn(p1, p2)))));
}

// One thread per frame. DP = D padded to a multiple of 4 (padding contributes exact zeros).
template <int DP>
__global__ void __launch_bounds__(256) ll_kernel(
    const float* __restrict__ X, long long f0, long long nf, int D, int Mact,
    const int* __restrict__ act, const float* __restrict__ mu, const float* __restrict__ icov,
    const float* __restrict__ logG, const float* __restrict__ logW, float minLL,
    float* __restrict__ G, long long ldg, float* __restrict__ ll, double* __restrict__ llpart,
    int* __restrict__ flag) {
  constexpr int Q = DP / 4;
  __shared__ float4 s_par[kCompTile][2 * Q];
  __shared__ float s_c[kCompTile], s_lw[kCompTile];
  __shared__ double s_red[8];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < nf;
  float x[DP];
#pragma unroll
  for (int d = 0; d < DP; ++d) x[d] = (valid && d < D) ? X[(size_t)(f0 + i) * D + d] : 0.0f;

  float maxLL = minLL, sumLL = minLL;
  for (int t0 = 0; t0 < Mact; t0 += kCompTile) {
    const int nt = min(kCompTile, Mact - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < nt * DP; e += blockDim.x) {
      int j = e / DP, d = e - j * DP;
      int m = act[t0 + j];
      float mv = d < D ? mu[(size_t)m * D + d] : 0.0f;
      float iv = d < D ? icov[(size_t)m * D + d] : 0.0f;
      float* row = reinterpret_cast<float*>(&s_par[j][0]);
      row[(d >> 2) * 8 + (d & 3)] = mv;
      row[(d >> 2) * 8 + 4 + (d & 3)] = iv;
    }
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
      int m = act[t0 + j];
      s_c[j] = logG[m];
      s_lw[j] = logW[m];
    }
    __syncthreads();
    for (int j = 0; j < nt; ++j) {
      float e = 0.0f;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        float4 mq = s_par[j][2 * q], iq = s_par[j][2 * q + 1];
        float t;
        t = __fsub_rn(x[4 * q + 0], mq.x); t = __fmul_rn(t, t); t = __fmul_rn(t, iq.x); e = __fadd_rn(e, t);
        t = __fsub_rn(x[4 * q + 1], mq.y); t = __fmul_rn(t, t); t = __fmul_rn(t, iq.y); e = __fadd_rn(e, t);
        t = __fsub_rn(x[4 * q + 2], mq.z); t = __fmul_rn(t, t); t = __fmul_rn(t, iq.z); e = __fadd_rn(e, t);
        t = __fsub_rn(x[4 * q + 3], mq.w); t = __fmul_rn(t, t); t = __fmul_rn(t, iq.w); e = __fadd_rn(e, t);
      }
      float s = __fsub_rn(s_c[j], __fmul_rn(0.5f, e));
      if (!isfinite(s)) s = minLL;
      float g = __fadd_rn(s, s_lw[j]);
      if (G != nullptr && valid) G[(size_t)(t0 + j) * ldg + i] = g;
      if (maxLL < g) maxLL = g;
      add_log(sumLL, g);
    }
  }
  float l = (maxLL == minLL) ? minLL : sumLL;
  if (valid) {
    if (maxLL == minLL) flag[1] = 1;
    ll[f0 + i] = l;
  }
  double v = warp_sum(valid ? (double)l : 0.0);
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += s_red[k];
    llpart[blockIdx.x] = t;
  }
}

// Generic fallback for D > 128: the frame is re-read from global memory (L1 resident).
__global__ void __launch_bounds__(256) ll_kernel_large(
    const float* __restrict__ X, long long f0, long long nf, int D, int Mact,
    const int* __restrict__ act, const float* __restrict__ mu, const float* __restrict__ icov,
    const float* __restrict__ logG, const float* __restrict__ logW, float minLL,
    float* __restrict__ G, long long ldg, float* __restrict__ ll, double* __restrict__ llpart,
    int* __restrict__ flag) {
  __shared__ double s_red[8];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < nf;
  const float* x = X + (size_t)(f0 + (valid ? i : 0)) * D;
  float maxLL = minLL, sumLL = minLL;
  for (int j = 0; j < Mact; ++j) {
    int m = act[j];
    const float* mm = mu + (size_t)m * D;
    const float* ic = icov + (size_t)m * D;
    float e = 0.0f;
    for (int d = 0; d < D; ++d) {
      float t = __fsub_rn(x[d], mm[d]);
      t = __fmul_rn(t, t);
      t = __fmul_rn(t, ic[d]);
      e = __fadd_rn(e, t);
    }
    float s = __fsub_rn(logG[m], __fmul_rn(0.5f, e));
    if (!isfinite(s)) s = minLL;
    float g = __fadd_rn(s, logW[m]);
    if (G != nullptr && valid) G[(size_t)j * ldg + i] = g;
    if (maxLL < g) maxLL = g;
    add_log(sumLL, g);
  }
  float l = (maxLL == minLL) ? minLL : sumLL;
  if (valid) {
    if (maxLL == minLL) flag[1] = 1;
    ll[f0 + i] = l;
  }
  double v = warp_sum(valid ? (double)l : 0.0);
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += s_red[k];
    llpart[blockIdx.x] = t;
  }
}

// One warp per (active component j, frame slice s). DW = ceil(D / 32) dims per lane.
template <int DW>
__global__ void __launch_bounds__(128) stats_kernel(
    const float* __restrict__ X, long long f0, long long nf, int D, int Mact,
    const float* __restrict__ G, long long ldg, const float* __restrict__ ll, float minLL,
    float minGamma, int single_comp, int flags, int slices, long long slice_len,
    double* __restrict__ part) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x;
  const int s = blockIdx.y * (blockDim.x >> 5) + warp;
  if (s >= slices) return;
  const bool fm = (flags & GMM_ACC_MEAN) != 0, fv = (flags & GMM_ACC_VAR) != 0;
  const bool probs_only = (flags & GMM_ACC_PROBS_ONLY) != 0;
  const long long a = (long long)s * slice_len;
  const long long b = min(nf, a + slice_len);
  double n = 0.0, F[DW], S[DW];
#pragma unroll
  for (int q = 0; q < DW; ++q) F[q] = S[q] = 0.0;
  const float* Gj = G + (size_t)j * ldg;
  for (long long f = a; f < b; f += 32) {
    const long long fi = f + lane;
    float gam = 0.0f;
    bool kept = false;
    if (fi < b) {
      float g = Gj[fi];
      float l = ll[f0 + fi];
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
      n += (double)gb;
      if (probs_only) continue;
      const float* xr = X + (size_t)(f0 + f + src) * D;
#pragma unroll
      for (int q = 0; q < DW; ++q) {
        int d = lane + 32 * q;
        if (d < D) {
          float xv = xr[d];
          float p = __fmul_rn(gb, xv);
          if (fm) F[q] += (double)p;
          if (fv) S[q] += (double)__fmul_rn(p, xv);
        }
      }
    }
  }
  double* out = part + ((size_t)s * Mact + j) * (size_t)(1 + 2 * D);
  if (lane == 0) out[0] = n;
#pragma unroll
  for (int q = 0; q < DW; ++q) {
    int d = lane + 32 * q;
    if (d < D) {
      out[1 + d] = F[q];
      out[1 + D + d] = S[q];
    }
  }
}

// stats[n | F | S] (caller order) += sum over slices of part (fixed order).
__global__ void reduce_kernel(int M, int D, int Mact, const int* __restrict__ act, int slices,
                              const double* __restrict__ part, double* __restrict__ stats) {
  const int E = 1 + 2 * D;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)Mact * E) return;
  int j = (int)(t / E), e = (int)(t - (long long)j * E);
  double s = 0.0;
  for (int k = 0; k < slices; ++k) s += part[((size_t)k * Mact + j) * E + e];
  int m = act[j];
  size_t dst;
  if (e == 0) dst = (size_t)m;
  else if (e <= D) dst = (size_t)M + (size_t)m * D + (e - 1);
  else dst = (size_t)M + (size_t)M * D + (size_t)m * D + (e - 1 - D);
  stats[dst] += s;
}

// stats[tot] += sum of block partials (single block, fixed order).
__global__ void ll_total_kernel(int nblocks, const double* __restrict__ llpart,
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

template <int DP>
void launch_ll(Ctx* c, long long f0, long long nf, float* G, long long ldg, float* llout,
               int blocks) {
  GMM_LAUNCH(c, "plain_ll_kernel");
  ll_kernel<DP><<<blocks, 256, 0, c->stream>>>(c->X, f0, nf, c->D, c->Mact, c->act, c->mu,
                                                c->icov, c->logG, c->logW, c->minLL, G, ldg,
                                                llout, c->llpart, c->flag);
}

template <int DW>
void launch_stats(Ctx* c, long long f0, long long nf, long long ldg, int flags, int slices,
                  long long slice_len) {
  GMM_LAUNCH(c, "plain_stats_kernel");
  dim3 grid(c->Mact, (slices + 3) / 4);
  stats_kernel<DW><<<grid, 128, 0, c->stream>>>(c->X, f0, nf, c->D, c->Mact, c->logits, ldg,
                                                c->ll, c->minLL, c->minGamma, c->Mact == 1,
                                                flags, slices, slice_len, c->part);
}

}  // namespace

int plain_precompute_async(Ctx* c) {
  {
    GMM_LAUNCH(c, "active_list_kernel");
    active_list_kernel<<<1, 32, 0, c->stream>>>(c->M, c->w, c->act, c->flag + 4);
  }
  {
    GMM_LAUNCH(c, "precompute_kernel");
    precompute_kernel<<<(c->M + 127) / 128, 128, 0, c->stream>>>(
        c->M, c->D, c->w, c->var, c->min_var, c->minLL, c->icov, c->logG, c->logW, c->flag);
  }
  return GMM_OK;
}

int plain_precompute(Ctx* c) {
  {
    GMM_LAUNCH(c, "active_list_kernel");
    active_list_kernel<<<1, 32, 0, c->stream>>>(c->M, c->w, c->act, c->flag + 4);
  }
  {
    GMM_LAUNCH(c, "precompute_kernel");
    precompute_kernel<<<(c->M + 127) / 128, 128, 0, c->stream>>>(
        c->M, c->D, c->w, c->var, c->min_var, c->minLL, c->icov, c->logG, c->logW, c->flag);
  }
  cudaError_t e = cudaMemcpyAsync(c->hflag, c->flag, 8 * sizeof(int), cudaMemcpyDeviceToHost,
                                  c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpyAsync(flags)");
  int rc = sync(c, "model precompute");
  if (rc) return rc;
  c->Mact = c->hflag[4];
  if (c->hflag[0]) {
    // insertModel throws on a variance below min_var (OL_GMMStatsEstimator.cpp:287-296)
    cudaMemsetAsync(c->flag, 0, sizeof(int), c->stream);
    return fail(c, GMM_ERR_MODEL, "insertModel(): model contains very low variances (< min_var)");
  }
  c->model_dirty = false;
  return GMM_OK;
}

// The diagonal model's log joints of frames [f0, f0 + nf): raw values into G [Mact][ldg] (when
// G is not null), frame LLs into llout[f0 + i], per-256-frame-block LL partials into c->llpart.
// Returns the number of blocks.
int plain_ll_chunk(Ctx* c, long long f0, long long nf, float* G, long long ldg, float* llout) {
  const int D = c->D;
  const int blocks = (int)((nf + 255) / 256);
  if (D <= 16) launch_ll<16>(c, f0, nf, G, ldg, llout, blocks);
  else if (D <= 32) launch_ll<32>(c, f0, nf, G, ldg, llout, blocks);
  else if (D <= 40) launch_ll<40>(c, f0, nf, G, ldg, llout, blocks);
  else if (D <= 64) launch_ll<64>(c, f0, nf, G, ldg, llout, blocks);
  else if (D <= 128) launch_ll<128>(c, f0, nf, G, ldg, llout, blocks);
  else {
    GMM_LAUNCH(c, "plain_ll_kernel_large");
    ll_kernel_large<<<blocks, 256, 0, c->stream>>>(c->X, f0, nf, D, c->Mact, c->act, c->mu, c->icov,
                                                   c->logG, c->logW, c->minLL, G, ldg, llout, c->llpart,
                                                   c->flag);
  }
  return blocks;
}

// One E-step over the resident features. want_stats: accumulate statistics into c->stats
// (zeroed by the caller); ll_out_dev: optional per-frame LL destination (device, N floats).
int plain_estep(Ctx* c, int flags, bool want_stats, float* ll_out_dev) {
  const long long N = c->N;
  const int D = c->D;
  if (c->Mact <= 0) return fail(c, GMM_ERR_STATE, "no component with non-zero weight");
  // frame chunk so that the log-posterior buffer stays within 4 GiB
  const size_t budget = (size_t)4 << 30;
  long long chunk = want_stats ? (long long)(budget / ((size_t)c->Mact * sizeof(float))) : N;
  chunk = chunk / 256 * 256;
  if (chunk < 256) chunk = 256;
  if (chunk > N) chunk = N;
  if (want_stats) {
    size_t need = (size_t)c->Mact * (size_t)chunk * sizeof(float);
    if (need > c->logits_cap) {
      dfree(c, c->logits, c->logits_cap);
      c->logits = nullptr;
      c->logits_cap = 0;
      int rc = dalloc(c, (void**)&c->logits, need, "log-posterior buffer");
      if (rc) return rc;
      c->logits_cap = need;
    }
  }
  float* llbuf = ll_out_dev ? ll_out_dev : c->ll;
  const int E = 1 + 2 * D;
  for (long long f0 = 0; f0 < N; f0 += chunk) {
    const long long nf = (N - f0 < chunk) ? N - f0 : chunk;
    const int blocks = (int)((nf + 255) / 256);
    if ((size_t)blocks > c->llpart_cap) return fail(c, GMM_ERR_STATE, "llpart too small");
    plain_ll_chunk(c, f0, nf, want_stats ? c->logits : nullptr, chunk, llbuf);
    if (want_stats) {
      GMM_LAUNCH(c, "ll_total_kernel");
      ll_total_kernel<<<1, 1024, 0, c->stream>>>(blocks, c->llpart,
                                                  c->stats + (size_t)c->M * (1 + 2 * D));
    }
    if (!want_stats) continue;
    // frame slices: aim for ~64 warps per SM in total, at least 256 frames per slice
    long long target = 152LL * 64 / c->Mact;
    long long slices = target < 1 ? 1 : target;
    if (slices > nf / 256) slices = nf / 256;
    if (slices < 1) slices = 1;
    slices = (slices + 3) / 4 * 4;
    long long slice_len = (nf + slices - 1) / slices;
    slice_len = (slice_len + 31) / 32 * 32;
    size_t need = (size_t)slices * c->Mact * E * sizeof(double);
    if (need > c->part_cap) {
      dfree(c, c->part, c->part_cap);
      c->part = nullptr;
      c->part_cap = 0;
      int rc = dalloc(c, (void**)&c->part, need, "partial statistics");
      if (rc) return rc;
      c->part_cap = need;
    }
    const int DW = (D + 31) / 32;
    switch (DW) {
      case 1: launch_stats<1>(c, f0, nf, chunk, flags, (int)slices, slice_len); break;
      case 2: launch_stats<2>(c, f0, nf, chunk, flags, (int)slices, slice_len); break;
      case 3: launch_stats<3>(c, f0, nf, chunk, flags, (int)slices, slice_len); break;
      case 4: launch_stats<4>(c, f0, nf, chunk, flags, (int)slices, slice_len); break;
      default:
        if (DW <= 8) launch_stats<8>(c, f0, nf, chunk, flags, (int)slices, slice_len);
        else if (DW <= 16) launch_stats<16>(c, f0, nf, chunk, flags, (int)slices, slice_len);
        else launch_stats<32>(c, f0, nf, chunk, flags, (int)slices, slice_len);
    }
    {
      GMM_LAUNCH(c, "reduce_kernel");
      long long tot = (long long)c->Mact * E;
      reduce_kernel<<<(int)((tot + 255) / 256), 256, 0, c->stream>>>(
          c->M, D, c->Mact, c->act, (int)slices, c->part, c->stats);
    }
    if (c->robust && c->aux) {
      const int rc = robust_chunk(c, c->M, D, c->Mact, c->act, f0, nf, chunk, c->aux);
      if (rc) return rc;
    }
  }
  return GMM_OK;
}

// Per-speaker FP32-path statistics: one plain E-step per speaker over its frame range (the
// reference's one-speaker-at-a-time AdaptModel loop, projects/Model_ADAPT/Model_ADAPT.cpp:170-240),
// each into its own block [n (M) | F (M x D) | S (M x D) | totLL | pad].
int plain_speaker_stats(Ctx* c, int S, const long long* offs, int flags, double** out, size_t* bytes) {
  const int M = c->M, D = c->D;
  const size_t stride = (size_t)M * (1 + 2 * D) + 2;
  *bytes = sizeof(double) * stride * (size_t)(S > 0 ? S : 1);
  *out = nullptr;
  int rc = dalloc(c, (void**)out, *bytes, "per-speaker statistics");
  if (rc) return rc;
  double* d_stats = *out;
  cudaMemsetAsync(d_stats, 0, *bytes, c->stream);
  const float* X0 = c->X;
  const long long N0 = c->N;
  double* stats0 = c->stats;
  for (int s = 0; s < S && !rc; ++s) {
    c->X = X0 + (size_t)offs[s] * D;
    c->N = offs[s + 1] - offs[s];
    c->stats = d_stats + (size_t)s * stride;
    if (c->N > 0) rc = plain_estep(c, flags, true, nullptr);
  }
  c->X = X0;
  c->N = N0;
  c->stats = stats0;
  if (rc) {
    cudaStreamSynchronize(c->stream);
    dfree(c, *out, *bytes);
    *out = nullptr;
  }
  return rc;
}

// Batched MAP with FP32 statistics: the per-speaker plain E-steps, then one M-step launch for all.
int plain_map_batch(Ctx* c, const MapBatch& b) {
  double* d_stats = nullptr;
  size_t bytes = 0;
  int rc = plain_speaker_stats(c, b.S, b.offs, b.flags, &d_stats, &bytes);
  if (rc) return rc;
  rc = mstep_map_batch(c, b, d_stats, nullptr);
  if (!rc) rc = sync(c, "batched MAP (FP32 statistics)");
  cudaStreamSynchronize(c->stream);
  dfree(c, d_stats, bytes);
  return rc;
}

}  // namespace gmm

// ---------------------------------------------------------------------------------------------
// Allocation-free E-step (gmm_accumulate_noalloc). Some callers cannot let this library call
// cudaMalloc: an application whose framework owns the whole device-memory pool, or a
// latency-critical loop where an allocation (and the implicit device synchronisation of a
// cudaFree) is not allowed once it runs. For them the plain FP32 E-step below works entirely in
// one fixed scratch array that lives in this file for the life of the process.
// ---------------------------------------------------------------------------------------------
namespace gmm {
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;  // 32 MiB per device
constexpr int kNoAllocMaxMix = 4096;
constexpr int kNoAllocMaxDim = 128;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace
}  // namespace gmm

extern "C" int gmm_accumulate_noalloc(const float* dX, long long N, int D, int M, const float* dw,
                                      const float* dmu, const float* dvar, float min_loglike,
                                      float min_gamma, float min_var, int flags, double* d_stats,
                                      void* stream) {
  using namespace gmm;
  if (N < 0 || M < 1 || D < 1 || !dw || !dmu || !dvar || !d_stats || (N > 0 && !dX))
    return fail(nullptr, GMM_ERR_ARG, "gmm_accumulate_noalloc: bad argument");
  if (M > kNoAllocMaxMix || D > kNoAllocMaxDim)
    return fail(nullptr, GMM_ERR_UNSUPPORTED,
                "gmm_accumulate_noalloc: at most 4096 components and 128 dimensions "
                "(fixed 32 MiB scratch)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return fail(nullptr, GMM_ERR_CUDA, "gmm_accumulate_noalloc: no current CUDA device");
  // The scratch array's address in the current device's context, looked up on every call (no
  // cache): it is valid for this context only, and a cudaDeviceReset gives the device a new one.
  void* scratch = nullptr;
  e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(nullptr, GMM_ERR_CUDA,
                std::string("gmm_accumulate_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  }
  unsigned char* base = static_cast<unsigned char*>(scratch);
  const int E = 1 + 2 * D;

  // carve the scratch: flags | active list | icov | logG | logW | partials | LL | LL partials | posteriors
  size_t off = 0;
  Ctx c;
  c.device = dev;
  c.stream = static_cast<cudaStream_t>(stream);
  c.minLL = min_loglike;
  c.minGamma = min_gamma;
  c.min_var = min_var;
  c.M = M;
  c.D = D;
  c.Dx = D;
  c.N = N;
  c.X = dX;
  c.w = const_cast<float*>(dw);
  c.mu = const_cast<float*>(dmu);
  c.var = const_cast<float*>(dvar);
  c.stats = d_stats;
  int hflag[16] = {0};
  c.hflag = hflag;
  c.flag = reinterpret_cast<int*>(base + off); off = align_up(off + 16 * sizeof(int), 256);
  c.act = reinterpret_cast<int*>(base + off); off = align_up(off + sizeof(int) * M, 256);
  c.icov = reinterpret_cast<float*>(base + off); off = align_up(off + sizeof(float) * (size_t)M * D, 256);
  c.logG = reinterpret_cast<float*>(base + off); off = align_up(off + sizeof(float) * M, 256);
  c.logW = reinterpret_cast<float*>(base + off); off = align_up(off + sizeof(float) * M, 256);

  // calls share the scratch: clear what must start at zero (flags) and the caller's output
  e = cudaMemsetAsync(c.flag, 0, 16 * sizeof(int), c.stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(d_stats, 0, sizeof(double) * ((size_t)M * E + 1), c.stream);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "gmm_accumulate_noalloc: cudaMemsetAsync");
  int rc = plain_precompute(&c);
  if (rc) return fail(nullptr, rc, c.err);
  if (c.Mact <= 0) return fail(nullptr, GMM_ERR_STATE, "gmm_accumulate_noalloc: no component with non-zero weight");

  // The rest of the scratch: per-slice partial statistics [slices][Mact][E] (FP64), then a frame
  // chunk of posteriors [Mact][chunk] + LL [chunk] + LL partials [chunk / 256]. The partials get
  // as many slices as the frames want (as gmm_accumulate picks them), at most half of what is
  // left and at least one; the model must leave room for one slice and 256 frames.
  const size_t avail = kNoAllocScratchBytes - off;
  const size_t slice_bytes = sizeof(double) * (size_t)c.Mact * E;
  const size_t frame_bytes = sizeof(float) * (size_t)c.Mact + sizeof(float) + sizeof(double);
  const size_t min_chunk_bytes = frame_bytes * 256 + 3 * 256;
  if (align_up(slice_bytes, 256) + min_chunk_bytes > avail)
    return fail(nullptr, GMM_ERR_UNSUPPORTED,
                "gmm_accumulate_noalloc: model too large for the 32 MiB scratch (one slice of statistics "
                "and 256 frames of posteriors do not fit)");
  long long slice_cap = (long long)((avail - min_chunk_bytes) / slice_bytes);
  const long long half_cap = (long long)((avail / 2) / slice_bytes);
  if (half_cap >= 1 && half_cap < slice_cap) slice_cap = half_cap;
  c.part = reinterpret_cast<double*>(base + off);
  off = align_up(off + slice_bytes * (size_t)slice_cap, 256);
  long long chunk = (long long)((kNoAllocScratchBytes - off - 3 * 256) / frame_bytes);
  chunk = chunk / 256 * 256;
  if (chunk > N) chunk = (N + 255) / 256 * 256;
  if (chunk < 256) chunk = 256;
  c.logits = reinterpret_cast<float*>(base + off); off = align_up(off + sizeof(float) * (size_t)c.Mact * chunk, 256);
  c.ll = reinterpret_cast<float*>(base + off); off = align_up(off + sizeof(float) * (size_t)chunk, 256);
  c.llpart = reinterpret_cast<double*>(base + off); off = align_up(off + sizeof(double) * (size_t)(chunk / 256 + 1), 256);
  if (off > kNoAllocScratchBytes) return fail(nullptr, GMM_ERR_UNSUPPORTED, "gmm_accumulate_noalloc: scratch layout overflow");
  c.llpart_cap = (size_t)(chunk / 256 + 1);

  for (long long f0 = 0; f0 < N; f0 += chunk) {
    const long long nf = (N - f0 < chunk) ? N - f0 : chunk;
    const int blocks = (int)((nf + 255) / 256);
    // per-chunk frame index space: the kernels address X and LL as [f0 + i]; the LL buffer
    // holds one chunk, so point it one chunk back
    float* llbuf = c.ll - f0;
    if (D <= 16) launch_ll<16>(&c, f0, nf, c.logits, chunk, llbuf, blocks);
    else if (D <= 32) launch_ll<32>(&c, f0, nf, c.logits, chunk, llbuf, blocks);
    else if (D <= 40) launch_ll<40>(&c, f0, nf, c.logits, chunk, llbuf, blocks);
    else if (D <= 64) launch_ll<64>(&c, f0, nf, c.logits, chunk, llbuf, blocks);
    else launch_ll<128>(&c, f0, nf, c.logits, chunk, llbuf, blocks);
    ll_total_kernel<<<1, 1024, 0, c.stream>>>(blocks, c.llpart, c.stats + (size_t)M * E);
    // frame slices as gmm_accumulate picks them (about 64 warps per SM, at least 256 frames
    // each, a multiple of 4), then at most what the carved partials hold
    long long slices = 152LL * 64 / c.Mact;
    if (slices > nf / 256) slices = nf / 256;
    if (slices < 1) slices = 1;
    slices = (slices + 3) / 4 * 4;
    if (slices > slice_cap) slices = slice_cap;
    long long slice_len = (nf + slices - 1) / slices;
    slice_len = (slice_len + 31) / 32 * 32;
    // the statistics kernel reads LL as ll[f0 + i] from c.ll
    c.ll = llbuf;
    const int DW = (D + 31) / 32;
    switch (DW) {
      case 1: launch_stats<1>(&c, f0, nf, chunk, flags, (int)slices, slice_len); break;
      case 2: launch_stats<2>(&c, f0, nf, chunk, flags, (int)slices, slice_len); break;
      case 3: launch_stats<3>(&c, f0, nf, chunk, flags, (int)slices, slice_len); break;
      default: launch_stats<4>(&c, f0, nf, chunk, flags, (int)slices, slice_len); break;
    }
    c.ll = llbuf + f0;
    const long long tot = (long long)c.Mact * E;
    reduce_kernel<<<(int)((tot + 255) / 256), 256, 0, c.stream>>>(M, D, c.Mact, c.act, (int)slices,
                                                                  c.part, c.stats);
  }
  e = cudaStreamSynchronize(c.stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "gmm_accumulate_noalloc");
  return GMM_OK;
}
