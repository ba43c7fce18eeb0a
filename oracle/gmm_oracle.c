/*
 * CPU oracle for the GMM hot path -- TEST INFRASTRUCTURE ONLY (see gmm_oracle.h).
 * Compiled with -ffp-contract=off so that every float expression rounds exactly as in an
 * x86-64 build of the reference estimator, on any host.
 *
 * Reference anchors (paths inside GMMTeam/GMM/GMM/lib_bmssr):
 *   model precompute      trainer/OL_GMMStatsEstimator.cpp:234-313 (insertModel)
 *   component log-like    trainer/OL_GMMStatsEstimator.cpp:563-588 (computeMixLogLike)
 *   frame log-like        trainer/OL_GMMStatsEstimator.cpp:444-510 (getLikeAndGammas)
 *   log-add               trainer/OL_GMMStatsEstimator.cpp:1449-1458 (addLog, LPDIF = 15)
 *   posteriors            trainer/OL_GMMStatsEstimator.cpp:515-558 (compGammas)
 *   stat accumulation     trainer/OL_GMMStatsEstimator.cpp:1334-1378 (accumulateStats(vec))
 *   frame loop + totals   trainer/OL_GMMStatsEstimator.cpp:1105-1193 (accumulateStats(batch))
 *   thread split + merge  trainer/OL_GMMStatsEstimator.cpp:884-971 (accumulateStatsMT),
 *                         model/OL_GMMStats.cpp:99-145 (operator+=)
 */
#include "gmm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define MINUS_LOG_2PI (-1.837877066409345)
#define LPDIF 15.0f
#define MIN_FRAMES_FOR_THREAD 100
#define MIN_IND_SAMPLES 2.0

int orc_em_update_nind(int M, int D, float* w, float* mu, float* var, const double* n,
                       const double* F, const double* S, long long totN, int upW, int upM, int upV,
                       float min_var, const double* nind);
int orc_full_em_update_nind(int M, int D, float* w, float* mu, float* cov, const double* n,
                            const double* F, const double* Sp, long long totN, int upW, int upM, int upV,
                            const double* nind);

int orc_rearrange_order(int M, const float* w, int* order) {
  int nz = 0, z = 1;
  for (int m = 0; m < M; ++m) {
    if (w[m] > 0) order[nz++] = m;
    else order[M - z++] = m;
  }
  return nz;
}

/* ---------------------------------------------------------------- float port ---------- */

typedef struct {
  int M, D;
  const float* w;
  const float* mu;
  float* icov;      /* M*D, 1/var */
  float* logGconst; /* M */
  float* logW;      /* M */
  const orc_opts* o;
} model32;

static int prep32(model32* m, int M, int D, const float* w, const float* mu, const float* var,
                  const orc_opts* o) {
  m->M = M;
  m->D = D;
  m->w = w;
  m->mu = mu;
  m->o = o;
  m->icov = (float*)malloc(sizeof(float) * (size_t)M * D);
  m->logGconst = (float*)malloc(sizeof(float) * (size_t)M);
  m->logW = (float*)malloc(sizeof(float) * (size_t)M);
  for (int c = 0; c < M; ++c) {
    float wc = w[c];
    m->logW[c] = (wc > 0) ? logf(wc) : o->minLogLike;
    if (!(wc > 0)) { m->logGconst[c] = 0.0f; continue; }
    float acc = 0.0f;
    for (int d = 0; d < D; ++d) {
      float v = var[(size_t)c * D + d];
      if (v < o->min_var) return 1;
      m->icov[(size_t)c * D + d] = 1.0f / v;
      acc += logf(v);
    }
    m->logGconst[c] = (float)(MINUS_LOG_2PI * D / 2 - acc / 2);
  }
  return 0;
}

static void free32(model32* m) {
  free(m->icov);
  free(m->logGconst);
  free(m->logW);
}

static inline void add_log(float* p1, float p2) {
  if (*p1 - LPDIF > p2) return;
  if (*p1 > p2) *p1 = *p1 + logf(1.0f + expf(p2 - *p1));
  else *p1 = p2 + logf(1.0f + expf(*p1 - p2));
}

static inline float mix_loglike(const model32* m, int c, const float* x) {
  const float* mean = m->mu + (size_t)c * m->D;
  const float* ic = m->icov + (size_t)c * m->D;
  float e = 0.0f;
  for (int d = 0; d < m->D; ++d) {
    float diff = x[d] - mean[d];
    float t = diff * diff;
    t = t * ic[d];
    e = e + t;
  }
  float ll = m->logGconst[c] - 0.5f * e;
  if (!isfinite(ll)) return m->o->minLogLike;
  return ll;
}

/* getLikeAndGammas: g[c] = unnormalised log posterior; returns frame log-likelihood. */
static float like_and_gammas(const model32* m, const float* x, float* g, int* trouble) {
  float minLL = m->o->minLogLike;
  float maxLL = minLL, sumLL = minLL;
  for (int c = 0; c < m->M; ++c) {
    if (!(m->w[c] > 0)) continue;
    if (m->logW[c] == minLL) { g[c] = minLL; continue; }
    g[c] = mix_loglike(m, c, x) + m->logW[c];
    if (maxLL < g[c]) maxLL = g[c];
    add_log(&sumLL, g[c]);
  }
  if (maxLL == minLL) { *trouble = 1; return minLL; }
  return sumLL;
}

static int count_active(int M, const float* w) {
  int k = 0;
  for (int c = 0; c < M; ++c) k += (w[c] > 0);
  return k;
}

/* compGammas */
static float comp_gammas(const model32* m, const float* x, float* g, int nactive, int* trouble) {
  float ll = like_and_gammas(m, x, g, trouble);
  if (nactive == 1) {
    for (int c = 0; c < m->M; ++c)
      if (m->w[c] > 0) { g[c] = 1.0f; break; }
    return ll;
  }
  float minLL = m->o->minLogLike;
  if (ll == minLL) {
    for (int c = 0; c < m->M; ++c)
      if (m->w[c] > 0) g[c] = m->o->minGamma;
  } else {
    for (int c = 0; c < m->M; ++c) {
      if (!(m->w[c] > 0)) continue;
      g[c] = (float)(g[c] > minLL) * expf(g[c] - ll);
    }
  }
  return ll;
}

typedef struct {
  const model32* m;
  const float* X;
  long long first, count;
  int flags;
  double *n, *F, *S;
  double totLL;
  long long totN;
  float* out;
  int trouble;
  int nactive;
} job32;

static void acc_range(job32* j) {
  const model32* m = j->m;
  int D = m->D, M = m->M;
  float* g = (float*)malloc(sizeof(float) * (size_t)(M > 0 ? M : 1));
  int fm = (j->flags & ORC_ACC_MEAN) != 0, fv = (j->flags & ORC_ACC_VAR) != 0;
  int probsOnly = (j->flags & ORC_ACC_PROBS_ONLY) != 0;
  float minGamma = m->o->minGamma;
  for (long long i = 0; i < j->count; ++i) {
    const float* x = j->X + (size_t)(j->first + i) * D;
    float ll = comp_gammas(m, x, g, j->nactive, &j->trouble);
    j->totLL += (double)ll;
    for (int c = 0; c < M; ++c) {
      if (!(m->w[c] > 0)) continue;
      float gc = g[c];
      if (gc <= minGamma) continue;
      j->n[c] += (double)gc;
      if (probsOnly) continue;
      for (int k = 0; k < D; ++k) {
        if (fm) j->F[(size_t)c * D + k] += (double)(gc * x[k]);
        if (fv) {
          float t = gc * x[k];
          t = t * x[k];
          j->S[(size_t)c * D + k] += (double)t;
        }
      }
    }
  }
  j->totN += j->count;
  free(g);
}

static void ll_range(job32* j) {
  const model32* m = j->m;
  float* g = (float*)malloc(sizeof(float) * (size_t)(m->M > 0 ? m->M : 1));
  for (long long i = 0; i < j->count; ++i) {
    const float* x = j->X + (size_t)(j->first + i) * m->D;
    j->out[j->first + i] = like_and_gammas(m, x, g, &j->trouble);
  }
  free(g);
}

static void* acc_thread(void* p) { acc_range((job32*)p); return NULL; }
static void* ll_thread(void* p) { ll_range((job32*)p); return NULL; }

/* Split exactly as accumulateStatsMT / compVecsLogLikeMT: T = min(N/100, threads) workers,
 * N/T frames each, the last takes the remainder. */
static int split_threads(long long N, int threads) {
  long long t = N / MIN_FRAMES_FOR_THREAD;
  if (t > threads) t = threads;
  return (int)t;
}

int orc32_loglikes(const float* X, long long N, int D, int M, const float* w, const float* mu,
                   const float* var, const orc_opts* o, float* out, int* stability_trouble) {
  if (N < 0 || D <= 0 || M <= 0) return 2;
  model32 m;
  int rc = prep32(&m, M, D, w, mu, var, o);
  if (rc) { free32(&m); return rc; }
  int T = split_threads(N, o->threads);
  int trouble = 0;
  if (T < 2) {
    job32 j = {&m, X, 0, N, 0, 0, 0, 0, 0.0, 0, out, 0, 0};
    ll_range(&j);
    trouble = j.trouble;
  } else {
    job32* jobs = (job32*)calloc((size_t)T, sizeof(job32));
    pthread_t* th = (pthread_t*)calloc((size_t)T, sizeof(pthread_t));
    long long part = N / T, shift = 0;
    for (int t = 0; t < T; ++t) {
      long long cnt = (t + 1 == T) ? N - shift : part;
      job32 j = {&m, X, shift, cnt, 0, 0, 0, 0, 0.0, 0, out, 0, 0};
      jobs[t] = j;
      shift += cnt;
      pthread_create(&th[t], NULL, ll_thread, &jobs[t]);
    }
    for (int t = 0; t < T; ++t) { pthread_join(th[t], NULL); trouble |= jobs[t].trouble; }
    free(jobs);
    free(th);
  }
  if (stability_trouble) *stability_trouble = trouble;
  free32(&m);
  return 0;
}

int orc32_accumulate(const float* X, long long N, int D, int M, const float* w, const float* mu,
                     const float* var, const orc_opts* o, int flags, double* n, double* F,
                     double* S, double* totLL, long long* totN) {
  if (N < 0 || D <= 0 || M <= 0) return 2;
  model32 m;
  int rc = prep32(&m, M, D, w, mu, var, o);
  if (rc) { free32(&m); return rc; }
  int nactive = count_active(M, w);
  size_t MD = (size_t)M * D;
  int T = split_threads(N, o->threads);
  if (T < 2) {
    job32 j = {&m, X, 0, N, flags, n, F, S, *totLL, *totN, NULL, 0, nactive};
    acc_range(&j);
    *totLL = j.totLL;
    *totN = j.totN;
  } else {
    job32* jobs = (job32*)calloc((size_t)T, sizeof(job32));
    pthread_t* th = (pthread_t*)calloc((size_t)T, sizeof(pthread_t));
    long long part = N / T, shift = 0;
    for (int t = 0; t < T; ++t) {
      long long cnt = (t + 1 == T) ? N - shift : part;
      job32 j = {&m, X, shift, cnt, flags, n, F, S, *totLL, *totN, NULL, 0, nactive};
      if (t > 0) {
        j.n = (double*)calloc((size_t)M, sizeof(double));
        j.F = (double*)calloc(MD, sizeof(double));
        j.S = (double*)calloc(MD, sizeof(double));
        j.totLL = 0.0;
        j.totN = 0;
      }
      jobs[t] = j;
      shift += cnt;
      pthread_create(&th[t], NULL, acc_thread, &jobs[t]);
    }
    pthread_join(th[0], NULL);
    int fm = (flags & (ORC_ACC_MEAN | ORC_ACC_VAR)) != 0, fv = (flags & ORC_ACC_VAR) != 0;
    /* GMMStats::operator+= in thread order: per component mixProb, then per dim mean, var */
    for (int t = 1; t < T; ++t) {
      pthread_join(th[t], NULL);
      for (int c = 0; c < M; ++c) {
        n[c] += jobs[t].n[c];
        for (int k = 0; k < D; ++k) {
          if (fm) F[(size_t)c * D + k] += jobs[t].F[(size_t)c * D + k];
          if (fv) S[(size_t)c * D + k] += jobs[t].S[(size_t)c * D + k];
        }
      }
      jobs[0].totN += jobs[t].totN;
      jobs[0].totLL += jobs[t].totLL;
      free(jobs[t].n);
      free(jobs[t].F);
      free(jobs[t].S);
    }
    *totLL = jobs[0].totLL;
    *totN = jobs[0].totN;
    free(jobs);
    free(th);
  }
  free32(&m);
  return 0;
}

/* ---------------------------------------------------------------- FP64 oracle --------- */

typedef struct {
  int M, D;
  const float* w;
  const float* mu;
  const float* var;
  double* logc; /* log w - D/2 log 2pi - 1/2 sum log var */
} model64;

static int prep64(model64* m, int M, int D, const float* w, const float* mu, const float* var,
                  const orc_opts* o) {
  m->M = M; m->D = D; m->w = w; m->mu = mu; m->var = var;
  m->logc = (double*)malloc(sizeof(double) * (size_t)M);
  for (int c = 0; c < M; ++c) {
    if (!(w[c] > 0)) { m->logc[c] = 0; continue; }
    double s = 0;
    for (int d = 0; d < D; ++d) {
      double v = var[(size_t)c * D + d];
      if (v < o->min_var) return 1;
      s += log(v);
    }
    m->logc[c] = log((double)w[c]) + MINUS_LOG_2PI * D / 2.0 - 0.5 * s;
  }
  return 0;
}

/* returns frame LL (or -inf if no active component); g[c] = log joint, -inf for skipped */
static double frame64(const model64* m, const float* x, double* g) {
  double mx = -INFINITY;
  for (int c = 0; c < m->M; ++c) {
    if (!(m->w[c] > 0)) { g[c] = -INFINITY; continue; }
    const float* mean = m->mu + (size_t)c * m->D;
    const float* v = m->var + (size_t)c * m->D;
    double e = 0;
    for (int d = 0; d < m->D; ++d) {
      double diff = (double)x[d] - (double)mean[d];
      e += diff * diff / (double)v[d];
    }
    g[c] = m->logc[c] - 0.5 * e;
    if (g[c] > mx) mx = g[c];
  }
  if (mx == -INFINITY) return mx;
  double s = 0;
  for (int c = 0; c < m->M; ++c)
    if (g[c] > -INFINITY) s += exp(g[c] - mx);
  return mx + log(s);
}

int orc64_loglikes(const float* X, long long N, int D, int M, const float* w, const float* mu,
                   const float* var, const orc_opts* o, double* out) {
  model64 m;
  int rc = prep64(&m, M, D, w, mu, var, o);
  if (rc) { free(m.logc); return rc; }
  double* g = (double*)malloc(sizeof(double) * (size_t)M);
  for (long long i = 0; i < N; ++i) out[i] = frame64(&m, X + (size_t)i * D, g);
  free(g);
  free(m.logc);
  return 0;
}

typedef struct {
  const model64* m;
  const float* X;
  long long f0, f1;
  int D, M, nactive, fm, fv, probsOnly;
  const orc_opts* o;
  double *n, *F, *S, tl;
} acc64_job;

static void* acc64_thread(void* arg) {
  acc64_job* j = (acc64_job*)arg;
  const model64* m = j->m;
  const int M = j->M, D = j->D;
  double* g = (double*)malloc(sizeof(double) * (size_t)M);
  for (long long i = j->f0; i < j->f1; ++i) {
    const float* x = j->X + (size_t)i * D;
    double ll = frame64(m, x, g);
    if (ll == -INFINITY) { j->tl += (double)j->o->minLogLike; continue; }
    j->tl += ll;
    for (int c = 0; c < M; ++c) {
      if (!(m->w[c] > 0)) continue;
      double gc = (j->nactive == 1) ? 1.0 : exp(g[c] - ll);
      if (gc <= (double)j->o->minGamma) continue;
      j->n[c] += gc;
      if (j->probsOnly) continue;
      for (int k = 0; k < D; ++k) {
        double xv = x[k];
        if (j->fm) j->F[(size_t)c * D + k] += gc * xv;
        if (j->fv) j->S[(size_t)c * D + k] += gc * xv * xv;
      }
    }
  }
  free(g);
  return NULL;
}

/* FP64 statistics. With o->threads = T > 1 the frames are split into T contiguous ranges whose
 * private sums are added in range order (a precision reference: only the FP64 summation order
 * depends on T). */
int orc64_accumulate(const float* X, long long N, int D, int M, const float* w, const float* mu,
                     const float* var, const orc_opts* o, int flags, double* n, double* F,
                     double* S, double* totLL, long long* totN) {
  model64 m;
  int rc = prep64(&m, M, D, w, mu, var, o);
  if (rc) { free(m.logc); return rc; }
  int T = o->threads < 1 ? 1 : o->threads;
  if (N < (long long)T * 64) T = 1;
  acc64_job* jobs = (acc64_job*)calloc((size_t)T, sizeof(acc64_job));
  pthread_t* th = (pthread_t*)calloc((size_t)T, sizeof(pthread_t));
  for (int t = 0; t < T; ++t) {
    acc64_job* j = &jobs[t];
    j->m = &m; j->X = X; j->D = D; j->M = M; j->o = o;
    j->f0 = N * t / T; j->f1 = N * (t + 1) / T;
    j->nactive = count_active(M, w);
    j->fm = (flags & ORC_ACC_MEAN) != 0;
    j->fv = (flags & ORC_ACC_VAR) != 0;
    j->probsOnly = (flags & ORC_ACC_PROBS_ONLY) != 0;
    if (T == 1) {
      j->n = n; j->F = F; j->S = S; j->tl = *totLL;
    } else {
      j->n = (double*)calloc((size_t)M, sizeof(double));
      j->F = (double*)calloc((size_t)M * D, sizeof(double));
      j->S = (double*)calloc((size_t)M * D, sizeof(double));
      j->tl = 0.0;
    }
  }
  if (T == 1) {
    acc64_thread(&jobs[0]);
    *totLL = jobs[0].tl;
  } else {
    for (int t = 0; t < T; ++t) pthread_create(&th[t], NULL, acc64_thread, &jobs[t]);
    for (int t = 0; t < T; ++t) pthread_join(th[t], NULL);
    double tl = *totLL;
    for (int t = 0; t < T; ++t) {
      for (int c = 0; c < M; ++c) n[c] += jobs[t].n[c];
      for (size_t e = 0; e < (size_t)M * D; ++e) {
        F[e] += jobs[t].F[e];
        S[e] += jobs[t].S[e];
      }
      tl += jobs[t].tl;
      free(jobs[t].n);
      free(jobs[t].F);
      free(jobs[t].S);
    }
    *totLL = tl;
  }
  *totN += N;
  free(jobs);
  free(th);
  free(m.logc);
  return 0;
}

/* ---------------------------------------------------------------- M-step ------------- */

static float reset_var_value(void) {
  /* GMMMixture::Reset (OL_GMModel.cpp:73-83) fills diagonal variances with memset(.., 1, ..):
   * every byte 0x01. */
  unsigned int bits = 0x01010101u;
  float f;
  memcpy(&f, &bits, sizeof f);
  return f;
}

int orc_em_update(int M, int D, float* w, float* mu, float* var, const double* n,
                  const double* F, const double* S, long long totN, int upW, int upM, int upV,
                  float min_var) {
  return orc_em_update_nind(M, D, w, mu, var, n, F, S, totN, upW, upM, upV, min_var, NULL);
}

/* UpdateModelEM with the kill rule on `nind` (the robust independent-frame counts of
 * MakeRobustStats) instead of the occupancies when nind is not NULL. */
int orc_em_update_nind(int M, int D, float* w, float* mu, float* var, const double* n,
                       const double* F, const double* S, long long totN, int upW, int upM, int upV,
                       float min_var, const double* nind) {
  int changed = 0, nzero = 0;
  double corr = 0.0;
  float* mean = (float*)malloc(sizeof(float) * (size_t)D);
  float rv = reset_var_value();
  unsigned int tot = (unsigned int)totN; /* GMMStats::_totalAccSamples is unsigned int */
  for (int j = 0; j < M; ++j) {
    if (w[j] == 0.0f) { ++nzero; continue; }
    double mp = n[j];
    if ((nind ? nind[j] : mp) < MIN_IND_SAMPLES) {
      for (int k = 0; k < D; ++k) { mu[(size_t)j * D + k] = 0.0f; var[(size_t)j * D + k] = rv; }
      w[j] = 0.0f;
      changed = 1;
      continue;
    }
    if (upW) {
      w[j] = (float)(mp / tot);
      changed = 1;
    }
    corr += w[j];
    if (upM || upV) {
      for (int k = 0; k < D; ++k) mean[k] = (float)(F[(size_t)j * D + k] / mp);
      if (upV) {
        for (int k = 0; k < D; ++k) {
          float v = (float)(S[(size_t)j * D + k] / mp - pow((double)mean[k], 2));
          if (v < min_var) v = min_var;
          var[(size_t)j * D + k] = v;
        }
      }
      if (upM) memcpy(mu + (size_t)j * D, mean, sizeof(float) * (size_t)D);
    }
  }
  if (changed && corr > 0.0)
    for (int j = 0; j < M; ++j) w[j] = (float)(w[j] / corr);
  free(mean);
  return M - nzero;
}

int orc64_em_update(int M, int D, const float* w, const double* n, const double* F,
                    const double* S, long long totN, int upW, int upM, int upV, double min_var,
                    double* ow, double* omu, double* ovar) {
  int nzero = 0;
  double corr = 0.0;
  for (int j = 0; j < M; ++j) {
    ow[j] = w[j];
    if (w[j] == 0.0f) { ++nzero; continue; }
    double mp = n[j];
    if (mp < MIN_IND_SAMPLES) { ow[j] = 0.0; continue; }
    if (upW) ow[j] = mp / (double)totN;
    corr += ow[j];
    for (int k = 0; k < D; ++k) {
      double mk = F[(size_t)j * D + k] / mp;
      if (upM) omu[(size_t)j * D + k] = mk;
      if (upV) {
        double v = S[(size_t)j * D + k] / mp - mk * mk;
        ovar[(size_t)j * D + k] = v < min_var ? min_var : v;
      }
    }
  }
  if (corr > 0.0)
    for (int j = 0; j < M; ++j) ow[j] /= corr;
  return M - nzero;
}

void orc_map_update(int M, int D, float* w, float* mu, float* var, const float* ubm_w,
                    const float* ubm_mu, const float* ubm_var, const double* n, const double* F,
                    const double* S, long long totN, int tau, int upW, int upM, int upV,
                    float min_var) {
  double corr = 0.0;
  unsigned int tot = (unsigned int)totN;
  float* am = (float*)malloc(sizeof(float) * (size_t)D);
  float* av = (float*)malloc(sizeof(float) * (size_t)D);
  for (int j = 0; j < M; ++j) {
    if (ubm_w[j] == 0) continue;
    double mp = n[j];
    if (!(mp > 0.0f)) continue;
    const float* um = ubm_mu + (size_t)j * D;
    const float* uv = ubm_var + (size_t)j * D;
    double alfa = mp / (mp + tau);
    if (upW && tot > 0) {
      float aw = (float)(alfa * (mp / tot) + (1 - alfa) * ubm_w[j]);
      w[j] = aw;
      corr += aw;
    }
    if (upM || upV) {
      for (int k = 0; k < D; ++k)
        am[k] = (float)(alfa * F[(size_t)j * D + k] / mp + (1 - alfa) * um[k]);
      if (upV) {
        for (int k = 0; k < D; ++k) {
          float second = uv[k] + um[k] * um[k];
          float msq = am[k] * am[k];
          av[k] = (float)(alfa * S[(size_t)j * D + k] / mp + (1 - alfa) * second - msq);
          if (av[k] < min_var) av[k] = min_var;
        }
      }
      memcpy(mu + (size_t)j * D, am, sizeof(float) * (size_t)D);
      if (upV) memcpy(var + (size_t)j * D, av, sizeof(float) * (size_t)D);
    }
  }
  if (upW && corr != 0) {
    float fc = (float)corr;
    for (int j = 0; j < M; ++j) w[j] = w[j] / fc;
  }
  free(am);
  free(av);
}

void orc_gj_invert(int n, double* a) {
  for (int k = 0; k < n; ++k) {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        if (i != k && j != k) a[i * n + j] -= a[k * n + j] * a[i * n + k] / a[k * n + k];
    for (int j = 0; j < n; ++j)
      if (j != k) a[k * n + j] = -a[k * n + j] / a[k * n + k];
    for (int i = 0; i < n; ++i)
      if (i != k) a[i * n + k] = a[i * n + k] / a[k * n + k];
    a[k * n + k] = 1.0 / a[k * n + k];
  }
}

int orc_mllr_w(int M, int D, const float* mu, const float* var, const float* ubm_mu,
               const float* ubm_var, const double* n, const double* F, int ubm_init,
               float min_var, double* W) {
  int E = D + 1;
  if (M < E) return 3;
  int active = 0;
  double occ = 0.0;
  for (int m = 0; m < M; ++m)
    if (n[m] > 0) { ++active; occ += n[m]; }
  if (active < E) return 3;
  if (occ * D < (double)D * E) return 3;
  double* G = (double*)malloc(sizeof(double) * (size_t)E * E);
  double* k = (double*)malloc(sizeof(double) * (size_t)E);
  double* G0 = NULL;
  double* k0 = NULL;
  if (ubm_init) {
    /* prepareKiGiInitMatrices: per row i, prior terms from every UBM component */
    G0 = (double*)calloc((size_t)D * E * E, sizeof(double));
    k0 = (double*)calloc((size_t)D * E, sizeof(double));
    for (int m = 0; m < M; ++m) {
      const float* v = ubm_var + (size_t)m * D;
      const float* me = ubm_mu + (size_t)m * D;
      for (int r = 0; r < D; ++r) {
        double cG = (v[r] < min_var) ? (double)(1 / min_var) : (double)(1 / v[r]);
        double ck = me[r] * cG;
        double* Gr = G0 + (size_t)r * E * E;
        double* kr = k0 + (size_t)r * E;
        for (int d = 0; d < D; ++d) {
          kr[d] += ck * me[d];
          Gr[D * E + d] += cG * me[d];
          Gr[d * E + D] += cG * me[d];
          for (int dd = 0; dd < D; ++dd) Gr[d * E + dd] += cG * me[d] * me[dd];
          Gr[d * E + d] += cG * v[d];
        }
        Gr[E * E - 1] += cG;
        kr[D] += ck;
      }
    }
  }
  for (int i = 0; i < D; ++i) {
    if (ubm_init) {
      memcpy(G, G0 + (size_t)i * E * E, sizeof(double) * (size_t)E * E);
      memcpy(k, k0 + (size_t)i * E, sizeof(double) * (size_t)E);
    } else {
      memset(G, 0, sizeof(double) * (size_t)E * E);
      memset(k, 0, sizeof(double) * (size_t)E);
    }
    for (int m = 0; m < M; ++m) {
      double mp = n[m];
      if (!(mp > 0)) continue;
      const float* mv = var + (size_t)m * D;
      const float* mm = mu + (size_t)m * D;
      double cm = F[(size_t)m * D + i] / mv[i];
      double cv = mp / mv[i];
      for (int a = 0; a < D; ++a) {
        k[a] += cm * mm[a];
        for (int b = a; b < D; ++b) {
          G[a * E + b] += cv * mm[a] * mm[b];
          G[b * E + a] = G[a * E + b];
        }
        G[a * E + D] += cv * mm[a];
        G[D * E + a] = G[a * E + D];
      }
      k[D] += cm;
      G[D * E + D] += cv;
    }
    orc_gj_invert(E, G);
    for (int a = 0; a < E; ++a) {
      double s = 0.0;
      for (int b = 0; b < E; ++b) s += G[a * E + b] * k[b];
      W[(size_t)i * E + a] = s;
    }
  }
  free(G);
  free(k);
  free(G0);
  free(k0);
  return 0;
}

void orc_mllr_apply(int M, int D, const float* mu, const double* W, float* omu) {
  int E = D + 1;
  for (int m = 0; m < M; ++m) {
    const float* x = mu + (size_t)m * D;
    for (int k = 0; k < D; ++k) {
      double v = 0.0;
      for (int kk = 0; kk < D; ++kk) v += W[(size_t)k * E + kk] * x[kk];
      omu[(size_t)m * D + k] = (float)(v + W[(size_t)k * E + D]);
    }
  }
}

/* ---------------------------------------------------------------- full covariance ------ */
/* The full-covariance branch of the reference (OL_GMMStatsEstimator.cpp:155-229 getCovInverse /
 * getLogDet, :593-620 computeMixLogLikeFullCov, :1334-1378 accumulateStats with _fFullVar;
 * OL_ModelAdapt.cpp:905-917 UpdateModelEM, :1074-1086 UpdateModelMAP). The reference inverts
 * and factors with single-precision LAPACK (ACML spotrf/spotri, not vendored); this restatement
 * works in double: Cholesky factor L (cov = L L^T), log det = 2 sum log L_ii, and
 * (x-mu)^T cov^-1 (x-mu) = |L^-1 (x-mu)|^2 by forward substitution. Second-order statistics
 * are the packed upper triangle in row order: S[k][kk] for kk >= k at k*D + kk - k(k+1)/2. */

/* Cholesky of each active component's covariance, in double. chol: M*D*D (lower, row-major),
 * logdet: M. Returns 4 if a covariance is not positive definite. */
int orc64_full_prepare(int M, int D, const float* w, const float* cov, double* chol, double* logdet) {
  for (int c = 0; c < M; ++c) {
    double* L = chol + (size_t)c * D * D;
    memset(L, 0, sizeof(double) * (size_t)D * D);
    logdet[c] = 0.0;
    if (!(w[c] > 0)) continue;
    const float* A = cov + (size_t)c * D * D;
    for (int j = 0; j < D; ++j) {
      double s = A[(size_t)j * D + j];
      for (int k = 0; k < j; ++k) s -= L[(size_t)j * D + k] * L[(size_t)j * D + k];
      if (!(s > 0.0)) return 4;
      const double ljj = sqrt(s);
      L[(size_t)j * D + j] = ljj;
      for (int i = j + 1; i < D; ++i) {
        double t = A[(size_t)i * D + j];
        for (int k = 0; k < j; ++k) t -= L[(size_t)i * D + k] * L[(size_t)j * D + k];
        L[(size_t)i * D + j] = t / ljj;
      }
      logdet[c] += 2.0 * log(ljj);
    }
  }
  return 0;
}

static double full_frame64(int M, int D, const float* w, const float* mu, const double* chol,
                           const double* logc, const float* x, double* g, double* y) {
  double mx = -INFINITY;
  for (int c = 0; c < M; ++c) {
    if (!(w[c] > 0)) { g[c] = -INFINITY; continue; }
    const float* mean = mu + (size_t)c * D;
    const double* L = chol + (size_t)c * D * D;
    double e = 0.0;
    for (int i = 0; i < D; ++i) {  /* y = L^-1 (x - mu) */
      double t = (double)x[i] - (double)mean[i];
      for (int k = 0; k < i; ++k) t -= L[(size_t)i * D + k] * y[k];
      y[i] = t / L[(size_t)i * D + i];
      e += y[i] * y[i];
    }
    g[c] = logc[c] - 0.5 * e;
    if (g[c] > mx) mx = g[c];
  }
  if (mx == -INFINITY) return mx;
  double s = 0;
  for (int c = 0; c < M; ++c)
    if (g[c] > -INFINITY) s += exp(g[c] - mx);
  return mx + log(s);
}

static int full_model64(int M, int D, const float* w, const float* cov, double** chol, double** logc) {
  *chol = (double*)malloc(sizeof(double) * (size_t)M * D * D);
  *logc = (double*)malloc(sizeof(double) * (size_t)M);
  double* logdet = (double*)malloc(sizeof(double) * (size_t)M);
  int rc = orc64_full_prepare(M, D, w, cov, *chol, logdet);
  for (int c = 0; c < M; ++c)
    (*logc)[c] = (w[c] > 0) ? log((double)w[c]) + MINUS_LOG_2PI * D / 2.0 - 0.5 * logdet[c] : 0.0;
  free(logdet);
  return rc;
}

int orc64_full_loglikes(const float* X, long long N, int D, int M, const float* w, const float* mu,
                        const float* cov, double* out) {
  double *chol, *logc;
  int rc = full_model64(M, D, w, cov, &chol, &logc);
  if (!rc) {
    double* g = (double*)malloc(sizeof(double) * (size_t)M);
    double* y = (double*)malloc(sizeof(double) * (size_t)D);
    for (long long i = 0; i < N; ++i) out[i] = full_frame64(M, D, w, mu, chol, logc, X + (size_t)i * D, g, y);
    free(g);
    free(y);
  }
  free(chol);
  free(logc);
  return rc;
}

/* FP64 statistics for a full-covariance model into zeroed n[M], F[M*D], Sp[M*D(D+1)/2]. */
int orc64_full_accumulate(const float* X, long long N, int D, int M, const float* w, const float* mu,
                          const float* cov, const orc_opts* o, int flags, double* n, double* F,
                          double* Sp, double* totLL, long long* totN) {
  double *chol, *logc;
  int rc = full_model64(M, D, w, cov, &chol, &logc);
  if (rc) { free(chol); free(logc); return rc; }
  const int fm = (flags & ORC_ACC_MEAN) != 0, fv = (flags & ORC_ACC_VAR) != 0;
  const int probsOnly = (flags & ORC_ACC_PROBS_ONLY) != 0;
  const int nactive = count_active(M, w);
  const size_t P = (size_t)D * (D + 1) / 2;
  double* g = (double*)malloc(sizeof(double) * (size_t)M);
  double* y = (double*)malloc(sizeof(double) * (size_t)D);
  for (long long i = 0; i < N; ++i) {
    const float* x = X + (size_t)i * D;
    double ll = full_frame64(M, D, w, mu, chol, logc, x, g, y);
    if (ll == -INFINITY) { *totLL += (double)o->minLogLike; continue; }
    *totLL += ll;
    for (int c = 0; c < M; ++c) {
      if (!(w[c] > 0)) continue;
      double gc = (nactive == 1) ? 1.0 : exp(g[c] - ll);
      if (gc <= (double)o->minGamma) continue;
      n[c] += gc;
      if (probsOnly) continue;
      size_t e = 0;
      for (int k = 0; k < D; ++k) {
        if (fm) F[(size_t)c * D + k] += gc * x[k];
        if (fv)
          for (int kk = k; kk < D; ++kk) Sp[(size_t)c * P + e++] += gc * (double)x[k] * (double)x[kk];
      }
    }
  }
  *totN += N;
  free(g);
  free(y);
  free(chol);
  free(logc);
  return 0;
}

/* UpdateModelEM for full covariances (OL_ModelAdapt.cpp:858-931): as the diagonal update, the
 * covariance (float)(S/n - mean_k*mean_kk) with a float product of the float means, symmetric,
 * no floor; a killed component gets mean 0 and the identity (GMMMixture::Reset). */
int orc_full_em_update(int M, int D, float* w, float* mu, float* cov, const double* n,
                       const double* F, const double* Sp, long long totN, int upW, int upM, int upV) {
  return orc_full_em_update_nind(M, D, w, mu, cov, n, F, Sp, totN, upW, upM, upV, NULL);
}

int orc_full_em_update_nind(int M, int D, float* w, float* mu, float* cov, const double* n,
                            const double* F, const double* Sp, long long totN, int upW, int upM, int upV,
                            const double* nind) {
  int changed = 0, nzero = 0;
  double corr = 0.0;
  const size_t P = (size_t)D * (D + 1) / 2;
  float* mean = (float*)malloc(sizeof(float) * (size_t)D);
  for (int j = 0; j < M; ++j) {
    if (w[j] == 0.0f) { ++nzero; continue; }
    const double mp = n[j];
    float* C = cov + (size_t)j * D * D;
    if ((nind ? nind[j] : mp) < 2.0) {
      for (int k = 0; k < D; ++k) mu[(size_t)j * D + k] = 0.0f;
      for (int e = 0; e < D * D; ++e) C[e] = 0.0f;
      for (int k = 0; k < D; ++k) C[(size_t)k * D + k] = 1.0f;
      w[j] = 0.0f;
      changed = 1;
      continue;
    }
    if (upW) {
      w[j] = (float)(mp / (double)(unsigned int)totN);
      changed = 1;
    }
    corr += w[j];
    if (upM || upV) {
      for (int k = 0; k < D; ++k) mean[k] = (float)(F[(size_t)j * D + k] / mp);
      if (upV) {
        size_t e = 0;
        for (int k = 0; k < D; ++k)
          for (int kk = k; kk < D; ++kk) {
            const float mm = mean[k] * mean[kk];
            const float v = (float)(Sp[(size_t)j * P + e++] / mp - (double)mm);
            C[(size_t)k * D + kk] = v;
            C[(size_t)kk * D + k] = v;
          }
      }
      if (upM) memcpy(mu + (size_t)j * D, mean, sizeof(float) * (size_t)D);
    }
  }
  if (changed && corr > 0.0)
    for (int j = 0; j < M; ++j) w[j] = (float)((double)w[j] / corr);
  free(mean);
  return M - nzero;
}

/* UpdateModelMAP, tau > 0, full covariances (OL_ModelAdapt.cpp:1024-1099). */
void orc_full_map_update(int M, int D, float* w, float* mu, float* cov, const float* ubm_w,
                         const float* ubm_mu, const float* ubm_cov, const double* n, const double* F,
                         const double* Sp, long long totN, int tau, int upW, int upM, int upV) {
  double corr = 0.0;
  const size_t P = (size_t)D * (D + 1) / 2;
  float* am = (float*)malloc(sizeof(float) * (size_t)D);
  for (int j = 0; j < M; ++j) {
    if (ubm_w[j] == 0.0f) continue;
    const double mp = n[j];
    if (!(mp > 0.0)) continue;
    const float* um = ubm_mu + (size_t)j * D;
    const float* uc = ubm_cov + (size_t)j * D * D;
    const double alfa = mp / (mp + tau);
    if (upW && totN > 0) {
      const float aw = (float)(alfa * (mp / (double)(unsigned int)totN) + (1 - alfa) * ubm_w[j]);
      w[j] = aw;
      corr += aw;
    }
    if (upM || upV) {
      for (int k = 0; k < D; ++k) am[k] = (float)(alfa * F[(size_t)j * D + k] / mp + (1 - alfa) * um[k]);
      if (upV) {
        float* C = cov + (size_t)j * D * D;
        size_t e = 0;
        for (int k = 0; k < D; ++k)
          for (int kk = k; kk < D; ++kk) {
            const float second = uc[(size_t)k * D + kk] + um[k] * um[kk];
            const float msq = am[k] * am[kk];
            const float v = (float)(alfa * Sp[(size_t)j * P + e++] / mp + (1 - alfa) * second - msq);
            C[(size_t)k * D + kk] = v;
            C[(size_t)kk * D + k] = v;
          }
      }
      memcpy(mu + (size_t)j * D, am, sizeof(float) * (size_t)D);
    }
  }
  if (upW && corr != 0.0)
    for (int j = 0; j < M; ++j) w[j] = w[j] / (float)corr;
  free(am);
}

/* ---------------------------------------------------------------- fMLLR -------------- */

/* FP64 E-step of a diagonal model with full (packed upper-triangle) second-order statistics,
 * as ComputeW_fMLLR gathers them (AccumulateStats with varFull, OL_ModelAdapt.cpp:1626-1628). */
int orc64_accumulate_fullstats(const float* X, long long N, int D, int M, const float* w,
                               const float* mu, const float* var, const orc_opts* o, double* n,
                               double* F, double* Sp, double* totLL, long long* totN) {
  model64 m;
  int rc = prep64(&m, M, D, w, mu, var, o);
  if (rc) { free(m.logc); return rc; }
  const int nactive = count_active(M, w);
  const size_t P = (size_t)D * (D + 1) / 2;
  double* g = (double*)malloc(sizeof(double) * (size_t)M);
  for (long long i = 0; i < N; ++i) {
    const float* x = X + (size_t)i * D;
    double ll = frame64(&m, x, g);
    if (ll == -INFINITY) { *totLL += (double)o->minLogLike; continue; }
    *totLL += ll;
    for (int c = 0; c < M; ++c) {
      if (!(w[c] > 0)) continue;
      double gc = (nactive == 1) ? 1.0 : exp(g[c] - ll);
      if (gc <= (double)o->minGamma) continue;
      n[c] += gc;
      size_t e = 0;
      for (int k = 0; k < D; ++k) {
        F[(size_t)c * D + k] += gc * x[k];
        for (int kk = k; kk < D; ++kk) Sp[(size_t)c * P + e++] += gc * (double)x[k] * (double)x[kk];
      }
    }
  }
  *totN += N;
  free(g);
  free(m.logc);
  return 0;
}

/* Determinant by elimination with partial pivoting (MATRIX::_Det_Gen + pivot,
 * Matrix4_LMa.cpp:1925-1962, 2091-2120). a is overwritten. */
static double det_gen(int n, double* a) {
  double det = 1.0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double amax = -1.0;
    for (int i = k; i < n; ++i) {
      const double t = fabs(a[i * n + k]);
      if (t > amax && t != 0.0) { amax = t; p = i; }
    }
    if (a[p * n + k] == 0.0) return 0.0;
    if (p != k) {
      for (int j = 0; j < n; ++j) { double t = a[p * n + j]; a[p * n + j] = a[k * n + j]; a[k * n + j] = t; }
      det = -det;
    }
    det = det * a[k * n + k];
    for (int i = k + 1; i < n; ++i) {
      const double piv = a[i * n + k] / a[k * n + k];
      for (int j = k + 1; j < n; ++j) a[i * n + j] -= piv * a[k * n + j];
    }
  }
  return det;
}

/* ComputeW_fMLLR (OL_ModelAdapt.cpp:1614-1719) with ComputeKiGi_fMLLR (:1794-1848) and
 * EstimateAb_fmllr (:1721-1792): per row i, G_i = sum_m (1/var_mi) [S_m F_m; F_m^T n_m] and
 * k_i = sum_m (mu_mi/var_mi) [F_m; n_m] (the coefficients as float quotients), G_i inverted by
 * pivot-free Gauss-Jordan; then `iters` passes over the rows starting from A = I, b = 0: the
 * cofactors of A at the start of the pass (inv(A) det(A)), the quadratic in the row's scale
 * factor and the root that maximises the row's auxiliary function. W = [A | b], D x (D+1).
 * Returns 0, 3 (CheckInvertibility), or 5 (a negative discriminant or a zero root). */
int orc_fmllr_w(int M, int D, const float* mu, const float* var, const double* n, const double* F,
                const double* Sp, long long totN, int iters, double* W) {
  const int E = D + 1;
  const size_t P = (size_t)D * (D + 1) / 2;
  if (M < E) return 3;
  int active = 0;
  double occ = 0.0;
  for (int m = 0; m < M; ++m)
    if (n[m] > 0) { ++active; occ += n[m]; }
  if (active < E) return 3;
  if (occ * D < (double)D * E) return 3;
  double* G = (double*)calloc((size_t)D * E * E, sizeof(double));
  double* Gi = (double*)malloc(sizeof(double) * (size_t)D * E * E);
  double* K = (double*)calloc((size_t)D * E, sizeof(double));
  for (int i = 0; i < D; ++i) {
    double* g = G + (size_t)i * E * E;
    double* k = K + (size_t)i * E;
    for (int m = 0; m < M; ++m) {
      const double mp = n[m];
      if (!(mp > 0)) continue;
      const float fv = 1.0f / var[(size_t)m * D + i];
      const float fm = mu[(size_t)m * D + i] / var[(size_t)m * D + i];
      const double cv = fv, cm = fm;
      const double* Fm = F + (size_t)m * D;
      const double* Sm = Sp + (size_t)m * P;
      size_t e = 0;
      for (int a = 0; a < D; ++a) {
        k[a] += cm * Fm[a];
        for (int b = a; b < D; ++b) {
          g[a * E + b] += cv * Sm[e++];
          g[b * E + a] = g[a * E + b];
        }
        g[a * E + D] += cv * Fm[a];
        g[D * E + a] = g[a * E + D];
      }
      k[D] += cm * mp;
      g[D * E + D] += cv * mp;
    }
    memcpy(Gi + (size_t)i * E * E, g, sizeof(double) * (size_t)E * E);
    orc_gj_invert(E, Gi + (size_t)i * E * E);
  }
  double* A = (double*)calloc((size_t)D * D, sizeof(double));
  double* b = (double*)calloc((size_t)D, sizeof(double));
  double* cofm = (double*)malloc(sizeof(double) * (size_t)D * D);
  double* tmp = (double*)malloc(sizeof(double) * (size_t)D * D);
  double* c = (double*)calloc((size_t)E, sizeof(double));
  double* foo = (double*)malloc(sizeof(double) * (size_t)E);
  double* wv = (double*)malloc(sizeof(double) * (size_t)E);
  double* w2 = (double*)malloc(sizeof(double) * 2 * (size_t)E);
  int rc = 0;
  for (int d = 0; d < D; ++d) A[d * D + d] = 1.0;
  const double aa = (double)(float)totN;
  for (int it = 0; it < iters && !rc; ++it) {
    memcpy(cofm, A, sizeof(double) * (size_t)D * D);
    orc_gj_invert(D, cofm);
    memcpy(tmp, A, sizeof(double) * (size_t)D * D);
    const double det = det_gen(D, tmp);
    for (int e = 0; e < D * D; ++e) cofm[e] *= det;
    for (int i = 0; i < D && !rc; ++i) {
      const double* g = G + (size_t)i * E * E;
      const double* gi = Gi + (size_t)i * E * E;
      const double* k = K + (size_t)i * E;
      for (int a = 0; a < D; ++a) c[a] = cofm[a * D + i];
      c[D] = 0.0;
      for (int q = 0; q < E; ++q) {
        double s = 0.0;
        for (int p = 0; p < E; ++p) s += c[p] * gi[p * E + q];
        foo[q] = s;
      }
      double bb = 0.0, cc = 0.0;
      for (int q = 0; q < E; ++q) bb += foo[q] * k[q];
      for (int q = 0; q < E; ++q) cc += foo[q] * c[q];
      bb *= -1.0;
      cc *= -1.0;
      const double sqrtD = sqrt(bb * bb - 4 * aa * cc);
      if (sqrtD < 0 || isnan(sqrtD)) { rc = 5; break; }
      const double f[2] = {(-bb + sqrtD) / (2 * aa), (-bb - sqrtD) / (2 * aa)};
      double Q[2];
      for (int j = 0; j < 2; ++j) {
        if (f[j] == 0) { rc = 5; break; }
        for (int a = 0; a <= D; ++a) wv[a] = c[a] / f[j] + k[a];
        double* wj = w2 + (size_t)j * E;
        for (int q = 0; q < E; ++q) {
          double s = 0.0;
          for (int p = 0; p < E; ++p) s += wv[p] * gi[p * E + q];
          wj[q] = s;
        }
        Q[j] = 0.0;
        for (int a = 0; a <= D; ++a) {
          double s = 0.0;
          for (int q = 0; q < E; ++q) s += g[a * E + q] * wj[q];
          Q[j] += wj[a] * (k[a] - 0.5 * s);
        }
      }
      if (rc) break;
      const double* best = w2 + (size_t)(Q[0] > Q[1] ? 0 : 1) * E;
      for (int a = 0; a < D; ++a) A[i * D + a] = best[a];
      b[i] = best[D];
    }
  }
  if (!rc)
    for (int i = 0; i < D; ++i) {
      for (int j = 0; j < D; ++j) W[(size_t)i * E + j] = A[i * D + j];
      W[(size_t)i * E + D] = b[i];
    }
  free(G); free(Gi); free(K); free(A); free(b); free(cofm); free(tmp); free(c); free(foo); free(wv); free(w2);
  return rc;
}

/* ---------------------------------------------------------------- robust statistics ---- */

/* Auxiliary statistics of --robust (GMMStatsEstimator::accumulateAuxStats, no-pruning branch,
 * OL_GMMStatsEstimator.cpp:1253-1286, driven per consecutive frame pair by accumulateStats
 * :1175-1188, one thread): for frames i >= 1, with the posteriors of frames i and i-1,
 * gs = 1 / sum_m [g_m > minGamma] g_m over g_m = post_i,m post_i-1,m; aux2_m += sqrt(post_i,m)
 * when post_i,m > minGamma; for g = gs post_i,m post_i-1,m > minGamma: aux_m[k] += g |x_i,k -
 * x_i-1,k| and aux3_m += g. Posteriors in FP64 here (the diagonal or the full model). */
int orc64_aux_stats(const float* X, long long N, int D, int M, const float* w, const float* mu,
                    const float* var, int full, const orc_opts* o, double* aux, double* aux2, double* aux3) {
  model64 m;
  double *chol = NULL, *logc = NULL;
  int rc = 0;
  if (full) rc = full_model64(M, D, w, var, &chol, &logc);
  else rc = prep64(&m, M, D, w, mu, var, o);
  if (rc) { if (full) { free(chol); free(logc); } else free(m.logc); return rc; }
  const int nactive = count_active(M, w);
  double* g = (double*)malloc(sizeof(double) * (size_t)M);
  double* y = (double*)malloc(sizeof(double) * (size_t)D);
  double* p0 = (double*)calloc((size_t)M, sizeof(double));
  double* p1 = (double*)calloc((size_t)M, sizeof(double));
  for (long long i = 0; i < N; ++i) {
    const float* x = X + (size_t)i * D;
    const double ll = full ? full_frame64(M, D, w, mu, chol, logc, x, g, y) : frame64(&m, x, g);
    for (int c = 0; c < M; ++c) {
      if (!(w[c] > 0)) { p1[c] = 0.0; continue; }
      if (nactive == 1) p1[c] = 1.0;
      else if (ll == -INFINITY) p1[c] = (double)o->minGamma;
      else p1[c] = exp(g[c] - ll);
    }
    if (i > 0) {
      double gs = 0.0;
      for (int c = 0; c < M; ++c) {
        if (!(w[c] > 0)) continue;
        const double gg = p1[c] * p0[c];
        if (gg > o->minGamma) gs += gg;
      }
      if (gs > 0) gs = 1.0 / gs;
      const float* xp = x - D;
      for (int c = 0; c < M; ++c) {
        if (!(w[c] > 0)) continue;
        const double gg = gs * p1[c] * p0[c];
        if (p1[c] > o->minGamma) aux2[c] += sqrt(p1[c]);
        if (gg <= o->minGamma) continue;
        for (int k = 0; k < D; ++k) aux[(size_t)c * D + k] += gg * fabs((double)x[k] - (double)xp[k]);
        aux3[c] += gg;
      }
    }
    double* t = p0; p0 = p1; p1 = t;
  }
  free(g); free(y); free(p0); free(p1);
  if (full) { free(chol); free(logc); } else free(m.logc);
  return 0;
}

static float diag_cov_multiplier(double nind) {
  if (nind < 2) return (float)pow(pow((1.0 + (1.0 / (2.0 - 1.25))), 3.5), (3 - nind));
  return (float)pow((1.0 + (1.0 / (nind - 1.25))), 3.5);
}

static float offdiag_cov_multiplier(double nind, int D) {
  if (nind < 2) return 0.0f;
  return (float)(1 - pow(((double)D / (D - 1 + nind)), 1.4));
}

/* GetNIndFrames + MakeRobustStats (OL_ModelAdapt.cpp:468-588): the per-component count of
 * independent frames from the auxiliary statistics, and the second-order statistics pulled
 * toward the squared means with the diagonal / off-diagonal multipliers. S is [M][D] (diagonal)
 * or [M][D(D+1)/2] (full, packed) and is modified in place; nind receives the counts.
 * Returns 6 if a global variance is zero (the reference throws). */
int orc_make_robust(int M, int D, int full, const double* n, const double* F, double* S,
                    const double* aux, const double* aux2, const double* aux3, double* nind) {
  const size_t P = full ? (size_t)D * (D + 1) / 2 : (size_t)D;
  double* gstd = (double*)calloc((size_t)D, sizeof(double));
  double* gmean = (double*)calloc((size_t)D, sizeof(double));
  double gmp = 0.0, sumNg = 0.0;
  for (int m = 0; m < M; ++m) {
    gmp += n[m];
    size_t shift = 0;
    for (int d = 0; d < D; ++d) {
      gmean[d] += F[(size_t)m * D + d];
      if (full) {
        shift += (size_t)d;
        gstd[d] += S[(size_t)m * P + (size_t)d * D + d - shift];
      } else {
        gstd[d] += S[(size_t)m * P + d];
      }
    }
    nind[m] = 0;
    sumNg += aux2[m];
  }
  int rc = 0;
  for (int d = 0; d < D; ++d) {
    gmean[d] /= gmp;
    gstd[d] = sqrt(gstd[d] / gmp - gmean[d] * gmean[d]);
    if (gstd[d] == 0) rc = 6;
  }
  if (!rc) {
    for (int m = 0; m < M; ++m) {
      if (n[m] == 0 || aux3[m] == 0) {
        nind[m] = 0;
      } else {
        for (int d = 0; d < D; ++d) nind[m] += aux[(size_t)m * D + d] / aux3[m] / gstd[d];
        nind[m] /= D;
        nind[m] = pow(nind[m] / 1.12, 3);
        nind[m] = 1 + (aux2[m] * gmp / sumNg - 1) * nind[m];
      }
    }
    for (int j = 0; j < M; ++j) {
      float dc = diag_cov_multiplier(nind[j]);
      dc *= nind[j] / (nind[j] - 1);
      double* Sj = S + (size_t)j * P;
      const double* Fj = F + (size_t)j * D;
      if (full) {
        const float odc = offdiag_cov_multiplier(nind[j], D);
        size_t shift = 0;
        for (int k = 0; k < D - 1; ++k) {
          shift += (size_t)k;
          Sj[(size_t)k * D + k - shift] = dc * Sj[(size_t)k * D + k - shift] + (1 - dc) * pow(Fj[k], 2.0) / n[j];
          for (int kk = k + 1; kk < D; ++kk)
            Sj[(size_t)k * D + kk - shift] = odc * Sj[(size_t)k * D + kk - shift] + (1 - odc) * Fj[k] * Fj[kk] / n[j];
        }
        Sj[P - 1] = dc * Sj[P - 1] + (1 - dc) * pow(Fj[D - 1], 2.0) / n[j];
      } else {
        for (int k = 0; k < D; ++k) Sj[k] = dc * Sj[k] + (1 - dc) * pow(Fj[k], 2.0) / n[j];
      }
    }
  }
  free(gstd);
  free(gmean);
  return rc;
}
