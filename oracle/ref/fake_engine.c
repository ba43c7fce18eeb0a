/*
 * A CPU stand-in for the subset of the gmm_gb300 C ABI that GMMStatsEstimator_GB300
 * (oracle/ref/gb300_adapter.hpp) calls. TEST INFRASTRUCTURE ONLY: it lets the adapter run
 * inside the reference's own CModelAdapt on a machine without a GPU, so that a test can check
 * the adapter's bookkeeping (model group and slots, rearranged component order, GMMStats +=
 * semantics, totals, flags) against the reference's CPU estimator. The arithmetic is the
 * oracle's port of the reference CPU estimator (orc32_*, single thread), which is pinned
 * bit-for-bit to the reference, so with the reference estimator also on one thread both runs
 * must agree exactly. Entry points the adapter only needs for full covariances or feature files
 * report GMM_ERR_UNSUPPORTED.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/gmm_gb300.h"
#include "../gmm_oracle.h"

#define FAKE_MAX_SLOTS 64

typedef struct {
  int M, D;
  float *w, *mu, *var;
} fake_slot;

struct gmm_ctx {
  char err[256];
  float minLL, minGamma, min_var;
  fake_slot slots[FAKE_MAX_SLOTS];
  fake_slot cur; /* the model in use (a copy of a slot) */
  float* X;
  long long N;
  int Dx;
};

static char g_create_err[256] = "";

static int fake_fail(gmm_handle h, int code, const char* msg) {
  snprintf(h ? h->err : g_create_err, 256, "%s", msg);
  return code;
}

static void slot_free(fake_slot* s) {
  free(s->w);
  free(s->mu);
  free(s->var);
  memset(s, 0, sizeof(*s));
}

static int slot_copy(fake_slot* dst, int M, int D, const float* w, const float* mu, const float* var) {
  slot_free(dst);
  dst->w = (float*)malloc(sizeof(float) * (size_t)M);
  dst->mu = (float*)malloc(sizeof(float) * (size_t)M * D);
  dst->var = (float*)malloc(sizeof(float) * (size_t)M * D);
  if (!dst->w || !dst->mu || !dst->var) return 1;
  memcpy(dst->w, w, sizeof(float) * (size_t)M);
  memcpy(dst->mu, mu, sizeof(float) * (size_t)M * D);
  memcpy(dst->var, var, sizeof(float) * (size_t)M * D);
  dst->M = M;
  dst->D = D;
  return 0;
}

static orc_opts fake_opts(gmm_handle h) {
  orc_opts o;
  o.minLogLike = h->minLL;
  o.minGamma = h->minGamma;
  o.min_var = h->min_var;
  o.threads = 1;
  return o;
}

int gmm_create(int device, gmm_handle* out) {
  (void)device;
  if (!out) return fake_fail(NULL, GMM_ERR_ARG, "gmm_create: null output pointer");
  *out = (gmm_handle)calloc(1, sizeof(struct gmm_ctx));
  if (!*out) return fake_fail(NULL, GMM_ERR_NOMEM, "gmm_create: out of host memory");
  (*out)->minLL = -1e20f;
  (*out)->minGamma = 1e-4f;
  (*out)->min_var = 1e-6f;
  return GMM_OK;
}

int gmm_destroy(gmm_handle h) {
  if (!h) return GMM_OK;
  for (int i = 0; i < FAKE_MAX_SLOTS; ++i) slot_free(&h->slots[i]);
  slot_free(&h->cur);
  free(h->X);
  free(h);
  return GMM_OK;
}

const char* gmm_last_error(gmm_handle h) { return h ? h->err : g_create_err; }

int gmm_set_precision(gmm_handle h, int mode) {
  (void)mode;
  return h ? GMM_OK : GMM_ERR_ARG;
}

int gmm_set_options(gmm_handle h, float min_loglike, float min_gamma, float min_var) {
  if (!h) return GMM_ERR_ARG;
  h->minLL = min_loglike;
  h->minGamma = min_gamma;
  h->min_var = min_var;
  return GMM_OK;
}

int gmm_upload_model_slot(gmm_handle h, int slot, int M, int D, const float* w, const float* mu,
                          const float* var) {
  if (!h) return GMM_ERR_ARG;
  if (slot < 0 || slot >= FAKE_MAX_SLOTS || M < 1 || D < 1 || !w || !mu || !var)
    return fake_fail(h, GMM_ERR_ARG, "gmm_upload_model_slot: bad argument");
  for (int i = 0; i < FAKE_MAX_SLOTS; ++i)
    if (i != slot && h->slots[i].w && h->slots[i].D != D)
      return fake_fail(h, GMM_ERR_ARG, "gmm_upload_model_slot: models of a group must have the same dimension");
  return slot_copy(&h->slots[slot], M, D, w, mu, var) ? fake_fail(h, GMM_ERR_NOMEM, "out of host memory")
                                                      : GMM_OK;
}

int gmm_select_model(gmm_handle h, int slot) {
  if (!h) return GMM_ERR_ARG;
  if (slot < 0 || slot >= FAKE_MAX_SLOTS || !h->slots[slot].w)
    return fake_fail(h, GMM_ERR_ARG, "gmm_select_model: no model in that slot");
  const fake_slot* s = &h->slots[slot];
  return slot_copy(&h->cur, s->M, s->D, s->w, s->mu, s->var) ? fake_fail(h, GMM_ERR_NOMEM, "out of host memory")
                                                             : GMM_OK;
}

int gmm_clear_model_slots(gmm_handle h) {
  if (!h) return GMM_ERR_ARG;
  for (int i = 0; i < FAKE_MAX_SLOTS; ++i) slot_free(&h->slots[i]);
  return GMM_OK;
}

int gmm_upload_features(gmm_handle h, const float* X, long long N, int D) {
  if (!h) return GMM_ERR_ARG;
  if (N < 0 || D < 1 || (N > 0 && !X)) return fake_fail(h, GMM_ERR_ARG, "gmm_upload_features: bad argument");
  free(h->X);
  h->X = (float*)malloc(sizeof(float) * (size_t)(N > 0 ? N : 1) * D);
  if (!h->X) return fake_fail(h, GMM_ERR_NOMEM, "out of host memory");
  if (N > 0) memcpy(h->X, X, sizeof(float) * (size_t)N * D);
  h->N = N;
  h->Dx = D;
  return GMM_OK;
}

int gmm_accumulate(gmm_handle h, int flags, double* n, double* F, double* S, double* tot_loglike,
                   long long* tot_frames) {
  if (!h) return GMM_ERR_ARG;
  if (!h->cur.w) return fake_fail(h, GMM_ERR_STATE, "gmm_accumulate: no model");
  if (!h->X || h->Dx != h->cur.D) return fake_fail(h, GMM_ERR_STATE, "gmm_accumulate: no features of the model's D");
  const int M = h->cur.M, D = h->cur.D;
  double* nn = (double*)calloc((size_t)M, sizeof(double));
  double* FF = (double*)calloc((size_t)M * D, sizeof(double));
  double* SS = (double*)calloc((size_t)M * D, sizeof(double));
  double tl = 0.0;
  long long tn = 0;
  orc_opts o = fake_opts(h);
  int rc = (nn && FF && SS) ? orc32_accumulate(h->X, h->N, D, M, h->cur.w, h->cur.mu, h->cur.var, &o, flags,
                                               nn, FF, SS, &tl, &tn)
                            : 2;
  if (rc == 0) {
    if (n) memcpy(n, nn, sizeof(double) * (size_t)M);
    if (F) memcpy(F, FF, sizeof(double) * (size_t)M * D);
    if (S) memcpy(S, SS, sizeof(double) * (size_t)M * D);
    if (tot_loglike) *tot_loglike = tl;
    if (tot_frames) *tot_frames = tn;
  }
  free(nn);
  free(FF);
  free(SS);
  if (rc == 1) return fake_fail(h, GMM_ERR_MODEL, "model contains very low variances");
  return rc ? fake_fail(h, GMM_ERR_ARG, "gmm_accumulate: bad arguments") : GMM_OK;
}

int gmm_loglikes(gmm_handle h, float* out) {
  if (!h) return GMM_ERR_ARG;
  if (!h->cur.w || !h->X || h->Dx != h->cur.D) return fake_fail(h, GMM_ERR_STATE, "gmm_loglikes: no model or features");
  int trouble = 0;
  orc_opts o = fake_opts(h);
  int rc = orc32_loglikes(h->X, h->N, h->cur.D, h->cur.M, h->cur.w, h->cur.mu, h->cur.var, &o, out, &trouble);
  if (rc == 1) return fake_fail(h, GMM_ERR_MODEL, "model contains very low variances");
  return rc ? fake_fail(h, GMM_ERR_ARG, "gmm_loglikes: bad arguments") : GMM_OK;
}

static int unsupported(gmm_handle h, const char* what) { return fake_fail(h, GMM_ERR_UNSUPPORTED, what); }

int gmm_upload_model_full(gmm_handle h, int M, int D, const float* w, const float* mu, const float* cov) {
  (void)M; (void)D; (void)w; (void)mu; (void)cov;
  return unsupported(h, "fake engine: no full covariances");
}
int gmm_accumulate_full(gmm_handle h, int flags, double* n, double* F, double* Sp, double* tot_loglike,
                        long long* tot_frames) {
  (void)flags; (void)n; (void)F; (void)Sp; (void)tot_loglike; (void)tot_frames;
  return unsupported(h, "fake engine: no full covariances");
}
int gmm_loglikes_full(gmm_handle h, float* out) {
  (void)out;
  return unsupported(h, "fake engine: no full covariances");
}
int gmm_accumulate_files(gmm_handle h, int flags, int n_files, const char* const* paths, int prm_type,
                         unsigned int dwnsmp, double buffer_gb, int* files_used) {
  (void)flags; (void)n_files; (void)paths; (void)prm_type; (void)dwnsmp; (void)buffer_gb; (void)files_used;
  return unsupported(h, "fake engine: no feature files");
}
int gmm_read_stats(gmm_handle h, double* n, double* F, double* S, double* tot_loglike, long long* tot_frames) {
  (void)n; (void)F; (void)S; (void)tot_loglike; (void)tot_frames;
  return unsupported(h, "fake engine: no device statistics");
}
