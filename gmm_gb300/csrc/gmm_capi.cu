// C ABI of the GB300 GMM statistics engine (declared in include/gmm_gb300.h).
//
// A handle owns one non-blocking CUDA stream and keeps the model, the features, the FP64
// statistics and all scratch resident on its device. Host round trips happen only where a
// result is returned to the caller; gmm_em_iterate runs the whole EM loop on the device.
#include <string.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include <atomic>
#include <condition_variable>
#include <mutex>
#include <thread>

#include "gmm_internal.cuh"

namespace gmm {

static std::string g_create_err;

int fail(Ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_err = msg;
  return code;
}

int cuda_fail(Ctx* c, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();  // clear a non-sticky error
  return fail(c, e == cudaErrorMemoryAllocation ? GMM_ERR_NOMEM : GMM_ERR_CUDA, m);
}

int dalloc(Ctx* c, void** p, size_t bytes, const char* what) {
  *p = nullptr;
  if (bytes == 0) return GMM_OK;
  if (c->budget && c->allocated + bytes > c->budget)
    return fail(c, GMM_ERR_NOMEM, std::string(what) + ": over the handle's device-memory budget");
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_fail(c, e, what);
  }
  c->allocated += bytes;
  return GMM_OK;
}

void dfree(Ctx* c, void* p, size_t bytes) {
  if (!p) return;
  cudaFree(p);
  c->allocated = c->allocated >= bytes ? c->allocated - bytes : 0;
}

int scratch(Ctx* c, int slot, size_t bytes, const char* what, void** out) {
  Ctx::Scratch& b = c->scratch[slot];
  if (bytes > b.cap) {
    cudaStreamSynchronize(c->stream);  // the old buffer may still be read by queued work
    dfree(c, b.p, b.cap);
    b.p = nullptr;
    b.cap = 0;
    int rc = dalloc(c, &b.p, bytes, what);
    if (rc) return rc;
    b.cap = bytes;
  }
  *out = bytes ? b.p : nullptr;
  return GMM_OK;
}

int sync(Ctx* c, const char* what) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  return GMM_OK;
}

LaunchScope::LaunchScope(Ctx* ctx, const char* name) : c(ctx) {
  ++c->launches;
  if (!c->profile) return;
  for (auto& k : c->timers)
    if (k.name == name) { t = &k; break; }
  if (!t) {
    c->timers.emplace_back();
    t = &c->timers.back();
    t->name = name;
  }
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, c->stream);
}

LaunchScope::~LaunchScope() {
  if (!t) return;
  cudaEventRecord(b, c->stream);
  t->pending.emplace_back(a, b);
  t->launches++;
}

static void drain_timers(Ctx* c) {
  for (auto& k : c->timers) {
    for (auto& ev : k.pending) {
      cudaEventSynchronize(ev.second);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, ev.first, ev.second);
      k.ms += ms;
      cudaEventDestroy(ev.first);
      cudaEventDestroy(ev.second);
    }
    k.pending.clear();
  }
}

static void free_slot(Ctx* c, ModelSlot& s) {
  const size_t md = sizeof(float) * (size_t)s.M * s.D, m1 = sizeof(float) * (size_t)s.M;
  dfree(c, s.w, m1);
  dfree(c, s.mu, md);
  dfree(c, s.var, md);
  s = ModelSlot();
}

static void free_model(Ctx* c) {
  size_t md = sizeof(float) * (size_t)c->M * c->D, m1 = sizeof(float) * (size_t)c->M;
  dfree(c, c->w, m1); dfree(c, c->mu, md); dfree(c, c->var, md);
  dfree(c, c->icov, md); dfree(c, c->logG, m1); dfree(c, c->logW, m1);
  dfree(c, c->act, sizeof(int) * (size_t)c->M);
  dfree(c, c->pw, m1); dfree(c, c->pmu, md); dfree(c, c->pvar, md);
  dfree(c, c->bw, m1); dfree(c, c->bmu, md); dfree(c, c->bvar, md);
  dfree(c, c->stats, sizeof(double) * ((size_t)c->M * (1 + 2 * c->D) + 2));
  c->w = c->mu = c->var = c->icov = c->logG = c->logW = nullptr;
  c->pw = c->pmu = c->pvar = c->bw = c->bmu = c->bvar = nullptr;
  c->act = nullptr;
  c->stats = nullptr;
  c->have_prior = false;
  c->stats_valid = false;
}

static int ensure_model(Ctx* c, int M, int D) {
  if (c->w && c->M == M && c->D == D) return GMM_OK;
  free_model(c);
  c->M = M;
  c->D = D;
  size_t md = sizeof(float) * (size_t)M * D, m1 = sizeof(float) * (size_t)M;
  int rc = 0;
  rc |= dalloc(c, (void**)&c->w, m1, "model weights");
  if (!rc) rc |= dalloc(c, (void**)&c->mu, md, "model means");
  if (!rc) rc |= dalloc(c, (void**)&c->var, md, "model variances");
  if (!rc) rc |= dalloc(c, (void**)&c->icov, md, "inverse variances");
  if (!rc) rc |= dalloc(c, (void**)&c->logG, m1, "log constants");
  if (!rc) rc |= dalloc(c, (void**)&c->logW, m1, "log weights");
  if (!rc) rc |= dalloc(c, (void**)&c->act, sizeof(int) * (size_t)M, "active list");
  if (!rc) rc |= dalloc(c, (void**)&c->bw, m1, "model backup");
  if (!rc) rc |= dalloc(c, (void**)&c->bmu, md, "model backup");
  if (!rc) rc |= dalloc(c, (void**)&c->bvar, md, "model backup");
  if (!rc) rc |= dalloc(c, (void**)&c->stats, sizeof(double) * ((size_t)M * (1 + 2 * D) + 2), "statistics");
  if (rc) { int code = rc; free_model(c); c->M = c->D = 0; return code; }
  c->tcx_valid = c->tcx_valid && (c->tcx.K != 0);
  return GMM_OK;
}

static void free_features(Ctx* c) {
  dfree(c, c->Xown, sizeof(float) * (size_t)c->N * c->Dx);
  c->Xown = nullptr;
  c->X = nullptr;
  dfree(c, c->ll, c->ll_cap);
  c->ll = nullptr;
  c->ll_cap = 0;
  dfree(c, c->llpart, c->llpart_cap * sizeof(double));
  c->llpart = nullptr;
  c->llpart_cap = 0;
  c->N = 0;
  c->tcx_valid = false;
}

static int alloc_frame_buffers(Ctx* c, long long N) {
  size_t llb = sizeof(float) * (size_t)(N + 256);
  int rc = dalloc(c, (void**)&c->ll, llb, "per-frame log-likelihoods");
  if (rc) return rc;
  c->ll_cap = llb;
  size_t np = (size_t)((N + 255) / 256) + 1024;
  rc = dalloc(c, (void**)&c->llpart, np * sizeof(double), "log-likelihood partial sums");
  if (rc) return rc;
  c->llpart_cap = np;
  return GMM_OK;
}

static int estep(Ctx* c, int flags, bool want_stats, float* ll_dev) {
  if (!c->w) return fail(c, GMM_ERR_STATE, "no model uploaded");
  if (!c->X) return fail(c, GMM_ERR_STATE, "no features uploaded");
  if (c->Dx != c->D)
    return fail(c, GMM_ERR_ARG, "Inconsistent model & feature vector - different dimensions");
  int rc;
  if (c->model_dirty) {
    rc = plain_precompute(c);
    if (rc) return rc;
  }
  // robust statistics need the per-frame posteriors, which only the plain E-step writes out
  if (c->precision == GMM_PREC_TC && !(c->robust && want_stats)) return tc_estep(c, flags, want_stats, ll_dev);
  return plain_estep(c, flags, want_stats, ll_dev);
}

static int accumulate_device(Ctx* c, int flags) {
  if (!c->w) return fail(c, GMM_ERR_STATE, "no model uploaded");
  if (!c->X) return fail(c, GMM_ERR_STATE, "no features uploaded");
  cudaError_t e = cudaMemsetAsync(c->stats, 0, sizeof(double) * ((size_t)c->M * (1 + 2 * c->D) + 2),
                                  c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemsetAsync(stats)");
  c->stats_valid = false;
  c->aux_valid = false;
  if (c->robust) {
    const int rc = ensure_aux(c, &c->aux, &c->aux_cap, c->M, c->D);
    if (rc) return rc;
  }
  int rc = estep(c, flags, true, nullptr);
  if (rc) return rc;
  c->tot_frames = c->N;
  c->acc_flags = flags;
  c->stats_valid = true;
  c->aux_valid = c->robust;
  return GMM_OK;
}

static int stage(Ctx* c, size_t bytes) {
  if (bytes <= c->hstage_cap) return GMM_OK;
  if (c->hstage) cudaFreeHost(c->hstage);
  c->hstage = nullptr;
  c->hstage_cap = 0;
  cudaError_t e = cudaMallocHost((void**)&c->hstage, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMallocHost(staging)");
  c->hstage_cap = bytes;
  return GMM_OK;
}

static int read_stats(Ctx* c, double* n, double* F, double* S, double* tl, long long* tn) {
  if (!c->stats_valid) return fail(c, GMM_ERR_STATE, "no statistics accumulated");
  size_t cnt = (size_t)c->M * (1 + 2 * c->D) + 1;
  int rc = stage(c, cnt * sizeof(double));
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(c->hstage, c->stats, cnt * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpyAsync(stats)");
  rc = sync(c, "read statistics");
  if (rc) return rc;
  const size_t M = c->M, MD = (size_t)c->M * c->D;
  if (n) memcpy(n, c->hstage, M * sizeof(double));
  if (F) memcpy(F, c->hstage + M, MD * sizeof(double));
  if (S) memcpy(S, c->hstage + M + MD, MD * sizeof(double));
  if (tl) *tl = c->hstage[M + 2 * MD];
  if (tn) *tn = c->tot_frames;
  return GMM_OK;
}

}  // namespace gmm

using namespace gmm;

extern "C" {

int gmm_create(int device, gmm_handle* out) {
  if (!out) return fail(nullptr, GMM_ERR_ARG, "gmm_create: null output pointer");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return fail(nullptr, GMM_ERR_CUDA, "gmm_create: no CUDA device is available");
  if (device < 0 || device >= n) return fail(nullptr, GMM_ERR_ARG, "gmm_create: device id out of range");
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(nullptr, GMM_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  gmm_ctx* c = new (std::nothrow) gmm_ctx();
  if (!c) return fail(nullptr, GMM_ERR_NOMEM, "gmm_create: out of host memory");
  c->device = device;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete c; return fail(nullptr, GMM_ERR_CUDA, "cudaStreamCreate failed"); }
  if (dalloc(c, (void**)&c->flag, 16 * sizeof(int), "flags") ||
      cudaMallocHost((void**)&c->hflag, 16 * sizeof(int)) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return fail(nullptr, GMM_ERR_NOMEM, "gmm_create: flag allocation failed");
  }
  cudaMemset(c->flag, 0, 16 * sizeof(int));
  *out = c;
  return GMM_OK;
}

int gmm_destroy(gmm_handle h) {
  if (!h) return GMM_OK;
  gmm_ctx* c = h;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  drain_timers(c);
  full_destroy(c);
  sched_free(c);
  for (auto& s : c->slots) free_slot(c, s);
  dfree(c, c->aux, c->aux_cap);
  dfree(c, c->gs, c->gs_cap * sizeof(float));
  dfree(c, c->gprev, c->gprev_cap * sizeof(float));
  dfree(c, c->nind, c->nind_cap * sizeof(double));
  for (auto& b : c->scratch) dfree(c, b.p, b.cap);
  free_model(c);
  free_features(c);
  dfree(c, c->logits, c->logits_cap);
  dfree(c, c->part, c->part_cap);
  dfree(c, c->tcpart, c->tcpart_cap);
  dfree(c, c->tcm.planes, 0);
  dfree(c, c->tcm.comp_of_row, 0);
  dfree(c, c->tcm.cent, 0);
  if (c->em_graph) cudaGraphExecDestroy(c->em_graph);
  if (c->map_graph) cudaGraphExecDestroy(c->map_graph);
  dfree(c, c->ll_hist, 0);
  dfree(c, c->tcm.ll2, 0);
  dfree(c, c->tcx.planes, 0);
  dfree(c, c->tc_err, 0);
  dfree(c, c->tc_llpart, 0);
  dfree(c, c->flag, 0);
  if (c->hflag) cudaFreeHost(c->hflag);
  if (c->hstage) cudaFreeHost(c->hstage);
  for (cudaEvent_t ev : c->copy_events) cudaEventDestroy(ev);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  cudaStreamDestroy(c->stream);
  delete c;
  return GMM_OK;
}

const char* gmm_last_error(gmm_handle h) { return h ? h->err.c_str() : g_create_err.c_str(); }

int gmm_set_options(gmm_handle h, float min_loglike, float min_gamma, float min_var) {
  if (!h) return GMM_ERR_ARG;
  h->minLL = min_loglike;
  h->minGamma = min_gamma;
  h->min_var = min_var;
  h->model_dirty = true;
  return GMM_OK;
}

int gmm_set_precision(gmm_handle h, int mode) {
  if (!h) return GMM_ERR_ARG;
  if (mode != GMM_PREC_FP32 && mode != GMM_PREC_TC) return fail(h, GMM_ERR_ARG, "unknown precision mode");
  if (mode == GMM_PREC_TC && h->D > 0 && !tc_supported(h->D))
    return fail(h, GMM_ERR_UNSUPPORTED, "tensor-core path supports 1 <= D <= 63");
  h->precision = mode;
  return GMM_OK;
}

int gmm_set_autotune(gmm_handle h, int on) {
  if (!h) return GMM_ERR_ARG;
  h->autotune = on != 0;
  if (!on) h->tuned_waves.clear();
  return GMM_OK;
}

int gmm_set_wait_limit(gmm_handle h, long long cycles) {
  if (!h) return GMM_ERR_ARG;
  h->wait_limit = cycles > 0 ? cycles : kDefaultWaitLimit;
  // the captured EM iteration and batched MAP hold the old limit as a kernel argument
  if (h->em_graph) cudaGraphExecDestroy(h->em_graph);
  h->em_graph = nullptr;
  if (h->map_graph) cudaGraphExecDestroy(h->map_graph);
  h->map_graph = nullptr;
  return GMM_OK;
}

int gmm_set_tile_schedule(gmm_handle h, int mode) {
  if (!h) return GMM_ERR_ARG;
  if (mode < 0 || mode > 2) return fail(h, GMM_ERR_ARG, "gmm_set_tile_schedule: mode must be 0, 1 or 2");
  h->sched.mode = mode;
  if (h->em_graph) cudaGraphExecDestroy(h->em_graph);  // the captured iteration has the old schedule
  h->em_graph = nullptr;
  return GMM_OK;
}

int gmm_autotune_choice(gmm_handle h, int* n, long long* keys, int* waves, int cap) {
  if (!h || !n) return GMM_ERR_ARG;
  int k = 0;
  for (const auto& kv : h->tuned_waves) {
    if (k < cap && keys) keys[k] = kv.first;
    if (k < cap && waves) waves[k] = kv.second;
    ++k;
  }
  *n = k;
  return GMM_OK;
}

int gmm_set_memory_budget(gmm_handle h, size_t bytes) {
  if (!h) return GMM_ERR_ARG;
  h->budget = bytes;
  return GMM_OK;
}

int gmm_get_stream(gmm_handle h, void** stream) {
  if (!h || !stream) return GMM_ERR_ARG;
  *stream = (void*)h->stream;
  return GMM_OK;
}

int gmm_upload_model(gmm_handle h, int M, int D, const float* w, const float* mu, const float* var) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!w || !mu || !var) return fail(c, GMM_ERR_ARG, "gmm_upload_model: null array");
  if (M < 1 || M > kMaxMix || D < 1 || D > kMaxDim)
    return fail(c, GMM_ERR_ARG, "gmm_upload_model: M must be in [1, 32767] and D in [1, 1024]");
  if (c->precision == GMM_PREC_TC && !tc_supported(D))
    return fail(c, GMM_ERR_UNSUPPORTED, "tensor-core path supports 1 <= D <= 63");
  cudaSetDevice(c->device);
  int rc = ensure_model(c, M, D);
  if (rc) return rc;
  size_t md = sizeof(float) * (size_t)M * D;
  cudaMemcpyAsync(c->w, w, sizeof(float) * M, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->mu, mu, md, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->var, var, md, cudaMemcpyHostToDevice, c->stream);
  c->stats_valid = false;
  c->model_dirty = true;
  return plain_precompute(c);
}

int gmm_upload_model_slot(gmm_handle h, int slot, int M, int D, const float* w, const float* mu,
                          const float* var) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!w || !mu || !var) return fail(c, GMM_ERR_ARG, "gmm_upload_model_slot: null array");
  if (slot < 0 || slot >= kMaxModelSlots)
    return fail(c, GMM_ERR_ARG, "gmm_upload_model_slot: slot must be in [0, 4096)");
  if (M < 1 || M > kMaxMix || D < 1 || D > kMaxDim)
    return fail(c, GMM_ERR_ARG, "gmm_upload_model_slot: M must be in [1, 32767] and D in [1, 1024]");
  for (size_t i = 0; i < c->slots.size(); ++i)
    if ((int)i != slot && c->slots[i].w && c->slots[i].D != D)
      return fail(c, GMM_ERR_ARG, "gmm_upload_model_slot: models of a group must have the same dimension");
  cudaSetDevice(c->device);
  if ((size_t)slot >= c->slots.size()) c->slots.resize(slot + 1);
  ModelSlot& s = c->slots[slot];
  if (s.w && (s.M != M || s.D != D)) free_slot(c, s);
  if (!s.w) {
    const size_t md = sizeof(float) * (size_t)M * D, m1 = sizeof(float) * (size_t)M;
    int rc = dalloc(c, (void**)&s.w, m1, "model slot weights");
    if (!rc) rc = dalloc(c, (void**)&s.mu, md, "model slot means");
    if (!rc) rc = dalloc(c, (void**)&s.var, md, "model slot variances");
    if (rc) {
      s.M = M;
      s.D = D;
      free_slot(c, s);
      return rc;
    }
    s.M = M;
    s.D = D;
  }
  const size_t md = sizeof(float) * (size_t)M * D;
  cudaMemcpyAsync(s.w, w, sizeof(float) * M, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(s.mu, mu, md, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(s.var, var, md, cudaMemcpyHostToDevice, c->stream);
  return sync(c, "gmm_upload_model_slot");
}

int gmm_select_model(gmm_handle h, int slot) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (slot < 0 || (size_t)slot >= c->slots.size() || !c->slots[slot].w)
    return fail(c, GMM_ERR_ARG, "gmm_select_model: no model in slot " + std::to_string(slot));
  const ModelSlot& s = c->slots[slot];
  if (c->precision == GMM_PREC_TC && !tc_supported(s.D))
    return fail(c, GMM_ERR_UNSUPPORTED, "tensor-core path supports 1 <= D <= 63");
  cudaSetDevice(c->device);
  int rc = ensure_model(c, s.M, s.D);
  if (rc) return rc;
  const size_t md = sizeof(float) * (size_t)s.M * s.D;
  cudaMemcpyAsync(c->w, s.w, sizeof(float) * s.M, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(c->mu, s.mu, md, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(c->var, s.var, md, cudaMemcpyDeviceToDevice, c->stream);
  c->stats_valid = false;
  c->model_dirty = true;
  return plain_precompute(c);
}

int gmm_clear_model_slots(gmm_handle h) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& s : c->slots) free_slot(c, s);
  c->slots.clear();
  return GMM_OK;
}

int gmm_set_prior(gmm_handle h, const float* w, const float* mu, const float* var) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!c->w) return fail(c, GMM_ERR_STATE, "upload a model before its prior");
  size_t md = sizeof(float) * (size_t)c->M * c->D, m1 = sizeof(float) * (size_t)c->M;
  if (!c->pw) {
    int rc = dalloc(c, (void**)&c->pw, m1, "prior weights");
    if (!rc) rc = dalloc(c, (void**)&c->pmu, md, "prior means");
    if (!rc) rc = dalloc(c, (void**)&c->pvar, md, "prior variances");
    if (rc) return rc;
  }
  if (w && mu && var) {
    cudaMemcpyAsync(c->pw, w, m1, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->pmu, mu, md, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->pvar, var, md, cudaMemcpyHostToDevice, c->stream);
  } else {  // NULLs: the current resident model becomes the prior
    cudaMemcpyAsync(c->pw, c->w, m1, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(c->pmu, c->mu, md, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(c->pvar, c->var, md, cudaMemcpyDeviceToDevice, c->stream);
  }
  c->have_prior = true;
  return sync(c, "gmm_set_prior");
}

int gmm_read_model(gmm_handle h, float* w, float* mu, float* var) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!c->w) return fail(c, GMM_ERR_STATE, "no model uploaded");
  size_t md = sizeof(float) * (size_t)c->M * c->D;
  if (w) cudaMemcpyAsync(w, c->w, sizeof(float) * c->M, cudaMemcpyDeviceToHost, c->stream);
  if (mu) cudaMemcpyAsync(mu, c->mu, md, cudaMemcpyDeviceToHost, c->stream);
  if (var) cudaMemcpyAsync(var, c->var, md, cudaMemcpyDeviceToHost, c->stream);
  return sync(c, "gmm_read_model");
}

int gmm_upload_features(gmm_handle h, const float* X, long long N, int D) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!X && N > 0) return fail(c, GMM_ERR_ARG, "gmm_upload_features: null array");
  if (N < 0 || D < 1 || D > kMaxDim) return fail(c, GMM_ERR_ARG, "gmm_upload_features: bad N or D");
  cudaSetDevice(c->device);
  size_t bytes = sizeof(float) * (size_t)N * D;
  int rc = GMM_OK;
  const bool reuse = c->Xown && c->N == N && c->Dx == D && c->ll;
  if (!reuse) {
    free_features(c);
    rc = dalloc(c, (void**)&c->Xown, bytes, "features");
    if (rc) return rc;
  }
  c->tcx_valid = false;
  if (bytes) {
    cudaError_t e = cudaMemcpyAsync(c->Xown, X, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpyAsync(features)");
  }
  c->X = c->Xown;
  c->N = N;
  c->Dx = D;
  if (!reuse) {
    rc = alloc_frame_buffers(c, N);
    if (rc) return rc;
  }
  c->stats_valid = false;
  return sync(c, "gmm_upload_features");
}

int gmm_upload_features_device(gmm_handle h, const float* dX, long long N, int D) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!dX && N > 0) return fail(c, GMM_ERR_ARG, "gmm_upload_features_device: null array");
  if (N < 0 || D < 1 || D > kMaxDim) return fail(c, GMM_ERR_ARG, "gmm_upload_features_device: bad N or D");
  cudaSetDevice(c->device);
  free_features(c);
  c->X = dX;
  c->N = N;
  c->Dx = D;
  c->stats_valid = false;
  return alloc_frame_buffers(c, N);
}

int gmm_accumulate_device(gmm_handle h, int flags) {
  if (!h) return GMM_ERR_ARG;
  cudaSetDevice(h->device);
  int rc = accumulate_device(h, flags);
  if (rc) return rc;
  return sync(h, "gmm_accumulate");
}

int gmm_accumulate_host(gmm_handle h, int flags, const float* X, long long N, int D) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!X && N > 0) return fail(c, GMM_ERR_ARG, "gmm_accumulate_host: null array");
  if (N < 0 || D < 1 || D > kMaxDim) return fail(c, GMM_ERR_ARG, "gmm_accumulate_host: bad N or D");
  cudaSetDevice(c->device);
  const bool streamed = c->precision == GMM_PREC_TC && !c->robust && c->w && D == c->D && tc_supported(D) && N > 0;
  if (!streamed) {  // the plain path (or a robust E-step): upload, then the E-step
    int rc = gmm_upload_features(h, X, N, D);
    if (!rc) rc = gmm_accumulate_device(h, flags);
    return rc;
  }
  // the handle's own feature buffer, filled by the E-step's chunked copies
  const bool reuse = c->Xown && c->N == N && c->Dx == D && c->ll;
  if (!reuse) {
    free_features(c);
    int rc = dalloc(c, (void**)&c->Xown, sizeof(float) * (size_t)N * D, "features");
    if (!rc) {
      c->N = N;
      c->Dx = D;
      rc = alloc_frame_buffers(c, N);
    }
    if (rc) return rc;
  }
  c->X = c->Xown;
  c->N = N;
  c->Dx = D;
  c->tcx_valid = false;
  cudaError_t e = cudaMemsetAsync(c->stats, 0, sizeof(double) * ((size_t)c->M * (1 + 2 * c->D) + 2), c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemsetAsync(stats)");
  c->stats_valid = false;
  if (c->model_dirty) {
    const int rc = plain_precompute(c);
    if (rc) return rc;
  }
  const int rc = tc_estep_streamed(c, X, flags, 8);
  if (rc) return rc;
  c->tot_frames = c->N;
  c->acc_flags = flags;
  c->stats_valid = true;
  return GMM_OK;
}

int gmm_read_stats(gmm_handle h, double* n, double* F, double* S, double* tl, long long* tn) {
  if (!h) return GMM_ERR_ARG;
  return read_stats(h, n, F, S, tl, tn);
}

int gmm_accumulate(gmm_handle h, int flags, double* n, double* F, double* S, double* tl,
                   long long* tn) {
  if (!h) return GMM_ERR_ARG;
  cudaSetDevice(h->device);
  int rc = accumulate_device(h, flags);
  if (rc) return rc;
  return read_stats(h, n, F, S, tl, tn);
}

int gmm_loglikes(gmm_handle h, float* out) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (!out && c->N > 0) return fail(c, GMM_ERR_ARG, "gmm_loglikes: null output");
  cudaSetDevice(c->device);
  int rc = estep(c, 0, false, c->ll);
  if (rc) return rc;
  if (c->N > 0) {
    cudaError_t e = cudaMemcpyAsync(out, c->ll, sizeof(float) * (size_t)c->N,
                                    cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemcpyAsync(loglikes)");
  }
  return sync(c, "gmm_loglikes");
}

int gmm_read_aux(gmm_handle h, int full, double* aux, double* aux2, double* aux3) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  const double* src = nullptr;
  int M = 0, D = 0;
  if (full) {
    if (!c->full || !full_aux(c, &src, &M, &D)) return fail(c, GMM_ERR_STATE, "no auxiliary statistics accumulated");
  } else {
    if (!c->aux_valid) return fail(c, GMM_ERR_STATE, "no auxiliary statistics accumulated");
    src = c->aux;
    M = c->M;
    D = c->D;
  }
  cudaSetDevice(c->device);
  if (aux) cudaMemcpyAsync(aux, src, sizeof(double) * (size_t)M * D, cudaMemcpyDeviceToHost, c->stream);
  if (aux2) cudaMemcpyAsync(aux2, src + (size_t)M * D, sizeof(double) * M, cudaMemcpyDeviceToHost, c->stream);
  if (aux3) cudaMemcpyAsync(aux3, src + (size_t)M * D + M, sizeof(double) * M, cudaMemcpyDeviceToHost, c->stream);
  return sync(c, "gmm_read_aux");
}

int gmm_em_update(gmm_handle h, int upW, int upM, int upV, int* alive) {
  if (!h) return GMM_ERR_ARG;
  cudaSetDevice(h->device);
  int a = 0;
  int rc = mstep_em(h, upW, upM, upV, &a);
  if (rc) return rc;
  if (alive) *alive = a;
  return GMM_OK;
}

int gmm_map_update(gmm_handle h, int tau, int upW, int upM, int upV) {
  if (!h) return GMM_ERR_ARG;
  if (tau < 0) return fail(h, GMM_ERR_ARG, "tau must be >= 0");
  cudaSetDevice(h->device);
  if (tau == 0) return gmm_em_update(h, upW, upM, upV, nullptr);
  int rc = mstep_map(h, tau, upW, upM, upV);
  if (rc) return rc;
  return sync(h, "gmm_map_update");
}

// Common checks of the batched entry points: speakers own resident frame ranges.
static int check_speakers(Ctx* c, const char* fn, int S, const long long* offs) {
  const std::string f(fn);
  if (S < 0 || (S > 0 && !offs)) return fail(c, GMM_ERR_ARG, f + ": bad speaker count or offsets");
  if (!c->w) return fail(c, GMM_ERR_STATE, "no model uploaded");
  if (!c->X && c->N > 0) return fail(c, GMM_ERR_STATE, "no features uploaded");
  if (c->Dx != c->D && c->N > 0)
    return fail(c, GMM_ERR_ARG, "Inconsistent model & feature vector - different dimensions");
  if (S == 0) return GMM_OK;
  if (offs[0] < 0 || offs[S] > c->N) return fail(c, GMM_ERR_ARG, f + ": offsets outside the resident frames");
  for (int s = 0; s < S; ++s)
    if (offs[s + 1] < offs[s]) return fail(c, GMM_ERR_ARG, f + ": offsets must be non-decreasing");
  cudaSetDevice(c->device);
  if (c->model_dirty) return plain_precompute(c);
  return GMM_OK;
}

static int map_batch(Ctx* c, int S, const long long* offs, int tau, int upW, int upM, int upV,
                     float* w, float* mu, float* var, double* ll, bool dev_out, const float* Xh = nullptr) {
  if (tau < 1) return fail(c, GMM_ERR_ARG, "gmm_map_batch: tau must be >= 1");
  int rc = check_speakers(c, "gmm_map_batch", S, offs);
  if (rc || S == 0) return rc;
  const int M = c->M, D = c->D;
  const size_t bw = sizeof(float) * (size_t)S * M, bmu = bw * D, bll = sizeof(double) * S;
  const size_t boffs = sizeof(long long) * (S + 1);
  MapBatch b;
  b.S = S;
  b.tau = tau;
  b.upW = upW;
  b.upM = upM;
  b.upV = upV;
  b.flags = (upM ? GMM_ACC_MEAN : 0) | (upV ? GMM_ACC_VAR : 0) | ((upW && !upM && !upV) ? GMM_ACC_PROBS_ONLY : 0);
  b.offs = offs;
  b.Xh = Xh;
  long long* d_offs = nullptr;
  float *ow = nullptr, *omu = nullptr, *ovar = nullptr;
  double* oll = nullptr;
  rc = scratch(c, SC_OFFS, boffs, "speaker offsets", (void**)&d_offs);
  if (!rc) rc = scratch(c, SC_AW, bw, "adapted weight scratch", (void**)&b.aw);
  // device staging for host outputs; weights and log-likelihoods are always computed
  if (!rc && !(dev_out && w)) rc = scratch(c, SC_W, bw, "adapted weights", (void**)&ow);
  if (!rc && !dev_out && mu) rc = scratch(c, SC_MU, bmu, "adapted means", (void**)&omu);
  if (!rc && !dev_out && var) rc = scratch(c, SC_VAR, bmu, "adapted variances", (void**)&ovar);
  if (!rc && !(dev_out && ll)) rc = scratch(c, SC_LL, bll, "speaker log-likelihoods", (void**)&oll);
  if (!rc) {
    b.d_offs = d_offs;
    b.w = ow ? ow : w;
    b.mu = dev_out ? mu : omu;
    b.var = dev_out ? var : ovar;
    b.ll = oll ? oll : ll;
    cudaMemcpyAsync(d_offs, offs, boffs, cudaMemcpyHostToDevice, c->stream);
    rc = c->precision == GMM_PREC_TC ? tc_map_batch(c, b) : plain_map_batch(c, b);
  }
  if (!rc && !dev_out) {
    if (w) cudaMemcpyAsync(w, b.w, bw, cudaMemcpyDeviceToHost, c->stream);
    if (mu) cudaMemcpyAsync(mu, b.mu, bmu, cudaMemcpyDeviceToHost, c->stream);
    if (var) cudaMemcpyAsync(var, b.var, bmu, cudaMemcpyDeviceToHost, c->stream);
    if (ll) cudaMemcpyAsync(ll, b.ll, bll, cudaMemcpyDeviceToHost, c->stream);
  }
  if (!rc) rc = sync(c, "gmm_map_batch");
  cudaStreamSynchronize(c->stream);
  return rc;
}

int gmm_map_batch(gmm_handle h, int S, const long long* offs, int tau, int upW, int upM, int upV,
                  float* w, float* mu, float* var, double* ll) {
  if (!h) return GMM_ERR_ARG;
  return map_batch(h, S, offs, tau, upW, upM, upV, w, mu, var, ll, false);
}

int gmm_map_batch_device(gmm_handle h, int S, const long long* offs, int tau, int upW, int upM,
                         int upV, float* d_w, float* d_mu, float* d_var, double* d_ll) {
  if (!h) return GMM_ERR_ARG;
  return map_batch(h, S, offs, tau, upW, upM, upV, d_w, d_mu, d_var, d_ll, true);
}

static int mllr_batch(Ctx* c, int S, const long long* offs, int ubm_init, double* W, int* status,
                      float* mu_out, double* ll, const float* Xh) {
  int rc = check_speakers(c, "gmm_mllr_batch", S, offs);
  if (rc || S == 0) return rc;
  const int M = c->M, D = c->D, E = D + 1;
  const size_t bW = sizeof(double) * (size_t)S * D * E, bst = sizeof(int) * S, bmu = sizeof(float) * (size_t)S * M * D;
  const size_t bll = sizeof(double) * S, boffs = sizeof(long long) * (S + 1);
  double *dW = nullptr, *dll = nullptr;
  int* dst = nullptr;
  float* dmu = nullptr;
  long long* doffs = nullptr;
  rc = scratch(c, SC_MLLR_W, bW, "MLLR transforms", (void**)&dW);
  if (!rc) rc = scratch(c, SC_MLLR_ST, bst, "MLLR status", (void**)&dst);
  if (!rc) rc = scratch(c, SC_LL, bll, "speaker log-likelihoods", (void**)&dll);
  if (!rc) rc = scratch(c, SC_OFFS, boffs, "speaker offsets", (void**)&doffs);
  if (!rc && mu_out) rc = scratch(c, SC_MU, bmu, "MLLR adapted means", (void**)&dmu);
  if (!rc) {
    cudaMemcpyAsync(doffs, offs, boffs, cudaMemcpyHostToDevice, c->stream);
    if (c->precision == GMM_PREC_TC) {
      SpeakerStats ss;
      rc = tc_speaker_stats(c, S, offs, doffs, dll, false, Xh, &ss);  // n and F only
      if (!rc) rc = mstep_mllr_batch(c, S, nullptr, &ss, ubm_init, dW, dst, dmu, nullptr);
      tc_free_speaker_stats(c, &ss);
    } else {
      double* stats = nullptr;
      size_t bytes = 0;
      rc = plain_speaker_stats(c, S, offs, GMM_ACC_MEAN, &stats, &bytes);
      if (!rc) rc = mstep_mllr_batch(c, S, stats, nullptr, ubm_init, dW, dst, dmu, dll);
      cudaStreamSynchronize(c->stream);
      dfree(c, stats, bytes);
    }
  }
  if (!rc) {
    if (W) cudaMemcpyAsync(W, dW, bW, cudaMemcpyDeviceToHost, c->stream);
    if (status) cudaMemcpyAsync(status, dst, bst, cudaMemcpyDeviceToHost, c->stream);
    if (mu_out) cudaMemcpyAsync(mu_out, dmu, bmu, cudaMemcpyDeviceToHost, c->stream);
    if (ll) cudaMemcpyAsync(ll, dll, bll, cudaMemcpyDeviceToHost, c->stream);
    rc = sync(c, "gmm_mllr_batch");
  }
  cudaStreamSynchronize(c->stream);
  return rc;
}

int gmm_mllr_batch(gmm_handle h, int S, const long long* offs, int ubm_init, double* W, int* status,
                   float* mu_out, double* ll) {
  if (!h) return GMM_ERR_ARG;
  return mllr_batch(h, S, offs, ubm_init, W, status, mu_out, ll, nullptr);
}

// The features of a batched call from host memory. On the tensor-core path the handle's own
// feature buffer is prepared here and filled by the call's chunked copies (*streamed = true);
// otherwise the frames are uploaded now.
static int batch_host_frames(gmm_handle h, const char* what, const float* X, long long N, int D, bool* streamed) {
  Ctx* c = h;
  if (!X && N > 0) return fail(c, GMM_ERR_ARG, std::string(what) + ": null array");
  if (N < 0 || D < 1 || D > kMaxDim) return fail(c, GMM_ERR_ARG, std::string(what) + ": bad N or D");
  cudaSetDevice(c->device);
  *streamed = c->precision == GMM_PREC_TC && c->w && D == c->D && tc_supported(D) && N > 0;
  if (!*streamed) return gmm_upload_features(h, X, N, D);
  const bool reuse = c->Xown && c->N == N && c->Dx == D && c->ll;
  if (!reuse) {
    free_features(c);
    int rc = dalloc(c, (void**)&c->Xown, sizeof(float) * (size_t)N * D, "features");
    if (!rc) {
      c->N = N;
      c->Dx = D;
      rc = alloc_frame_buffers(c, N);
    }
    if (rc) return rc;
  }
  c->X = c->Xown;
  c->N = N;
  c->Dx = D;
  c->tcx_valid = false;
  c->stats_valid = false;
  return GMM_OK;
}

int gmm_map_batch_host(gmm_handle h, const float* X, long long N, int D, int S, const long long* offs, int tau,
                       int up_weight, int up_mean, int up_var, float* w, float* mu, float* var, double* ll) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  bool streamed = false;
  int rc = batch_host_frames(h, "gmm_map_batch_host", X, N, D, &streamed);
  if (rc) return rc;
  return map_batch(c, S, offs, tau, up_weight, up_mean, up_var, w, mu, var, ll, false, streamed ? X : nullptr);
}

int gmm_mllr_batch_host(gmm_handle h, const float* X, long long N, int D, int S, const long long* offs,
                        int ubm_init, double* W, int* status, float* mu_out, double* ll) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  bool streamed = false;
  int rc = batch_host_frames(h, "gmm_mllr_batch_host", X, N, D, &streamed);
  if (rc) return rc;
  return mllr_batch(c, S, offs, ubm_init, W, status, mu_out, ll, streamed ? X : nullptr);
}

// File-by-file accumulation (accumulateStatsMT(CFileList&, ...), OL_GMMStatsEstimator.cpp:641-698):
// a loader thread fills two page-locked batch buffers in turn while the device accumulates the
// other one.
int gmm_accumulate_files(gmm_handle h, int flags, int n_files, const char* const* paths, int prm_type,
                         unsigned int dwnsmp, double buffer_gb, int* files_used) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (n_files < 0 || (n_files > 0 && !paths)) return fail(c, GMM_ERR_ARG, "gmm_accumulate_files: bad file list");
  if (prm_type < GMM_PRM_SVES || prm_type > GMM_PRM_RAW)
    return fail(c, GMM_ERR_ARG, "accumulateStatsMT(): Unknown input data type specified");
  if (!c->w) return fail(c, GMM_ERR_STATE, "no model uploaded");
  cudaSetDevice(c->device);
  free_features(c);
  cudaMemsetAsync(c->stats, 0, sizeof(double) * ((size_t)c->M * (1 + 2 * c->D) + 2), c->stream);
  c->stats_valid = false;

  struct Slot {
    float* h = nullptr;
    size_t cap = 0;  // floats
    long long n = 0;
    int D = 0, files = 0;
  } slot[2];
  std::mutex mu;
  std::condition_variable cv;
  int produced = 0, consumed = 0;
  bool done = false, abort_load = false;
  int lrc = GMM_OK;
  std::string lerr;
  const double limit = buffer_gb * 1024.0 * 1024.0 * 1024.0;
  const int Dm = c->D;

  std::thread loader([&] {
    cudaSetDevice(c->device);
    Slot* b = nullptr;
    auto acquire = [&]() -> bool {
      std::unique_lock<std::mutex> lk(mu);
      cv.wait(lk, [&] { return abort_load || produced - consumed < 2; });
      if (abort_load) return false;
      b = &slot[produced % 2];
      b->n = 0;
      b->D = 0;
      b->files = 0;
      return true;
    };
    auto publish = [&] {
      std::lock_guard<std::mutex> lk(mu);
      ++produced;
      cv.notify_all();
    };
    int rc = GMM_OK;
    std::string err;
    if (acquire()) {
      for (int f = 0; f < n_files && rc == GMM_OK; ++f) {
        long long N = 0;
        int D = 0;
        const int hr = param_header(paths[f], prm_type, dwnsmp, &N, &D, &err);
        if (hr < 0 || (hr == GMM_OK && N == 0)) continue;  // missing or empty: skipped
        if (hr) { rc = hr; break; }
        if (D != Dm) {
          rc = GMM_ERR_ARG;
          err = std::string("Inconsistent model & feature vector - different dimensions (") + paths[f] + ")";
          break;
        }
        const size_t need = (size_t)(b->n + N) * D;
        if (need > b->cap) {
          float* nb = nullptr;
          const size_t cap = need + need / 2;
          if (cudaMallocHost((void**)&nb, cap * sizeof(float)) != cudaSuccess) {
            rc = GMM_ERR_NOMEM;
            err = "gmm_accumulate_files: page-locked batch buffer";
            break;
          }
          if (b->n) std::memcpy(nb, b->h, (size_t)b->n * D * sizeof(float));
          if (b->h) cudaFreeHost(b->h);
          b->h = nb;
          b->cap = cap;
        }
        const int r = param_read(paths[f], prm_type, dwnsmp, b->h + (size_t)b->n * D, &err);
        if (r < 0) continue;
        if (r) { rc = r; break; }
        b->n += N;
        b->D = D;
        ++b->files;
        if ((double)b->n * D * sizeof(float) >= limit) {
          publish();
          if (!acquire()) break;
        }
      }
      if (rc == GMM_OK && b && b->n > 0) publish();
    }
    std::lock_guard<std::mutex> lk(mu);
    if (rc) {
      lrc = rc;
      lerr = err;
    }
    done = true;
    cv.notify_all();
  });

  float* dX[2] = {nullptr, nullptr};
  size_t dcap[2] = {0, 0};
  int rc = GMM_OK, used = 0;
  long long total = 0;
  for (int k = 0; rc == GMM_OK; ++k) {
    Slot* b;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv.wait(lk, [&] { return produced > consumed || done; });
      if (produced == consumed) break;
      b = &slot[consumed % 2];
    }
    const int d = k % 2;
    const size_t bytes = (size_t)b->n * b->D * sizeof(float);
    if (bytes > dcap[d]) {
      dfree(c, dX[d], dcap[d]);
      dX[d] = nullptr;
      dcap[d] = 0;
      rc = dalloc(c, (void**)&dX[d], bytes, "feature batch");
      if (rc) break;
      dcap[d] = bytes;
    }
    if ((size_t)(b->n + 256) * sizeof(float) > c->ll_cap) {
      dfree(c, c->ll, c->ll_cap);
      c->ll = nullptr;
      c->ll_cap = 0;
      dfree(c, c->llpart, c->llpart_cap * sizeof(double));
      c->llpart = nullptr;
      c->llpart_cap = 0;
      rc = alloc_frame_buffers(c, b->n);
      if (rc) break;
    }
    cudaMemcpyAsync(dX[d], b->h, bytes, cudaMemcpyHostToDevice, c->stream);
    c->X = dX[d];
    c->N = b->n;
    c->Dx = b->D;
    c->tcx_valid = false;
    rc = estep(c, flags, true, nullptr);  // adds into the statistics
    if (!rc) rc = sync(c, "gmm_accumulate_files");
    total += b->n;
    used += b->files;
    std::lock_guard<std::mutex> lk(mu);
    ++consumed;
    cv.notify_all();
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    abort_load = true;
    cv.notify_all();
  }
  loader.join();
  cudaStreamSynchronize(c->stream);
  for (int d = 0; d < 2; ++d) {
    dfree(c, dX[d], dcap[d]);
    if (slot[d].h) cudaFreeHost(slot[d].h);
  }
  // the batches were transient: no resident features remain
  c->X = nullptr;
  c->N = 0;
  c->tcx_valid = false;
  if (rc == GMM_OK && lrc) rc = fail(c, lrc, lerr);
  if (rc) return rc;
  c->tot_frames = total;
  c->acc_flags = flags;
  c->stats_valid = true;
  if (files_used) *files_used = used;
  return GMM_OK;
}

// One EM iteration of gmm_em_iterate as device work only (no host readback), in the order of
// the eager loop below: rearrange, precompute, statistics, LL record, backup, update, restore.
static int em_iteration_device(Ctx* c, int flags, int upW, int upM, int upV) {
  int rc = mstep_rearrange(c);
  if (!rc) rc = plain_precompute_async(c);
  if (!rc) {
    cudaError_t e = cudaMemsetAsync(c->stats, 0, sizeof(double) * ((size_t)c->M * (1 + 2 * c->D) + 2), c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemsetAsync(stats)");
    rc = tc_estep(c, flags, true, nullptr);
  }
  if (rc) return rc;
  c->tot_frames = c->N;
  c->acc_flags = flags;
  c->stats_valid = true;
  rc = record_iteration_ll(c);
  const size_t md = sizeof(float) * (size_t)c->M * c->D, m1 = sizeof(float) * (size_t)c->M;
  cudaMemcpyAsync(c->bw, c->w, m1, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(c->bmu, c->mu, md, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(c->bvar, c->var, md, cudaMemcpyDeviceToDevice, c->stream);
  if (!rc) rc = mstep_em(c, upW, upM, upV, nullptr);
  if (!rc) rc = mstep_em_restore(c);
  return rc;
}

// gmm_em_iterate on the tensor-core path: the first iteration runs eagerly (it allocates what
// the kernels need), the others replay a CUDA graph of one iteration captured from the stream.
// Shapes are fixed at all M components, so components that die stay as padding rows.
static int em_iterate_graph(Ctx* c, int iters, int upW, int upM, int upV, double* ll, int* alive) {
  const int flags = (upM ? GMM_ACC_MEAN : 0) | (upV ? GMM_ACC_VAR : 0) |
                    ((upW && !upM && !upV) ? GMM_ACC_PROBS_ONLY : 0);
  // the model as given is checked once, as insertModel does (later models come from the update,
  // which floors variances at min_var)
  int rc = plain_precompute(c);
  if (rc) return rc;
  if (!c->tcx_valid || c->tcx.planes == nullptr) {
    c->static_shapes = false;
    rc = tc_estep(c, flags, false, nullptr);  // builds the feature planes
    if (rc) return rc;
  }
  if (iters > c->ll_hist_cap) {
    dfree(c, c->ll_hist, sizeof(double) * (c->ll_hist_cap + 1));
    c->ll_hist = nullptr;
    c->ll_hist_cap = 0;
    rc = dalloc(c, (void**)&c->ll_hist, sizeof(double) * (iters + 1), "EM log-likelihood history");
    if (rc) return rc;
    c->ll_hist_cap = iters;
  }
  cudaMemsetAsync(c->ll_hist, 0, sizeof(double) * (c->ll_hist_cap + 1), c->stream);
  const bool prof = c->profile;
  c->static_shapes = true;
  rc = em_iteration_device(c, flags, upW, upM, upV);
  if (!rc) rc = sync(c, "EM iteration");
  // the graph holds these buffers by address: any change means a new capture
  const long long key[] = {c->M, c->D, c->N, flags | upW << 4 | upM << 5 | upV << 6,
                           (long long)(size_t)c->X, (long long)(size_t)c->w, (long long)(size_t)c->mu,
                           (long long)(size_t)c->var, (long long)(size_t)c->stats, (long long)(size_t)c->act,
                           (long long)(size_t)c->flag, (long long)(size_t)c->icov, (long long)(size_t)c->logG,
                           (long long)(size_t)c->logW, (long long)(size_t)c->bw, (long long)(size_t)c->bmu,
                           (long long)(size_t)c->bvar, (long long)(size_t)c->tcm.planes,
                           (long long)(size_t)c->tcm.comp_of_row, (long long)(size_t)c->tcm.ll2,
                           (long long)(size_t)c->tcm.cent,
                           (long long)(size_t)c->tcx.planes, (long long)(size_t)c->tcpart,
                           (long long)(size_t)c->tc_llpart, (long long)(size_t)c->tc_err,
                           (long long)(size_t)c->ll_hist, (long long)c->ll_hist_cap,
                           (long long)c->tcpart_cap, (long long)c->tc_llpart_cap,
                           (long long)(size_t)c->sched.planes, (long long)(size_t)c->sched.lists};
  static_assert(sizeof(key) == sizeof(c->em_graph_key), "graph key size");
  if (!rc && iters > 1 && (c->em_graph == nullptr || std::memcmp(key, c->em_graph_key, sizeof(key)) != 0)) {
    if (c->em_graph) cudaGraphExecDestroy(c->em_graph);
    c->em_graph = nullptr;
    c->profile = false;  // no timing events inside the graph
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
      rc = em_iteration_device(c, flags, upW, upM, upV);
      e = cudaStreamEndCapture(c->stream, &g);
      if (!rc && e == cudaSuccess) e = cudaGraphInstantiate(&c->em_graph, g, 0);
      if (g) cudaGraphDestroy(g);
    }
    c->profile = prof;
    if (!rc && e != cudaSuccess) rc = cuda_fail(c, e, "EM iteration graph");
    if (!rc) std::memcpy(c->em_graph_key, key, sizeof(key));
  }
  for (int it = 1; it < iters && !rc; ++it) {
    cudaError_t e = cudaGraphLaunch(c->em_graph, c->stream);
    if (e != cudaSuccess) rc = cuda_fail(c, e, "cudaGraphLaunch");
    c->launches += 1;
  }
  c->static_shapes = false;
  c->model_dirty = true;
  int herr = 0;
  if (!rc) {
    if (ll) cudaMemcpyAsync(ll, c->ll_hist, sizeof(double) * iters, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(c->hflag, c->flag, 8 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(&herr, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    rc = sync(c, "gmm_em_iterate");
  }
  if (!rc && herr) {
    c->tcx_valid = false;  // kernels that gave up may have left the feature planes half built
    cudaMemsetAsync(c->tc_err, 0, sizeof(int), c->stream);
    rc = fail(c, GMM_ERR_TIMEOUT, "tensor-core E-step: a bounded device wait expired");
  }
  if (!rc && alive) *alive = c->hflag[2];
  return rc;
}

int gmm_em_iterate(gmm_handle h, int iters, int upW, int upM, int upV, double* ll, int* alive) {
  if (!h) return GMM_ERR_ARG;
  Ctx* c = h;
  if (iters < 0) return fail(c, GMM_ERR_ARG, "iters must be >= 0");
  cudaSetDevice(c->device);
  if (c->precision == GMM_PREC_TC && iters > 0 && !c->robust) {
    if (!c->w) return fail(c, GMM_ERR_STATE, "no model uploaded");
    if (!c->X || c->N == 0) return fail(c, GMM_ERR_STATE, "no features uploaded");
    if (c->Dx != c->D) return fail(c, GMM_ERR_ARG, "Inconsistent model & feature vector - different dimensions");
    if (!tc_supported(c->D)) return fail(c, GMM_ERR_UNSUPPORTED, "tensor-core path supports 1 <= D <= 63");
    return em_iterate_graph(c, iters, upW, upM, upV, ll, alive);
  }
  const int flags = (upM ? GMM_ACC_MEAN : 0) | (upV ? GMM_ACC_VAR : 0) |
                    ((upW && !upM && !upV) ? GMM_ACC_PROBS_ONLY : 0);
  const size_t md = sizeof(float) * (size_t)c->M * c->D, m1 = sizeof(float) * (size_t)c->M;
  const size_t tot_idx = (size_t)c->M * (1 + 2 * c->D);
  int last_alive = 0;
  for (int it = 0; it < iters; ++it) {
    // insertModel: zero-weight components move behind the others (GMModel::RearrangeMixtures)
    int rc = mstep_rearrange(c);
    if (rc) return rc;
    rc = plain_precompute(c);
    if (rc) return rc;
    rc = accumulate_device(c, flags);
    if (rc) return rc;
    if (ll) {
      rc = sync(c, "EM iteration");
      if (rc) return rc;
      cudaMemcpy(&ll[it], c->stats + tot_idx, sizeof(double), cudaMemcpyDeviceToHost);
    }
    // IterEM keeps a copy of the model; UpdateModelMAP restores it if no component survives
    cudaMemcpyAsync(c->bw, c->w, m1, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(c->bmu, c->mu, md, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(c->bvar, c->var, md, cudaMemcpyDeviceToDevice, c->stream);
    rc = mstep_em(c, upW, upM, upV, &last_alive);
    if (rc) return rc;
    if (last_alive == 0) {
      cudaMemcpyAsync(c->w, c->bw, m1, cudaMemcpyDeviceToDevice, c->stream);
      cudaMemcpyAsync(c->mu, c->bmu, md, cudaMemcpyDeviceToDevice, c->stream);
      cudaMemcpyAsync(c->var, c->bvar, md, cudaMemcpyDeviceToDevice, c->stream);
    }
  }
  if (alive) *alive = last_alive;
  return sync(c, "gmm_em_iterate");
}

int gmm_mllr_estimate(gmm_handle h, int ubm_init, double* W) {
  if (!h || !W) return GMM_ERR_ARG;
  cudaSetDevice(h->device);
  return mstep_mllr(h, ubm_init, W);
}

int gmm_mllr_apply(gmm_handle h, const double* W) {
  if (!h || !W) return GMM_ERR_ARG;
  if (!h->w) return fail(h, GMM_ERR_STATE, "no model uploaded");
  cudaSetDevice(h->device);
  return mstep_mllr_apply(h, W);
}

int gmm_profile_enable(gmm_handle h, int on) {
  if (!h) return GMM_ERR_ARG;
  h->profile = on != 0;
  return GMM_OK;
}

int gmm_profile_reset(gmm_handle h) {
  if (!h) return GMM_ERR_ARG;
  drain_timers(h);
  h->timers.clear();
  return GMM_OK;
}

int gmm_profile_read(gmm_handle h, int cap, const char** names, double* ms, long long* launches) {
  if (!h) return -GMM_ERR_ARG;
  drain_timers(h);
  int n = (int)h->timers.size();
  for (int i = 0; i < n && i < cap; ++i) {
    if (names) names[i] = h->timers[i].name.c_str();
    if (ms) ms[i] = h->timers[i].ms;
    if (launches) launches[i] = h->timers[i].launches;
  }
  return n;
}

long long gmm_launch_count(gmm_handle h) { return h ? h->launches : 0; }

}  // extern "C"
