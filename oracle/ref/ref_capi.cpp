// Test-only C entry points around the reference's own CPU estimator and re-estimation
// driver, compiled unmodified from the reference sources (GMM/lib_bmssr) by oracle/Makefile.
// The resulting oracle/_ref/libgmmref.so is a checker used by tests and by the fixture
// generator in tests/golden; nothing in the product links or loads it.
//
// The reference classes keep the routines the tests need (UpdateModelEM, IterEM, IterMAP,
// IterW_MLLR, the _stats member) protected or private, so this translation unit opens
// them up with the preprocessor before including the headers. No reference code is
// changed; the calls below go through the same member functions trainGMM uses:
//   - E-step:   GMMStatsEstimator{,_SSE}<double>::accumulateStatsMT
//               (lib_bmssr/trainer/OL_GMMStatsEstimator.cpp:884-971)
//   - scoring:  compVecsLogLikeMT (OL_GMMStatsEstimator.cpp:811-879)
//   - EM loop:  CModelAdapt::IterEM / UpdateModelEM (OL_ModelAdapt.cpp:1276-1296, 823-949)
//   - MAP loop: CModelAdapt::IterMAP / UpdateModelMAP (OL_ModelAdapt.cpp:1298-1317, 993-1106)
//   - MLLR:     CModelAdapt::IterW_MLLR / AdaptModelMLLR (OL_ModelAdapt.cpp:1365-1415, 1583-1612)
#include <cstring>
#include <cstdio>
#include <vector>
#include <string>
#include <stdexcept>
// Standard headers first, so the access override below only reaches the reference classes.
#include <sstream>
#include <fstream>
#include <iostream>
#include <iomanip>
#include <list>
#include <map>
#include <new>
#include <limits>
#include <thread>
#include <mutex>
#include <functional>
#include <ext/hash_map>
#include <hash_map>
#include <boost/thread.hpp>
#include <boost/program_options.hpp>

#define private public
#define protected public
#include "general/my_inttypes.h"
#include "general/Exception.h"
#include "trainer/OL_ModelAdapt.h"
#include "trainer/OL_GMMStatsEstimator_SSE.h"
#undef private
#undef protected

GMModel* make_model_full(int M, int D, const float* w, const float* mu, const float* cov);
void read_model_full(GMModel* g, int M, int D, float* w, float* mu, float* cov);
extern "C" int ref_train_full(const float* X, long N, int D, int nummix, int iters_em, float split_x,
                              float split_th, float ll_th, int verbosity, int threads, int fullcov, float* w,
                              float* mu, float* var);

namespace {

// Builds a diagonal GMModel from flat arrays (w[M], mu[M*D], var[M*D]).
GMModel* make_model(int M, int D, const float* w, const float* mu, const float* var) {
  GMModel* g = new GMModel(D, M, false);
  for (int m = 0; m < M; ++m)
    g->SetMixParam(m, const_cast<float*>(mu + (size_t)m * D), const_cast<float*>(var + (size_t)m * D), w[m]);
  return g;
}

void read_model(GMModel* g, int M, int D, float* w, float* mu, float* var) {
  for (int m = 0; m < M; ++m) {
    w[m] = g->GetMixtureWeight(m);
    memcpy(mu + (size_t)m * D, g->GetMixtureMean(m), sizeof(float) * D);
    memcpy(var + (size_t)m * D, g->GetMixtureVar(m), sizeof(float) * D);
  }
}

std::vector<float*> rows(const float* X, long N, int D) {
  std::vector<float*> r((size_t)N);
  for (long i = 0; i < N; ++i) r[(size_t)i] = const_cast<float*>(X + (size_t)i * D);
  return r;
}

GMMStatsEstimator<double>* make_estimator(int sse, int threads) {
  GMMStatsEstimator<double>* e;
  if (sse) e = new GMMStatsEstimator_SSE<double>;
  else e = new GMMStatsEstimator<double>;
  e->_numThreads = threads;
  e->_verbosity = 0;
  return e;
}

thread_local std::string g_err;

void fill_param(Param& p, const float* X, long N, int D) {
  std::vector<float*> r = rows(X, N, D);
  std::vector<float> cf((size_t)N, 1.0f);
  p.ExportInternal<float>(r.data(), (unsigned)N, (unsigned)D, cf.data());
}

CModelAdapt::OPTIONS base_options(int threads, int sse) {
  CModelAdapt::OPTIONS opt;
  opt._numThreads = threads;
  opt._SSEacc = sse != 0;
  opt._verbosity = 0;
  opt._saveMixOcc = false;
  opt._delMix = 0.0f;
  return opt;
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// Per-frame log-likelihoods (a11). Returns 0 on success.
int ref_loglikes(const float* X, long N, int D, int M, const float* w, const float* mu,
                 const float* var, int threads, int sse, float* out) {
  try {
    GMModel* g = make_model(M, D, w, mu, var);
    GMMStatsEstimator<double>* e = make_estimator(sse, threads);
    e->insertModel(*g);
    std::vector<float*> r = rows(X, N, D);
    e->compVecsLogLikeMT(r.data(), (unsigned)N, (unsigned)D, out);
    delete e;
    delete g;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
}

// One E-step (a2-a6). flags: bit0 mean stats, bit1 var stats, bit2 occupancies only.
// order[k] receives the original index of the component stored at position k after
// GMModel::RearrangeMixtures; the statistics are returned in that (rearranged) order.
int ref_accumulate(const float* X, long N, int D, int M, const float* w, const float* mu,
                   const float* var, int threads, int sse, int flags, double* n, double* F,
                   double* S, double* totLL, unsigned* totSamples, int* order) {
  try {
    std::vector<float> wtag(w, w + M);
    GMModel* g = make_model(M, D, w, mu, var);
    // Tag each component with its original index through its first mean coordinate copy.
    std::vector<float*> before((size_t)M);
    for (int m = 0; m < M; ++m) before[(size_t)m] = g->GetMixtureMean(m);
    GMMStatsEstimator<double>* e = make_estimator(sse, threads);
    e->insertModel(*g);
    for (int k = 0; k < M; ++k) {
      order[k] = -1;
      for (int m = 0; m < M; ++m)
        if (g->GetMixtureMean(k) == before[(size_t)m]) order[k] = m;
    }
    bool probsOnly = (flags & 4) != 0;
    bool fm = (flags & 1) != 0, fv = (flags & 2) != 0;
    GMMStats<double> st(D, M, fm || fv, fv, false, false);
    st.reset();
    e->setAccFlags(probsOnly, fm, fv, false, false);
    std::vector<float*> r = rows(X, N, D);
    e->accumulateStatsMT(r.data(), (unsigned)N, (unsigned)D, st);
    for (int m = 0; m < M; ++m) {
      n[m] = st.getProb(m);
      for (int d = 0; d < D; ++d) {
        if (F) F[(size_t)m * D + d] = (fm || fv) ? st.getMean(m)[d] : 0.0;
        if (S) S[(size_t)m * D + d] = fv ? st.getVar(m)[d] : 0.0;
      }
    }
    *totLL = st.getTotLogLike();
    *totSamples = st.getTotAccSamples();
    delete e;
    delete g;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
}

// `iters` EM iterations through CModelAdapt::IterEM (tau = 0 MAP-type driver, which is the
// trainGMM --type 2 --tau 0 route). Model arrays are updated in place (component order after
// the reference's rearrangement). ll[i] = total log-likelihood accumulated in iteration i.
int ref_em(const float* X, long N, int D, int M, float* w, float* mu, float* var, int iters,
           int upW, int upM, int upV, int threads, int sse, double* ll, int* order) {
  try {
    GMModel* ubm = make_model(M, D, w, mu, var);
    std::vector<float*> before((size_t)M);
    for (int m = 0; m < M; ++m) before[(size_t)m] = ubm->GetMixtureMean(m);
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = base_options(threads, sse);
    opt._adaptType = MAP;
    opt._tau = 0;
    opt._iterCountEM = iters;
    opt._iterCountMAP = 0;
    opt._AdaptWeightBool = upW != 0;
    opt._AdaptMeanBool = upM != 0;
    opt._AdaptVarBool = upV != 0;
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    cm.Initialize(ubm);
    GMModel* model = new GMModel(ubm);
    for (int it = 0; it < iters; ++it) {
      cm.IterEM(model, 1);
      ll[it] = cm._stats.getTotLogLike();
    }
    // the estimator rearranged `model` in place; report the permutation relative to input
    for (int k = 0; k < M; ++k) order[k] = k;
    read_model(model, M, D, w, mu, var);
    delete model;
    delete ubm;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
  catch (Exception* ex) { g_err = ex->m_strDescription; delete ex; return 2; }
}

// MAP adaptation through CModelAdapt::IterMAP with relevance factor tau (a9).
int ref_map(const float* X, long N, int D, int M, const float* w, const float* mu, const float* var,
            int tau, int iters, int upW, int upM, int upV, int threads, int sse, float* ow,
            float* omu, float* ovar, double* ll) {
  try {
    GMModel* ubm = make_model(M, D, w, mu, var);
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = base_options(threads, sse);
    opt._adaptType = MAP;
    opt._tau = tau;
    opt._iterCountEM = 0;
    opt._iterCountMAP = iters;
    opt._AdaptWeightBool = upW != 0;
    opt._AdaptMeanBool = upM != 0;
    opt._AdaptVarBool = upV != 0;
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    cm.Initialize(ubm);
    GMModel* model = new GMModel(ubm);
    for (int it = 0; it < iters; ++it) {
      cm.IterMAP(model, 1);
      if (ll) ll[it] = cm._stats.getTotLogLike();
    }
    read_model(model, M, D, ow, omu, ovar);
    delete model;
    delete ubm;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
  catch (Exception* ex) { g_err = ex->m_strDescription; delete ex; return 2; }
}

// Global MLLR mean transform (a10): W is D x (D+1) row-major; omu receives A*mu+b.
int ref_mllr(const float* X, long N, int D, int M, const float* w, const float* mu, const float* var,
             int iters, int ubm_init, int threads, int sse, double* W, float* omu) {
  try {
    GMModel* ubm = make_model(M, D, w, mu, var);
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = base_options(threads, sse);
    opt._adaptType = MLLR;
    opt._iterMLLR = iters;
    opt._mllrUBMInit = ubm_init != 0;
    opt._applyTransforms = true;
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    cm.Initialize(ubm);
    cm._UBM = ubm;
    MATRIX* Wm = cm.IterW_MLLR(ubm, iters, NULL);
    for (int i = 0; i < D; ++i)
      for (int j = 0; j <= D; ++j) W[(size_t)i * (D + 1) + j] = Wm->GetXY(i, j);
    GMModel* ad = cm.AdaptModelMLLR(ubm, Wm);
    for (int m = 0; m < M; ++m) memcpy(omu + (size_t)m * D, ad->GetMixtureMean(m), sizeof(float) * D);
    delete ad;
    Wm->Delete();
    delete Wm;
    delete ubm;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
  catch (Exception* ex) { g_err = ex->m_strDescription; delete ex; return 2; }
}

// Train from scratch: CModelAdapt::TrainFromScratch (OL_ModelAdapt.cpp:667-821) with the
// splitting of splitMultipleGaussians / splitGaussian (:590-665). Outputs the final model in
// its final (rearranged) component order.
int ref_train(const float* X, long N, int D, int nummix, int iters_em, float split_x, float split_th,
              float ll_th, int verbosity, int threads, float* w, float* mu, float* var) {
  return ref_train_full(X, N, D, nummix, iters_em, split_x, split_th, ll_th, verbosity, threads, 0, w, mu, var);
}

// ref_train with full covariances (fullcov = 1: var receives [nummix][D][D]).
int ref_train_full(const float* X, long N, int D, int nummix, int iters_em, float split_x, float split_th,
                   float ll_th, int verbosity, int threads, int fullcov, float* w, float* mu, float* var) {
  try {
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = base_options(threads, 0);
    opt._adaptType = FROM_SCRATCH;
    opt._iterCountEM = iters_em;
    opt._splitXpercAtOnce = split_x;
    opt._splitTh = split_th;
    opt._llTh = ll_th;
    opt._verbosity = verbosity;
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    std::streambuf* old = std::cout.rdbuf();
    std::ostringstream sink;
    std::cout.rdbuf(sink.rdbuf());  // the reference reports progress on stdout when verbose
    try {
      cm.TrainFromScratch((unsigned)nummix, fullcov != 0, NULL, "ref_train", false);
    } catch (...) {
      std::cout.rdbuf(old);
      throw;
    }
    std::cout.rdbuf(old);
    if (fullcov) read_model_full(cm._modelSP, nummix, D, w, mu, var);
    else read_model(cm._modelSP, nummix, D, w, mu, var);
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
  catch (Exception* ex) { g_err = ex->m_strDescription; delete ex; return 2; }
}

// Param::Load (param/OL_Param.cpp:224-243 -> Load / LoadHTK / LoadRaw): one feature file.
// out = NULL: only *N and *D. Returns the loader's status (-1: file not found), -2 on exception.
int ref_param_load(const char* path, int type, unsigned int dwnsmp, float* out, long long cap,
                   long long* N, int* D) {
  try {
    Param p;
    int rc = p.Load(path, type, dwnsmp);
    if (rc) return rc;
    *N = p.GetNumberOfVectors();
    *D = (int)p.GetVectorDim();
    if (out && *N > 0) {
      if (*N > cap) return -3;
      float** v = *p.GetVectors();
      for (long long i = 0; i < *N; ++i) memcpy(out + (size_t)i * *D, v[i], sizeof(float) * *D);
    }
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -2;
  } catch (Exception* e) {
    g_err = "reference exception";
    return -2;
  }
}

}  // extern "C"



// ---- full covariances (cov: M*D*D row-major). The factor and inverse go through the shim's
// restatement of spotrf / spotri (oracle/ref/shim/acml.h).

namespace {
}  // namespace

GMModel* make_model_full(int M, int D, const float* w, const float* mu, const float* cov) {
  GMModel* g = new GMModel(D, M, true);
  for (int m = 0; m < M; ++m)
    g->SetMixParam(m, const_cast<float*>(mu + (size_t)m * D), const_cast<float*>(cov + (size_t)m * D * D), w[m]);
  return g;
}
void read_model_full(GMModel* g, int M, int D, float* w, float* mu, float* cov) {
  for (int m = 0; m < M; ++m) {
    w[m] = g->GetMixtureWeight(m);
    memcpy(mu + (size_t)m * D, g->GetMixtureMean(m), sizeof(float) * D);
    memcpy(cov + (size_t)m * D * D, g->GetMixtureVar(m), sizeof(float) * D * D);
  }
}

extern "C" {

int ref_full_loglikes(const float* X, long N, int D, int M, const float* w, const float* mu,
                      const float* cov, int threads, float* out) {
  try {
    GMModel* g = make_model_full(M, D, w, mu, cov);
    GMMStatsEstimator<double>* e = make_estimator(0, threads);
    e->insertModel(*g);
    std::vector<float*> r = rows(X, N, D);
    e->compVecsLogLikeMT(r.data(), (unsigned)N, (unsigned)D, out);
    delete e;
    delete g;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
}

// E-step with full second-order statistics: Sp[M][D(D+1)/2] packed upper triangle, in the
// rearranged order (order[k] = original index at slot k).
int ref_full_accumulate(const float* X, long N, int D, int M, const float* w, const float* mu,
                        const float* cov, int threads, int flags, double* n, double* F, double* Sp,
                        double* totLL, unsigned* totSamples, int* order) {
  try {
    GMModel* g = make_model_full(M, D, w, mu, cov);
    std::vector<float*> before((size_t)M);
    for (int m = 0; m < M; ++m) before[(size_t)m] = g->GetMixtureMean(m);
    GMMStatsEstimator<double>* e = make_estimator(0, threads);
    e->insertModel(*g);
    for (int k = 0; k < M; ++k) {
      order[k] = -1;
      for (int m = 0; m < M; ++m)
        if (g->GetMixtureMean(k) == before[(size_t)m]) order[k] = m;
    }
    const bool probsOnly = (flags & 4) != 0, fm = (flags & 1) != 0, fv = (flags & 2) != 0;
    GMMStats<double> st(D, M, fm || fv, fv, fv, false);
    st.reset();
    e->setAccFlags(probsOnly, fm, fv, fv, false);
    std::vector<float*> r = rows(X, N, D);
    e->accumulateStatsMT(r.data(), (unsigned)N, (unsigned)D, st);
    const size_t P = (size_t)D * (D + 1) / 2;
    for (int m = 0; m < M; ++m) {
      n[m] = st.getProb(m);
      for (int d = 0; d < D; ++d) F[(size_t)m * D + d] = (fm || fv) ? st.getMean(m)[d] : 0.0;
      for (size_t q = 0; q < P; ++q) Sp[(size_t)m * P + q] = fv ? st.getVar(m)[q] : 0.0;
    }
    *totLL = st.getTotLogLike();
    *totSamples = st.getTotAccSamples();
    delete e;
    delete g;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
}

// EM iterations (IterEM, tau = 0) or MAP iterations (IterMAP, tau > 0) on a full-covariance
// model; the model arrays receive the result (rearranged order). ll[i]: total LL of iteration i.
int ref_full_adapt(const float* X, long N, int D, int M, float* w, float* mu, float* cov, int tau,
                   int iters, int upW, int upM, int upV, int threads, double* ll) {
  try {
    GMModel* ubm = make_model_full(M, D, w, mu, cov);
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = base_options(threads, 0);
    opt._adaptType = MAP;
    opt._tau = tau;
    opt._iterCountEM = tau == 0 ? iters : 0;
    opt._iterCountMAP = tau == 0 ? 0 : iters;
    opt._AdaptWeightBool = upW != 0;
    opt._AdaptMeanBool = upM != 0;
    opt._AdaptVarBool = upV != 0;
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    cm.Initialize(ubm);
    GMModel* model = new GMModel(ubm);
    for (int it = 0; it < iters; ++it) {
      if (tau == 0) cm.IterEM(model, 1);
      else cm.IterMAP(model, 1);
      ll[it] = cm._stats.getTotLogLike();
    }
    read_model_full(model, M, D, w, mu, cov);
    delete model;
    delete ubm;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
  catch (Exception* ex) { g_err = ex->m_strDescription; delete ex; return 2; }
}

}  // extern "C"

extern "C" {

// fMLLR (CModelAdapt::ComputeW_fMLLR, OL_ModelAdapt.cpp:1614-1719) of a diagonal UBM: W is
// D x (D+1) row-major; n, F, Sp receive the E-step statistics it used (packed full second order).
int ref_fmllr(const float* X, long N, int D, int M, const float* w, const float* mu, const float* var,
              int threads, double* W, double* n, double* F, double* Sp, double* totLL) {
  try {
    GMModel* ubm = make_model(M, D, w, mu, var);
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = base_options(threads, 0);
    opt._adaptType = fMLLR;
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    cm.Initialize(ubm);
    cm._UBM = ubm;
    MATRIX* Wm = cm.ComputeW_fMLLR(ubm);
    for (int i = 0; i < D; ++i)
      for (int j = 0; j <= D; ++j) W[(size_t)i * (D + 1) + j] = Wm->GetXY(i, j);
    const size_t P = (size_t)D * (D + 1) / 2;
    for (int m = 0; m < M; ++m) {
      n[m] = cm._stats.getProb(m);
      for (int d = 0; d < D; ++d) F[(size_t)m * D + d] = cm._stats.getMean(m)[d];
      for (size_t q = 0; q < P; ++q) Sp[(size_t)m * P + q] = cm._stats.getVar(m)[q];
    }
    *totLL = cm._stats.getTotLogLike();
    Wm->Delete();
    delete Wm;
    delete ubm;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
  catch (Exception* ex) { g_err = ex->m_strDescription; delete ex; return 2; }
}

}  // extern "C"

extern "C" {

// CModelAdapt::AdaptModel (OL_ModelAdapt.cpp:1163-1226) of a diagonal UBM with the given
// adaptation type (2 MAP, 4 MLLR+MAP), iterations and flags; the adapted model out.
int ref_adapt_model(const float* X, long N, int D, int M, const float* w, const float* mu, const float* var,
                    int type, int tau, int it_em, int it_map, int it_mllr, int mllr_init, int upW, int upM,
                    int upV, int threads, float* ow, float* omu, float* ovar) {
  try {
    GMModel* ubm = make_model(M, D, w, mu, var);
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = base_options(threads, 0);
    opt._adaptType = type;
    opt._tau = tau;
    opt._iterCountEM = it_em;
    opt._iterCountMAP = it_map;
    opt._iterMLLR = it_mllr;
    opt._mllrUBMInit = mllr_init != 0;  // the OPTIONS default is true, the command line's false
    opt._AdaptWeightBool = upW != 0;
    opt._AdaptMeanBool = upM != 0;
    opt._AdaptVarBool = upV != 0;
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    cm.AdaptModel(ubm);
    GMModel* model = cm.PickUpClientModel();
    if (!model) throw std::runtime_error("no adapted model");
    read_model(model, M, D, ow, omu, ovar);
    delete model;
    delete ubm;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
  catch (Exception* ex) { g_err = ex->m_strDescription; delete ex; return 2; }
}

}  // extern "C"

extern "C" {

// E-step with the --robust auxiliary statistics (accumulateAuxStats) of a diagonal (full = 0,
// var [M][D]) or full-covariance (full = 1, var [M][D][D]) model, one thread; order as
// ref_accumulate.
int ref_aux_accumulate(const float* X, long N, int D, int M, const float* w, const float* mu,
                       const float* var, int full, double* aux, double* aux2, double* aux3, int* order) {
  try {
    GMModel* g = full ? make_model_full(M, D, w, mu, var) : make_model(M, D, w, mu, var);
    std::vector<float*> before((size_t)M);
    for (int m = 0; m < M; ++m) before[(size_t)m] = g->GetMixtureMean(m);
    GMMStatsEstimator<double>* e = make_estimator(0, 1);
    e->insertModel(*g);
    for (int k = 0; k < M; ++k) {
      order[k] = -1;
      for (int m = 0; m < M; ++m)
        if (g->GetMixtureMean(k) == before[(size_t)m]) order[k] = m;
    }
    GMMStats<double> st(D, M, true, true, full != 0, true);
    st.reset();
    e->setAccFlags(false, true, true, full != 0, true);
    std::vector<float*> r = rows(X, N, D);
    e->accumulateStatsMT(r.data(), (unsigned)N, (unsigned)D, st);
    for (int m = 0; m < M; ++m) {
      for (int d = 0; d < D; ++d) aux[(size_t)m * D + d] = st[m].aux[d];
      aux2[m] = st[m].aux2;
      aux3[m] = st[m].aux3;
    }
    delete e;
    delete g;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
}

// EM (tau = 0) or MAP iterations with --robust on a diagonal or full-covariance model, one
// thread; the model arrays receive the result (rearranged order).
int ref_robust_adapt(const float* X, long N, int D, int M, float* w, float* mu, float* var, int full, int tau,
                     int iters, int upW, int upM, int upV, double* ll) {
  try {
    GMModel* ubm = full ? make_model_full(M, D, w, mu, var) : make_model(M, D, w, mu, var);
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = base_options(1, 0);
    opt._adaptType = MAP;
    opt._tau = tau;
    opt._iterCountEM = tau == 0 ? iters : 0;
    opt._iterCountMAP = tau == 0 ? 0 : iters;
    opt._AdaptWeightBool = upW != 0;
    opt._AdaptMeanBool = upM != 0;
    opt._AdaptVarBool = upV != 0;
    opt._robustCov = true;
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    cm.Initialize(ubm);
    GMModel* model = new GMModel(ubm);
    for (int it = 0; it < iters; ++it) {
      if (tau == 0) cm.IterEM(model, 1);
      else cm.IterMAP(model, 1);
      ll[it] = cm._stats.getTotLogLike();
    }
    if (full) read_model_full(model, M, D, w, mu, var);
    else read_model(model, M, D, w, mu, var);
    delete model;
    delete ubm;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
  catch (Exception* ex) { g_err = ex->m_strDescription; delete ex; return 2; }
}

}  // extern "C"

extern "C" {

// Global MLLR of a full-covariance UBM (IterW_MLLR + AdaptModelMLLR): W D x (D+1), omu = A mu + b.
int ref_full_mllr(const float* X, long N, int D, int M, const float* w, const float* mu, const float* cov,
                  int iters, int ubm_init, int threads, double* W, float* omu) {
  try {
    GMModel* ubm = make_model_full(M, D, w, mu, cov);
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = base_options(threads, 0);
    opt._adaptType = MLLR;
    opt._iterMLLR = iters;
    opt._mllrUBMInit = ubm_init != 0;
    opt._applyTransforms = true;
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    cm.Initialize(ubm);
    cm._UBM = ubm;
    MATRIX* Wm = cm.IterW_MLLR(ubm, iters, NULL);
    for (int i = 0; i < D; ++i)
      for (int j = 0; j <= D; ++j) W[(size_t)i * (D + 1) + j] = Wm->GetXY(i, j);
    GMModel* ad = cm.AdaptModelMLLR(ubm, Wm);
    for (int m = 0; m < M; ++m) memcpy(omu + (size_t)m * D, ad->GetMixtureMean(m), sizeof(float) * D);
    delete ad;
    Wm->Delete();
    delete Wm;
    delete ubm;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
  catch (Exception* ex) { g_err = ex->m_strDescription; delete ex; return 2; }
}

}  // extern "C"

extern "C" {

// fMLLR of a full-covariance UBM (ComputeW_fMLLR with GetMixtureVarDiag): W D x (D+1).
int ref_fmllr_full(const float* X, long N, int D, int M, const float* w, const float* mu, const float* cov,
                   double* W) {
  try {
    GMModel* ubm = make_model_full(M, D, w, mu, cov);
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = base_options(1, 0);
    opt._adaptType = fMLLR;
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    cm.Initialize(ubm);
    cm._UBM = ubm;
    MATRIX* Wm = cm.ComputeW_fMLLR(ubm);
    for (int i = 0; i < D; ++i)
      for (int j = 0; j <= D; ++j) W[(size_t)i * (D + 1) + j] = Wm->GetXY(i, j);
    Wm->Delete();
    delete Wm;
    delete ubm;
    return 0;
  } catch (std::exception& ex) { g_err = ex.what(); return 1; }
  catch (Exception* ex) { g_err = ex->m_strDescription; delete ex; return 2; }
}

}  // extern "C"
