// Test-only C entry points that run the reference's CModelAdapt, compiled unmodified from the
// reference sources (lib_bmssr/trainer/OL_ModelAdapt.cpp, included below) with _CUDA defined,
// so that its estimator switch (--CUDA, InitializeEstimator, OL_ModelAdapt.cpp:248-267)
// constructs GMMStatsEstimator_GB300 through oracle/ref/gb300_shim. oracle/Makefile links this
// file twice: against the engine (libgmm_gb300.so) and against oracle/ref/fake_engine.c (the
// oracle's CPU port behind the same C ABI). Nothing in the product links or loads it.
//
// The access override below opens the reference classes to this file (CModelAdapt's options
// and statistics) and stands in for the one friend line GMMStats gets for the adapter
// (lib_bmssr/model/OL_GMMStats.h:115-116).
#include <cstring>
#include <cstdio>
#include <vector>
#include <string>
#include <stdexcept>
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
#include "trainer/OL_ModelAdapt.cpp"
#undef private
#undef protected

namespace {

thread_local std::string g_err;

GMModel* make_model(int M, int D, const float* w, const float* mu, const float* var) {
  GMModel* g = new GMModel(D, M, false);
  for (int m = 0; m < M; ++m)
    g->SetMixParam(m, const_cast<float*>(mu + (size_t)m * D), const_cast<float*>(var + (size_t)m * D), w[m]);
  return g;
}

void read_model(GMModel* g, int M, int D, float* w, float* mu, float* var) {
  for (int m = 0; m < M; ++m) {
    w[m] = g->GetMixtureWeight(m);
    std::memcpy(mu + (size_t)m * D, g->GetMixtureMean(m), sizeof(float) * D);
    std::memcpy(var + (size_t)m * D, g->GetMixtureVar(m), sizeof(float) * D);
  }
}

CModelAdapt::OPTIONS em_options(int iters, int gb300) {
  CModelAdapt::OPTIONS opt;
  opt._numThreads = 1;
  opt._SSEacc = false;
  opt._CUDAacc = gb300 != 0;  // the --CUDA switch: the GB300 estimator in this build
  opt._cudaGPUid = 0;
  opt._verbosity = 0;
  opt._saveMixOcc = false;
  opt._delMix = 0.0f;
  opt._adaptType = MAP;
  opt._tau = 0;
  opt._iterCountEM = iters;
  opt._iterCountMAP = 0;
  opt._AdaptWeightBool = true;
  opt._AdaptMeanBool = true;
  opt._AdaptVarBool = true;
  return opt;
}

void fill_param(Param& p, const float* X, long N, int D) {
  std::vector<float*> r((size_t)N);
  for (long i = 0; i < N; ++i) r[(size_t)i] = const_cast<float*>(X + (size_t)i * D);
  std::vector<float> cf((size_t)N, 1.0f);
  p.ExportInternal<float>(r.data(), (unsigned)N, (unsigned)D, cf.data());
}

int copy_msg(const std::string& s, char* out, int cap) {
  if (out && cap > 0) {
    std::strncpy(out, s.c_str(), (size_t)cap - 1);
    out[cap - 1] = 0;
  }
  return 0;
}

}  // namespace

extern "C" {

const char* adt_last_error() { return g_err.c_str(); }

// CModelAdapt with the --CUDA switch: InitializeEstimator constructs the estimator. Returns 0
// and getEstimationType() in `out`, or 1 and the message of the std::runtime_error it threw.
int adt_initialize(char* out, int cap) {
  try {
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = em_options(1, 1);
    cm.SetOptions(opt);
    cm.InitializeEstimator();
    copy_msg(cm._estimator->getEstimationType(), out, cap);
    return 0;
  } catch (std::runtime_error& e) {
    copy_msg(e.what(), out, cap);
    return 1;
  } catch (std::exception& e) {
    copy_msg(e.what(), out, cap);
    return 2;
  }
}

// `iters` EM iterations through CModelAdapt::IterEM (trainGMM --type 2 --tau 0), one thread,
// with the GB300 estimator (gb300 != 0) or the reference's CPU estimator. The model arrays are
// updated in place (the reference's rearranged order); ll[i] = total log-likelihood of iteration i.
int adt_em(const float* X, long N, int D, int M, float* w, float* mu, float* var, int iters, int gb300,
           double* ll, char* type, int cap) {
  try {
    GMModel* ubm = make_model(M, D, w, mu, var);
    CModelAdapt cm;
    CModelAdapt::OPTIONS opt = em_options(iters, gb300);
    cm.SetOptions(opt);
    Param p;
    fill_param(p, X, N, D);
    cm.InsertData(p, false);
    cm.Initialize(ubm);
    copy_msg(cm._estimator->getEstimationType(), type, cap);
    GMModel* model = new GMModel(ubm);
    for (int it = 0; it < iters; ++it) {
      cm.IterEM(model, 1);
      ll[it] = cm._stats.getTotLogLike();
    }
    read_model(model, M, D, w, mu, var);
    delete model;
    delete ubm;
    return 0;
  } catch (std::exception& ex) {
    g_err = ex.what();
    return 1;
  } catch (Exception* ex) {
    g_err = ex->m_strDescription;
    delete ex;
    return 2;
  }
}

// A model group on one estimator: insertModel for each of the K models (first = true for the
// first one), then for each n of sel[0..n_sel): setModelToBeUsed(n) and one accumulateStatsMT
// into fresh GMMStats (mean and variance statistics). With fresh != 0 every selection instead
// gets a new estimator holding model n alone. Models are packed [K][M] / [K][M][D]; outputs
// [n_sel][M], [n_sel][M][D], [n_sel][M][D], [n_sel] in each model's rearranged order.
int adt_group(int gb300, int fresh, const float* X, long N, int D, int M, int K, const float* w,
              const float* mu, const float* var, int n_sel, const int* sel, double* n_out, double* F_out,
              double* S_out, double* tl_out, char* type, int cap) {
  std::vector<GMModel*> models;
  GMMStatsEstimator<double>* est = nullptr;
  auto make_est = [&]() {
    GMMStatsEstimator<double>* e;
    if (gb300) e = new GMMStatsEstimator_CUDA<double>(0);
    else e = new GMMStatsEstimator<double>;
    e->_numThreads = 1;
    e->_verbosity = 0;
    return e;
  };
  try {
    for (int k = 0; k < K; ++k)
      models.push_back(make_model(M, D, w + (size_t)k * M, mu + (size_t)k * M * D, var + (size_t)k * M * D));
    if (!fresh) {
      est = make_est();
      for (int k = 0; k < K; ++k) est->insertModel(*models[(size_t)k], k == 0);
    }
    std::vector<float*> rows((size_t)N);
    for (long i = 0; i < N; ++i) rows[(size_t)i] = const_cast<float*>(X + (size_t)i * D);
    for (int s = 0; s < n_sel; ++s) {
      if (fresh) {
        delete est;
        est = make_est();
        est->insertModel(*models[(size_t)sel[s]], true);
      } else {
        est->setModelToBeUsed((unsigned)sel[s]);
      }
      copy_msg(est->getEstimationType(), type, cap);
      GMMStats<double> st(D, M, true, true, false, false);
      st.reset();
      est->setAccFlags(false, true, true, false, false);
      est->accumulateStatsMT(rows.data(), (unsigned)N, (unsigned)D, st);
      for (int m = 0; m < M; ++m) {
        n_out[(size_t)s * M + m] = st.getProb(m);
        for (int d = 0; d < D; ++d) {
          F_out[((size_t)s * M + m) * D + d] = st.getMean(m)[d];
          S_out[((size_t)s * M + m) * D + d] = st.getVar(m)[d];
        }
      }
      tl_out[s] = st.getTotLogLike();
    }
    delete est;
    for (GMModel* g : models) delete g;
    return 0;
  } catch (std::exception& ex) {
    g_err = ex.what();
    delete est;
    for (GMModel* g : models) delete g;
    return 1;
  }
}

}  // extern "C"
