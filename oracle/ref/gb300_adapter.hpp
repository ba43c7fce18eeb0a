// GMMStatsEstimator_GB300<TS>: the reference-side binding of the gmm_gb300 engine.
//
// This is the header a maintainer adds to the reference (lib_bmssr/trainer/), beside the
// estimators it replaces. It derives from the reference's GMMStatsEstimator<TS, float, float>
// (lib_bmssr/trainer/OL_GMMStatsEstimator.h:57-182) and overrides the same virtual functions as
// the reference's CUDA estimator (OL_GMMStatsEstimator_CUDA.h:39-61), forwarding each to the
// C ABI of include/gmm_gb300.h:
//   insertModel        OL_GMMStatsEstimator.cpp:234-313  -> gmm_upload_model_slot + gmm_select_model
//   setModelToBeUsed   OL_GMMStatsEstimator.cpp:318-325  -> gmm_select_model (device-to-device)
//   accumulateStatsMT  OL_GMMStatsEstimator.cpp:884-971  -> gmm_upload_features + gmm_accumulate
//   accumulateStatsMT (file list)         :641-698       -> gmm_accumulate_files + gmm_read_stats
//   compVecsLogLikeMT  OL_GMMStatsEstimator.cpp:811-879  -> gmm_loglikes
// The base class keeps its own bookkeeping (rearranged model order, the low-variance check,
// the model group, the accumulation flags); the engine receives the rearranged arrays.
//
// Two lines of the reference change with it: GMMStats<T> names the class a friend (next to
// GMMStatsEstimator_CUDA, lib_bmssr/model/OL_GMMStats.h:115-116), because the E-step adds its
// totals into GMMStats' private _totLogLike and _totalAccSamples as the reference estimators
// do; and the estimator switch constructs it (CModelAdapt::InitializeEstimator,
// OL_ModelAdapt.cpp:248-267; getLogLike's switch, projects/GetLogLikeGMM/main.cpp:119-135).
//
// In this repository the header is compiled against the reference headers by oracle/Makefile
// (target `adapter`) and exercised by tests/test_adapter.py; it is not part of the engine.
#ifndef GMM_GB300_ADAPTER_HPP
#define GMM_GB300_ADAPTER_HPP

#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "gmm_gb300.h"
#include "trainer/OL_GMMStatsEstimator.h"

template <typename TS>
class GMMStatsEstimator_GB300 : public GMMStatsEstimator<TS, float, float> {
  typedef GMMStatsEstimator<TS, float, float> Base;

 public:
  explicit GMMStatsEstimator_GB300(int GPU_id = 0, int precision = GMM_PREC_TC)
      : _gpu(GPU_id < 0 ? 0 : GPU_id), _precision(precision) {
    if (gmm_create(_gpu, &_h) != GMM_OK)
      throw std::runtime_error(std::string("GMMStatsEstimator_GB300: ") + gmm_last_error(nullptr));
    if (gmm_set_precision(_h, precision) != GMM_OK) {
      const std::string msg = gmm_last_error(_h);
      gmm_destroy(_h);
      throw std::runtime_error("GMMStatsEstimator_GB300: " + msg);
    }
    this->_estimType = "GB300";
  }
  virtual ~GMMStatsEstimator_GB300() { gmm_destroy(_h); }

  // Rearranges the model and checks its variances in the base class (which throws as the
  // reference does), then stores it in the next device slot of the group and puts it in use.
  virtual void insertModel(GMModel& model, bool first = true) {
    Base::insertModel(model, first);
    if (first) {
      check(gmm_clear_model_slots(_h));
      _full.clear();
    }
    const int slot = (int)_full.size();
    const int M = (int)model.GetNumberOfMixtures(), D = (int)model.GetDimension();
    check(gmm_set_options(_h, this->_minLogLike, this->_minGamma, this->_min_var));
    if (model.GetFullCovStatus()) {
      // full covariances: no device slot; the arrays are uploaded whenever the model is selected
      _full.push_back(flat_model(model, true));
      upload_full(_full.back(), M, D);
    } else {
      const FlatModel f = flat_model(model, false);
      check(gmm_upload_model_slot(_h, slot, M, D, f.w.data(), f.mu.data(), f.var.data()));
      _full.push_back(FlatModel());
      check(gmm_select_model(_h, slot));
    }
    _fullInUse = model.GetFullCovStatus();
  }

  virtual void setModelToBeUsed(unsigned int n) {
    Base::setModelToBeUsed(n);  // the group's host-side state (_model, _nummix, ...)
    if (n >= _full.size()) throw std::runtime_error("setModelToBeUsed(): no such model");
    check(gmm_set_options(_h, this->_minLogLike, this->_minGamma, this->_min_var));
    _fullInUse = this->_model->GetFullCovStatus();
    if (_fullInUse)
      upload_full(_full[n], (int)this->_model->GetNumberOfMixtures(), (int)this->_model->GetDimension());
    else
      check(gmm_select_model(_h, (int)n));
  }

  virtual void accumulateStatsMT(float** vecs, unsigned int N, unsigned int dim, GMMStats<TS>& gmms) {
    if (!this->_modelIn) throw std::logic_error("accumulateStatsMT(): None model inserted! \n\t");
    if (!this->_flagsSet) this->setAccFlags(gmms);
    if (!gmms.isAllocated()) {
      gmms.alloc(this->_dim, this->_nummixAlloc, this->_fMean, this->_fVar, this->_fFullVar, false);
      gmms.reset();
    }
    if (dim != this->_dim || dim != gmms.getDim())
      throw std::logic_error("accumulateStats(): Inconsistent model & feature dimensions!");
    this->checkProperAllocation(gmms);
    // setSameDataFlag(): the frames of the previous call are still resident on the device
    if (!(this->_fSameDataProvided && _resident == vecs && _residentN == N)) upload(vecs, N, dim);
    this->_fSameDataProvided = false;
    const int flags = this->_fMixProbOnly ? GMM_ACC_PROBS_ONLY
                                          : ((this->_fMean ? GMM_ACC_MEAN : 0) | (this->_fVar ? GMM_ACC_VAR : 0));
    const int M = (int)this->_nummixAlloc;
    std::vector<double> n((size_t)M), F((size_t)M * dim), S((size_t)M * gmms.getVarDim());
    double tl = 0.0;
    long long tn = 0;
    if (_fullInUse)
      check(gmm_accumulate_full(_h, flags, n.data(), F.data(), S.data(), &tl, &tn));
    else
      check(gmm_accumulate(_h, flags, n.data(), F.data(), S.data(), &tl, &tn));
    add_stats(gmms, n, F, S, tl, tn);
  }

  // File-by-file accumulation: the engine reads the files on a loader thread and overlaps
  // the copies with the E-step (batches of _memoryBuffDataGB).
  virtual void accumulateStatsMT(CFileList& list, GMMStats<TS>& gmms, int prm_type, unsigned int dwnsmp = 1) {
    if (!this->_modelIn) throw std::logic_error("accumulateStatsMT(): None model inserted! \n\t");
    if (_fullInUse) throw std::runtime_error("accumulateStatsMT(CFileList): diagonal models only");
    if (!this->_flagsSet) this->setAccFlags(gmms);
    if (!gmms.isAllocated()) {
      gmms.alloc(this->_dim, this->_nummixAlloc, this->_fMean, this->_fVar, this->_fFullVar, false);
      gmms.reset();
    }
    this->checkProperAllocation(gmms);
    std::vector<const char*> paths;
    for (unsigned int i = 0; i < list.ListLength(); ++i) paths.push_back(list.GetItemName(i));
    const int flags = this->_fMixProbOnly ? GMM_ACC_PROBS_ONLY
                                          : ((this->_fMean ? GMM_ACC_MEAN : 0) | (this->_fVar ? GMM_ACC_VAR : 0));
    int used = 0;
    check(gmm_accumulate_files(_h, flags, (int)paths.size(), paths.data(), prm_type, dwnsmp,
                               this->_memoryBuffDataGB > 0 ? this->_memoryBuffDataGB : 1.0, &used));
    const int M = (int)this->_nummixAlloc, D = (int)this->_dim;
    std::vector<double> n((size_t)M), F((size_t)M * D), S((size_t)M * D);
    double tl = 0.0;
    long long tn = 0;
    check(gmm_read_stats(_h, n.data(), F.data(), S.data(), &tl, &tn));
    _resident = nullptr;  // the file batches are not resident afterwards
    add_stats(gmms, n, F, S, tl, tn);
  }

  virtual void compVecsLogLikeMT(float** vecs, unsigned int N, unsigned int dim, float* outLogLikes) {
    if (!this->_modelIn) throw std::logic_error("compVecsLogLikeMT(): None model inserted! \n\t");
    if (dim != this->_dim) throw std::logic_error("compVecsLogLike(): Inconsistent model & feature dimensions!");
    if (!(this->_fSameDataProvided && _resident == vecs && _residentN == N)) upload(vecs, N, dim);
    this->_fSameDataProvided = false;
    check(_fullInUse ? gmm_loglikes_full(_h, outLogLikes) : gmm_loglikes(_h, outLogLikes));
  }

  virtual GMMStatsEstimator<TS, float, float>* getNewInstance() {
    return new GMMStatsEstimator_GB300<TS>(_gpu, _precision);
  }

 private:
  struct FlatModel {
    std::vector<float> w, mu, var;
  };

  void check(int rc) const {
    if (rc != GMM_OK) throw std::runtime_error(std::string("GMMStatsEstimator_GB300: ") + gmm_last_error(_h));
  }

  // The model's arrays in its (rearranged) component order; full covariances as D x D blocks.
  static FlatModel flat_model(GMModel& model, bool full) {
    const unsigned int M = model.GetNumberOfMixtures(), D = model.GetDimension();
    const unsigned int V = full ? D * D : D;
    FlatModel f;
    f.w.resize(M);
    f.mu.resize((size_t)M * D);
    f.var.resize((size_t)M * V);
    for (unsigned int m = 0; m < M; ++m) {
      f.w[m] = model.GetMixtureWeight(m);
      const float* mu = model.GetMixtureMean(m);
      const float* var = full ? model.GetMixtureVar(m) : model.GetMixtureVarDiag(m);
      for (unsigned int d = 0; d < D; ++d) f.mu[(size_t)m * D + d] = mu[d];
      for (unsigned int v = 0; v < V; ++v) f.var[(size_t)m * V + v] = var[v];
    }
    return f;
  }

  void upload_full(const FlatModel& f, int M, int D) {
    check(gmm_upload_model_full(_h, M, D, f.w.data(), f.mu.data(), f.var.data()));
  }

  // The frames go to the device as one block: directly when vecs[i] are consecutive rows of one
  // array (Param keeps them so), else gathered into one host block first.
  void upload(float** vecs, unsigned int N, unsigned int dim) {
    bool contiguous = true;
    for (unsigned int i = 1; i < N && contiguous; ++i) contiguous = vecs[i] == vecs[0] + (size_t)i * dim;
    if (N == 0 || contiguous) {
      check(gmm_upload_features(_h, N ? vecs[0] : nullptr, (long long)N, (int)dim));
    } else {
      std::vector<float> block((size_t)N * dim);
      for (unsigned int i = 0; i < N; ++i)
        for (unsigned int d = 0; d < dim; ++d) block[(size_t)i * dim + d] = vecs[i][d];
      check(gmm_upload_features(_h, block.data(), (long long)N, (int)dim));
    }
    _resident = vecs;
    _residentN = N;
  }

  // GMMStats is only ever added to (OL_GMMStats.cpp:99-145): n into mixProb, F into mean, S into
  // var (the packed upper triangle for full covariances, GMMStats' own _allFV layout), the totals.
  static void add_stats(GMMStats<TS>& gmms, const std::vector<double>& n, const std::vector<double>& F,
                        const std::vector<double>& S, double tl, long long tn) {
    // the allocation flags directly: GMMStats::getAllocStatus falls off its end without a
    // return statement (OL_GMMStats.cpp:382-389), which GCC compiles into a trap
    const bool allM = gmms._allM, allV = gmms._allV;
    const unsigned int M = gmms.getMixNum(), D = gmms.getDim(), V = gmms.getVarDim();
    for (unsigned int m = 0; m < M; ++m) {
      typename GMMStats<TS>::mixStats& ms = gmms[m];
      ms.mixProb += (TS)n[m];
      if (allM)
        for (unsigned int d = 0; d < D; ++d) ms.mean[d] += (TS)F[(size_t)m * D + d];
      if (allV)
        for (unsigned int v = 0; v < V; ++v) ms.var[v] += (TS)S[(size_t)m * V + v];
    }
    gmms._totLogLike += (TS)tl;
    gmms._totalAccSamples += (unsigned int)tn;
  }

  gmm_handle _h = nullptr;
  int _gpu, _precision;
  std::vector<FlatModel> _full;  // per inserted model: its arrays if it has full covariances
  bool _fullInUse = false;
  float** _resident = nullptr;   // the frames last uploaded (identity of the caller's rows)
  unsigned int _residentN = 0;

  GMMStatsEstimator_GB300(const GMMStatsEstimator_GB300<TS>&);
  GMMStatsEstimator_GB300<TS>& operator=(const GMMStatsEstimator_GB300<TS>&);
};

#endif
