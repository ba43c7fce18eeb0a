// C++ host side of the GB300 engine, in the shape of the reference's lib_bmssr classes:
// GMModel (model/OL_GMModel.h:69-136), GMMStats (model/OL_GMMStats.h:44-148), the estimator
// interface GMMStatsEstimator (trainer/OL_GMMStatsEstimator.h:57-182) and the re-estimation driver
// CModelAdapt (trainer/OL_ModelAdapt.h). Everything computes through the C ABI of gmm_gb300.h;
// nothing here runs on the CPU except file I/O, argument checks and the O(M D) Gaussian split.
// Errors are thrown as std::runtime_error, as the reference's estimators do.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "gmm_gb300.h"

namespace gmmgb {

// GMM with diagonal (var [M][D]) or full (var [M][D][D], row-major) covariances, with the
// file's normalisation coefficients.
class GMModel {
 public:
  GMModel() = default;
  // zero weights, components in GMMMixture::Reset state (mean 0; variances of bytes 0x01 for a
  // diagonal model, the identity for a full one; OL_GMModel.cpp:73-83)
  GMModel(int dim, int nummix, bool full_cov = false);
  int GetDimension() const { return dim_; }
  int GetNumberOfMixtures() const { return (int)w_.size(); }
  bool GetFullCovStatus() const { return full_; }
  int DimVar() const { return full_ ? dim_ * dim_ : dim_; }
  float GetMixtureWeight(int m) const { return w_[(size_t)m]; }
  void SetMixWeight(int m, float w) { w_[(size_t)m] = w; }
  float* GetMixtureMean(int m) { return &mu_[(size_t)m * dim_]; }
  float* GetMixtureVar(int m) { return &var_[(size_t)m * DimVar()]; }
  const float* GetMixtureMean(int m) const { return &mu_[(size_t)m * dim_]; }
  const float* GetMixtureVar(int m) const { return &var_[(size_t)m * DimVar()]; }
  std::vector<float>& weights() { return w_; }
  std::vector<float>& means() { return mu_; }
  std::vector<float>& vars() { return var_; }
  const std::vector<float>& weights() const { return w_; }
  const std::vector<float>& means() const { return mu_; }
  const std::vector<float>& vars() const { return var_; }
  // GMModel::RearrangeMixtures (OL_GMModel.cpp:857-885): non-zero weights keep their order, the
  // k-th zero-weight component goes to slot M-1-k. Returns the number of zero-weight components.
  int RearrangeMixtures();
  // GMModel::Load / Save (text: WriteTXT / ReadTXT, OL_GMModel.cpp:475-547, 627-753; binary
  // "GMM-DB-VN": WriteBIN / ReadBIN, :551-624, 757-853; a full model's text weight line ends in
  // " F" and its binary dimension is negated). Zero-weight components are not saved.
  void Load(const std::string& path, bool txt);
  void Save(const std::string& path, bool txt) const;

 private:
  int dim_ = 0;
  bool full_ = false;
  std::vector<float> norm_, w_, mu_, var_;
};

// GMMStats<double>: occupation n [M], first order F [M][D], second order S [M][varsize] with
// varsize = D, or D(D+1)/2 (the packed upper triangle in row order) for a full-covariance model.
// The estimator only ever adds into it (OL_GMMStats.cpp:99-145).
struct GMMStats {
  int M = 0, D = 0;
  bool full = false;
  std::vector<double> n, F, S;
  double totLogLike = 0.0;
  long long totalAccSamples = 0;
  int varsize() const { return full ? D * (D + 1) / 2 : D; }
  void alloc(int M_, int D_, bool full_ = false);
  void reset();
  // GMMStats<double>::save / load (OL_GMMStats.cpp:493-778): binary = seven int32 (mixProb,
  // mean, var and full-var flags, dim, varsize, nummix) then per component n, F[D], S[varsize]
  // as doubles; text = the same header line, a blank line, then per component "n", " F..",
  // " S..", blank, in ostream's default 6-digit format.
  void save(const std::string& path, bool txt) const;
  void load(const std::string& path, bool txt);
};

// The same layout for single-precision records (GMMStats<float>), as CModelAdapt::Save writes a
// model or an MLLR transform with --save-in-stat-form (OL_ModelAdapt.cpp:1946-1987); `mean` or
// `var` may be null (not saved).
void save_stats_float(const std::string& path, bool txt, int dim, int nummix, const float* mixprob,
                      const float* mean, const float* var);

// GMMStatsEstimator implemented on one GB300: the virtuals the reference's estimators override
// (insertModel, accumulateStatsMT, compVecsLogLikeMT) and its public knobs.
class GMMStatsEstimatorGB300 {
 public:
  explicit GMMStatsEstimatorGB300(int gpu_id = 0, int precision = GMM_PREC_TC);
  ~GMMStatsEstimatorGB300();
  GMMStatsEstimatorGB300(const GMMStatsEstimatorGB300&) = delete;
  GMMStatsEstimatorGB300& operator=(const GMMStatsEstimatorGB300&) = delete;

  float _minLogLike = -1e20f, _minGamma = 1e-4f, _min_var = 1e-6f;

  // insertModel (OL_GMMStatsEstimator.cpp:234-313): rearranges `model` in place, checks the
  // variances (a full model: factors its covariances) and makes the model resident.
  void insertModel(GMModel& model, bool first = true);
  void setAccFlags(bool mixProbsOnly, bool mean, bool var);
  void setSameDataFlag() { same_data_ = true; }
  // accumulateStatsMT (:884-971): frames [N][dim] in one block; statistics are added into gmms.
  void accumulateStatsMT(const float* vecs, unsigned N, unsigned dim, GMMStats& gmms);
  // compVecsLogLikeMT (:811-879): per-frame log-likelihoods into out [N].
  void compVecsLogLikeMT(const float* vecs, unsigned N, unsigned dim, float* out);
  gmm_handle handle() const { return h_; }
  void check(int rc) const;

 private:
  void upload(const float* vecs, unsigned N, unsigned dim);
  gmm_handle h_ = nullptr;
  int M_ = 0;
  bool full_ = false;
  int flags_ = GMM_ACC_MEAN | GMM_ACC_VAR;
  bool same_data_ = false;
  const float* last_ = nullptr;
  unsigned last_n_ = 0;
};

// The options of CModelAdapt::OPTIONS on the diagonal hot path (defaults of GetOptions,
// OL_ModelAdapt.cpp:2032-2132).
enum AdaptType { FROM_SCRATCH = 0, MLLR = 1, MAP = 2, FMLLR = 3, MLLR_MAP = 4 };
struct AdaptOptions {
  int adaptType = MAP;
  int tau = 0;
  int iterCountEM = 0, iterCountMAP = 0;
  bool AdaptWeightBool = false, AdaptMeanBool = true, AdaptVarBool = false;
  int iterMLLR = 1;
  int iterfMLLR = 20;  // _iter_fMLLR (OL_ModelAdapt.cpp:190)
  bool mllrUBMInit = false, applyTransforms = false, saveTransforms = false;
  std::string transformFileExt = ".mat";
  float min_var = 1e-6f;
  float splitXpercAtOnce = 0.0f, splitTh = 0.0f, llTh = 0.0f;
  bool robustCov = false;  // --robust
  int verbosity = 0;
  int precision = GMM_PREC_TC;
  int gpu = 0;
};

// CModelAdapt for MAP (incl. EM with tau = 0), MLLR and training from scratch, on the device.
class ModelAdapt {
 public:
  explicit ModelAdapt(const AdaptOptions& opt);
  ~ModelAdapt();
  void InsertData(const float* X, long long N, int D);
  // InsertData(CFileList*) (file-by-file mode): every E-step streams the files through
  // gmm_accumulate_files in batches of at most buffer_gb instead of keeping the frames resident.
  void InsertFiles(const std::vector<std::string>& paths, int prm_type, unsigned dwnsmp, double buffer_gb);
  // AdaptModel (OL_ModelAdapt.cpp:1163-1226): MAP (IterEM then IterMAP), MLLR, fMLLR or MLLR+MAP.
  void AdaptModel(const GMModel& ubm);
  // TrainFromScratch (OL_ModelAdapt.cpp:667-821); `init` (optional) is the model the splitting
  // starts from instead of the global Gaussian and decides diagonal vs full; fullcov trains full
  // covariance matrices (splits along the leading eigenvector, sign: largest component positive).
  void TrainFromScratch(int nummix, const GMModel* init = nullptr, bool fullcov = false);
  const GMModel& GetModel() const { return model_; }
  const std::vector<double>& GetW() const { return W_; }  // (f)MLLR transform D x (D+1)
  bool ModelTrained() const { return trained_; }
  long long NumFrames() const { return N_; }
  // CModelAdapt::Save (OL_ModelAdapt.cpp:1930-1989): the MLLR transform (when it is the result,
  // or saveTransforms is set) to FileName with its extension replaced by transformFileExt, and
  // the adapted / trained model to FileName.
  void Save(const std::string& FileName, bool save_txt, bool save_in_stat_form = false) const;
  // SaveTRNMatrices (OL_ModelAdapt.cpp:1900-1928): " MLLR" / " fMLLR", " 1\tD D+1", rows of " value".
  void SaveTRNMatrices(const std::string& FileName) const;
  std::vector<double> ll_history;

 private:
  void upload_model(GMModel& m);
  void set_prior(const GMModel& ubm);
  double total_ll();
  int em_update();
  void read_model(GMModel& m);
  void estep(int flags);
  void check(int rc) const;
  void IterEM(GMModel& model, int iters);
  void IterMAP(GMModel& model, const GMModel& ubm, int iters);
  std::vector<double> ComputeW_MLLR(GMModel& model, const GMModel& ubm);
  std::vector<double> IterW_MLLR(const GMModel& ubm);
  GMModel AdaptModelMLLR(const GMModel& model, const std::vector<double>& W);
  void splitMultipleGaussians(GMModel& model);
  AdaptOptions o_;
  gmm_handle h_ = nullptr;
  std::vector<float> X_;
  long long N_ = 0;
  int D_ = 0;
  bool uploaded_ = false, trained_ = false, full_ = false;
  std::vector<std::string> files_;
  int prm_type_ = 0;
  unsigned dwnsmp_ = 1;
  double buffer_gb_ = 0.05;
  GMModel model_;
  std::vector<double> W_;
};

// Feature files (SVES / HTK / RAW) through gmm_read_param.
std::vector<float> read_features(const std::string& path, int prm_type, unsigned dwnsmp, long long* N, int* D);

}  // namespace gmmgb
