// Implementation of gmm_host.hpp: model files, the estimator over the C ABI, and the
// re-estimation driver (EM / MAP / MLLR / training from scratch).
#include "gmm_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <sstream>

namespace gmmgb {

namespace {

float reset_var() {
  // GMMMixture::Reset fills the variances with memset(.., 1, ..) (OL_GMModel.cpp:73-83)
  uint32_t bits = 0x01010101u;
  float f;
  std::memcpy(&f, &bits, sizeof f);
  return f;
}

void fail(const std::string& m) { throw std::runtime_error(m); }

}  // namespace

// ------------------------------------------------------------------ GMModel

GMModel::GMModel(int dim, int nummix, bool full_cov)
    : dim_(dim), full_(full_cov), norm_((size_t)dim, 1.0f), w_((size_t)nummix, 0.0f),
      mu_((size_t)nummix * dim, 0.0f),
      var_((size_t)nummix * (full_cov ? dim * dim : dim), full_cov ? 0.0f : reset_var()) {
  if (full_cov)
    for (int m = 0; m < nummix; ++m)
      for (int d = 0; d < dim; ++d) var_[((size_t)m * dim + d) * dim + d] = 1.0f;
}

int GMModel::RearrangeMixtures() {
  const int M = GetNumberOfMixtures(), V = DimVar();
  std::vector<int> order((size_t)M);
  int nz = 0, z = 1;
  for (int m = 0; m < M; ++m) {
    if (w_[(size_t)m] > 0.0f) order[(size_t)nz++] = m;
    else order[(size_t)(M - z++)] = m;
  }
  std::vector<float> w((size_t)M), mu(mu_.size()), var(var_.size());
  for (int k = 0; k < M; ++k) {
    const int m = order[(size_t)k];
    w[(size_t)k] = w_[(size_t)m];
    std::memcpy(&mu[(size_t)k * dim_], &mu_[(size_t)m * dim_], sizeof(float) * dim_);
    std::memcpy(&var[(size_t)k * V], &var_[(size_t)m * V], sizeof(float) * V);
  }
  w_.swap(w);
  mu_.swap(mu);
  var_.swap(var);
  return z - 1;
}

void GMModel::Load(const std::string& path, bool txt) {
  if (txt) {
    std::ifstream f(path);
    if (!f) fail("GMModel::Load(): cannot open " + path);
    std::vector<std::string> lines;
    std::string ln;
    while (std::getline(f, ln)) {
      const size_t a = ln.find_first_not_of(" \t\r"), b = ln.find_last_not_of(" \t\r");
      lines.push_back(a == std::string::npos ? std::string() : ln.substr(a, b - a + 1));
    }
    size_t i = 0;
    auto num = [&](size_t k) -> double {
      if (k >= lines.size()) fail("GMModel::Load(): truncated file " + path);
      return std::stod(lines[k]);
    };
    dim_ = (int)num(i++);
    norm_.assign((size_t)dim_, 0.0f);
    for (int d = 0; d < dim_; ++d) norm_[(size_t)d] = (float)num(i++);
    const int M = (int)num(i++);
    w_.assign((size_t)M, 0.0f);
    mu_.clear();
    var_.clear();
    for (int m = 0; m < M; ++m) {
      std::istringstream head(lines.at(i));
      std::string tok, kind;
      head >> tok >> kind;
      full_ = kind == "F";
      w_[(size_t)m] = (float)std::stod(tok);
      i += 2;
      for (int d = 0; d < dim_; ++d) mu_.push_back((float)num(i + d));
      i += dim_ + 1;
      if (full_) {  // each row: the diagonal element, then the D values of the row
        for (int r = 0; r < dim_; ++r) {
          if (i + r >= lines.size()) fail("GMModel::Load(): truncated file " + path);
          std::istringstream row(lines[i + r]);
          double v = 0.0;
          row >> v;
          for (int c = 0; c < dim_; ++c) {
            if (!(row >> v)) fail("GMModel::Load(): short covariance row in " + path);
            var_.push_back((float)v);
          }
        }
      } else {
        for (int d = 0; d < dim_; ++d) var_.push_back((float)num(i + d));
      }
      i += dim_ + 1;
    }
  } else {
    std::ifstream f(path, std::ios::binary);
    if (!f) fail("GMModel::Load(): cannot open " + path);
    char tag[9];
    int16_t D = 0, M = 0;
    f.read(tag, 9);
    if (!f || std::memcmp(tag, "GMM-DB-VN", 9) != 0) fail("GMModel::Load(): not a GMM-DB-VN file: " + path);
    f.read(reinterpret_cast<char*>(&D), 2);
    full_ = D < 0;
    dim_ = full_ ? -D : D;
    const int V = DimVar();
    norm_.assign((size_t)dim_, 0.0f);
    f.read(reinterpret_cast<char*>(norm_.data()), sizeof(float) * dim_);
    f.read(reinterpret_cast<char*>(&M), 2);
    w_.assign((size_t)M, 0.0f);
    mu_.assign((size_t)M * dim_, 0.0f);
    var_.assign((size_t)M * V, 0.0f);
    f.read(reinterpret_cast<char*>(w_.data()), sizeof(float) * M);
    for (int m = 0; m < M; ++m) {
      f.read(reinterpret_cast<char*>(&mu_[(size_t)m * dim_]), sizeof(float) * dim_);
      f.read(reinterpret_cast<char*>(&var_[(size_t)m * V]), sizeof(float) * V);
    }
    if (!f) fail("GMModel::Load(): truncated file " + path);
  }
}

void GMModel::Save(const std::string& path, bool txt) const {
  std::vector<int> keep;
  for (int m = 0; m < GetNumberOfMixtures(); ++m)
    if (w_[(size_t)m] != 0.0f) keep.push_back(m);
  const int V = DimVar();
  if (txt) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) fail("GMModel::Save(): cannot open " + path);
    std::fprintf(f, "%d\n", dim_);
    for (float v : norm_) std::fprintf(f, "%15e\n", v);
    std::fprintf(f, "%d\n", (int)keep.size());
    for (int m : keep) {
      std::fprintf(f, full_ ? "%15e F\n\n" : "%15e\n\n", w_[(size_t)m]);
      for (int d = 0; d < dim_; ++d) std::fprintf(f, "%15e\n", mu_[(size_t)m * dim_ + d]);
      std::fprintf(f, "\n");
      const float* C = &var_[(size_t)m * V];
      if (full_) {
        for (int r = 0; r < dim_; ++r) {
          std::fprintf(f, "%15e", C[(size_t)r * dim_ + r]);
          for (int c = 0; c < dim_; ++c) std::fprintf(f, " %15e", C[(size_t)r * dim_ + c]);
          std::fprintf(f, "\n");
        }
      } else {
        for (int d = 0; d < dim_; ++d) std::fprintf(f, "%15e\n", C[d]);
      }
      std::fprintf(f, "\n");
    }
    std::fclose(f);
  } else {
    std::ofstream f(path, std::ios::binary);
    if (!f) fail("GMModel::Save(): cannot open " + path);
    const int16_t D = (int16_t)(full_ ? -dim_ : dim_), M = (int16_t)keep.size();
    f.write("GMM-DB-VN", 9);
    f.write(reinterpret_cast<const char*>(&D), 2);
    f.write(reinterpret_cast<const char*>(norm_.data()), sizeof(float) * dim_);
    f.write(reinterpret_cast<const char*>(&M), 2);
    for (int m : keep) f.write(reinterpret_cast<const char*>(&w_[(size_t)m]), sizeof(float));
    for (int m : keep) {
      f.write(reinterpret_cast<const char*>(&mu_[(size_t)m * dim_]), sizeof(float) * dim_);
      f.write(reinterpret_cast<const char*>(&var_[(size_t)m * V]), sizeof(float) * V);
    }
  }
}

// ------------------------------------------------------------------ GMMStats

void GMMStats::alloc(int M_, int D_, bool full_) {
  M = M_;
  D = D_;
  full = full_;
  n.assign((size_t)M, 0.0);
  F.assign((size_t)M * D, 0.0);
  S.assign((size_t)M * varsize(), 0.0);
  totLogLike = 0.0;
  totalAccSamples = 0;
}

void GMMStats::reset() { alloc(M, D, full); }

namespace {

// The header and records of the GMMStats file layout, for T = double or float.
template <typename T>
void write_stats(const std::string& path, bool txt, int dim, int nummix, const T* mp, const T* mean,
                 const T* var, int varsize) {
  FILE* f = std::fopen(path.c_str(), txt ? "w" : "wb");
  if (!f) fail("save(): Unable to open file " + path);
  const int32_t hdr[7] = {1, mean != nullptr, var != nullptr, var != nullptr && varsize != dim, dim,
                          var ? varsize : 0, nummix};
  bool ok = true;
  if (txt) {
    ok = std::fprintf(f, "%d %d %d %d %d %d %d\n\n", hdr[0], hdr[1], hdr[2], hdr[3], hdr[4], hdr[5], hdr[6]) > 0;
    for (int m = 0; ok && m < nummix; ++m) {
      ok = std::fprintf(f, "%g\n", (double)mp[m]) > 0;
      if (mean) {
        for (int d = 0; ok && d < dim; ++d) ok = std::fprintf(f, " %g", (double)mean[(size_t)m * dim + d]) > 0;
        ok = ok && std::fputc('\n', f) != EOF;
      }
      if (var) {
        for (int d = 0; ok && d < varsize; ++d) ok = std::fprintf(f, " %g", (double)var[(size_t)m * varsize + d]) > 0;
        ok = ok && std::fputc('\n', f) != EOF;
      }
      ok = ok && std::fputc('\n', f) != EOF;
    }
  } else {
    ok = std::fwrite(hdr, sizeof hdr, 1, f) == 1;
    for (int m = 0; ok && m < nummix; ++m) {
      ok = std::fwrite(&mp[m], sizeof(T), 1, f) == 1;
      if (ok && mean) ok = std::fwrite(&mean[(size_t)m * dim], sizeof(T), (size_t)dim, f) == (size_t)dim;
      if (ok && var) ok = std::fwrite(&var[(size_t)m * varsize], sizeof(T), (size_t)varsize, f) == (size_t)varsize;
    }
  }
  if (std::fclose(f) != 0 || !ok) fail("save(): Exception writing file " + path);
}

}  // namespace

void GMMStats::save(const std::string& path, bool txt) const {
  write_stats<double>(path, txt, D, M, n.data(), F.data(), S.data(), varsize());
}

void GMMStats::load(const std::string& path, bool txt) {
  std::ifstream f(path, txt ? std::ios::in : std::ios::binary);
  if (!f) fail("load(): Unable to open file " + path);
  int32_t h[7] = {0, 0, 0, 0, 0, 0, 0};
  if (txt) {
    for (int k = 0; k < 7; ++k) f >> h[k];
  } else {
    f.read(reinterpret_cast<char*>(h), sizeof h);
  }
  if (!f) fail("load(): Exception reading file " + path);
  alloc(h[6], h[4], h[3] != 0);
  const int varsize = h[5];
  if (h[2] && varsize != this->varsize()) fail("load(): inconsistent statistics sizes in " + path);
  for (int m = 0; m < M; ++m) {
    double* Fm = &F[(size_t)m * D];
    double* Sm = &S[(size_t)m * varsize];
    if (txt) {
      if (h[0]) f >> n[(size_t)m];
      if (h[1])
        for (int d = 0; d < D; ++d) f >> Fm[d];
      if (h[2])
        for (int d = 0; d < varsize; ++d) f >> Sm[d];
    } else {
      if (h[0]) f.read(reinterpret_cast<char*>(&n[(size_t)m]), sizeof(double));
      if (h[1]) f.read(reinterpret_cast<char*>(Fm), sizeof(double) * D);
      if (h[2]) f.read(reinterpret_cast<char*>(Sm), sizeof(double) * varsize);
    }
    if (!f) fail("load(): Exception reading file " + path);
  }
}

void save_stats_float(const std::string& path, bool txt, int dim, int nummix, const float* mixprob,
                      const float* mean, const float* var) {
  write_stats<float>(path, txt, dim, nummix, mixprob, mean, var, dim);
}

// ------------------------------------------------------------------ estimator

GMMStatsEstimatorGB300::GMMStatsEstimatorGB300(int gpu_id, int precision) {
  if (gmm_create(gpu_id < 0 ? 0 : gpu_id, &h_)) throw std::runtime_error(gmm_last_error(nullptr));
  check(gmm_set_precision(h_, precision));
}

GMMStatsEstimatorGB300::~GMMStatsEstimatorGB300() { gmm_destroy(h_); }

void GMMStatsEstimatorGB300::check(int rc) const {
  if (rc) throw std::runtime_error(gmm_last_error(h_));
}

void GMMStatsEstimatorGB300::insertModel(GMModel& model, bool) {
  model.RearrangeMixtures();
  check(gmm_set_options(h_, _minLogLike, _minGamma, _min_var));
  full_ = model.GetFullCovStatus();
  if (full_)
    check(gmm_upload_model_full(h_, model.GetNumberOfMixtures(), model.GetDimension(), model.weights().data(),
                                model.means().data(), model.vars().data()));
  else
    check(gmm_upload_model(h_, model.GetNumberOfMixtures(), model.GetDimension(), model.weights().data(),
                           model.means().data(), model.vars().data()));
  M_ = model.GetNumberOfMixtures();
}

void GMMStatsEstimatorGB300::setAccFlags(bool mixProbsOnly, bool mean, bool var) {
  flags_ = (mean ? GMM_ACC_MEAN : 0) | (var ? GMM_ACC_VAR : 0) | (mixProbsOnly ? GMM_ACC_PROBS_ONLY : 0);
}

void GMMStatsEstimatorGB300::upload(const float* vecs, unsigned N, unsigned dim) {
  // the frames stay resident while the caller says they did not change (setSameDataFlag)
  if (!(same_data_ && vecs == last_ && N == last_n_)) check(gmm_upload_features(h_, vecs, N, (int)dim));
  last_ = vecs;
  last_n_ = N;
  same_data_ = false;
}

void GMMStatsEstimatorGB300::accumulateStatsMT(const float* vecs, unsigned N, unsigned dim, GMMStats& gmms) {
  if (M_ == 0) fail("accumulateStatsMT(): None model inserted!");
  upload(vecs, N, dim);
  // the estimator allocates the statistics when the caller did not (OL_GMMStatsEstimator.cpp:1108-1112)
  if (gmms.M == 0) gmms.alloc(M_, (int)dim, full_);
  if (gmms.M != M_ || gmms.D != (int)dim || gmms.full != full_)
    fail("accumulateStatsMT(): statistics and model sizes differ");
  const int M = M_;
  std::vector<double> n, F, S;
  double tl = 0.0;
  long long tn = 0;
  n.assign((size_t)M, 0.0);
  F.assign((size_t)M * dim, 0.0);
  S.assign((size_t)M * gmms.varsize(), 0.0);
  if (full_)  // full second-order statistics imply variance statistics (OL_GMMStatsEstimator.cpp:410-412)
    check(gmm_accumulate_full(h_, flags_ | GMM_ACC_VAR, n.data(), F.data(), S.data(), &tl, &tn));
  else
    check(gmm_accumulate(h_, flags_, n.data(), F.data(), S.data(), &tl, &tn));
  for (size_t k = 0; k < n.size(); ++k) gmms.n[k] += n[k];
  for (size_t k = 0; k < F.size(); ++k) gmms.F[k] += F[k];
  for (size_t k = 0; k < S.size(); ++k) gmms.S[k] += S[k];
  gmms.totLogLike += tl;
  gmms.totalAccSamples += tn;
}

void GMMStatsEstimatorGB300::compVecsLogLikeMT(const float* vecs, unsigned N, unsigned dim, float* out) {
  upload(vecs, N, dim);
  check(full_ ? gmm_loglikes_full(h_, out) : gmm_loglikes(h_, out));
}

// ------------------------------------------------------------------ ModelAdapt

ModelAdapt::ModelAdapt(const AdaptOptions& opt) : o_(opt) {
  if (gmm_create(o_.gpu, &h_)) throw std::runtime_error(gmm_last_error(nullptr));
  check(gmm_set_precision(h_, o_.precision));
  check(gmm_set_robust(h_, o_.robustCov));
}

ModelAdapt::~ModelAdapt() { gmm_destroy(h_); }

void ModelAdapt::check(int rc) const {
  if (rc) throw std::runtime_error(gmm_last_error(h_));
}

void ModelAdapt::InsertData(const float* X, long long N, int D) {
  X_.assign(X, X + (size_t)N * D);
  N_ = N;
  D_ = D;
  uploaded_ = false;
  files_.clear();
}

void ModelAdapt::InsertFiles(const std::vector<std::string>& paths, int prm_type, unsigned dwnsmp, double buffer_gb) {
  files_.clear();
  N_ = 0;
  D_ = 0;
  for (const auto& p : paths) {  // headers only: frame counts and the dimension
    long long n = 0;
    int d = 0;
    if (gmm_read_param(p.c_str(), prm_type, dwnsmp, nullptr, 0, &n, &d) || n == 0) continue;
    if (D_ && d != D_) fail("InsertData(): feature files of different dimensions");
    D_ = d;
    N_ += n;
    files_.push_back(p);
  }
  prm_type_ = prm_type;
  dwnsmp_ = dwnsmp;
  buffer_gb_ = buffer_gb;
  X_.clear();
  uploaded_ = false;
}

void ModelAdapt::upload_model(GMModel& m) {
  if (N_ == 0) fail("AdaptModel(): Insert adaptation data first!");
  if (!uploaded_ && files_.empty()) {
    check(gmm_upload_features(h_, X_.data(), N_, D_));
    uploaded_ = true;
  }
  check(gmm_set_options(h_, -1e20f, 1e-4f, o_.min_var));
  full_ = m.GetFullCovStatus();
  if (full_ && !files_.empty()) fail("AdaptModel(): file-by-file accumulation supports diagonal models only");
  if (full_)
    check(gmm_upload_model_full(h_, m.GetNumberOfMixtures(), m.GetDimension(), m.weights().data(),
                                m.means().data(), m.vars().data()));
  else
    check(gmm_upload_model(h_, m.GetNumberOfMixtures(), m.GetDimension(), m.weights().data(), m.means().data(),
                           m.vars().data()));
}

// The device-side M-step / readback entry points of the current model's family.
void ModelAdapt::set_prior(const GMModel& u) {
  check(full_ ? gmm_set_prior_full(h_, u.weights().data(), u.means().data(), u.vars().data())
              : gmm_set_prior(h_, u.weights().data(), u.means().data(), u.vars().data()));
}

double ModelAdapt::total_ll() {
  double tl = 0.0;
  long long tn = 0;
  check(full_ ? gmm_read_stats_full(h_, nullptr, nullptr, nullptr, &tl, &tn)
              : gmm_read_stats(h_, nullptr, nullptr, nullptr, &tl, &tn));
  return tl;
}

int ModelAdapt::em_update() {
  int alive = 0;
  check(full_ ? gmm_em_update_full(h_, o_.AdaptWeightBool, o_.AdaptMeanBool, o_.AdaptVarBool, &alive)
              : gmm_em_update(h_, o_.AdaptWeightBool, o_.AdaptMeanBool, o_.AdaptVarBool, &alive));
  return alive;
}

void ModelAdapt::read_model(GMModel& m) {
  check(full_ ? gmm_read_model_full(h_, m.weights().data(), m.means().data(), m.vars().data())
              : gmm_read_model(h_, m.weights().data(), m.means().data(), m.vars().data()));
}

void ModelAdapt::estep(int flags) {
  if (full_) {  // a full model always gathers full second-order statistics
    check(gmm_accumulate_full_device(h_, flags | GMM_ACC_VAR));
    return;
  }
  if (files_.empty()) {
    check(gmm_accumulate_device(h_, flags));
    return;
  }
  std::vector<const char*> p;
  for (const auto& f : files_) p.push_back(f.c_str());
  int used = 0;
  check(gmm_accumulate_files(h_, flags, (int)p.size(), p.data(), prm_type_, dwnsmp_, buffer_gb_, &used));
}

void ModelAdapt::IterEM(GMModel& model, int iters) {
  if (files_.empty() && !model.GetFullCovStatus()) {
    upload_model(model);  // gmm_em_iterate rearranges on the device each iteration, as insertModel
    std::vector<double> ll((size_t)std::max(iters, 1));
    int alive = 0;
    check(gmm_em_iterate(h_, iters, o_.AdaptWeightBool, o_.AdaptMeanBool, o_.AdaptVarBool, ll.data(), &alive));
    ll_history.insert(ll_history.end(), ll.begin(), ll.begin() + iters);
    check(gmm_read_model(h_, model.weights().data(), model.means().data(), model.vars().data()));
    return;
  }
  // file by file, or a full-covariance model: insertModel + E-step + UpdateModelEM per iteration
  // (IterEM, OL_ModelAdapt.cpp:1276-1296); all components killed -> the model before the update
  const int flags = GMM_ACC_MEAN | GMM_ACC_VAR;
  for (int it = 0; it < iters; ++it) {
    model.RearrangeMixtures();
    upload_model(model);
    estep(flags);
    ll_history.push_back(total_ll());
    if (em_update() == 0) continue;
    read_model(model);
  }
}

void ModelAdapt::IterMAP(GMModel& model, const GMModel& ubm, int iters) {
  const int flags = (o_.AdaptMeanBool ? GMM_ACC_MEAN : 0) | (o_.AdaptVarBool ? GMM_ACC_VAR : 0) |
                    ((o_.AdaptWeightBool && !o_.AdaptMeanBool && !o_.AdaptVarBool) ? GMM_ACC_PROBS_ONLY : 0);
  for (int it = 0; it < iters; ++it) {
    model.RearrangeMixtures();
    upload_model(model);
    set_prior(ubm);
    estep(flags);
    ll_history.push_back(total_ll());
    if (o_.tau == 0) {
      if (em_update() == 0) {
        model = ubm;
        continue;
      }
    } else {
      check(full_ ? gmm_map_update_full(h_, o_.tau, o_.AdaptWeightBool, o_.AdaptMeanBool, o_.AdaptVarBool)
                  : gmm_map_update(h_, o_.tau, o_.AdaptWeightBool, o_.AdaptMeanBool, o_.AdaptVarBool));
    }
    read_model(model);
  }
}

std::vector<double> ModelAdapt::ComputeW_MLLR(GMModel& model, const GMModel& ubm) {
  // a full-covariance model uses its covariance diagonals (GetMixtureVarDiag)
  model.RearrangeMixtures();
  upload_model(model);
  set_prior(ubm);
  estep(GMM_ACC_MEAN);
  std::vector<double> W((size_t)D_ * (D_ + 1));
  check(full_ ? gmm_mllr_estimate_full(h_, o_.mllrUBMInit, W.data()) : gmm_mllr_estimate(h_, o_.mllrUBMInit, W.data()));
  return W;
}

GMModel ModelAdapt::AdaptModelMLLR(const GMModel& model, const std::vector<double>& W) {
  GMModel out = model;
  upload_model(out);
  check(full_ ? gmm_mllr_apply_full(h_, W.data()) : gmm_mllr_apply(h_, W.data()));
  read_model(out);
  return out;
}

namespace {
// CModelAdapt::UpdateMLLRMatrix (OL_ModelAdapt.cpp:1319-1340): [A|b] <- [A_new A | A_new b + b_new].
std::vector<double> compose(const std::vector<double>& Ws, const std::vector<double>& Wn, int D) {
  const int E = D + 1;
  std::vector<double> out((size_t)D * E, 0.0);
  for (int k = 0; k < D; ++k) {
    for (int x = 0; x < D; ++x) {
      double s = 0.0;
      for (int y = 0; y < D; ++y) s += Wn[(size_t)k * E + y] * Ws[(size_t)y * E + x];
      out[(size_t)k * E + x] += s;
      out[(size_t)k * E + D] += Wn[(size_t)k * E + x] * Ws[(size_t)x * E + D];
    }
    out[(size_t)k * E + D] += Wn[(size_t)k * E + D];
  }
  return out;
}
}  // namespace

// IterW_MLLR (OL_ModelAdapt.cpp:1365-1415): iterMLLR transforms, each estimated on the model the
// previous ones produced, composed into one.
std::vector<double> ModelAdapt::IterW_MLLR(const GMModel& ubm) {
  GMModel u = ubm;
  std::vector<double> W = ComputeW_MLLR(u, ubm);
  if (o_.iterMLLR > 1) {
    GMModel sp = AdaptModelMLLR(ubm, W);
    for (int it = 1; it < o_.iterMLLR - 1; ++it) {
      std::vector<double> Wt = ComputeW_MLLR(sp, ubm);
      sp = AdaptModelMLLR(sp, Wt);
      W = compose(W, Wt, D_);
    }
    std::vector<double> Wt = ComputeW_MLLR(sp, ubm);
    W = compose(W, Wt, D_);
  }
  return W;
}

void ModelAdapt::AdaptModel(const GMModel& ubm) {
  if (o_.adaptType == MAP) {
    GMModel model = ubm;
    if (o_.iterCountEM) IterEM(model, o_.iterCountEM);
    if (o_.iterCountMAP) IterMAP(model, ubm, o_.iterCountMAP);
    model_ = model;
    trained_ = true;
  } else if (o_.adaptType == MLLR) {
    W_ = IterW_MLLR(ubm);
    if (o_.applyTransforms) {
      model_ = AdaptModelMLLR(ubm, W_);
      trained_ = true;
    }
  } else if (o_.adaptType == MLLR_MAP) {
    // MLLR of the UBM, then AdaptModelMAP of the transformed model against the original UBM
    // (OL_ModelAdapt.cpp:1190-1205); without enough data for MLLR, MAP alone
    GMModel model = ubm;
    try {
      model = AdaptModelMLLR(ubm, IterW_MLLR(ubm));
    } catch (const std::runtime_error& e) {
      if (std::string(e.what()).find("CheckInvertibility") == std::string::npos) throw;
      std::fprintf(stderr, "[WARNING: not enough data to perform MLLR adaptation -> only MAP performed]\n");
      model = ubm;
    }
    if (o_.iterCountEM) IterEM(model, o_.iterCountEM);
    if (o_.iterCountMAP) IterMAP(model, ubm, o_.iterCountMAP);
    model_ = model;
    trained_ = true;
  } else if (o_.adaptType == FMLLR) {  // ComputeW_fMLLR(_UBM): the transform is the result
    GMModel u = ubm;
    u.RearrangeMixtures();
    upload_model(u);
    W_.assign((size_t)D_ * (D_ + 1), 0.0);
    check(full_ ? gmm_fmllr_estimate_full(h_, o_.iterfMLLR, W_.data())
                : gmm_fmllr_estimate(h_, o_.iterfMLLR, W_.data()));
  } else {
    fail("AdaptModel(): use TrainFromScratch for --type 0");
  }
}

namespace {
// GetGaussStats (OL_ModelAdapt.cpp:951-990)
void gauss_stats(const GMModel& m, bool get_list, int* i_max, std::vector<int>* zero, std::vector<int>* srt) {
  *i_max = 0;
  float wm = 0.0f;
  zero->clear();
  srt->clear();
  for (int k = m.GetNumberOfMixtures() - 1; k >= 0; --k) {
    const float w = m.GetMixtureWeight(k);
    if (wm < w) {
      wm = w;
      *i_max = k;
    }
    if (w == 0.0f) {
      zero->push_back(k);
      continue;
    }
    if (get_list) {
      size_t p = 0;
      while (p < srt->size() && m.GetMixtureWeight((*srt)[p]) > w) ++p;
      srt->insert(srt->begin() + (long)p, k);
    }
  }
}

// Largest eigenvalue and its unit eigenvector of a symmetric n x n matrix by cyclic Jacobi
// rotations in double (getEigValVecs, OL_ModelAdapt.cpp:73-160, asks LAPACK for this pair). The
// eigenvector's sign is not fixed by the problem: its largest-magnitude component is made positive.
void leading_eigenpair(const float* a, int n, float* lam, float* v) {
  std::vector<double> A((size_t)n * n), V((size_t)n * n, 0.0);
  for (size_t e = 0; e < A.size(); ++e) A[e] = a[e];
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[(size_t)p * n + q] * A[(size_t)p * n + q];
    if (off < 1e-30) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double theta = (A[(size_t)q * n + q] - A[(size_t)p * n + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = c * akp - sn * akq;
          A[(size_t)k * n + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = c * apk - sn * aqk;
          A[(size_t)q * n + k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vkp - sn * vkq;
          V[(size_t)k * n + q] = sn * vkp + c * vkq;
        }
      }
  }
  int best = 0;
  for (int i = 1; i < n; ++i)
    if (A[(size_t)i * n + i] > A[(size_t)best * n + best]) best = i;
  int big = 0;
  for (int i = 1; i < n; ++i)
    if (std::fabs(V[(size_t)i * n + best]) > std::fabs(V[(size_t)big * n + best])) big = i;
  const double sg = V[(size_t)big * n + best] < 0 ? -1.0 : 1.0;
  for (int i = 0; i < n; ++i) v[i] = (float)(sg * V[(size_t)i * n + best]);
  *lam = (float)A[(size_t)best * n + best];
}

// splitGaussian (OL_ModelAdapt.cpp:612-665): the new component takes the covariance, both take
// half the weight; the means move by +-sqrt(var)/2 (diagonal) or by +-sqrt(lambda) v along the
// leading eigenvector (full).
void split_gaussian(GMModel& model, int m2, int mnew) {
  const int D = model.GetDimension();
  std::memcpy(model.GetMixtureVar(mnew), model.GetMixtureVar(m2), sizeof(float) * model.DimVar());
  const float w = model.GetMixtureWeight(m2) / 2.0f;
  model.SetMixWeight(mnew, w);
  model.SetMixWeight(m2, w);
  float* m = model.GetMixtureMean(m2);
  float* mn = model.GetMixtureMean(mnew);
  std::vector<float> shift((size_t)D);
  if (model.GetFullCovStatus()) {
    float lam = 0.0f;
    std::vector<float> v((size_t)D);
    leading_eigenpair(model.GetMixtureVar(m2), D, &lam, v.data());
    if (lam < 0) fail("splitGaussian(): covariance matrix not positive definite!");
    for (int d = 0; d < D; ++d) shift[(size_t)d] = std::sqrt(lam) * v[(size_t)d];
  } else {
    for (int d = 0; d < D; ++d) shift[(size_t)d] = (float)(std::sqrt((double)model.GetMixtureVar(m2)[d]) * 0.5);
  }
  for (int d = 0; d < D; ++d) {
    mn[d] = m[d] + shift[(size_t)d];
    m[d] -= shift[(size_t)d];
  }
}
}  // namespace

void ModelAdapt::splitMultipleGaussians(GMModel& model) {
  int i_max = 0;
  std::vector<int> zero, srt;
  gauss_stats(model, o_.splitXpercAtOnce > 0.0f, &i_max, &zero, &srt);
  const unsigned n_split =
      (unsigned)std::ceil(o_.splitXpercAtOnce * (float)(model.GetNumberOfMixtures() - (int)zero.size()));
  if (n_split < 2) {
    split_gaussian(model, i_max, zero.front());
    return;
  }
  const float th = o_.splitTh * model.GetMixtureWeight(i_max);
  for (size_t n = 0; n < srt.size(); ++n) {
    if (model.GetMixtureWeight(srt[n]) < th || n >= zero.size() || n >= n_split) break;
    split_gaussian(model, srt[n], zero[n]);
  }
}

void ModelAdapt::TrainFromScratch(int nummix, const GMModel* init_model, bool fullcov) {
  if (N_ <= 3) fail("TrainFromScratch(): Not enough data to model training.");
  if (init_model) fullcov = init_model->GetFullCovStatus();  // the init model decides
  const int D = D_;
  GMModel init;
  int max_iter = nummix;
  auto em_all = [&](int* alive) {  // UpdateModelEM with every parameter updated
    check(full_ ? gmm_em_update_full(h_, 1, 1, 1, alive) : gmm_em_update(h_, 1, 1, 1, alive));
  };
  if (!init_model) {
    // global Gaussian: one component, every posterior 1 (identity covariance for a full model)
    init = GMModel(D, 1, fullcov);
    init.SetMixWeight(0, 1.0f);
    if (!fullcov)
      for (int d = 0; d < D; ++d) init.GetMixtureVar(0)[d] = 1.0f;
    upload_model(init);
    estep(GMM_ACC_MEAN | GMM_ACC_VAR);
    int alive = 0;
    em_all(&alive);
    if (alive == 0) fail("trainFromScratch(): amount of data too low to estimate a model, or data are constant!");
    read_model(init);
  } else {
    init = *init_model;
    if (init.GetDimension() != D) fail("trainFromScratch(): init model and data dimensions differ!");
    if (nummix <= init.GetNumberOfMixtures())
      fail("trainFromScratch(): init model already contains specified number of Gaussians!");
    max_iter = nummix - init.GetNumberOfMixtures();
  }
  if (nummix < 2) max_iter = 0;
  GMModel model(D, nummix, fullcov);
  for (int m = 0; m < init.GetNumberOfMixtures(); ++m) {
    model.SetMixWeight(m, init.GetMixtureWeight(m));
    std::memcpy(model.GetMixtureMean(m), init.GetMixtureMean(m), sizeof(float) * D);
    std::memcpy(model.GetMixtureVar(m), init.GetMixtureVar(m), sizeof(float) * model.DimVar());
  }
  const int iters_em = (o_.iterCountEM < 2 && o_.llTh > 0.0f) ? 2 : o_.iterCountEM;
  const float lowest = -std::numeric_limits<float>::max();
  float ll[3] = {lowest, lowest, lowest};
  GMModel m2, m3;
  int non_zero = init.GetNumberOfMixtures();
  for (int it = 0; it < max_iter; ++it) {
    for (int e = 0; e < iters_em; ++e) {
      model.RearrangeMixtures();
      upload_model(model);
      estep(GMM_ACC_MEAN | GMM_ACC_VAR);
      if (o_.verbosity)  // the reference only tracks the average LL when verbose
        ll[0] = (float)(total_ll() / (double)N_);
      if (non_zero > 1) {
        em_all(&non_zero);
        read_model(model);
      }
      if (non_zero < 2) {
        if (non_zero < 1) model = init;
        break;
      }
    }
    if (non_zero == 0 || non_zero == nummix) break;
    if (o_.llTh > 0.0f) {
      const float mx = std::max(ll[1], ll[2]);
      if (it > 2 && ll[0] - mx < o_.llTh) {
        if (mx > ll[0]) model = (mx == ll[1]) ? m2 : m3;
        break;
      }
      m3 = m2;
      m2 = model;
      ll[2] = ll[1];
      ll[1] = ll[0];
    }
    if (it < max_iter - 1) {
      splitMultipleGaussians(model);
      non_zero += 1;
    }
  }
  model.RearrangeMixtures();
  model_ = model;
  trained_ = true;
}

void ModelAdapt::SaveTRNMatrices(const std::string& FileName) const {
  std::string out = FileName;
  const size_t dot = out.rfind('.');
  if (dot != std::string::npos) out.erase(dot);
  out += o_.transformFileExt;
  FILE* f = std::fopen(out.c_str(), "w");
  if (!f) fail("Save(): Unable to open output file " + out + "!");
  const int E = D_ + 1;
  std::fprintf(f, o_.adaptType == FMLLR ? " fMLLR\n 1\t%d %d\n" : " MLLR\n 1\t%d %d\n", D_, E);
  for (int i = 0; i < D_; ++i) {  // the reference streams a float matrix with ostream defaults (%g)
    for (int j = 0; j < E; ++j) std::fprintf(f, " %g", (double)(float)W_[(size_t)i * E + j]);
    std::fprintf(f, "\n");
  }
  std::fclose(f);
}

void ModelAdapt::Save(const std::string& FileName, bool save_txt, bool save_in_stat_form) const {
  const bool trn = !W_.empty();
  if (!trained_ && !trn) fail("Save(): Missing client model or transformation matrix!");
  if (trn && (!trained_ || o_.saveTransforms || o_.adaptType == FMLLR)) {
    if (!save_in_stat_form) {
      SaveTRNMatrices(FileName);
    } else {  // D records of dimension D+1: occupancy 1, "mean" = the row of W
      std::vector<float> one((size_t)D_, 1.0f), rows(W_.size());
      for (size_t k = 0; k < W_.size(); ++k) rows[k] = (float)W_[k];
      save_stats_float(FileName, save_txt, D_ + 1, D_, one.data(), rows.data(), nullptr);
    }
  }
  if (trained_) {
    if (!save_in_stat_form)
      model_.Save(FileName, save_txt);
    else {  // every component slot, zero weights included; variances = the diagonal (GetMixtureVarDiag)
      const int D = model_.GetDimension(), M = model_.GetNumberOfMixtures();
      std::vector<float> diag((size_t)M * D);
      for (int m = 0; m < M; ++m)
        for (int d = 0; d < D; ++d)
          diag[(size_t)m * D + d] = model_.GetFullCovStatus() ? model_.GetMixtureVar(m)[(size_t)d * D + d]
                                                              : model_.GetMixtureVar(m)[d];
      save_stats_float(FileName, save_txt, D, M, model_.weights().data(), model_.means().data(), diag.data());
    }
  }
}

// ------------------------------------------------------------------ feature files

std::vector<float> read_features(const std::string& path, int prm_type, unsigned dwnsmp, long long* N, int* D) {
  if (gmm_read_param(path.c_str(), prm_type, dwnsmp, nullptr, 0, N, D))
    fail("Param::Load(): cannot read " + path);
  std::vector<float> X((size_t)(*N) * (*D));
  if (*N > 0 && gmm_read_param(path.c_str(), prm_type, dwnsmp, X.data(), *N, N, D))
    fail("Param::Load(): cannot read " + path);
  return X;
}

}  // namespace gmmgb
