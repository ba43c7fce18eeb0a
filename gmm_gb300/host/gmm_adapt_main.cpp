// gmm_adapt: the model-training / adaptation command line of projects/Model_ADAPT
// (Model_ADAPT.cpp:106-263) on one GB300, with the reference's option names
// (loadConfiguration / checkOptions, Model_ADAPT.cpp:276-475, and CModelAdapt::GetOptions,
// OL_ModelAdapt.cpp:2032-2132): train from scratch (no input model, --nummix), MAP / EM
// (--type 2), MLLR (--type 1), fMLLR (--type 3) or MLLR+MAP (--type 4) from SVES / HTK / RAW
// feature files; one model for all inputs
// (-o), one per input file (--model-file-mode) or one per class (-S, CLASS mode).
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "gmm_cli.hpp"
#include "gmm_host.hpp"

using gmmgb::cli::FLAG;
using gmmgb::cli::MULTI;
using gmmgb::cli::STR;

namespace {

std::vector<gmmgb::cli::Opt> options() {
  return {
      {"help", 'h', FLAG, "", "display this help"},
      {"config", 'c', STR, "", "configuration file (name = value lines; the command line wins)"},
      {"in-file", 'i', MULTI, "", "feature file(s) to adapt / train on; repeatable"},
      {"in-list", 'I', MULTI, "", "directory or list file with paths of feature files; repeatable"},
      {"model-file-mode", 0, FLAG, "0", "one model per input file, stored in --outDir with --outExt"},
      {"in-classes", 'S', MULTI, "", "CLASS mode: lines 'class_ID file_1 ... file_N'; one model per class"},
      {"outExt", 'x', STR, ".gmm", "extension of output models (model-file / CLASS mode)"},
      {"outDir", 'D', STR, "./", "directory of output models (model-file / CLASS mode)"},
      {"in-UBM", 'u', STR, "", "UBM / initial model (none: train from scratch)"},
      {"in-dir-UBM", 'U', STR, "", "directory with one initial model per output model"},
      {"nummix", 'g', STR, "0", "number of Gaussians when training from scratch"},
      {"full-cov", 0, FLAG, "0", "(FROM_SCRATCH) train full covariance matrices"},
      {"inExt-gmm", 'E', STR, ".gmm", "extension of models in --in-dir-UBM"},
      {"outFile", 'o', STR, "", "output model"},
      {"file-by-file", 'f', FLAG, "0", "stream the feature files each iteration instead of keeping them resident"},
      {"inExt", 'e', STR, "", "extension of input files when a list is a directory (default '.*')"},
      {"data-T", 0, STR, "0", "feature files in sves(0) / htk(1) / raw(2) format"},
      {"load-txt", 'L', FLAG, "0", "load models from text files"},
      {"save-txt", 'T', FLAG, "0", "save the model as a text file"},
      {"save-in-stat-form", 0, FLAG, "0", "save the model (or MLLR transform) in the GMMStats file layout"},
      {"dwnsmp", 0, STR, "1", "down-sample factor of the feature vectors"},
      {"verbosity", 'v', STR, "0", "verbose mode"},
      {"type", 't', STR, "2", "FROM_SCRATCH=0, MLLR=1, MAP=2, fMLLR=3, MLLR+MAP=4"},
      {"split-X", 0, STR, "0", "(FROM_SCRATCH) fraction of Gaussians split at once per round"},
      {"split-th", 0, STR, "0", "(FROM_SCRATCH) split only weights above split-th * max weight"},
      {"ll-Th", 0, STR, "0", "(FROM_SCRATCH) stop when the log-likelihood gain is below this"},
      {"robust", 'R', FLAG, "0", "(FROM_SCRATCH|MAP) robust statistics (independent-frame counts)"},
      {"it-EM", 0, STR, "0", "(MAP|FROM_SCRATCH) EM iterations"},
      {"it-MAP", 0, STR, "0", "(MAP) MAP iterations against the UBM"},
      {"mean", 'M', FLAG, "0", "(MAP) adapt means"},
      {"var", 'V', FLAG, "0", "(MAP) adapt variances"},
      {"weight", 'W', FLAG, "0", "(MAP) adapt weights"},
      {"tau", 'r', STR, "0", "(MAP) relevance factor"},
      {"min-var", 0, STR, "1e-06", "minimal variance of the model"},
      {"numThrd", 0, STR, "1", "accepted for compatibility; the GPU estimator ignores it"},
      {"prm-buffer", 0, STR, "0.05", "feature batch size in GB with --file-by-file"},
      {"GPU-id", 'G', STR, "0", "GPU to use"},
      {"SSE", 0, FLAG, "0", "accepted for compatibility; ignored"},
      {"CUDA", 0, FLAG, "0", "accepted for compatibility; ignored"},
      {"mat-ext", 'X', STR, ".mat", "(MLLR) extension of the transform file"},
      {"apply-trn", 'a', FLAG, "0", "(MLLR) transform the model with the estimated matrix and save it"},
      {"save-trn", 's', FLAG, "0", "(MLLR) save the transform matrix"},
      {"mllr-init", 0, FLAG, "0", "(MLLR) add UBM statistics to the MLLR accumulators"},
      {"it-mllr", 0, STR, "1", "(MLLR) MLLR iterations"},
      {"precision", 0, STR, "tc", "E-step arithmetic: tc (split-bf16 tensor cores) | fp32 (plain FP32)"},
  };
}

int prm_type(int t) {
  if (t == 0) return GMM_PRM_SVES;
  if (t == 1) return GMM_PRM_HTK;
  if (t == 2) return GMM_PRM_RAW;
  throw std::runtime_error("--data-T must be 0 (sves), 1 (htk) or 2 (raw)");
}

struct Job {
  std::string name, out;  // model name (for --in-dir-UBM) and output path
  std::vector<std::string> files;
};

}  // namespace

int main(int argc, char** argv) {
  try {
    gmmgb::cli::Parser P(options());
    P.parse(argc, argv);
    if (P.get_bool("help")) {
      P.help("gmm_adapt: GMM training / MAP / MLLR adaptation on one GB300\nOptions:");
      return 0;
    }
    const bool class_mode = P.count("in-classes");
    if (class_mode && P.count("in-file"))
      throw std::runtime_error("MLF mode (-S with -i) is not supported; use CLASS mode (-S with -I)");
    if (!class_mode && !P.count("in-file") && !P.count("in-list"))
      throw std::runtime_error("LoadConfiguration(): input not specified (options -i | -I)!");
    const bool each = P.get_bool("model-file-mode");
    if (!class_mode && !each && !P.count("outFile"))
      throw std::runtime_error("LoadConfiguration(): \"outFile\" not specified!");
    if (P.count("in-UBM") && P.count("in-dir-UBM"))
      throw std::runtime_error("LoadConfiguration(): Both options \"in-UBM\" and \"in-dir-UBM\" specified!");
    const bool no_model = !P.count("in-UBM") && !P.count("in-dir-UBM");
    const int nummix = P.get_int("nummix");
    const bool from_scratch = nummix > 0;  // Model_ADAPT.cpp:392: --nummix selects training
    if (no_model && !from_scratch)
      throw std::runtime_error("LoadConfiguration(): None input model specified (\"in-UBM\" or \"in-dir-UBM\") and \"nummix\" < 1!");
    std::string in_ext = P.get("inExt");
    if (in_ext.empty() && !class_mode) in_ext = ".*";

    gmmgb::AdaptOptions o;
    o.adaptType = from_scratch ? gmmgb::FROM_SCRATCH : P.get_int("type");
    if (o.adaptType < gmmgb::FROM_SCRATCH || o.adaptType > gmmgb::MLLR_MAP)
      throw std::runtime_error("--type must be 0 (from scratch), 1 (MLLR), 2 (MAP), 3 (fMLLR) or 4 (MLLR+MAP)");
    o.tau = P.get_int("tau");
    o.iterCountEM = P.get_int("it-EM");
    o.iterCountMAP = P.get_int("it-MAP");
    o.AdaptMeanBool = P.get_bool("mean");
    o.AdaptVarBool = P.get_bool("var");
    o.AdaptWeightBool = P.get_bool("weight");
    o.iterMLLR = P.get_int("it-mllr");
    o.mllrUBMInit = P.get_bool("mllr-init");
    o.applyTransforms = P.get_bool("apply-trn");
    o.saveTransforms = P.get_bool("save-trn");
    o.transformFileExt = P.get("mat-ext");
    o.min_var = P.get_float("min-var");
    o.splitXpercAtOnce = P.get_float("split-X");
    o.splitTh = P.get_float("split-th");
    o.llTh = P.get_float("ll-Th");
    o.robustCov = P.get_bool("robust");
    o.verbosity = P.get_int("verbosity");
    o.precision = P.get("precision") == "fp32" ? GMM_PREC_FP32 : GMM_PREC_TC;
    o.gpu = P.get_int("GPU-id") < 0 ? 0 : P.get_int("GPU-id");
    const int type = prm_type(P.get_int("data-T"));
    const unsigned dwnsmp = P.get_uint("dwnsmp");
    const bool load_txt = P.get_bool("load-txt"), save_txt = P.get_bool("save-txt");
    const bool file_by_file = P.get_bool("file-by-file");
    const std::string out_dir = P.get("outDir"), out_ext = P.get("outExt");

    // the jobs: (model name, output path, feature files)  (Model_ADAPT.cpp:125-177)
    std::vector<Job> jobs;
    if (class_mode) {
      const std::vector<std::string> lists = P.all("in-list");
      const std::string prefix = lists.empty() || lists[0].empty() ? std::string() : lists[0] + "/";
      for (const auto& cf : P.all("in-classes")) {
        std::ifstream f(cf);
        if (!f) throw std::runtime_error("loadFileLists(): file " + cf + " could not be opened for reading");
        std::string ln;
        while (std::getline(f, ln)) {
          for (char& ch : ln)
            if (std::string(", ;:*!\r\t").find(ch) != std::string::npos) ch = ' ';
          std::istringstream is(ln);
          std::string id, e;
          if (!(is >> id)) continue;
          Job j;
          j.name = gmmgb::cli::basename_noext(id);
          while (is >> e) {
            if (!in_ext.empty()) {  // boost::filesystem::change_extension
              const size_t sl = e.rfind('/'), dot = e.rfind('.');
              if (dot != std::string::npos && (sl == std::string::npos || dot > sl)) e.erase(dot);
              e += in_ext;
            }
            j.files.push_back(prefix + e);
          }
          if (j.files.empty()) continue;
          j.out = out_dir + "/" + j.name + out_ext;
          jobs.push_back(j);
        }
      }
    } else {
      std::vector<std::string> files;
      for (const auto& f : P.all("in-file")) {
        if (gmmgb::cli::is_file(f)) files.push_back(f);
        else std::cerr << "WARNING: input file " << f << " not found" << std::endl;
      }
      for (const auto& l : P.all("in-list"))
        if (!l.empty()) gmmgb::cli::read_list(l, in_ext, &files);
      if (each) {
        for (const auto& f : files) jobs.push_back({gmmgb::cli::basename_noext(f), "", {f}});
        for (auto& j : jobs) j.out = out_dir + "/" + j.name + out_ext;
      } else if (!files.empty()) {
        jobs.push_back({gmmgb::cli::basename_noext(P.get("outFile")), P.get("outFile"), files});
      }
    }
    if (jobs.empty()) {
      std::printf("Non input files found!\n");
      return 1;
    }

    for (const auto& j : jobs) {
      gmmgb::GMModel ubm;
      if (!no_model) {  // loadUBM (Model_ADAPT.cpp:598-623)
        bool ok = false;
        if (P.count("in-dir-UBM")) {
          try {
            ubm.Load(P.get("in-dir-UBM") + "/" + j.name + P.get("inExt-gmm"), load_txt);
            ok = true;
          } catch (const std::exception&) {
          }
        }
        if (!ok && P.count("in-UBM")) ubm.Load(P.get("in-UBM"), load_txt);
        else if (!ok) throw std::runtime_error("UBM failed to load: [" + P.get("in-UBM") + "] | [" + j.name + "]");
      }
      gmmgb::ModelAdapt ma(o);
      if (file_by_file) {
        ma.InsertFiles(j.files, type, dwnsmp, P.get_float("prm-buffer"));
        if (ma.NumFrames() == 0) {
          std::cerr << " WARNING: none data, adaptation skipped!" << std::endl;
          continue;
        }
      } else {  // fillAdaptationWithData (Model_ADAPT.cpp:566-593): all frames, file after file
        std::vector<float> X;
        long long N = 0;
        int D = 0;
        for (const auto& f : j.files) {
          long long n = 0;
          int d = 0;
          std::vector<float> x;
          try {
            x = gmmgb::read_features(f, type, dwnsmp, &n, &d);
          } catch (const std::exception&) {
            if (o.verbosity > 1) std::cout << "File " << f << " could not be opened -> skipped" << std::endl;
            continue;
          }
          if (n == 0) continue;
          if (D && d != D) throw std::runtime_error("feature files of different dimensions");
          D = d;
          X.insert(X.end(), x.begin(), x.end());
          N += n;
        }
        if (N == 0) {
          std::cerr << " WARNING: none data, adaptation skipped!" << std::endl;
          continue;
        }
        ma.InsertData(X.data(), N, D);
      }
      if (from_scratch) ma.TrainFromScratch(nummix, no_model ? nullptr : &ubm, P.get_bool("full-cov"));
      else ma.AdaptModel(ubm);
      ma.Save(j.out, save_txt, P.get_bool("save-in-stat-form"));
      if (o.verbosity)
        for (size_t i = 0; i < ma.ll_history.size(); ++i)
          std::printf(" [%s] E-step %zu: total log-likelihood %.17g\n", j.name.c_str(), i, ma.ll_history[i]);
    }
    return 0;
  } catch (const std::exception& e) {
    std::cout << "ERROR: " << e.what() << std::endl;
    return 1;
  }
}
