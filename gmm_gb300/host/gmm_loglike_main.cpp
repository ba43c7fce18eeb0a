// gmm_loglike: the scoring command line of projects/GetLogLikeGMM (main.cpp:100-200) on one
// GB300, with the reference's option names (LoadConfiguration, main.cpp:262-390). Per input
// file: with --for-each the per-frame log-likelihoods are written to --outDir (saveMat layout,
// text with --save-txt); otherwise the file's mean log-likelihood goes to standard output as
// "<file>\t<mean>".
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "gmm_cli.hpp"
#include "gmm_host.hpp"

using gmmgb::cli::FLAG;
using gmmgb::cli::MULTI;
using gmmgb::cli::STR;

int main(int argc, char** argv) {
  try {
    gmmgb::cli::Parser P({
        {"help", 'h', FLAG, "", "display this help"},
        {"config", 'c', STR, "", "configuration file (name = value lines; the command line wins)"},
        {"in-file", 'i', MULTI, "", "feature file(s); repeatable"},
        {"in-list", 'I', MULTI, "", "directory or list file with feature files; repeatable"},
        {"in-GMM", 'g', STR, "", "the GMM"},
        {"for-each", 'f', FLAG, "0", "write the log-likelihood of every frame to --outDir"},
        {"outDir", 'o', STR, "", "output directory (--for-each)"},
        {"inExt", 'e', STR, ".*", "extension of input files when a list is a directory"},
        {"outExt", 'x', STR, ".logL", "extension of output files (--for-each)"},
        {"load-txt", 'L', FLAG, "0", "load the GMM from a text file"},
        {"save-txt", 'T', FLAG, "0", "save log-likelihoods as text (--for-each)"},
        {"data-T", 0, STR, "0", "feature files in sves(0) / htk(1) / raw(2) format"},
        {"SSE", 0, FLAG, "0", "accepted for compatibility; ignored"},
        {"CUDA", 0, FLAG, "0", "accepted for compatibility; ignored"},
        {"GPU-id", 'G', STR, "0", "GPU to use"},
        {"numThrd", 0, STR, "1", "accepted for compatibility; the GPU estimator ignores it"},
        {"dwnsmp", 0, STR, "1", "down-sample factor of the feature vectors"},
        {"verbosity", 'v', STR, "0", "verbose mode"},
        {"precision", 0, STR, "tc", "E-step arithmetic: tc (split-bf16 tensor cores) | fp32 (plain FP32)"},
    });
    P.parse(argc, argv);
    if (P.get_bool("help")) {
      P.help("gmm_loglike: per-frame GMM log-likelihoods on one GB300\nOptions:");
      return 0;
    }
    if (!P.count("in-file") && !P.count("in-list"))
      throw std::runtime_error("LoadConfiguration(): input not specified (options -i | -I)!");
    if (!P.count("in-GMM")) throw std::runtime_error("LoadConfiguration(): \"in-GMM\" not specified!");
    const bool each = P.get_bool("for-each");
    if (each && !P.count("outDir")) throw std::runtime_error("LoadConfiguration(): \"outDir\" has to be specified!");
    const int dt = P.get_int("data-T");
    const int type = dt == 1 ? GMM_PRM_HTK : dt == 2 ? GMM_PRM_RAW : GMM_PRM_SVES;
    const unsigned dwnsmp = P.get_uint("dwnsmp");
    const int verbosity = P.get_int("verbosity");
    const bool save_txt = P.get_bool("save-txt");

    // loadFileLists (main.cpp:228-255)
    std::vector<std::string> files;
    for (const auto& f : P.all("in-file")) {
      if (gmmgb::cli::is_file(f)) files.push_back(f);
      else std::cout << "WARNING: input file " << f << " not found" << std::endl;
    }
    for (const auto& l : P.all("in-list"))
      if (!l.empty()) gmmgb::cli::read_list(l, P.get("inExt"), &files);
    if (files.empty()) throw std::runtime_error("None suitable input files found");

    gmmgb::GMModel g;
    try {
      g.Load(P.get("in-GMM"), P.get_bool("load-txt"));
    } catch (const std::exception&) {
      throw std::runtime_error("GMM model [" + P.get("in-GMM") + "] not found");
    }
    const int gpu = P.get_int("GPU-id");
    gmmgb::GMMStatsEstimatorGB300 est(gpu < 0 ? 0 : gpu, P.get("precision") == "fp32" ? GMM_PREC_FP32 : GMM_PREC_TC);
    est.insertModel(g);
    std::vector<float> ll;
    for (const auto& path : files) {
      long long N = 0;
      int D = 0;
      std::vector<float> X;
      try {
        X = gmmgb::read_features(path, type, dwnsmp, &N, &D);
      } catch (const std::exception&) {
        std::cerr << "WARNING: Param file [" << path << "] not found -> skipped!" << std::endl;
        continue;
      }
      if (N < 1) {
        if (verbosity > 1) std::cerr << "WARNING: Param file [" << path << "] empty" << std::endl;
        continue;
      }
      ll.resize((size_t)N);
      est.compVecsLogLikeMT(X.data(), (unsigned)N, (unsigned)D, ll.data());
      if (each) {
        gmmgb::cli::save_mat(gmmgb::cli::new_path(path, P.get("outDir"), P.get("outExt")), save_txt, ll.data(), 1,
                             (unsigned)N);
      } else {
        float mean = 0.0f;  // the reference sums in float, in frame order
        for (long long n = 0; n < N; ++n) mean += ll[(size_t)n];
        mean /= (float)N;
        std::printf("\r%s\t%g\n", path.c_str(), (double)mean);
      }
    }
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
}
