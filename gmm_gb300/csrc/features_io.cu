// Feature files: the three formats of the reference's Param loaders (param/OL_Param.cpp:224-580),
// read straight into a caller-provided (page-locked, when it is a staging buffer) float block.
//
//   SVES  "SV-ES-PARAM" (11 bytes), int32 dim, int32 nsamples, float CF[nsamples],
//         float vectors[nsamples][dim]; host byte order            (Param::Load, :245-340)
//   HTK   big-endian int32 nSamples, int32 sampPeriod, int16 sampSize (bytes per frame),
//         int16 parmKind, then big-endian float frames; dim = sampSize / 4   (Param::LoadHTK, :474-560)
//   RAW   int32 nsamples, int32 dim, then float frames; nsamples < 1 means "the rest of the
//         file"                                                      (Param::LoadRaw, :345-450)
//
// Down-sampling keeps frames 0, d, 2d, ...: nsamples / d + (nsamples % d > 0) frames.
#include <cstdio>
#include <cstring>
#include <string>

#include "gmm_internal.cuh"

namespace gmm {
namespace {

struct File {
  FILE* f = nullptr;
  explicit File(const char* p) : f(std::fopen(p, "rb")) {}
  ~File() {
    if (f) std::fclose(f);
  }
  bool read(void* dst, size_t n) { return std::fread(dst, 1, n, f) == n; }
  bool skip(long long n) { return n == 0 || std::fseek(f, (long)n, SEEK_CUR) == 0; }
};

uint32_t be32(const unsigned char* b) { return (uint32_t)b[0] << 24 | (uint32_t)b[1] << 16 | (uint32_t)b[2] << 8 | b[3]; }
uint16_t be16(const unsigned char* b) { return (uint16_t)(b[0] << 8 | b[1]); }

long long kept(long long nsamples, unsigned d) { return d > 1 ? nsamples / d + (nsamples % d > 0) : nsamples; }

}  // namespace

int param_header(const char* path, int type, unsigned dwnsmp, long long* N, int* D, std::string* err) {
  File file(path);
  if (!file.f) return -1;  // the reference skips a missing file with a warning
  if (type == GMM_PRM_SVES) {
    char h[11];
    int32_t dim, ns;
    if (!file.read(h, 11) || std::memcmp(h, "SV-ES-PARAM", 11) != 0) {
      *err = std::string("Param::Load(): file's ") + path + " format different from SV-ES-PARAM";
      return GMM_ERR_ARG;
    }
    if (!file.read(&dim, 4) || !file.read(&ns, 4)) {
      *err = std::string("Param::Load(): Error occured when reading file ") + path;
      return GMM_ERR_ARG;
    }
    *D = dim;
    *N = (ns > 0 && dim > 0) ? kept(ns, dwnsmp) : 0;
    if (*N == 0) *D = 0;
  } else if (type == GMM_PRM_HTK) {
    unsigned char h[12];
    if (!file.read(h, 12)) {
      *err = std::string("Param::LoadHTK(): Error occured when reading file ") + path;
      return GMM_ERR_ARG;
    }
    const long long ns = (long long)be32(h);
    const int dim = (int)(int16_t)be16(h + 8) / 4;
    *D = dim;
    *N = (ns > 0 && dim > 0) ? kept(ns, dwnsmp ? dwnsmp : 1) : 0;
    if (*N == 0) *D = 0;
  } else if (type == GMM_PRM_RAW) {
    int32_t ns, dim;
    if (!file.read(&ns, 4) || !file.read(&dim, 4)) {
      *err = std::string("Param::LoadRaw(): Error occured when reading file ") + path;
      return GMM_ERR_ARG;
    }
    long long n = ns;
    if (n < 1 && dim > 0) {
      std::fseek(file.f, 0, SEEK_END);
      const long long size = std::ftell(file.f) - 8;
      n = size / dim / (long long)sizeof(float);
    }
    *D = dim;
    *N = (n > 0 && dim > 0) ? kept(n, dwnsmp) : 0;
    if (*N == 0) *D = 0;
  } else {
    *err = "Param::Load(): Unknown input data type specified";
    return GMM_ERR_ARG;
  }
  return GMM_OK;
}

int param_read(const char* path, int type, unsigned dwnsmp, float* out, std::string* err) {
  long long N = 0;
  int D = 0;
  int rc = param_header(path, type, dwnsmp, &N, &D, err);
  if (rc) return rc;
  if (N == 0) return GMM_OK;
  File file(path);
  if (!file.f) return -1;
  const unsigned d = dwnsmp > 1 ? dwnsmp : 1;
  const size_t fb = (size_t)D * sizeof(float);
  bool ok = true;
  if (type == GMM_PRM_SVES) {
    int32_t ns;
    ok = file.skip(11 + 4) && file.read(&ns, 4) && file.skip((long long)ns * 4);  // header, CFs
    for (long long i = 0; ok && i < N; ++i) {
      ok = file.read(out + (size_t)i * D, fb);
      if (ok && i + 1 < N) ok = file.skip((long long)(d - 1) * (long long)fb);
    }
  } else if (type == GMM_PRM_HTK) {
    ok = file.skip(12);
    for (long long i = 0; ok && i < N; ++i) {
      unsigned char* b = reinterpret_cast<unsigned char*>(out + (size_t)i * D);
      ok = file.read(b, fb);
      for (int k = 0; ok && k < D; ++k) {  // big-endian floats to host order
        const uint32_t v = be32(b + 4 * k);
        std::memcpy(b + 4 * k, &v, 4);
      }
      if (ok && i + 1 < N) ok = file.skip((long long)(d - 1) * (long long)fb);
    }
  } else {
    ok = file.skip(8);
    for (long long i = 0; ok && i < N; ++i) {
      ok = file.read(out + (size_t)i * D, fb);
      if (ok && i + 1 < N) ok = file.skip((long long)(d - 1) * (long long)fb);
    }
  }
  if (!ok) {
    *err = std::string("Param::Load(): Error occured when reading file ") + path;
    return GMM_ERR_ARG;
  }
  return GMM_OK;
}

}  // namespace gmm

extern "C" int gmm_read_param(const char* path, int prm_type, unsigned int dwnsmp, float* out,
                              long long cap_frames, long long* N, int* D) {
  if (!path || !N || !D) return GMM_ERR_ARG;
  std::string err;
  int rc = gmm::param_header(path, prm_type, dwnsmp, N, D, &err);
  if (rc < 0) return GMM_ERR_ARG;  // missing file
  if (rc || !out) return rc;
  if (*N > cap_frames) return GMM_ERR_ARG;
  rc = gmm::param_read(path, prm_type, dwnsmp, out, &err);
  return rc < 0 ? GMM_ERR_ARG : rc;
}
