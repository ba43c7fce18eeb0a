// Build-only stand-in for the three ACML LAPACK routines the reference names. They are used
// only by the full-covariance path, which the oracle never exercises; calling one throws.
#ifndef ORACLE_SHIM_ACML_H
#define ORACLE_SHIM_ACML_H
#include <stdexcept>
inline void spotrf(char, int, float*, int, int*) { throw std::runtime_error("spotrf: full covariance is not part of the oracle"); }
inline void spotri(char, int, float*, int, int*) { throw std::runtime_error("spotri: full covariance is not part of the oracle"); }
inline void ssyevr(char, char, char, int, float*, int, float, float, int, int, float, int*, float*, float*, int, int*, int*) {
  throw std::runtime_error("ssyevr: full covariance is not part of the oracle");
}
#endif
