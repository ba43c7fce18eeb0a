// Build-only stand-in for the ACML LAPACK routines the reference names (ACML is not vendored
// with the reference; its version is unpinned). spotrf and spotri are restated here from the
// published unblocked LAPACK algorithms (xPOTF2 for the Cholesky factor; xTRTI2 then xLAUU2 for
// the inverse from it), in single precision, column-major, lower triangle -- the reference calls
// them with uplo 'L' on its row-major symmetric matrices. A vendor library may order the float
// operations differently, so full-covariance outputs of this build pin the reference's logic,
// not the last bits of ACML's arithmetic. ssyevr (eigenvectors for the full-covariance split of
// training from scratch) is not restated; calling it throws.
#ifndef ORACLE_SHIM_ACML_H
#define ORACLE_SHIM_ACML_H
#include <cmath>
#include <stdexcept>

namespace acml_shim {
inline float& at(float* a, int lda, int i, int j) { return a[i + (long)j * lda]; }
}  // namespace acml_shim

// Cholesky factor A = L L^T, L in the lower triangle (xPOTF2 order). info = j + 1 if the leading
// minor of order j + 1 is not positive definite.
inline void spotrf(char uplo, int n, float* a, int lda, int* info) {
  using acml_shim::at;
  if (uplo != 'L' && uplo != 'l') throw std::runtime_error("spotrf: only uplo = 'L' is restated");
  *info = 0;
  for (int j = 0; j < n; ++j) {
    float dot = 0.0f;
    for (int k = 0; k < j; ++k) dot += at(a, lda, j, k) * at(a, lda, j, k);
    float ajj = at(a, lda, j, j) - dot;
    if (ajj <= 0.0f || std::isnan(ajj)) {
      at(a, lda, j, j) = ajj;
      *info = j + 1;
      return;
    }
    ajj = std::sqrt(ajj);
    at(a, lda, j, j) = ajj;
    if (j < n - 1) {
      for (int c = 0; c < j; ++c) {  // A(j+1:n, j) -= A(j+1:n, 0:j) * A(j, 0:j)^T
        const float t = -at(a, lda, j, c);
        for (int i = j + 1; i < n; ++i) at(a, lda, i, j) += t * at(a, lda, i, c);
      }
      const float r = 1.0f / ajj;
      for (int i = j + 1; i < n; ++i) at(a, lda, i, j) *= r;
    }
  }
}

// Inverse of A from its Cholesky factor: inv(L) in place (xTRTI2, lower, non-unit), then
// inv(L)^T inv(L) into the lower triangle (xLAUU2).
inline void spotri(char uplo, int n, float* a, int lda, int* info) {
  using acml_shim::at;
  if (uplo != 'L' && uplo != 'l') throw std::runtime_error("spotri: only uplo = 'L' is restated");
  *info = 0;
  for (int j = 0; j < n; ++j)
    if (at(a, lda, j, j) == 0.0f) {
      *info = j + 1;
      return;
    }
  for (int j = n - 1; j >= 0; --j) {
    at(a, lda, j, j) = 1.0f / at(a, lda, j, j);
    const float ajj = -at(a, lda, j, j);
    if (j < n - 1) {
      const int m = n - j - 1;  // x = T x, T = A(j+1:n, j+1:n) lower, x = A(j+1:n, j)
      for (int jj = m - 1; jj >= 0; --jj) {
        const float xj = at(a, lda, j + 1 + jj, j);
        if (xj != 0.0f) {
          for (int ii = m - 1; ii > jj; --ii) at(a, lda, j + 1 + ii, j) += xj * at(a, lda, j + 1 + ii, j + 1 + jj);
          at(a, lda, j + 1 + jj, j) = xj * at(a, lda, j + 1 + jj, j + 1 + jj);
        }
      }
      for (int i = j + 1; i < n; ++i) at(a, lda, i, j) *= ajj;
    }
  }
  for (int i = 0; i < n; ++i) {
    const float aii = at(a, lda, i, i);
    if (i < n - 1) {
      float dot = 0.0f;
      for (int r = i; r < n; ++r) dot += at(a, lda, r, i) * at(a, lda, r, i);
      at(a, lda, i, i) = dot;
      for (int c = 0; c < i; ++c) at(a, lda, i, c) *= aii;  // y = aii * A(i, 0:i)
      for (int c = 0; c < i; ++c) {                          // y += A(i+1:n, 0:i)^T A(i+1:n, i)
        float t = 0.0f;
        for (int r = i + 1; r < n; ++r) t += at(a, lda, r, c) * at(a, lda, r, i);
        at(a, lda, i, c) += t;
      }
    } else {
      for (int c = 0; c <= i; ++c) at(a, lda, i, c) *= aii;
    }
  }
}

inline void ssyevr(char, char, char, int, float*, int, float, float, int, int, float, int*, float*, float*, int, int*, int*) {
  throw std::runtime_error("ssyevr: the full-covariance split of training from scratch is not restated");
}
#endif
