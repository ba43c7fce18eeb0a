// Build-only stand-in for the ACML LAPACK routines the reference names (ACML is not vendored
// with the reference; its version is unpinned). spotrf and spotri are restated here from the
// published unblocked LAPACK algorithms (xPOTF2 for the Cholesky factor; xTRTI2 then xLAUU2 for
// the inverse from it), in single precision, column-major, lower triangle -- the reference calls
// them with uplo 'L' on its row-major symmetric matrices. A vendor library may order the float
// operations differently, so full-covariance outputs of this build pin the reference's logic,
// not the last bits of ACML's arithmetic. ssyevr (the eigenvector of the full-covariance split of
// training from scratch) is restated for the largest eigenpair only, below.
#ifndef ORACLE_SHIM_ACML_H
#define ORACLE_SHIM_ACML_H
#include <cmath>
#include <stdexcept>
#include <vector>

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

// ssyevr for the one call the reference makes (getEigValVecs: jobz 'V', range 'I', il = iu = n):
// the largest eigenvalue of the symmetric matrix and its unit eigenvector, by cyclic Jacobi
// rotations in double. The eigenvector's sign is not fixed by the problem; this stand-in makes
// its largest-magnitude component positive (the convention the GB300 drivers use for the
// full-covariance split), where ACML's choice is unknown.
inline void ssyevr(char jobz, char range, char, int n, float* a, int lda, float, float, int il, int iu, float, int* m,
                   float* w, float* z, int, int*, int* info) {
  if (jobz != 'V' || range != 'I' || il != n || iu != n)
    throw std::runtime_error("ssyevr: only the largest eigenpair is restated");
  std::vector<double> A((size_t)n * n), V((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) A[(size_t)i * n + j] = a[i + (long)j * lda];
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
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- J^T A J, V <- V J
          const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = c * akp - s * akq;
          A[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = c * apk - s * aqk;
          A[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vkp - s * vkq;
          V[(size_t)k * n + q] = s * vkp + c * vkq;
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
  for (int i = 0; i < n; ++i) z[i] = (float)(sg * V[(size_t)i * n + best]);
  w[0] = (float)A[(size_t)best * n + best];
  *m = 1;
  *info = 0;
}
#endif
