/*
 * lapacke.h -- a stand-in for the LAPACKE C interface, for compiling the
 * reference's USE_PRECONDITIONER code (lapack_wrapper.cpp) on a machine
 * without LAPACK.  TEST INFRASTRUCTURE ONLY (oracle/build_ref.py).
 *
 * dgetrf: LU factorisation with partial pivoting, row-major, unit lower
 * triangle, ipiv 1-based (the LAPACK convention); dgetri: the inverse from
 * those factors, column by column through forward and back substitution.
 * The reference uses only these two (lapack_wrapper.cpp:29-42); the gesv
 * wrappers it also defines are never called on this path and report failure.
 * dgetrf keeps a copy of the matrix it was given, so the emulation can return
 * the reference's preconditioner block before its inversion.
 */
#ifndef SIPG_LAPACKE_EMUL_H
#define SIPG_LAPACKE_EMUL_H

#include <cmath>
#include <vector>

typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

namespace lapacke_emul {
inline std::vector<double>& last_factored() {
  static std::vector<double> v;
  return v;
}
}  // namespace lapacke_emul

inline lapack_int LAPACKE_sgesv(int, lapack_int, lapack_int, float*, lapack_int, lapack_int*, float*, lapack_int) {
  return -1;
}
inline lapack_int LAPACKE_dgesv(int, lapack_int, lapack_int, double*, lapack_int, lapack_int*, double*, lapack_int) {
  return -1;
}

inline lapack_int LAPACKE_dgetrf(int order, lapack_int m, lapack_int n, double* a, lapack_int lda, lapack_int* ipiv) {
  if (order != LAPACK_ROW_MAJOR || m != n) return -1;
  lapacke_emul::last_factored().assign(a, a + (size_t)n * lda);
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r * lda + c]) > std::fabs(a[piv * lda + c])) piv = r;
    ipiv[c] = piv + 1;
    if (a[piv * lda + c] == 0) return c + 1;
    if (piv != c)
      for (int k = 0; k < n; ++k) std::swap(a[c * lda + k], a[piv * lda + k]);
    for (int r = c + 1; r < n; ++r) {
      const double l = a[r * lda + c] / a[c * lda + c];
      a[r * lda + c] = l;
      for (int k = c + 1; k < n; ++k) a[r * lda + k] -= l * a[c * lda + k];
    }
  }
  return 0;
}

inline lapack_int LAPACKE_dgetri(int order, lapack_int n, double* a, lapack_int lda, const lapack_int* ipiv) {
  if (order != LAPACK_ROW_MAJOR) return -1;
  std::vector<double> inv((size_t)n * n), col(n);
  for (int j = 0; j < n; ++j) {
    // column j of P A^-1 = U^-1 L^-1 (P e_j): apply the row swaps to e_j
    for (int i = 0; i < n; ++i) col[i] = (i == j) ? 1.0 : 0.0;
    for (int i = 0; i < n; ++i) std::swap(col[i], col[ipiv[i] - 1]);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < i; ++k) col[i] -= a[i * lda + k] * col[k];
    for (int i = n - 1; i >= 0; --i) {
      for (int k = i + 1; k < n; ++k) col[i] -= a[i * lda + k] * col[k];
      col[i] /= a[i * lda + i];
    }
    for (int i = 0; i < n; ++i) inv[(size_t)i * n + j] = col[i];
  }
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) a[i * lda + k] = inv[(size_t)i * n + k];
  return 0;
}

#endif
