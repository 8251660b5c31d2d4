/* Column-major reference BLAS routines (dgemm_, zgemm_, dcopy_, zcopy_) with
 * the Fortran interface declared in src/atrip/Blas.hpp:24-57, for linking the
 * reference sources as a CPU oracle.  Straight triple loops: test
 * infrastructure, correctness over speed. */
#include <complex>
#include <cstring>

namespace {
template <typename F>
F op(char t, const F *a, int lda, int r, int c) {
  if (t == 'N' || t == 'n') return a[r + (long)c * lda];
  F v = a[c + (long)r * lda];
  if (t == 'C' || t == 'c') return std::conj(v);
  return v;
}
template <>
double op<double>(char t, const double *a, int lda, int r, int c) {
  return (t == 'N' || t == 'n') ? a[r + (long)c * lda] : a[c + (long)r * lda];
}
template <typename F>
void gemm(const char *ta, const char *tb, int m, int n, int k, F alpha,
          const F *A, int lda, const F *B, int ldb, F beta, F *C, int ldc) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      F s = F(0);
      for (int l = 0; l < k; ++l) s += op(*ta, A, lda, i, l) * op(*tb, B, ldb, l, j);
      F &c = C[i + (long)j * ldc];
      c = (beta == F(0) ? F(0) : beta * c) + alpha * s;
    }
}
} // namespace

extern "C" {
void dgemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k,
            double *alpha, const double *A, const int *lda, const double *B,
            const int *ldb, double *beta, double *C, const int *ldc) {
  gemm<double>(ta, tb, *m, *n, *k, *alpha, A, *lda, B, *ldb, *beta, C, *ldc);
}
void zgemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k,
            std::complex<double> *alpha, const std::complex<double> *A, const int *lda,
            const std::complex<double> *B, const int *ldb, std::complex<double> *beta,
            std::complex<double> *C, const int *ldc) {
  gemm<std::complex<double>>(ta, tb, *m, *n, *k, *alpha, A, *lda, B, *ldb, *beta, C, *ldc);
}
void dcopy_(int *n, const double *x, int *incx, double *y, int *incy) {
  for (int i = 0; i < *n; ++i) y[(long)i * *incy] = x[(long)i * *incx];
}
void zcopy_(int *n, const void *x, int *incx, void *y, int *incy) {
  const std::complex<double> *xs = (const std::complex<double> *)x;
  std::complex<double> *ys = (std::complex<double> *)y;
  for (int i = 0; i < *n; ++i) ys[(long)i * *incy] = xs[(long)i * *incx];
}
}
