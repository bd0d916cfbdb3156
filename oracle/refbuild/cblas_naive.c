/* Plain-loop CBLAS routines for the reference trainer oracle build.
 *
 * Test infrastructure only (see cblas.h).  Each routine follows the textbook
 * BLAS definition; speed is irrelevant because the oracle only checks small
 * cases.  Row-major and column-major storage are both handled by indexing
 * helpers rather than by transposing data.
 */
#include "cblas.h"
#include <math.h>
#include <stdlib.h>

/* Element (i, j) of an r x c matrix stored with leading dimension ld. */
static double at(enum CBLAS_ORDER o, const double *a, int ld, int i, int j) {
  return o == CblasRowMajor ? a[(size_t)i * ld + j] : a[(size_t)j * ld + i];
}
static double *ref(enum CBLAS_ORDER o, double *a, int ld, int i, int j) {
  return o == CblasRowMajor ? &a[(size_t)i * ld + j] : &a[(size_t)j * ld + i];
}
/* op(A)(i, j) for op = identity or transpose. */
static double op(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE t, const double *a, int ld, int i, int j) {
  return t == CblasNoTrans ? at(o, a, ld, i, j) : at(o, a, ld, j, i);
}

void cblas_dgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb,
                 int m, int n, int k, double alpha, const double *a, int lda,
                 const double *b, int ldb, double beta, double *c, int ldc) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0;
      for (int q = 0; q < k; ++q) s += op(o, ta, a, lda, i, q) * op(o, tb, b, ldb, q, j);
      double *cij = ref(o, c, ldc, i, j);
      *cij = (beta == 0 ? 0 : beta * *cij) + alpha * s;
    }
}

void cblas_dgemv(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, int m, int n,
                 double alpha, const double *a, int lda, const double *x, int incx,
                 double beta, double *y, int incy) {
  const int rows = ta == CblasNoTrans ? m : n, cols = ta == CblasNoTrans ? n : m;
  for (int i = 0; i < rows; ++i) {
    double s = 0;
    for (int j = 0; j < cols; ++j)
      s += (ta == CblasNoTrans ? at(o, a, lda, i, j) : at(o, a, lda, j, i)) * x[(size_t)j * incx];
    double *yi = &y[(size_t)i * incy];
    *yi = (beta == 0 ? 0 : beta * *yi) + alpha * s;
  }
}

void cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy) {
  for (int i = 0; i < n; ++i) y[(size_t)i * incy] += alpha * x[(size_t)i * incx];
}

void cblas_dger(enum CBLAS_ORDER o, int m, int n, double alpha, const double *x, int incx,
                const double *y, int incy, double *a, int lda) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) *ref(o, a, lda, i, j) += alpha * x[(size_t)i * incx] * y[(size_t)j * incy];
}

/* Upper triangle in row-major order is the lower triangle in column-major. */
static int in_triangle(enum CBLAS_ORDER o, enum CBLAS_UPLO u, int i, int j) {
  (void)o;
  return u == CblasUpper ? j >= i : j <= i;
}

void cblas_dsyr(enum CBLAS_ORDER o, enum CBLAS_UPLO u, int n, double alpha,
                const double *x, int incx, double *a, int lda) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      if (in_triangle(o, u, i, j)) *ref(o, a, lda, i, j) += alpha * x[(size_t)i * incx] * x[(size_t)j * incx];
}

void cblas_dsyrk(enum CBLAS_ORDER o, enum CBLAS_UPLO u, enum CBLAS_TRANSPOSE t,
                 int n, int k, double alpha, const double *a, int lda, double beta,
                 double *c, int ldc) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (!in_triangle(o, u, i, j)) continue;
      double s = 0;
      for (int q = 0; q < k; ++q)
        s += (t == CblasNoTrans ? at(o, a, lda, i, q) * at(o, a, lda, j, q)
                                : at(o, a, lda, q, i) * at(o, a, lda, q, j));
      double *cij = ref(o, c, ldc, i, j);
      *cij = (beta == 0 ? 0 : beta * *cij) + alpha * s;
    }
}

void cblas_dsymv(enum CBLAS_ORDER o, enum CBLAS_UPLO u, int n, double alpha,
                 const double *a, int lda, const double *x, int incx, double beta,
                 double *y, int incy) {
  for (int i = 0; i < n; ++i) {
    double s = 0;
    for (int j = 0; j < n; ++j) {
      const double aij = in_triangle(o, u, i, j) ? at(o, a, lda, i, j) : at(o, a, lda, j, i);
      s += aij * x[(size_t)j * incx];
    }
    double *yi = &y[(size_t)i * incy];
    *yi = (beta == 0 ? 0 : beta * *yi) + alpha * s;
  }
}

void cblas_dswap(int n, double *x, int incx, double *y, int incy) {
  for (int i = 0; i < n; ++i) {
    const double t = x[(size_t)i * incx];
    x[(size_t)i * incx] = y[(size_t)i * incy];
    y[(size_t)i * incy] = t;
  }
}

CBLAS_INDEX cblas_idamax(int n, const double *x, int incx) {
  CBLAS_INDEX best = 0;
  double v = -1;
  for (int i = 0; i < n; ++i)
    if (fabs(x[(size_t)i * incx]) > v) { v = fabs(x[(size_t)i * incx]); best = (CBLAS_INDEX)i; }
  return best;
}

void cblas_domatcopy(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE t, int rows, int cols,
                     double alpha, const double *a, int lda, double *b, int ldb) {
  for (int i = 0; i < rows; ++i)
    for (int j = 0; j < cols; ++j) {
      if (t == CblasNoTrans) *ref(o, b, ldb, i, j) = alpha * at(o, a, lda, i, j);
      else *ref(o, b, ldb, j, i) = alpha * at(o, a, lda, i, j);
    }
}
