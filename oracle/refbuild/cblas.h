/* Minimal CBLAS interface for building the reference trainer as an oracle.
 *
 * Test infrastructure only: the reference's own Fortran BLAS needs gfortran,
 * which is absent, so the oracle build links these plain-loop routines
 * (cblas_naive.c) instead.  Only the routines and enum names the reference
 * sources use are declared.  Nothing in the GPU product links this file.
 */
#ifndef SUS2_ORACLE_CBLAS_H
#define SUS2_ORACLE_CBLAS_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
typedef size_t CBLAS_INDEX;

void cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb,
                 int m, int n, int k, double alpha, const double *a, int lda,
                 const double *b, int ldb, double beta, double *c, int ldc);
void cblas_dgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, int m, int n,
                 double alpha, const double *a, int lda, const double *x, int incx,
                 double beta, double *y, int incy);
void cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy);
void cblas_dger(enum CBLAS_ORDER order, int m, int n, double alpha, const double *x, int incx,
                const double *y, int incy, double *a, int lda);
void cblas_dsyr(enum CBLAS_ORDER order, enum CBLAS_UPLO uplo, int n, double alpha,
                const double *x, int incx, double *a, int lda);
void cblas_dsyrk(enum CBLAS_ORDER order, enum CBLAS_UPLO uplo, enum CBLAS_TRANSPOSE trans,
                 int n, int k, double alpha, const double *a, int lda, double beta,
                 double *c, int ldc);
void cblas_dsymv(enum CBLAS_ORDER order, enum CBLAS_UPLO uplo, int n, double alpha,
                 const double *a, int lda, const double *x, int incx, double beta,
                 double *y, int incy);
void cblas_dswap(int n, double *x, int incx, double *y, int incy);
CBLAS_INDEX cblas_idamax(int n, const double *x, int incx);
void cblas_domatcopy(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, int rows, int cols,
                     double alpha, const double *a, int lda, double *b, int ldb);
#ifdef __cplusplus
}
#endif
#endif
