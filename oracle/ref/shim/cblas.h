/* Build shim for compiling the xerus reference as a test oracle.
 * Declares the CBLAS entry points the reference calls and binds them to the
 * prefixed symbols exported by SciPy's bundled OpenBLAS (LP64 build). */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
typedef enum CBLAS_ORDER CBLAS_LAYOUT;
double scipy_cblas_dasum(int n, const double *x, int incx);
double scipy_cblas_ddot(int n, const double *x, int incx, const double *y, int incy);
double scipy_cblas_dnrm2(int n, const double *x, int incx);
void scipy_cblas_dgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, int m, int n, double alpha,
                       const double *a, int lda, const double *x, int incx, double beta, double *y, int incy);
void scipy_cblas_dger(enum CBLAS_ORDER order, int m, int n, double alpha, const double *x, int incx,
                      const double *y, int incy, double *a, int lda);
void scipy_cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n, int k,
                       double alpha, const double *a, int lda, const double *b, int ldb, double beta, double *c, int ldc);
#ifdef __cplusplus
}
#endif
#define cblas_dasum scipy_cblas_dasum
#define cblas_ddot scipy_cblas_ddot
#define cblas_dnrm2 scipy_cblas_dnrm2
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_dger scipy_cblas_dger
#define cblas_dgemm scipy_cblas_dgemm
