/* Build shim for compiling the xerus reference as a test oracle.
 * Declares the LAPACKE entry points the reference calls and binds them to the
 * prefixed symbols exported by SciPy's bundled OpenBLAS (LP64 build). */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
lapack_int scipy_LAPACKE_dgesdd(int layout, char jobz, lapack_int m, lapack_int n, double *a, lapack_int lda,
                                double *s, double *u, lapack_int ldu, double *vt, lapack_int ldvt);
lapack_int scipy_LAPACKE_dgeqp3(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda, lapack_int *jpvt, double *tau);
lapack_int scipy_LAPACKE_dorgqr(int layout, lapack_int m, lapack_int n, lapack_int k, double *a, lapack_int lda, const double *tau);
lapack_int scipy_LAPACKE_dgeqrf(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda, double *tau);
lapack_int scipy_LAPACKE_dgerqf(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda, double *tau);
lapack_int scipy_LAPACKE_dorgrq(int layout, lapack_int m, lapack_int n, lapack_int k, double *a, lapack_int lda, const double *tau);
lapack_int scipy_LAPACKE_dgesv(int layout, lapack_int n, lapack_int nrhs, double *a, lapack_int lda, lapack_int *ipiv, double *b, lapack_int ldb);
lapack_int scipy_LAPACKE_dpotrf2(int layout, char uplo, lapack_int n, double *a, lapack_int lda);
lapack_int scipy_LAPACKE_dpotrs(int layout, char uplo, lapack_int n, lapack_int nrhs, const double *a, lapack_int lda, double *b, lapack_int ldb);
lapack_int scipy_LAPACKE_dsysv(int layout, char uplo, lapack_int n, lapack_int nrhs, double *a, lapack_int lda, lapack_int *ipiv, double *b, lapack_int ldb);
lapack_int scipy_LAPACKE_dgelsd(int layout, lapack_int m, lapack_int n, lapack_int nrhs, double *a, lapack_int lda, double *b,
                                lapack_int ldb, double *s, double rcond, lapack_int *rank);
lapack_int scipy_LAPACKE_dgelsy(int layout, lapack_int m, lapack_int n, lapack_int nrhs, double *a, lapack_int lda, double *b,
                                lapack_int ldb, lapack_int *jpvt, double rcond, lapack_int *rank);
#ifdef __cplusplus
}
#endif
#define LAPACKE_dgesdd scipy_LAPACKE_dgesdd
#define LAPACKE_dgeqp3 scipy_LAPACKE_dgeqp3
#define LAPACKE_dorgqr scipy_LAPACKE_dorgqr
#define LAPACKE_dgeqrf scipy_LAPACKE_dgeqrf
#define LAPACKE_dgerqf scipy_LAPACKE_dgerqf
#define LAPACKE_dorgrq scipy_LAPACKE_dorgrq
#define LAPACKE_dgesv scipy_LAPACKE_dgesv
#define LAPACKE_dpotrf2 scipy_LAPACKE_dpotrf2
#define LAPACKE_dpotrs scipy_LAPACKE_dpotrs
#define LAPACKE_dsysv scipy_LAPACKE_dsysv
#define LAPACKE_dgelsd scipy_LAPACKE_dgelsd
#define LAPACKE_dgelsy scipy_LAPACKE_dgelsy
