/*
 * oblas.h -- the BLAS/LAPACK subset the oracle calls.
 *
 * TEST INFRASTRUCTURE ONLY.  Two interchangeable back ends implement it:
 *   oblas_scipy.c  forwards to the LP64 OpenBLAS that ships inside scipy
 *                  (symbols scipy_dgemm_ ...), the same library the
 *                  reference C sources are linked against for pinning;
 *   oblas_naive.c  plain C loops, used when no such library is found.
 *
 * Argument meaning follows the Fortran BLAS the reference calls through
 * include/lapackapi_netlib.h:18-32 (column-major, leading dimensions),
 * with scalars by value.
 */
#ifndef DPLR_ORACLE_OBLAS_H
#define DPLR_ORACLE_OBLAS_H

void   ob_dgemv(char trans, int m, int n, double alpha, const double *a, int lda,
                const double *x, int incx, double beta, double *y, int incy);
void   ob_dgemm(char ta, char tb, int m, int n, int k, double alpha,
                const double *a, int lda, const double *b, int ldb,
                double beta, double *c, int ldc);
double ob_dnrm2(int n, const double *x, int incx);
double ob_ddot(int n, const double *x, int incx, const double *y, int incy);
void   ob_dscal(int n, double alpha, double *x, int incx);
void   ob_dcopy(int n, const double *x, int incx, double *y, int incy);
void   ob_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy);
/* LU with partial pivoting of an m x m matrix; returns LAPACK's info. */
int    ob_dgetrf(int m, double *a, int lda, int *ipiv);
/* Inverse from the LU factors, with LAPACK's workspace query; returns info. */
int    ob_dgetri(int m, double *a, int lda, int *ipiv);
/* Thread count of the back end (no-op for the loop back end). */
void   ob_set_threads(int n);
/* 1 when the optimised library is linked, 0 for the loop back end. */
int    ob_is_optimised(void);

#endif
