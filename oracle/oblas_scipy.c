/*
 * oblas_scipy.c -- oblas.h forwarded to scipy's bundled OpenBLAS (LP64).
 *
 * TEST INFRASTRUCTURE ONLY (oracle back end).  The library exports the
 * Fortran BLAS/LAPACK entry points with a `scipy_` prefix; the reference
 * sources are pinned against the very same library, so the oracle and
 * the reference make identical BLAS calls.
 */
#include "oblas.h"
#include <stdlib.h>

void scipy_dgemv_(const char *, const int *, const int *, const double *, const double *,
                  const int *, const double *, const int *, const double *, double *,
                  const int *);
void scipy_dgemm_(const char *, const char *, const int *, const int *, const int *,
                  const double *, const double *, const int *, const double *,
                  const int *, const double *, double *, const int *);
double scipy_dnrm2_(const int *, const double *, const int *);
double scipy_ddot_(const int *, const double *, const int *, const double *, const int *);
void scipy_dscal_(const int *, const double *, double *, const int *);
void scipy_dcopy_(const int *, const double *, const int *, double *, const int *);
void scipy_daxpy_(const int *, const double *, const double *, const int *, double *,
                  const int *);
void scipy_dgetrf_(const int *, const int *, double *, const int *, int *, int *);
void scipy_dgetri_(const int *, double *, const int *, const int *, double *,
                   const int *, int *);
void scipy_openblas_set_num_threads(int);

void ob_dgemv(char trans, int m, int n, double alpha, const double *a, int lda,
              const double *x, int incx, double beta, double *y, int incy)
{
    scipy_dgemv_(&trans, &m, &n, &alpha, a, &lda, x, &incx, &beta, y, &incy);
}

void ob_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *a,
              int lda, const double *b, int ldb, double beta, double *c, int ldc)
{
    scipy_dgemm_(&ta, &tb, &m, &n, &k, &alpha, a, &lda, b, &ldb, &beta, c, &ldc);
}

double ob_dnrm2(int n, const double *x, int incx) { return scipy_dnrm2_(&n, x, &incx); }

double ob_ddot(int n, const double *x, int incx, const double *y, int incy)
{
    return scipy_ddot_(&n, x, &incx, y, &incy);
}

void ob_dscal(int n, double alpha, double *x, int incx) { scipy_dscal_(&n, &alpha, x, &incx); }

void ob_dcopy(int n, const double *x, int incx, double *y, int incy)
{
    scipy_dcopy_(&n, x, &incx, y, &incy);
}

void ob_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy)
{
    scipy_daxpy_(&n, &alpha, x, &incx, y, &incy);
}

int ob_dgetrf(int m, double *a, int lda, int *ipiv)
{
    int info = 0;
    scipy_dgetrf_(&m, &m, a, &lda, ipiv, &info);
    return info;
}

int ob_dgetri(int m, double *a, int lda, int *ipiv)
{
    int info = 0, lwork = -1;
    double query = 0.0;
    scipy_dgetri_(&m, a, &lda, ipiv, &query, &lwork, &info);
    if (info != 0) return info;
    lwork = (int)query;
    if (lwork < 1) lwork = 1;
    double *work = (double *)malloc((size_t)lwork * sizeof(double));
    if (!work) return -1000;
    scipy_dgetri_(&m, a, &lda, ipiv, work, &lwork, &info);
    free(work);
    return info;
}

void ob_set_threads(int n) { scipy_openblas_set_num_threads(n); }
int ob_is_optimised(void) { return 1; }
