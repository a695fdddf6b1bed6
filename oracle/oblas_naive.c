/*
 * oblas_naive.c -- oblas.h in plain C loops.
 *
 * TEST INFRASTRUCTURE ONLY (oracle back end for hosts without an
 * optimised LP64 BLAS).  Semantics follow the Fortran reference BLAS:
 * beta == 0 overwrites the output without reading it; alpha == 0 only
 * scales; non-positive increments are not supported (the oracle never
 * passes them).
 */
#include "oblas.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define A_(i, j) a[(size_t)(j) * lda + (i)]

void ob_dgemv(char trans, int m, int n, double alpha, const double *a, int lda,
              const double *x, int incx, double beta, double *y, int incy)
{
    int tr = !(trans == 'N' || trans == 'n');
    int ylen = tr ? n : m, xlen = tr ? m : n;
    if (m <= 0 || n <= 0) {
        if (ylen > 0 && beta != 1.0)
            for (int i = 0; i < ylen; ++i) y[(size_t)i * incy] = beta == 0.0 ? 0.0 : beta * y[(size_t)i * incy];
        return;
    }
    for (int i = 0; i < ylen; ++i)
        y[(size_t)i * incy] = beta == 0.0 ? 0.0 : beta * y[(size_t)i * incy];
    if (alpha == 0.0) return;
    if (!tr) {
        for (int j = 0; j < xlen; ++j) {
            double t = alpha * x[(size_t)j * incx];
            for (int i = 0; i < m; ++i) y[(size_t)i * incy] += t * A_(i, j);
        }
    } else {
        for (int j = 0; j < n; ++j) {
            double s = 0.0;
            for (int i = 0; i < m; ++i) s += A_(i, j) * x[(size_t)i * incx];
            y[(size_t)j * incy] += alpha * s;
        }
    }
}

void ob_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *a,
              int lda, const double *b, int ldb, double beta, double *c, int ldc)
{
    int tra = !(ta == 'N' || ta == 'n'), trb = !(tb == 'N' || tb == 'n');
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) {
            double *cij = &c[(size_t)j * ldc + i];
            double s = 0.0;
            if (alpha != 0.0)
                for (int l = 0; l < k; ++l) {
                    double av = tra ? a[(size_t)i * lda + l] : a[(size_t)l * lda + i];
                    double bv = trb ? b[(size_t)l * ldb + j] : b[(size_t)j * ldb + l];
                    s += av * bv;
                }
            *cij = (beta == 0.0 ? 0.0 : beta * *cij) + alpha * s;
        }
}

double ob_dnrm2(int n, const double *x, int incx)
{
    double scale = 0.0, ssq = 1.0;
    for (int i = 0; i < n; ++i) {
        double v = fabs(x[(size_t)i * incx]);
        if (v == 0.0) continue;
        if (scale < v) { ssq = 1.0 + ssq * (scale / v) * (scale / v); scale = v; }
        else ssq += (v / scale) * (v / scale);
    }
    return scale * sqrt(ssq);
}

double ob_ddot(int n, const double *x, int incx, const double *y, int incy)
{
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += x[(size_t)i * incx] * y[(size_t)i * incy];
    return s;
}

void ob_dscal(int n, double alpha, double *x, int incx)
{
    if (incx <= 0) return;
    for (int i = 0; i < n; ++i) x[(size_t)i * incx] *= alpha;
}

void ob_dcopy(int n, const double *x, int incx, double *y, int incy)
{
    for (int i = 0; i < n; ++i) y[(size_t)i * incy] = x[(size_t)i * incx];
}

void ob_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy)
{
    if (alpha == 0.0) return;
    for (int i = 0; i < n; ++i) y[(size_t)i * incy] += alpha * x[(size_t)i * incx];
}

int ob_dgetrf(int m, double *a, int lda, int *ipiv)
{
    int info = 0;
    for (int j = 0; j < m; ++j) {
        int p = j;
        double best = fabs(A_(j, j));
        for (int i = j + 1; i < m; ++i)
            if (fabs(A_(i, j)) > best) { best = fabs(A_(i, j)); p = i; }
        ipiv[j] = p + 1;
        if (A_(p, j) == 0.0) { if (!info) info = j + 1; continue; }
        if (p != j)
            for (int c = 0; c < m; ++c) { double t = A_(j, c); A_(j, c) = A_(p, c); A_(p, c) = t; }
        double inv = 1.0 / A_(j, j);
        for (int i = j + 1; i < m; ++i) A_(i, j) *= inv;
        for (int c = j + 1; c < m; ++c) {
            double t = A_(j, c);
            if (t != 0.0)
                for (int i = j + 1; i < m; ++i) A_(i, c) -= A_(i, j) * t;
        }
    }
    return info;
}

int ob_dgetri(int m, double *a, int lda, int *ipiv)
{
    /* Solve A X = I column by column from the packed LU factors. */
    double *inv = (double *)malloc((size_t)m * m * sizeof(double));
    if (!inv) return -1000;
    for (int j = 0; j < m; ++j) if (A_(j, j) == 0.0) { free(inv); return j + 1; }
    for (int c = 0; c < m; ++c) {
        double *x = inv + (size_t)c * m;
        for (int i = 0; i < m; ++i) x[i] = (i == c) ? 1.0 : 0.0;
        for (int i = 0; i < m; ++i) {            /* row interchanges */
            int p = ipiv[i] - 1;
            if (p != i) { double t = x[i]; x[i] = x[p]; x[p] = t; }
        }
        for (int i = 0; i < m; ++i)              /* unit lower solve */
            for (int r = i + 1; r < m; ++r) x[r] -= A_(r, i) * x[i];
        for (int i = m - 1; i >= 0; --i) {       /* upper solve */
            x[i] /= A_(i, i);
            for (int r = 0; r < i; ++r) x[r] -= A_(r, i) * x[i];
        }
    }
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) A_(i, j) = inv[(size_t)j * m + i];
    free(inv);
    return 0;
}

void ob_set_threads(int n) { (void)n; }
int ob_is_optimised(void) { return 0; }
