/*
 * dplr_oracle.h -- CPU oracle for the DPLR apply / inverse path.
 *
 * TEST INFRASTRUCTURE ONLY.  These functions restate, step by step, the
 * algorithms of the reference DPLR sources so that the GPU library can be
 * checked against them.  Only the tests, the smoke check and the CPU
 * baseline of the benchmark load this code; the product never does.
 *
 * Every routine uses the DPlrMtx layout of include/dplr.h and the BLAS
 * calls of the reference (through oblas.h), so with the same BLAS the
 * results match the reference sources bit for bit.
 */
#ifndef DPLR_ORACLE_H
#define DPLR_ORACLE_H

#include "../include/dplr.h"

#ifdef __cplusplus
extern "C" {
#endif

void orc_ini(DPlrMtx *A);
void orc_inid(int m, DPlrMtx *A);
void orc_inilr(int m, DPlrMtx *A, int capacity);
void orc_inih(int m, DPlrMtx *A);
void orc_clr(DPlrMtx *A);
void orc_resizelr(DPlrMtx *A, int capacity);
long orc_nz(int m, DPlrMtx *A);
void orc_rnk(int m, DPlrMtx *A, int *ranks);
void orc_gep2d(int m, DPlrMtx *A, double *B, int ldb);

void orc_gepmv(char trans, int m, const double *alpha, DPlrMtx *A, const double *x,
               int incx, const double *beta, double *y, int incy);
void orc_gepdmm(char transa, char transb, int m, int n, const double *alpha, DPlrMtx *A,
                const double *B, int ldb, const double *beta, double *C, int ldc);
void orc_geprk(int m, int k, const double *alpha, const double *u, int ldu,
               const double *v, int ldv, const double *s, int incs, DPlrMtx *A, double eps);
void orc_geinv(int m, DPlrMtx *A, DPlrMtx *B, double eps, int *info);

/* Pivoted, sval-weighted Gram-Schmidt with truncation on one low-rank
 * factorisation u diag(sval) v^T (columns of length nnu and nnv).
 * Returns the new rank; survivors are compacted into columns 0..rank-1. */
int  orc_dortlr(int nnu, int nnv, double *u, double *v, int lrankini, double *sval,
                double eps, int niter);
void orc_reduce(int m, DPlrMtx *A, double eps);

/* Checker (not a restatement): rnorm[j] = ||b_j - A x_j||_2 with A x_j
 * evaluated in double-double arithmetic, absnorm[j] = || |A||x_j| ||_2,
 * for columns j < ncols, spread over nthreads threads (dd_resid.c).
 * Returns 0, or -1 on a bad argument or failed allocation. */
int  orc_resid_dd(int m, DPlrMtx *A, int ncols, const double *X, int ldx, const double *B,
                  int ldb, double *rnorm, double *absnorm, int nthreads);

/* Timing stand-in (not a restatement): B := a tree with the structure
 * DPLR's dplrgeinv gives inv(A) (own rank + the ranks of the ancestors'
 * corrections in every block, leaves unchanged), every entry `fill`
 * (shape.c).  Returns 0, or -1 on a malformed A or failed allocation. */
int  orc_inverse_shape(int m, const DPlrMtx *A, DPlrMtx *B, double fill);

/* Number of argument errors reported since load (the reference prints
 * them to stderr and returns without touching outputs). */
long orc_error_count(void);
void orc_set_threads(int n);
int  orc_blas_optimised(void);

#ifdef __cplusplus
}
#endif

#endif
