/*
 * dplr_oracle.c -- CPU restatement of the DPLR apply / inverse path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker of the GPU library, the
 * replay target of the golden vectors, and the timed CPU baseline.  The
 * product (libdplr_gb300.so) never links or calls it.
 *
 * Each routine cites the reference function whose steps it restates.
 * The BLAS calls (oblas.h) are the ones the reference makes, in the same
 * order and with the same arguments, so that with the same BLAS library
 * the results are bit-identical to the reference sources.
 */
#include "dplr_oracle.h"
#include "oblas.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static long g_errors = 0;

static void report(const char *fn, const char *what)
{
    ++g_errors;
    fprintf(stderr, "%s: %s\n", fn, what);
}

long orc_error_count(void) { return g_errors; }
void orc_set_threads(int n) { ob_set_threads(n); }
int orc_blas_optimised(void) { return ob_is_optimised(); }

/* ------------------------------------------------------------------ */
/* structure helpers                                                   */
/* ------------------------------------------------------------------ */

static double *nan_filled(size_t count)
{
    double *p = (double *)malloc(count * sizeof(double));
    if (!p) return NULL;
    double q = nan("");
    for (size_t i = 0; i < count; ++i) p[i] = q;
    return p;
}

/* dplrini, src/dplrini.c:18-30 */
void orc_ini(DPlrMtx *A)
{
    memset(A, 0, sizeof(*A));
    A->type = PLR_UMTX;
}

/* dplrinid, src/dplrini.c:35-74: NaN-filled dense leaf */
void orc_inid(int m, DPlrMtx *A)
{
    if (m < 0) { report("orc_inid", "invalid matrix size"); return; }
    A->type = PLR_DMTX;
    A->size = m;
    A->dd.d = NULL;
    if (m > 0) {
        A->dd.d = nan_filled((size_t)m * m);
        if (!A->dd.d) report("orc_inid", "memory allocation failed");
    }
}

/* dplrinilr, src/dplrini.c:80-134: NaN-filled low-rank block, rank 0 */
void orc_inilr(int m, DPlrMtx *A, int capacity)
{
    if (m < 0 || capacity < 0) { report("orc_inilr", "invalid size or capacity"); return; }
    A->type = PLR_LRMTX;
    A->size = m;
    A->dlr.rank = 0;
    A->dlr.capacity = capacity;
    A->dlr.u = A->dlr.v = A->dlr.sig = NULL;
    if (capacity > 0) {
        A->dlr.u = nan_filled((size_t)m * capacity);
        A->dlr.sig = nan_filled((size_t)capacity);
        A->dlr.v = nan_filled((size_t)m * capacity);
        if (!A->dlr.u || !A->dlr.v || !A->dlr.sig) report("orc_inilr", "memory allocation failed");
    }
}

/* dplrinih, src/dplrini.c:142-175: four untyped children */
void orc_inih(int m, DPlrMtx *A)
{
    if (m < 0) { report("orc_inih", "invalid size"); return; }
    if (m % 2 != 0) { report("orc_inih", "m must be even"); return; }
    A->type = PLR_HMTX;
    A->size = m;
    DPlrMtx **kids[4] = { &A->dh.nw, &A->dh.ne, &A->dh.se, &A->dh.sw };
    for (int i = 0; i < 4; ++i) {
        *kids[i] = (DPlrMtx *)malloc(sizeof(DPlrMtx));
        if (!*kids[i]) { report("orc_inih", "memory allocation failed"); return; }
        orc_ini(*kids[i]);
    }
}

/* dplrclr, src/dplrini.c:183-206: buffers only; child structs are kept */
void orc_clr(DPlrMtx *A)
{
    switch (A->type) {
    case PLR_DMTX: free(A->dd.d); break;
    case PLR_LRMTX: free(A->dlr.u); free(A->dlr.v); free(A->dlr.sig); break;
    case PLR_HMTX:
        orc_clr(A->dh.nw); orc_clr(A->dh.se); orc_clr(A->dh.ne); orc_clr(A->dh.sw);
        break;
    default: break;
    }
}

/* dplrresizelr, src/dplrresizelr.c:15-118: at least double, keep live cols */
void orc_resizelr(DPlrMtx *A, int capacity)
{
    if (A->type != PLR_LRMTX) { report("orc_resizelr", "invalid matrix type"); return; }
    if (A->size < 0) { report("orc_resizelr", "invalid matrix size"); return; }
    if (capacity < 0) { report("orc_resizelr", "invalid capacity"); return; }
    if (capacity < A->dlr.capacity) return;
    int grown = capacity > 2 * A->dlr.capacity ? capacity : 2 * A->dlr.capacity;
    size_t n = (size_t)A->size;
    double *u = nan_filled(n * grown), *v = nan_filled(n * grown), *s = nan_filled((size_t)grown);
    if (!u || !v || !s) { report("orc_resizelr", "memory allocation failed"); return; }
    if (A->dlr.rank > 0) {
        int live = A->dlr.rank * A->size;
        ob_dcopy(A->dlr.rank, A->dlr.sig, 1, s, 1);
        ob_dcopy(live, A->dlr.u, 1, u, 1);
        ob_dcopy(live, A->dlr.v, 1, v, 1);
    }
    if (A->dlr.capacity > 0) { free(A->dlr.u); free(A->dlr.v); free(A->dlr.sig); }
    A->dlr.capacity = grown;
    A->dlr.u = u;
    A->dlr.v = v;
    A->dlr.sig = s;
}

/* dplrnz, src/dplrnz.c:17-62 */
long orc_nz(int m, DPlrMtx *A)
{
    if (m < 0) { report("orc_nz", "invalid matrix size"); return -1; }
    if (A->size != m) { report("orc_nz", "invalid A size"); return -1; }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) { report("orc_nz", "invalid A type"); return -1; }
    if (A->type == PLR_DMTX) return (long)m * m;
    long nz = (long)m * (A->dh.ne->dlr.rank + A->dh.sw->dlr.rank);
    return nz + orc_nz(m / 2, A->dh.nw) + orc_nz(m / 2, A->dh.se);
}

/* dplrrnk, src/dplrrnk.c:22-57 */
void orc_rnk(int m, DPlrMtx *A, int *ranks)
{
    if (m < 0) { report("orc_rnk", "invalid matrix size"); return; }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) { report("orc_rnk", "invalid A type"); return; }
    if (A->size != m) { report("orc_rnk", "invalid A size"); return; }
    if (A->type != PLR_HMTX) return;
    int r = A->dh.ne->dlr.rank > A->dh.sw->dlr.rank ? A->dh.ne->dlr.rank : A->dh.sw->dlr.rank;
    if (ranks[0] < r) ranks[0] = r;
    if (A->dh.nw->type != PLR_DMTX && A->dh.se->type != PLR_DMTX) {
        orc_rnk(m / 2, A->dh.nw, ranks + 1);
        orc_rnk(m / 2, A->dh.se, ranks + 1);
    }
}

/* dplrlr2d / dplrgep2d, src/dplrp2d.c:18-138 */
static void lr_to_dense(int m, DPlrMtx *L, double *B, int ldb)
{
    if (L->dlr.rank == 0) {
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) B[(size_t)j * ldb + i] = 0.0;
        return;
    }
    int r = L->dlr.rank, len = m * r;
    double *t = (double *)malloc((size_t)len * sizeof(double));
    ob_dcopy(len, L->dlr.u, 1, t, 1);
    for (int k = 0; k < r; ++k) ob_dscal(m, L->dlr.sig[k], t + (size_t)k * m, 1);
    ob_dgemm('N', 'T', m, m, r, 1.0, t, m, L->dlr.v, m, 0.0, B, ldb);
    free(t);
}

void orc_gep2d(int m, DPlrMtx *A, double *B, int ldb)
{
    if (m < 0 || A->size != m || ldb < m || (A->type != PLR_DMTX && A->type != PLR_HMTX)) {
        report("orc_gep2d", "invalid arguments");
        return;
    }
    if (A->type == PLR_DMTX) {
        for (int j = 0; j < m; ++j) ob_dcopy(m, A->dd.d + (size_t)j * m, 1, B + (size_t)j * ldb, 1);
        return;
    }
    int h = m / 2;
    lr_to_dense(h, A->dh.ne, B + (size_t)ldb * h, ldb);
    lr_to_dense(h, A->dh.sw, B + h, ldb);
    orc_gep2d(h, A->dh.nw, B, ldb);
    orc_gep2d(h, A->dh.se, B + (size_t)ldb * h + h, ldb);
}

/* ------------------------------------------------------------------ */
/* apply: y := alpha op(A) x + beta y  (src/dplrpmv.c)                 */
/* ------------------------------------------------------------------ */

/* y := beta*y over m strided entries, zeroing for beta == 0
 * (src/dplrpmv.c:48-56, :142-150). */
static void scale_vector(int m, double beta, double *y, int incy)
{
    if (beta == 0.0) {
        for (int i = 0; i < m; ++i) y[(size_t)i * incy] = 0.0;
    } else {
        ob_dscal(m, beta, y, incy);
    }
}

/* One low-rank block; restates dplrlrmv, src/dplrpmv.c:19-105.  For op=N
 * the block contracts V with x and expands with U; op=T swaps the two. */
static void lr_times_vector(int tr, int m, const double *alpha, DPlrMtx *L, const double *x,
                            int incx, const double *beta, double *y, int incy)
{
    if (m < 0) { report("orc_lrmv", "invalid matrix size"); return; }
    if (L->type != PLR_LRMTX) { report("orc_lrmv", "invalid A type"); return; }
    if (L->size != m) { report("orc_lrmv", "invalid A size"); return; }
    if (L->dlr.rank == 0 || *alpha == 0.0) { scale_vector(m, *beta, y, incy); return; }

    const double *contract = tr ? L->dlr.u : L->dlr.v;
    const double *expand = tr ? L->dlr.v : L->dlr.u;
    int r = L->dlr.rank;
    double *t = (double *)malloc((size_t)r * sizeof(double));
    ob_dgemv('T', m, r, 1.0, contract, m, x, incx, 0.0, t, 1);
    for (int k = 0; k < r; ++k) t[k] *= L->dlr.sig[k];
    ob_dgemv('N', m, r, *alpha, expand, m, t, 1, *beta, y, incy);
    free(t);
}

/* Restates dplrpmv (src/dplrpmv.c:113-180) and dplrptmv (:188-254). */
static void h_times_vector(int tr, int m, const double *alpha, DPlrMtx *A, const double *x,
                           int incx, const double *beta, double *y, int incy)
{
    if (m < 0) { report("orc_pmv", "invalid matrix size"); return; }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) { report("orc_pmv", "invalid A type"); return; }
    if (A->size != m) { report("orc_pmv", "invalid A size"); return; }

    /* alpha == 0 scales y here AND again below (the reference does not
     * return early, src/dplrpmv.c:140-151), so y ends up beta^2 * y. */
    if (*alpha == 0.0) scale_vector(m, *beta, y, incy);

    if (A->type == PLR_DMTX) {
        ob_dgemv(tr ? 'T' : 'N', m, m, *alpha, A->dd.d, m, x, incx, *beta, y, incy);
        return;
    }
    int h = m / 2;
    const double one = 1.0;
    /* Block writing the top half of y, then the one writing the bottom
     * half: ne and sw for op=N (:166-167), sw and ne for op=T (:240-241). */
    DPlrMtx *to_top = tr ? A->dh.sw : A->dh.ne;
    DPlrMtx *to_bottom = tr ? A->dh.ne : A->dh.sw;
    lr_times_vector(tr, h, alpha, to_top, x + (size_t)h * incx, incx, beta, y, incy);
    lr_times_vector(tr, h, alpha, to_bottom, x, incx, beta, y + (size_t)h * incy, incy);
    h_times_vector(tr, h, alpha, A->dh.nw, x, incx, &one, y, incy);
    h_times_vector(tr, h, alpha, A->dh.se, x + (size_t)h * incx, incx, &one, y + (size_t)h * incy, incy);
}

/* dplrgepmv, src/dplrpmv.c:262-282: anything but N/n means transpose. */
void orc_gepmv(char trans, int m, const double *alpha, DPlrMtx *A, const double *x, int incx,
               const double *beta, double *y, int incy)
{
    h_times_vector(!(trans == 'N' || trans == 'n'), m, alpha, A, x, incx, beta, y, incy);
}

/* ------------------------------------------------------------------ */
/* apply to a dense block: C := alpha op(A) op(B) + beta C             */
/* (src/dplrpdmm.c)                                                    */
/* ------------------------------------------------------------------ */

static void scale_matrix(int m, int n, double beta, double *C, int ldc)
{
    if (beta == 0.0) {
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < m; ++i) C[(size_t)j * ldc + i] = 0.0;
    } else {
        for (int j = 0; j < n; ++j) ob_dscal(m, beta, C + (size_t)j * ldc, 1);
    }
}

/* One low-rank block; restates dplrldmm, src/dplrpdmm.c:23-166. */
static void lr_times_dense(int ta, int tb, int m, int n, const double *alpha, DPlrMtx *L,
                           const double *B, int ldb, const double *beta, double *C, int ldc)
{
    if (m < 0) { report("orc_ldmm", "invalid matrix size"); return; }
    if (L->type != PLR_LRMTX) { report("orc_ldmm", "invalid A type"); return; }
    if (L->size != m) { report("orc_ldmm", "invalid A size"); return; }
    if (m == 0 || n == 0) return;
    if (*alpha == 0.0 || L->dlr.rank == 0) { scale_matrix(m, n, *beta, C, ldc); return; }

    const double *contract = ta ? L->dlr.u : L->dlr.v;
    const double *expand = ta ? L->dlr.v : L->dlr.u;
    int r = L->dlr.rank;
    double *t = (double *)malloc((size_t)r * n * sizeof(double));
    ob_dgemm('T', tb ? 'T' : 'N', r, n, m, 1.0, contract, m, B, ldb, 0.0, t, r);
    for (int k = 0; k < r; ++k) ob_dscal(n, L->dlr.sig[k], t + k, r);
    ob_dgemm('N', 'N', m, n, r, *alpha, expand, m, t, r, *beta, C, ldc);
    free(t);
}

/* Restates dplrpdmm (:177), dplrptdmm (:253), dplrpdtmm (:320) and
 * dplrptdtmm (:387): the four differ only in the op of A (which block
 * feeds which half, dense leaf op) and in how B's second half is
 * addressed (row offset for op(B)=B, column offset for op(B)=B^T). */
static void h_times_dense(int ta, int tb, int m, int n, const double *alpha, DPlrMtx *A,
                          const double *B, int ldb, const double *beta, double *C, int ldc)
{
    if (m < 0) { report("orc_pdmm", "invalid matrix size"); return; }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) { report("orc_pdmm", "invalid A type"); return; }
    if (A->size != m) { report("orc_pdmm", "invalid A size"); return; }
    if (ldc < m) { report("orc_pdmm", "invalid leading dimensions"); return; }
    /* Only the (N,N) variant has this quick return (src/dplrpdmm.c:208). */
    if (!ta && !tb && (m == 0 || n == 0)) return;

    if (A->type == PLR_DMTX) {
        ob_dgemm(ta ? 'T' : 'N', tb ? 'T' : 'N', m, n, m, *alpha, A->dd.d, m, B, ldb, *beta, C, ldc);
        return;
    }
    int h = m / 2;
    const double one = 1.0;
    size_t second = tb ? (size_t)h * ldb : (size_t)h;
    DPlrMtx *to_top = ta ? A->dh.sw : A->dh.ne;
    DPlrMtx *to_bottom = ta ? A->dh.ne : A->dh.sw;
    lr_times_dense(ta, tb, h, n, alpha, to_top, B + second, ldb, beta, C, ldc);
    lr_times_dense(ta, tb, h, n, alpha, to_bottom, B, ldb, beta, C + h, ldc);
    h_times_dense(ta, tb, h, n, alpha, A->dh.nw, B, ldb, &one, C, ldc);
    h_times_dense(ta, tb, h, n, alpha, A->dh.se, B + second, ldb, &one, C + h, ldc);
}

/* dplrgepdmm, src/dplrpdmm.c:454-490 */
void orc_gepdmm(char transa, char transb, int m, int n, const double *alpha, DPlrMtx *A,
                const double *B, int ldb, const double *beta, double *C, int ldc)
{
    h_times_dense(!(transa == 'N' || transa == 'n'), !(transb == 'N' || transb == 'n'), m, n,
                  alpha, A, B, ldb, beta, C, ldc);
}

/* ------------------------------------------------------------------ */
/* rank-k update (src/dplrprk.c)                                       */
/* ------------------------------------------------------------------ */

/* Append k normalised column pairs to a low-rank block; restates the two
 * copy/normalise loops of dplrgeprk (src/dplrprk.c:99-142, :147-191). */
static void append_pairs(DPlrMtx *L, int len, int k, double alpha, const double *u, int ldu,
                         const double *v, int ldv, const double *s, int incs, double eps2)
{
    int r0 = L->dlr.rank;
    double mag = fabs(alpha);
    if (L->dlr.capacity < r0 + k) orc_resizelr(L, r0 + k);
    for (int i = 0; i < k; ++i) {
        double *uc = L->dlr.u + (size_t)(r0 + i) * len;
        double *vc = L->dlr.v + (size_t)(r0 + i) * len;
        ob_dcopy(len, u + (size_t)i * ldu, 1, uc, 1);
        ob_dcopy(len, v + (size_t)i * ldv, 1, vc, 1);
        double fu = ob_dnrm2(len, uc, 1), fv = ob_dnrm2(len, vc, 1);
        if (mag * s[(size_t)i * incs] * fu * fv < eps2) {
            L->dlr.sig[r0 + i] = 0.0;
        } else {
            L->dlr.sig[r0 + i] = mag * s[(size_t)i * incs] * fu * fv;
            ob_dscal(len, alpha > 0.0 ? 1.0 / fu : -1.0 / fu, uc, 1);
            ob_dscal(len, 1.0 / fv, vc, 1);
        }
    }
    L->dlr.rank += k;
}

/* dplrgeprk, src/dplrprk.c:21-199 (no recompression). */
void orc_geprk(int m, int k, const double *alpha, const double *u, int ldu, const double *v,
               int ldv, const double *s, int incs, DPlrMtx *A, double eps)
{
    if (m < 0) { report("orc_geprk", "invalid matrix size"); return; }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) { report("orc_geprk", "invalid A type"); return; }
    if (A->size != m) { report("orc_geprk", "invalid A size"); return; }
    if (ldu < m || ldv < m) { report("orc_geprk", "invalid leading dimensions"); return; }
    if (*alpha == 0.0 || k == 0) return;

    if (A->type == PLR_DMTX) {
        double *t = (double *)malloc((size_t)m * k * sizeof(double));
        for (int i = 0; i < k; ++i) {
            ob_dcopy(m, u + (size_t)i * ldu, 1, t + (size_t)i * m, 1);
            ob_dscal(m, s[(size_t)i * incs], t + (size_t)i * m, 1);
        }
        ob_dgemm('N', 'T', m, m, k, *alpha, t, m, v, ldv, 1.0, A->dd.d, m);
        free(t);
        return;
    }
    double eps2 = A->dh.nw->type == PLR_DMTX ? eps / 2.0 : eps / 4.0;
    int h = m / 2;
    /* ne holds rows of the top half and columns of the bottom half. */
    append_pairs(A->dh.ne, h, k, *alpha, u, ldu, v + h, ldv, s, incs, eps2);
    append_pairs(A->dh.sw, h, k, *alpha, u + h, ldu, v, ldv, s, incs, eps2);
    orc_geprk(h, k, alpha, u, ldu, v, ldv, s, incs, A->dh.nw, eps2);
    orc_geprk(h, k, alpha, u + h, ldu, v + h, ldv, s, incs, A->dh.se, eps2);
}

/* ------------------------------------------------------------------ */
/* inverse (src/dplrinv.c)                                             */
/* ------------------------------------------------------------------ */

/* dplrdinv, src/dplrinv.c:20-84: explicit inverse via getrf + getri. */
static void dense_inverse(int m, double *a, int lda, int *info)
{
    *info = -1;
    int *ipiv = (int *)malloc((size_t)(m > 0 ? m : 1) * sizeof(int));
    *info = ob_dgetrf(m, a, lda, ipiv);
    if (*info != 0) {
        fprintf(stderr, "orc_dinv: dgetrf() failed: %d\n", *info);
        free(ipiv);
        return;
    }
    *info = ob_dgetri(m, a, lda, ipiv);
    if (*info != 0) fprintf(stderr, "orc_dinv: dgetri() failed: %d\n", *info);
    free(ipiv);
}

/* Column normalisation of a factor pair with s = |u_i||v_i|, zeroed below
 * eps2 (src/dplrinv.c:333-369, :385-423). */
static void normalise_pairs(int len, int r, double *u, double *v, double *s, double eps2)
{
    for (int i = 0; i < r; ++i) {
        double *ui = u + (size_t)i * len, *vi = v + (size_t)i * len;
        double fu = ob_dnrm2(len, ui, 1), fv = ob_dnrm2(len, vi, 1);
        if (fu * fv < eps2) {
            s[i] = 0.0;
        } else {
            s[i] = fu * fv;
            ob_dscal(len, 1.0 / fu, ui, 1);
            ob_dscal(len, 1.0 / fv, vi, 1);
        }
    }
}

/* dplrgeinv, src/dplrinv.c:93-450. */
void orc_geinv(int m, DPlrMtx *A, DPlrMtx *B, double eps, int *info)
{
    if (m < 0) { report("orc_geinv", "invalid matrix size"); return; }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) { report("orc_geinv", "invalid A type"); return; }
    if (A->size != m) { report("orc_geinv", "invalid A size"); return; }
    *info = -1;

    if (A->type == PLR_DMTX) {
        if (B->type != PLR_DMTX || B->size != m) { orc_clr(B); orc_inid(m, B); }
        ob_dcopy(m * m, A->dd.d, 1, B->dd.d, 1);
        dense_inverse(m, B->dd.d, m, info);
        if (*info != 0) fprintf(stderr, "orc_geinv: failed to invert a dense matrix: %d\n", *info);
        return;
    }

    double eps2 = A->dh.nw->type == PLR_DMTX ? eps / 2.0 : eps / 4.0;
    if (B->type != PLR_HMTX || B->size != m) { orc_clr(B); orc_inih(m, B); }

    int h = m / 2;
    orc_geinv(h, A->dh.nw, B->dh.nw, eps2, info);
    if (*info != 0) { fprintf(stderr, "orc_geinv: failed to invert nw block: %d\n", *info); return; }
    orc_geinv(h, A->dh.se, B->dh.se, eps2, info);
    if (*info != 0) { fprintf(stderr, "orc_geinv: failed to invert se block: %d\n", *info); return; }

    DPlrMtx *ane = A->dh.ne, *asw = A->dh.sw, *bne = B->dh.ne, *bsw = B->dh.sw;
    if (bne->type != PLR_LRMTX || bne->size != h) { orc_clr(bne); orc_inilr(h, bne, ane->dlr.rank); }
    if (bsw->type != PLR_LRMTX || bsw->size != h) { orc_clr(bsw); orc_inilr(h, bsw, asw->dlr.rank); }
    if (bne->dlr.capacity < ane->dlr.rank) orc_resizelr(bne, ane->dlr.rank);
    if (bsw->dlr.capacity < asw->dlr.rank) orc_resizelr(bsw, asw->dlr.rank);

    int r1 = ane->dlr.rank, r2 = asw->dlr.rank, r = r1 + r2;
    if (r1 == 0 && r2 == 0) { *info = 0; return; }

    const double one = 1.0, zero = 0.0;
    double *u1 = (double *)malloc((size_t)h * r1 * sizeof(double));
    double *d1 = (double *)malloc((size_t)r1 * sizeof(double));
    double *v1 = (double *)malloc((size_t)h * r1 * sizeof(double));
    double *u2 = (double *)malloc((size_t)h * r2 * sizeof(double));
    double *d2 = (double *)malloc((size_t)r2 * sizeof(double));
    double *v2 = (double *)malloc((size_t)h * r2 * sizeof(double));

    /* Panels through the child inverses (src/dplrinv.c:253-263):
     *   u1 = inv(A_nw) U_ne,   u2 = inv(A_se) U_sw,
     *   B_ne.v = inv(A_se)^T V_ne,   B_sw.v = inv(A_nw)^T V_sw. */
    orc_gepdmm('N', 'N', h, r1, &one, B->dh.nw, ane->dlr.u, h, &zero, u1, h);
    orc_gepdmm('N', 'N', h, r2, &one, B->dh.se, asw->dlr.u, h, &zero, u2, h);
    orc_gepdmm('T', 'N', h, r1, &one, B->dh.se, ane->dlr.v, h, &zero, bne->dlr.v, h);
    orc_gepdmm('T', 'N', h, r2, &one, B->dh.nw, asw->dlr.v, h, &zero, bsw->dlr.v, h);
    ob_dcopy(h * r1, bne->dlr.v, 1, v1, 1);
    ob_dcopy(h * r2, bsw->dlr.v, 1, v2, 1);

    /* Capacitance X = [[diag(1/s_ne), V_ne^T u2], [V_sw^T u1, diag(1/s_sw)]]
     * (src/dplrinv.c:277-310), then X := inv(X). */
    double *X = (double *)malloc((size_t)r * r * sizeof(double));
    for (int j = 0; j < r1; ++j)
        for (int i = 0; i < r1; ++i) X[(size_t)j * r + i] = i == j ? 1.0 / ane->dlr.sig[i] : 0.0;
    for (int j = 0; j < r2; ++j)
        for (int i = 0; i < r2; ++i)
            X[(size_t)(r1 + j) * r + r1 + i] = i == j ? 1.0 / asw->dlr.sig[i] : 0.0;
    ob_dgemm('T', 'N', r1, r2, h, 1.0, ane->dlr.v, h, u2, h, 0.0, X + (size_t)r1 * r, r);
    ob_dgemm('T', 'N', r2, r1, h, 1.0, asw->dlr.v, h, u1, h, 0.0, X + r1, r);
    dense_inverse(r, X, r, info);
    if (*info != 0) {
        fprintf(stderr, "orc_geinv: failed to invert the Woodbury capacitance: %d\n", *info);
        return;
    }

    /* Off-diagonal blocks of the inverse (src/dplrinv.c:327-369). */
    ob_dgemm('N', 'N', h, r1, r1, -1.0, u1, h, X, r, 0.0, bne->dlr.u, h);
    ob_dgemm('N', 'N', h, r2, r2, -1.0, u2, h, X + (size_t)r1 * r + r1, r, 0.0, bsw->dlr.u, h);
    normalise_pairs(h, r1, bne->dlr.u, bne->dlr.v, bne->dlr.sig, eps2);
    bne->dlr.rank = r1;
    normalise_pairs(h, r2, bsw->dlr.u, bsw->dlr.v, bsw->dlr.sig, eps2);
    bsw->dlr.rank = r2;

    /* Corrections of the diagonal blocks (src/dplrinv.c:376-429):
     *   nw += (-u1 X12) v2^T,  se += (-u2 X21) v1^T. */
    double *keep = (double *)malloc((size_t)h * r1 * sizeof(double));
    ob_dcopy(h * r1, u1, 1, keep, 1);
    ob_dgemm('N', 'N', h, r1, r2, -1.0, u2, h, X + r1, r, 0.0, u1, h);
    ob_dgemm('N', 'N', h, r2, r1, -1.0, keep, h, X + (size_t)r1 * r, r, 0.0, u2, h);
    normalise_pairs(h, r2, u2, v2, d2, eps2);
    normalise_pairs(h, r1, u1, v1, d1, eps2);
    orc_geprk(h, r2, &one, u2, h, v2, h, d2, 1, B->dh.nw, eps2);
    orc_geprk(h, r1, &one, u1, h, v1, h, d1, 1, B->dh.se, eps2);

    free(X); free(u1); free(d1); free(v1); free(u2); free(d2); free(v2); free(keep);
    *info = 0;
}

/* ------------------------------------------------------------------ */
/* re-orthogonalisation (src/dortlr.f90, src/dplrreduce.c)             */
/* ------------------------------------------------------------------ */

/* One Gram-Schmidt pass over factor `a` (length na) with partner `b`
 * (length nb); restates the u-pass of dortlr (src/dortlr.f90:43-106),
 * whose v-pass (:110-170) is the same pass with the roles swapped.
 * Columns are visited in pivot order of decreasing sval; projections
 * removed from a column of `a` are folded into the pivot's partner
 * column of `b`; norms are RMS (|x|/sqrt(n)).  Returns the rank. */
static int gs_pass(int na, int nb, double *a, double *b, int *piv, int rank, double *sval,
                   double eps, double eps2)
{
    for (int j = 0; j < rank; ++j) {
        int kmax = j;
        double smax = -111.0;
        for (int k = j; k < rank; ++k)
            if (smax < sval[piv[k]]) { kmax = k; smax = sval[piv[k]]; }
        int t = piv[j]; piv[j] = piv[kmax]; piv[kmax] = t;
        int mm = piv[j];
        if (sval[mm] <= eps) return j;

        double *am = a + (size_t)mm * na, *bm = b + (size_t)mm * nb;
        for (int l = j + 1; l < rank; ++l) {
            int ll = piv[l];
            if (sval[ll] <= eps) { sval[ll] = 0.0; continue; }
            double *al = a + (size_t)ll * na, *bl = b + (size_t)ll * nb;
            double proj = ob_ddot(na, am, 1, al, 1) / na;
            ob_daxpy(na, -proj, am, 1, al, 1);
            double f1 = sqrt(ob_ddot(na, al, 1, al, 1) / na);
            if (f1 * sval[ll] > eps2) ob_dscal(na, 1.0 / f1, al, 1);
            proj = proj * sval[ll] / sval[mm];
            ob_daxpy(nb, proj, bl, 1, bm, 1);
            sval[ll] = sval[ll] * f1;
        }
        double f2 = sqrt(ob_ddot(nb, bm, 1, bm, 1) / nb);
        if (f2 * sval[mm] > eps2) ob_dscal(nb, 1.0 / f2, bm, 1);
        sval[mm] = sval[mm] * f2;
    }
    return rank;
}

/* dortlr, src/dortlr.f90:12-207, with the pivots initialised to the
 * identity as ortlrini does (src/ortlrini.f90:12-19) and the new rank
 * returned (the shipped C caller passes mismatched arguments). */
int orc_dortlr(int nnu, int nnv, double *u, double *v, int lrankini, double *sval, double eps,
               int niter)
{
    if (lrankini <= 0) return 0;
    int *piv = (int *)malloc((size_t)lrankini * sizeof(int));
    int *hole = (int *)malloc((size_t)lrankini * sizeof(int));
    for (int k = 0; k < lrankini; ++k) piv[k] = k;
    double eps2 = eps * eps;
    int rank = lrankini;
    for (int it = 0; it < niter; ++it) {
        rank = gs_pass(nnu, nnv, u, v, piv, rank, sval, eps, eps2);
        rank = gs_pass(nnv, nnu, v, u, piv, rank, sval, eps, eps2);
    }
    /* Compact survivors into slots 0..rank-1 (src/dortlr.f90:177-200). */
    int nh = 0;
    for (int l = rank; l < lrankini; ++l)
        if (piv[l] < rank) hole[nh++] = piv[l];
    int used = 0;
    for (int l = 0; l < rank; ++l) {
        if (piv[l] >= rank) {
            int dst = hole[used++];
            ob_dcopy(nnu, u + (size_t)piv[l] * nnu, 1, u + (size_t)dst * nnu, 1);
            ob_dcopy(nnv, v + (size_t)piv[l] * nnv, 1, v + (size_t)dst * nnv, 1);
            sval[dst] = sval[piv[l]];
            piv[l] = dst;
        }
    }
    free(piv);
    free(hole);
    return rank;
}

/* dplrreduce, src/dplrreduce.c:25-82: eps/4 per level, one iteration. */
void orc_reduce(int m, DPlrMtx *A, double eps)
{
    if (m < 0) { report("orc_reduce", "invalid matrix size"); return; }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) { report("orc_reduce", "invalid A type"); return; }
    if (A->size != m) { report("orc_reduce", "invalid A size"); return; }
    if (A->type == PLR_DMTX) return;
    double eps2 = eps / 4.0;
    int h = m / 2;
    DPlrMtx *blk[2] = { A->dh.ne, A->dh.sw };
    for (int i = 0; i < 2; ++i)
        blk[i]->dlr.rank = orc_dortlr(h, h, blk[i]->dlr.u, blk[i]->dlr.v, blk[i]->dlr.rank,
                                      blk[i]->dlr.sig, eps2, 1);
    orc_reduce(h, A->dh.nw, eps2);
    orc_reduce(h, A->dh.se, eps2);
}
