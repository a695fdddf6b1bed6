/*
 * dd_resid.c -- extended-precision residual of a PLR solve (TEST
 * INFRASTRUCTURE ONLY: a checker for the tests and the benchmark's CPU leg,
 * never part of the product).
 *
 * r_j = b_j - A x_j for selected columns, with A the PLR operator stored in
 * a DPlrMtx tree (include/dplr.h), evaluated in double-double arithmetic:
 * every product is split exactly with fma (TwoProd), every sum is kept as an
 * unevaluated hi + lo pair (Knuth's TwoSum).  The operator is the one the
 * reference's dplrgepdmm applies (src/dplrpdmm.c:177-241: leaves D x, and
 * per H node y[:m/2] += U_ne diag(sig) V_ne^T x[m/2:], y[m/2:] +=
 * U_sw diag(sig) V_sw^T x[:m/2]).  The rounding error of the result is
 * about n * 2^-104 |A||x|, i.e. below 1e-25 relative for the matrices here,
 * so the residual it reports is the exact residual of the stored operator
 * for every practical purpose, independent of any FP64 apply.
 *
 * Also returns || |A| |x_j| ||_2 (|A| taken entrywise on the factors: |U|
 * |sig| |V|^T), which bounds the rounding error of an FP64 apply.
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

#include "../include/dplr.h"

typedef struct { double hi, lo; } dd;

static inline dd two_sum(double a, double b)
{
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    dd r = {s, e};
    return r;
}

/* (a.hi + a.lo) + p * q, with the product split exactly by fma. */
static inline dd dd_add_prod(dd a, double p, double q)
{
    double ph = p * q;
    double pl = fma(p, q, -ph);
    dd s = two_sum(a.hi, ph);
    double lo = s.lo + a.lo + pl;
    return two_sum(s.hi, lo);
}

/* (a.hi + a.lo) + (t.hi + t.lo) * q */
static inline dd dd_add_ddprod(dd a, dd t, double q)
{
    double ph = t.hi * q;
    double pl = fma(t.hi, q, -ph) + t.lo * q;
    dd s = two_sum(a.hi, ph);
    double lo = s.lo + a.lo + pl;
    return two_sum(s.hi, lo);
}

typedef struct {
    const double *x;
    dd *y;
    double *ya;      /* |A||x| accumulator */
    dd *t;           /* rank scratch */
    double *ta;
} column_state;

static void lowrank_apply(int len, DPlrMtx *L, const double *x, dd *y, double *ya,
                          dd *t, double *ta)
{
    int r = L->dlr.rank;
    const double *u = L->dlr.u, *v = L->dlr.v, *s = L->dlr.sig;
    for (int k = 0; k < r; ++k) {
        dd acc = {0.0, 0.0};
        double aa = 0.0;
        const double *vk = v + (size_t)k * len;
        for (int i = 0; i < len; ++i) {
            acc = dd_add_prod(acc, vk[i], x[i]);
            aa += fabs(vk[i]) * fabs(x[i]);
        }
        /* t_k = sig_k * (V^T x)_k, kept in double-double */
        double ph = acc.hi * s[k];
        double pl = fma(acc.hi, s[k], -ph) + acc.lo * s[k];
        t[k] = two_sum(ph, pl);
        ta[k] = fabs(s[k]) * aa;
    }
    for (int k = 0; k < r; ++k) {
        const double *uk = u + (size_t)k * len;
        for (int i = 0; i < len; ++i) {
            y[i] = dd_add_ddprod(y[i], t[k], uk[i]);
            ya[i] += fabs(uk[i]) * ta[k];
        }
    }
}

static void tree_apply(int m, DPlrMtx *A, const double *x, dd *y, double *ya, dd *t, double *ta)
{
    if (A->type == PLR_DMTX) {
        const double *d = A->dd.d;
        for (int j = 0; j < m; ++j) {
            const double *dj = d + (size_t)j * m;
            double xj = x[j], axj = fabs(xj);
            for (int i = 0; i < m; ++i) {
                y[i] = dd_add_prod(y[i], dj[i], xj);
                ya[i] += fabs(dj[i]) * axj;
            }
        }
        return;
    }
    int h = m / 2;
    lowrank_apply(h, A->dh.ne, x + h, y, ya, t, ta);
    lowrank_apply(m - h, A->dh.sw, x, y + h, ya + h, t, ta);
    tree_apply(h, A->dh.nw, x, y, ya, t, ta);
    tree_apply(m - h, A->dh.se, x + h, y + h, ya + h, t, ta);
}

static int max_rank(DPlrMtx *A)
{
    if (A->type != PLR_HMTX)
        return 0;
    int r = A->dh.ne->dlr.rank > A->dh.sw->dlr.rank ? A->dh.ne->dlr.rank : A->dh.sw->dlr.rank;
    int a = max_rank(A->dh.nw), b = max_rank(A->dh.se);
    if (a > r) r = a;
    if (b > r) r = b;
    return r;
}

typedef struct {
    int m, ncols, ldx, ldb, rmax;
    DPlrMtx *A;
    const double *X, *B;
    double *rnorm, *absnorm;
    atomic_int next;
    atomic_int failed;
} job;

static void *worker(void *arg)
{
    job *J = (job *)arg;
    int m = J->m;
    dd *y = malloc(sizeof(dd) * (size_t)m);
    double *ya = malloc(sizeof(double) * (size_t)m);
    dd *t = malloc(sizeof(dd) * (size_t)(J->rmax + 1));
    double *ta = malloc(sizeof(double) * (size_t)(J->rmax + 1));
    if (!y || !ya || !t || !ta) {
        atomic_store(&J->failed, 1);
        free(y); free(ya); free(t); free(ta);
        return NULL;
    }
    for (;;) {
        int j = atomic_fetch_add(&J->next, 1);
        if (j >= J->ncols)
            break;
        memset(y, 0, sizeof(dd) * (size_t)m);
        memset(ya, 0, sizeof(double) * (size_t)m);
        const double *x = J->X + (size_t)j * J->ldx;
        const double *b = J->B + (size_t)j * J->ldb;
        tree_apply(m, J->A, x, y, ya, t, ta);
        double rr = 0.0, aa = 0.0;
        for (int i = 0; i < m; ++i) {
            /* r_i = b_i - y_i, then rounded once */
            dd d = two_sum(b[i], -y[i].hi);
            double ri = d.hi + (d.lo - y[i].lo);
            rr += ri * ri;
            aa += ya[i] * ya[i];
        }
        J->rnorm[j] = sqrt(rr);
        J->absnorm[j] = sqrt(aa);
    }
    free(y); free(ya); free(t); free(ta);
    return NULL;
}

/* For columns j < ncols of X (m x ncols, ld ldx) and B (ld ldb):
 * rnorm[j] = ||b_j - A x_j||_2 from a double-double evaluation of A x_j,
 * absnorm[j] = || |A||x_j| ||_2.  Columns are spread over nthreads threads.
 * Returns 0, or -1 on a bad argument or failed allocation. */
int orc_resid_dd(int m, DPlrMtx *A, int ncols, const double *X, int ldx, const double *B, int ldb,
                 double *rnorm, double *absnorm, int nthreads)
{
    if (m <= 0 || !A || A->size != m || ncols < 0 || ldx < m || ldb < m || nthreads < 1)
        return -1;
    job J;
    J.m = m; J.ncols = ncols; J.ldx = ldx; J.ldb = ldb; J.A = A; J.X = X; J.B = B;
    J.rnorm = rnorm; J.absnorm = absnorm; J.rmax = max_rank(A);
    atomic_init(&J.next, 0);
    atomic_init(&J.failed, 0);
    if (nthreads > ncols)
        nthreads = ncols > 0 ? ncols : 1;
    pthread_t *th = malloc(sizeof(pthread_t) * (size_t)nthreads);
    if (!th)
        return -1;
    int started = 0;
    for (int i = 0; i < nthreads; ++i) {
        if (pthread_create(&th[i], NULL, worker, &J) != 0)
            break;
        ++started;
    }
    if (started == 0)
        worker(&J);
    for (int i = 0; i < started; ++i)
        pthread_join(th[i], NULL);
    free(th);
    return atomic_load(&J.failed) ? -1 : 0;
}
