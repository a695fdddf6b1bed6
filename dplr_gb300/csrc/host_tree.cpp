// host_tree.cpp -- host-side structure helpers of the DPLR interface.
//
// These keep DPLR's semantics exactly (NaN-filled fresh buffers, at least
// doubling growth, buffers-only clearing) because the GPU inverse builds
// its output tree with them and callers rely on them:
//   dplrini      src/dplrini.c:18     dplrinid   src/dplrini.c:35
//   dplrinilr    src/dplrini.c:80     dplrinih   src/dplrini.c:142
//   dplrclr      src/dplrini.c:183    dplrresizelr src/dplrresizelr.c:15
//   dplrempty    src/dplrempty.c:18   dplrrnk    src/dplrrnk.c:22
//   dplrnz       src/dplrnz.c:17      dplrgep2d  src/dplrp2d.c:98
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/dplr.h"

static double *nan_block(size_t count)
{
    double *p = (double *)malloc(count * sizeof(double));
    if (!p) return nullptr;
    const double q = std::nan("");
    for (size_t i = 0; i < count; ++i) p[i] = q;
    return p;
}

extern "C" {

void dplrini(DPlrMtx *A)
{
    memset(A, 0, sizeof(*A));
    A->type = PLR_UMTX;
}

void dplrinid(int m, DPlrMtx *A)
{
    if (m < 0) {
        fprintf(stderr, "dplrinid: invalid matrix size\n");
        return;
    }
    A->type = PLR_DMTX;
    A->size = m;
    A->dd.d = nullptr;
    if (m > 0) {
        A->dd.d = nan_block((size_t)m * m);
        if (!A->dd.d) fprintf(stderr, "dplrinid: memory allocation failed\n");
    }
}

void dplrinilr(int m, DPlrMtx *A, int capacity)
{
    if (m < 0 || capacity < 0) {
        fprintf(stderr, "dplrinilr: invalid size or capacity\n");
        return;
    }
    A->type = PLR_LRMTX;
    A->size = m;
    A->dlr.rank = 0;
    A->dlr.capacity = capacity;
    A->dlr.u = A->dlr.v = A->dlr.sig = nullptr;
    if (capacity > 0) {
        A->dlr.u = nan_block((size_t)m * capacity);
        A->dlr.sig = nan_block((size_t)capacity);
        A->dlr.v = nan_block((size_t)m * capacity);
        if (!A->dlr.u || !A->dlr.v || !A->dlr.sig)
            fprintf(stderr, "dplrinilr: memory allocation failed\n");
    }
}

void dplrinih(int m, DPlrMtx *A)
{
    if (m < 0) {
        fprintf(stderr, "dplrinih: invalid size\n");
        return;
    }
    if (m % 2 != 0) {
        fprintf(stderr, "dplrinih: m must be even\n");
        return;
    }
    A->type = PLR_HMTX;
    A->size = m;
    DPlrMtx **kids[4] = {&A->dh.nw, &A->dh.ne, &A->dh.se, &A->dh.sw};
    for (DPlrMtx **k : kids) {
        *k = (DPlrMtx *)malloc(sizeof(DPlrMtx));
        if (!*k) {
            fprintf(stderr, "dplrinih: memory allocation failed\n");
            return;
        }
        dplrini(*k);
    }
}

void dplrclr(DPlrMtx *A)
{
    switch (A->type) {
    case PLR_DMTX:
        free(A->dd.d);
        break;
    case PLR_LRMTX:
        free(A->dlr.u);
        free(A->dlr.v);
        free(A->dlr.sig);
        break;
    case PLR_HMTX:
        dplrclr(A->dh.nw);
        dplrclr(A->dh.se);
        dplrclr(A->dh.ne);
        dplrclr(A->dh.sw);
        break;
    default:
        break;
    }
}

void dplrresizelr(DPlrMtx *A, int capacity)
{
    if (A->type != PLR_LRMTX) {
        fprintf(stderr, "dplrresizelr: invalid matrix type\n");
        return;
    }
    if (A->size < 0) {
        fprintf(stderr, "dplrresizelr: invalid matrix size\n");
        return;
    }
    if (capacity < 0) {
        fprintf(stderr, "dplrresizelr: invalid capacity\n");
        return;
    }
    if (capacity < A->dlr.capacity) return;
    const int grown = capacity > 2 * A->dlr.capacity ? capacity : 2 * A->dlr.capacity;
    const size_t n = (size_t)A->size;
    double *u = nan_block(n * grown), *v = nan_block(n * grown), *s = nan_block(grown);
    if (!u || !v || !s) {
        fprintf(stderr, "dplrresizelr: memory allocation failed\n");
        free(u);
        free(v);
        free(s);
        return;
    }
    if (A->dlr.rank > 0) {
        memcpy(s, A->dlr.sig, sizeof(double) * A->dlr.rank);
        memcpy(u, A->dlr.u, sizeof(double) * n * A->dlr.rank);
        memcpy(v, A->dlr.v, sizeof(double) * n * A->dlr.rank);
    }
    if (A->dlr.capacity > 0) {
        free(A->dlr.u);
        free(A->dlr.v);
        free(A->dlr.sig);
    }
    A->dlr.capacity = grown;
    A->dlr.u = u;
    A->dlr.v = v;
    A->dlr.sig = s;
}

void dplrempty(DPlrMtx *A, DPlrMtx *B)
{
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) {
        fprintf(stderr, "dplrempty: A must be a dense or hierarchical matrix\n");
        return;
    }
    dplrclr(B);
    if (A->type == PLR_DMTX) {
        dplrinid(A->size, B);
        return;
    }
    dplrinih(A->size, B);
    dplrinilr(A->size / 2, B->dh.ne, 0);
    dplrinilr(A->size / 2, B->dh.sw, 0);
    dplrempty(A->dh.nw, B->dh.nw);
    dplrempty(A->dh.se, B->dh.se);
}

void dplrrnk(int m, DPlrMtx *A, int *ranks)
{
    if (m < 0) {
        fprintf(stderr, "dplrrnk: invalid matrix size %d\n", m);
        return;
    }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) {
        fprintf(stderr, "dplrrnk: invalid A type\n");
        return;
    }
    if (A->size != m) {
        fprintf(stderr, "dplrrnk: invalid A size\n");
        return;
    }
    if (A->type != PLR_HMTX) return;
    const int r = A->dh.ne->dlr.rank > A->dh.sw->dlr.rank ? A->dh.ne->dlr.rank : A->dh.sw->dlr.rank;
    if (*ranks < r) *ranks = r;
    if (A->dh.nw->type != PLR_DMTX && A->dh.se->type != PLR_DMTX) {
        dplrrnk(m / 2, A->dh.nw, ranks + 1);
        dplrrnk(m / 2, A->dh.se, ranks + 1);
    }
}

long int dplrnz(int m, DPlrMtx *A)
{
    if (m < 0) {
        fprintf(stderr, "dplrnz: invalid matrix size %d\n", m);
        return -1;
    }
    if (A->size != m) {
        fprintf(stderr, "dplrnz: invalid A size\n");
        return -1;
    }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) {
        fprintf(stderr, "dplrnz: invalid A type\n");
        return -1;
    }
    if (A->type == PLR_DMTX) return (long)m * m;
    long nz = (long)m * (A->dh.ne->dlr.rank + A->dh.sw->dlr.rank);
    return nz + dplrnz(m / 2, A->dh.nw) + dplrnz(m / 2, A->dh.se);
}

static void lr_expand(int m, const DPlrMtx *L, double *B, int ldb)
{
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) {
            double s = 0.0;
            for (int k = 0; k < L->dlr.rank; ++k)
                s += L->dlr.u[(size_t)k * m + i] * L->dlr.sig[k] * L->dlr.v[(size_t)k * m + j];
            B[(size_t)j * ldb + i] = s;
        }
}

void dplrgep2d(int m, DPlrMtx *A, double *B, int ldb)
{
    if (m < 0 || A->size != m || ldb < m || (A->type != PLR_DMTX && A->type != PLR_HMTX)) {
        fprintf(stderr, "dplrgep2d: invalid arguments\n");
        return;
    }
    if (A->type == PLR_DMTX) {
        for (int j = 0; j < m; ++j) memcpy(B + (size_t)j * ldb, A->dd.d + (size_t)j * m, sizeof(double) * m);
        return;
    }
    const int h = m / 2;
    lr_expand(h, A->dh.ne, B + (size_t)ldb * h, ldb);
    lr_expand(h, A->dh.sw, B + h, ldb);
    dplrgep2d(h, A->dh.nw, B, ldb);
    dplrgep2d(h, A->dh.se, B + (size_t)ldb * h + h, ldb);
}

}  // extern "C"
