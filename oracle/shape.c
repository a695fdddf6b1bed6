/*
 * shape.c -- a stand-in tree with the structure of DPLR's explicit inverse
 * (TEST INFRASTRUCTURE ONLY: used by the benchmark's CPU legs to time the
 * reference's apply of inv(A) where forming inv(A) with dplrgeinv does not
 * finish in the time allowed; never part of the product).
 *
 * dplrgeinv (src/dplrinv.c:93) keeps A's tree.  At an H node with
 * off-diagonal ranks r1 (ne) and r2 (sw) it appends a rank-r2 correction to
 * every low-rank block of the nw subtree and a rank-r1 correction to every
 * block of the se subtree (dplrgeprk, src/dplrinv.c:428-429,
 * src/dplrprk.c:105-191), and nothing is recompressed.  So a block of the
 * inverse has its own rank plus the ranks of all corrections its ancestors
 * pushed to its side; its capacity is taken equal to that rank.  Leaves keep
 * their size.  The values are a constant: the time of a BLAS product does
 * not depend on them.
 */
#include <stdlib.h>

#include "../include/dplr.h"

static double *filled(size_t count, double v)
{
    double *p = malloc(sizeof(double) * (count ? count : 1));
    if (p)
        for (size_t i = 0; i < count; ++i)
            p[i] = v;
    return p;
}

static int build(int m, const DPlrMtx *A, DPlrMtx *B, int extra, double fill);

static int lowrank(int n, int rank, DPlrMtx *B, double fill)
{
    B->type = PLR_LRMTX;
    B->size = n;
    B->dlr.rank = rank;
    B->dlr.capacity = rank;
    B->dlr.u = filled((size_t)n * rank, fill);
    B->dlr.v = filled((size_t)n * rank, fill);
    B->dlr.sig = filled((size_t)rank, 1.0);
    return (B->dlr.u && B->dlr.v && B->dlr.sig) ? 0 : -1;
}

/* `extra`: ranks of the corrections the ancestors pushed into this subtree;
 * both off-diagonal blocks of every node below receive all of them. */
static int build(int m, const DPlrMtx *A, DPlrMtx *B, int extra, double fill)
{
    if (A->type == PLR_DMTX) {
        B->type = PLR_DMTX;
        B->size = m;
        B->dd.d = filled((size_t)m * m, fill);
        return B->dd.d ? 0 : -1;
    }
    if (A->type != PLR_HMTX)
        return -1;
    int h = m / 2;
    int r1 = A->dh.ne->dlr.rank, r2 = A->dh.sw->dlr.rank;
    B->type = PLR_HMTX;
    B->size = m;
    DPlrMtx **kids[4] = {&B->dh.nw, &B->dh.ne, &B->dh.se, &B->dh.sw};
    for (int i = 0; i < 4; ++i) {
        *kids[i] = calloc(1, sizeof(DPlrMtx));
        if (!*kids[i])
            return -1;
    }
    if (lowrank(h, r1 + extra, B->dh.ne, fill) || lowrank(h, r2 + extra, B->dh.sw, fill))
        return -1;
    if (build(h, A->dh.nw, B->dh.nw, extra + r2, fill))
        return -1;
    return build(m - h, A->dh.se, B->dh.se, extra + r1, fill);
}

/* B (an empty, dplrini'd node) := a tree shaped like DPLR's inv(A), every
 * entry `fill` (sig = 1).  Allocated with malloc like the reference's trees.
 * Returns 0, or -1 on a malformed A or a failed allocation (B may then be
 * partly built; free it as any tree). */
int orc_inverse_shape(int m, const DPlrMtx *A, DPlrMtx *B, double fill)
{
    if (!A || !B || A->size != m)
        return -1;
    return build(m, A, B, 0, fill);
}
