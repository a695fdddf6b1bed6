// host_ops.cpp -- DPLR's structure-level arithmetic on host trees:
//   dplrcpy   src/dplrcpy.c:19      B := A (B rebuilt when its shape differs)
//   dplrscal  src/dplrscal.c:17     A := alpha A
//   dplraxpy  src/dplraxpy.c:81     B := alpha A + B (low-rank parts append)
//   dplradpy  src/dplraxpy.c:141    B := alpha diag(D) + B
// They complete the drop-in interface (the plan mirrors of dplrscal and
// dplradpy, which keep a matrix on the device, are in ops.cu).  Argument
// checks, messages and the early returns on error are DPLR's, so a caller
// sees the same behaviour: invalid input leaves the outputs untouched.
// Low-rank blocks keep DPLR's sign convention: sig >= 0, a negative scale
// negates the u vectors.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/dplr.h"

namespace dg {
void recompress_after(int m, DPlrMtx *A);
}

extern "C" {

void dplrscal(int m, double *alpha, DPlrMtx *A)
{
    if (m < 0) {
        fprintf(stderr, "dplrscal: invalid matrix size\n");
        return;
    }
    if (A->size != m) {
        fprintf(stderr, "dplrscal: invalid A size %d\n", m);
        return;
    }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) {
        fprintf(stderr, "dplrscal: invalid A type\n");
        return;
    }
    const double a = *alpha;
    if (A->type == PLR_DMTX) {
        const size_t n = (size_t)m * m;
        for (size_t i = 0; i < n; ++i) A->dd.d[i] *= a;
        return;
    }
    // the ne and sw blocks: sig by |alpha|, and for alpha < 0 the u vectors
    // change sign (their m/2 x rank live columns)
    DPlrMtx *blk[2] = {A->dh.ne, A->dh.sw};
    for (DPlrMtx *L : blk) {
        const int r = L->dlr.rank;
        for (int k = 0; k < r; ++k) L->dlr.sig[k] *= std::fabs(a);
        if (a < 0.0) {
            const size_t n = (size_t)r * (m / 2);
            for (size_t i = 0; i < n; ++i) L->dlr.u[i] = -L->dlr.u[i];
        }
    }
    dplrscal(m / 2, alpha, A->dh.nw);
    dplrscal(m / 2, alpha, A->dh.se);
}

void dplrcpy(int m, DPlrMtx *A, DPlrMtx *B)
{
    if (m < 0) {
        fprintf(stderr, "dplrcpy: invalid matrix size %d\n", m);
        return;
    }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) {
        fprintf(stderr, "dplrcpy: invalid A type\n");
        return;
    }
    if (A->size != m) {
        fprintf(stderr, "dplrcpy: invalid A size\n");
        return;
    }
    if (A->type == PLR_DMTX) {
        if (B->type != PLR_DMTX || B->size != m) {
            dplrclr(B);
            dplrinid(m, B);
        }
        memcpy(B->dd.d, A->dd.d, (size_t)m * m * sizeof(double));
        return;
    }
    if (B->type != PLR_HMTX || B->size != m) {
        // fresh H node with empty low-rank blocks; the diagonal children are
        // shaped by the recursive calls
        dplrclr(B);
        dplrinih(m, B);
        dplrinilr(m / 2, B->dh.ne, 0);
        dplrinilr(m / 2, B->dh.sw, 0);
    }
    DPlrMtx *src[2] = {A->dh.ne, A->dh.sw}, *dst[2] = {B->dh.ne, B->dh.sw};
    for (int s = 0; s < 2; ++s) {
        const int r = src[s]->dlr.rank;
        if (dst[s]->dlr.capacity < r) dplrresizelr(dst[s], r);
        const size_t n = (size_t)r * (m / 2);
        memcpy(dst[s]->dlr.sig, src[s]->dlr.sig, (size_t)r * sizeof(double));
        memcpy(dst[s]->dlr.u, src[s]->dlr.u, n * sizeof(double));
        memcpy(dst[s]->dlr.v, src[s]->dlr.v, n * sizeof(double));
        dst[s]->dlr.rank = r;
    }
    dplrcpy(m / 2, A->dh.nw, B->dh.nw);
    dplrcpy(m / 2, A->dh.se, B->dh.se);
}

// B's low-rank block gains A's columns: u and v copied after B's live
// columns, sig scaled by |alpha|, u negated for alpha < 0.
static void lr_axpy(int m, double alpha, DPlrMtx *A, DPlrMtx *B)
{
    if (m < 0) {
        fprintf(stderr, "dplrlraxpy: invalid matrix size %d\n", m);
        return;
    }
    if (A->type != PLR_LRMTX || B->type != PLR_LRMTX) {
        fprintf(stderr, "dplrlraxpy: invalid matrix type\n");
        return;
    }
    if (A->size != m || B->size != m) {
        fprintf(stderr, "dplrlraxpy: invalid A or B size\n");
        return;
    }
    const int ra = A->dlr.rank, rb = B->dlr.rank;
    if (ra == 0) return;
    if (B->dlr.capacity < ra + rb) dplrresizelr(B, ra + rb);
    const size_t n = (size_t)m * ra, off = (size_t)rb * m;
    memcpy(B->dlr.u + off, A->dlr.u, n * sizeof(double));
    memcpy(B->dlr.v + off, A->dlr.v, n * sizeof(double));
    for (int k = 0; k < ra; ++k) B->dlr.sig[rb + k] = std::fabs(alpha) * A->dlr.sig[k];
    if (alpha < 0.0)
        for (size_t i = 0; i < n; ++i) B->dlr.u[off + i] = -B->dlr.u[off + i];
    B->dlr.rank = ra + rb;
}

static int axpy_tree(int m, double *alpha, DPlrMtx *A, DPlrMtx *B);

void dplraxpy(int m, double *alpha, DPlrMtx *A, DPlrMtx *B)
{
    // recompress only a B that was added to, and only when
    // dplr_gpu_set_recompress asked for it
    if (axpy_tree(m, alpha, A, B) == 0 && *alpha != 0.0) dg::recompress_after(m, B);
}

static int axpy_tree(int m, double *alpha, DPlrMtx *A, DPlrMtx *B)
{
    if (m < 0) {
        fprintf(stderr, "dplraxpy: invalid matrix size %d\n", m);
        return -1;
    }
    if (A->size != m || B->size != m) {
        fprintf(stderr, "dplraxpy: invalid A or B size\n");
        return -1;
    }
    if (A->type != B->type) {
        fprintf(stderr, "dplraxpy: A and B types do not match\n");
        return -1;
    }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) {
        fprintf(stderr, "dplraxpy: invalid A or B type\n");
        return -1;
    }
    const double a = *alpha;
    if (a == 0.0) return 0;
    if (A->type == PLR_DMTX) {
        const size_t n = (size_t)m * m;
        for (size_t i = 0; i < n; ++i) B->dd.d[i] += a * A->dd.d[i];
        return 0;
    }
    lr_axpy(m / 2, a, A->dh.ne, B->dh.ne);
    lr_axpy(m / 2, a, A->dh.sw, B->dh.sw);
    axpy_tree(m / 2, alpha, A->dh.nw, B->dh.nw);
    axpy_tree(m / 2, alpha, A->dh.se, B->dh.se);
    return 0;
}

void dplradpy(int m, double *alpha, double *D, DPlrMtx *B)
{
    if (m < 0) {
        fprintf(stderr, "dplradpy: invalid matrix size %d\n", m);
        return;
    }
    if (B->type != PLR_DMTX && B->type != PLR_HMTX) {
        fprintf(stderr, "dplradpy: invalid B type\n");
        return;
    }
    if (B->size != m) {
        fprintf(stderr, "dplradpy: invalid B size\n");
        return;
    }
    if (B->type == PLR_DMTX) {
        for (int i = 0; i < m; ++i) B->dd.d[(size_t)i * m + i] += *alpha * D[i];
        return;
    }
    dplradpy(m / 2, alpha, D, B->dh.nw);
    dplradpy(m / 2, alpha, D + m / 2, B->dh.se);
}

}  // extern "C"
