/*
 * dplr.h -- drop-in C interface of the GB300 DPLR library.
 *
 * The partitioned-low-rank (PLR, HODLR) matrix type and the public entry
 * points keep the layout and signatures of DPLR's own header, so code
 * written against DPLR compiles and links against libdplr_gb300.so
 * unchanged.  Reference: include/dplr.h:38-160 (prototypes) and
 * include/dplr_internal.h:32-115 (types, private helpers) of DPLR.
 *
 * Storage conventions (unchanged from DPLR):
 *   - all matrices are FP64, column-major, allocated with malloc;
 *   - an H node is a 2x2 block matrix: nw and se are H nodes or dense
 *     leaves, ne and sw are low-rank blocks U diag(sig) V^T;
 *   - a low-rank block of size n stores u and v as n x capacity arrays
 *     with leading dimension n, and sig[capacity]; only the first
 *     `rank` columns are live.  V is stored as V, not V^T;
 *   - ne maps x[m/2:m] to y[0:m/2]; sw maps x[0:m/2] to y[m/2:m].
 *
 * The apply, inverse, product and compression routines (dplrgepmv,
 * dplrgepdmm, dplrgeinv, dplrgeprk, dplrgeppmm, dplrreduce, dplrd2gep) run
 * on the GPU; the structural helpers run on the host.  GPU-specific
 * additions live in dplr_gb300.h.
 */
#ifndef DPLR_GB300_DPLR_H
#define DPLR_GB300_DPLR_H

#if defined(__GNUC__)
#define DPLR_API __attribute__((visibility("default")))
#else
#define DPLR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Node kind (DPLR include/dplr_internal.h:32-38). */
typedef enum
{
    PLR_UMTX = 0,   /* not yet populated */
    PLR_HMTX,       /* 2x2 hierarchical node */
    PLR_DMTX,       /* dense leaf */
    PLR_LRMTX       /* low-rank block */
} PlrMtxType;

typedef struct DPlrMtxStruct DPlrMtx;

/* 2x2 node: the four quadrants (dplr_internal.h:48-51). */
typedef struct
{
    DPlrMtx *nw, *ne, *se, *sw;
} DPlrHMtx;

/* Dense leaf: size x size, leading dimension size (dplr_internal.h:56-59). */
typedef struct
{
    double *d;
} DPlrDMtx;

/* Low-rank block U diag(sig) V^T (dplr_internal.h:64-70). */
typedef struct
{
    int rank;       /* live columns */
    int capacity;   /* allocated columns of u, v and entries of sig */
    double *u, *v;
    double *sig;
} DPlrLRMtx;

/* Generic node (dplr_internal.h:75-87). */
struct DPlrMtxStruct
{
    PlrMtxType type;
    int size;
    union
    {
        DPlrHMtx  dh;
        DPlrDMtx  dd;
        DPlrLRMtx dlr;
    };
};

/* ---- structure helpers (host) ------------------------------------- */

/* Make A an empty, untyped node.  Replaces dplrini, DPLR src/dplrini.c:18. */
DPLR_API void dplrini(DPlrMtx *A);

/* Free the buffers held by A and its subtree.  Replaces dplrclr,
 * src/dplrini.c:183 (like DPLR, child structs of H nodes are not freed). */
DPLR_API void dplrclr(DPlrMtx *A);

/* Dense m x m leaf, NaN-filled.  Replaces dplrinid, src/dplrini.c:35. */
DPLR_API void dplrinid(int m, DPlrMtx *A);

/* Low-rank block of size m and given capacity, NaN-filled, rank 0.
 * Replaces dplrinilr, src/dplrini.c:80. */
DPLR_API void dplrinilr(int m, DPlrMtx *A, int capacity);

/* H node of even size m with four untyped children.  Replaces dplrinih,
 * src/dplrini.c:142. */
DPLR_API void dplrinih(int m, DPlrMtx *A);

/* Grow the capacity of a low-rank block (at least doubling), keep the
 * live columns, NaN-fill the rest.  Replaces dplrresizelr,
 * src/dplrresizelr.c:15. */
DPLR_API void dplrresizelr(DPlrMtx *A, int capacity);

/* Empty copy of the structure of A into B.  Replaces dplrempty,
 * src/dplrempty.c:18. */
DPLR_API void dplrempty(DPlrMtx *A, DPlrMtx *B);

/* Maximum low-rank rank per level.  Replaces dplrrnk, src/dplrrnk.c:22. */
DPLR_API void dplrrnk(int m, DPlrMtx *A, int *ranks);

/* Stored entries (m*m per leaf, m*(r_ne+r_sw) per H node).  Replaces
 * dplrnz, src/dplrnz.c:17. */
DPLR_API long int dplrnz(int m, DPlrMtx *A);

/* Expand to a dense matrix B (ldb >= m).  Replaces dplrgep2d,
 * src/dplrp2d.c:98. */
DPLR_API void dplrgep2d(int m, DPlrMtx *A, double *B, int ldb);

/* B := A; B is rebuilt (dplrclr + dplrinid / dplrinih) where its type or
 * size differs, and low-rank capacities grow to A's ranks.  Replaces
 * dplrcpy, src/dplrcpy.c:19. */
DPLR_API void dplrcpy(int m, DPlrMtx *A, DPlrMtx *B);

/* A := alpha*A; low-rank blocks scale sig by |alpha| and negate u for
 * alpha < 0.  Replaces dplrscal, src/dplrscal.c:17. */
DPLR_API void dplrscal(int m, double *alpha, DPlrMtx *A);

/* B := alpha*A + B for PLR matrices of the same shape: leaves add, low-rank
 * blocks append A's columns (sig |alpha|, u negated for alpha < 0; capacity
 * grown as needed).  Replaces dplraxpy, src/dplraxpy.c:81. */
DPLR_API void dplraxpy(int m, double *alpha, DPlrMtx *A, DPlrMtx *B);

/* B := alpha*diag(D) + B (D: the m diagonal entries).  Replaces dplradpy,
 * src/dplraxpy.c:141. */
DPLR_API void dplradpy(int m, double *alpha, double *D, DPlrMtx *B);

/* ---- GPU hot path --------------------------------------------------- */

/* y := alpha*op(A)*x + beta*y.  Replaces dplrgepmv, src/dplrpmv.c:262. */
DPLR_API void dplrgepmv(char trans, int m, double *alpha, DPlrMtx *A,
               double *x, int incx, double *beta, double *y, int incy);

/* C := alpha*op(A)*op(B) + beta*C.  Replaces dplrgepdmm,
 * src/dplrpdmm.c:454. */
DPLR_API void dplrgepdmm(char transa, char transb, int m, int n, double *alpha,
                DPlrMtx *A, double *B, int ldb, double *beta,
                double *C, int ldc);

/* A += alpha * u diag(s) v^T on a PLR matrix.  Replaces dplrgeprk,
 * src/dplrprk.c:21. */
DPLR_API void dplrgeprk(int m, int k, double *alpha, double *u, int ldu,
               double *v, int ldv, double *s, int incs, DPlrMtx *A,
               double eps);

/* B := inv(A) by the recursive Woodbury formula.  Replaces dplrgeinv,
 * src/dplrinv.c:93. */
DPLR_API void dplrgeinv(int m, DPlrMtx *A, DPlrMtx *B, double eps, int *info);

/* C := alpha*op(A)*op(B) + beta*C for PLR matrices of one structure; the
 * low-rank blocks of C grow by the products' columns (normalised, zeroed
 * below eps/4 per level), nothing is recompressed.  Replaces dplrgeppmm,
 * src/dplrppmm.c:998. */
DPLR_API void dplrgeppmm(char transa, char transb, int m, double *alpha,
                DPlrMtx *A, DPlrMtx *B, double *beta, DPlrMtx *C,
                double eps);

/* Re-orthogonalise and truncate every low-rank block (eps/4 per level).
 * Replaces dplrreduce, src/dplrreduce.c:25, with the interface of the
 * Gram-Schmidt routine src/dortlr.f90:12 fixed (see dplr_gb300.h). */
DPLR_API void dplrreduce(int m, DPlrMtx *A, double eps);

/* Compress the dense m x m matrix A (lda >= m) into the PLR matrix B with
 * nlvl levels and absolute accuracy eps; each off-diagonal block is a
 * truncated SVD computed on the GPU (cuSOLVER gesvd), the threshold eps/2
 * on the last level and eps/4 above it.  B is rebuilt where its type or
 * size differs.  info = 0 on success, -1 on invalid arguments, the SVD's
 * info if it does not converge.  Replaces dplrd2gep, src/dplrd2p.c:186. */
DPLR_API void dplrd2gep(int m, double *A, int lda, DPlrMtx *B, double eps,
               int nlvl, int *info);

#ifdef __cplusplus
}
#endif

#endif /* DPLR_GB300_DPLR_H */
