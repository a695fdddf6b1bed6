/*
 * dplr_gb300.h -- GPU additions to the DPLR interface (libdplr_gb300.so).
 *
 * None of these exist in DPLR; the drop-in entry points of dplr.h are
 * built on them.  All pointers are plain C pointers; `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream); device
 * arrays are column-major FP64 with a leading dimension.
 *
 * A plan is a device-resident copy of one PLR matrix: a block table
 * (one descriptor per low-rank block and per dense leaf) plus one
 * contiguous factor pool in HBM.  Building a plan uploads the tree once;
 * every later apply or solve through the plan reads only device memory.
 * The drop-in dplrgepmv/dplrgepdmm upload the tree on every call unless
 * it was registered with dplr_gpu_register(), in which case they reuse
 * the registered plan (call dplr_gpu_register() again after modifying the
 * tree on the host).
 *
 * Every function returns 0 on success and a negative DPLR_GPU_E* code on
 * failure; dplr_gpu_last_error() describes the last failure of the
 * calling thread.  A plan must not be used by two threads at once;
 * distinct plans are independent.
 */
#ifndef DPLR_GB300_EXT_H
#define DPLR_GB300_EXT_H

#include "dplr.h"

#ifdef __cplusplus
extern "C" {
#endif

#define DPLR_GPU_OK          0
#define DPLR_GPU_EINVAL     -1   /* bad argument (size, type, stride ...) */
#define DPLR_GPU_ECUDA      -2   /* CUDA runtime error */
#define DPLR_GPU_ENOMEM     -3   /* device or host allocation failed */
#define DPLR_GPU_ESINGULAR  -4   /* zero pivot in a leaf or capacitance LU */
#define DPLR_GPU_ENOTCONV   -5   /* refinement did not reach the tolerance */
#define DPLR_GPU_ESTATE     -6   /* plan not factored / wrong state */

typedef struct dplr_gpu_plan_s *dplr_gpu_plan;
typedef struct dplr_gpu_graph_s *dplr_gpu_graph;

/* Thread-local description of the last failure ("" if none). */
DPLR_API const char *dplr_gpu_last_error(void);

/* Build a plan from an m x m host tree (upload of all factors). */
DPLR_API int dplr_gpu_plan_create(int m, const DPlrMtx *A, void *stream, dplr_gpu_plan *plan);
DPLR_API void dplr_gpu_plan_destroy(dplr_gpu_plan plan);
/* Re-upload factor values from the host tree (same structure and ranks). */
DPLR_API int dplr_gpu_plan_refresh(dplr_gpu_plan plan, const DPlrMtx *A, void *stream);
/* Size and stored entries (dplrnz) of the planned matrix. */
DPLR_API int dplr_gpu_plan_info(dplr_gpu_plan plan, int *m, long long *nnz, int *levels,
                       int *max_rank);
/* Device bytes held by the plan (factors, tables, factorisation, scratch). */
DPLR_API long long dplr_gpu_plan_device_bytes(dplr_gpu_plan plan);

/* Y := alpha*op(A)*X + beta*Y on device arrays (X: m x n, ldx >= m;
 * Y: m x n, ldy >= m).  beta == 0 does not read Y. */
DPLR_API int dplr_gpu_apply(dplr_gpu_plan plan, char trans, int n, double alpha, const double *X,
                   int ldx, double beta, double *Y, int ldy, void *stream);

/* FP64-accurate single-right-hand-side apply on the FP32 pipes.  Keeps a
 * second copy of the factors as float pairs (hi + lo: the leading 48 bits of
 * each double, 8 bytes per element); afterwards every op-N apply with one
 * right-hand side (dplr_gpu_apply, the drop-in dplrgepmv on a registered
 * plan) evaluates the products with error-free FP32 transformations and
 * compensated sums (relative error ~1e-14 of |A||x|), streaming the factors
 * at HBM speed instead of FP64-FMA speed.  Other applies keep the FP64
 * kernels.  The copy follows dplr_gpu_plan_refresh and dplr_gpu_pool_write
 * and is freed with the plan.  DPLR_GPU_EINVAL if the largest factor entry
 * is outside 2^+-50 (FP32 range). */
DPLR_API int dplr_gpu_prepare_pairs(dplr_gpu_plan plan, void *stream);

/* Device-resident structure arithmetic on a plan (no host round trip):
 * A := alpha*A (dplrscal's convention: sig scaled by |alpha|, u negated for
 * alpha < 0) and A := alpha*diag(D) + A with D on the device (m entries,
 * dplradpy).  The factorisation and sliced copies are dropped (rebuild them
 * as after dplr_gpu_pool_write); a float-pair copy is rebuilt. */
DPLR_API int dplr_gpu_scal(dplr_gpu_plan plan, double alpha, void *stream);
DPLR_API int dplr_gpu_adpy(dplr_gpu_plan plan, double alpha, const double *D, void *stream);

/* Structure arithmetic between device-resident plans (no host trees):
 * dplr_gpu_plan_copy makes *out a new plan equal to `plan` (DPLR's dplrcpy,
 * src/dplrcpy.c:19); dplr_gpu_axpy makes *out a new plan C = alpha A + B for
 * plans of one structure, with DPLR's dplraxpy layout (src/dplraxpy.c:17-138:
 * every low-rank block holds B's columns then A's, A's sig scaled by
 * |alpha| and its u negated for alpha < 0, rank r_A + r_B; leaves B +
 * alpha A; alpha == 0 gives a copy of B); dplr_gpu_gep2d writes the dense
 * m x m matrix into the device array D (ld ldd, DPLR's dplrgep2d,
 * src/dplrp2d.c:98; zero outside the trees of a batch).  New plans are not
 * factored and hold no sliced copies. */
DPLR_API int dplr_gpu_plan_copy(dplr_gpu_plan plan, void *stream, dplr_gpu_plan *out);
DPLR_API int dplr_gpu_axpy(double alpha, dplr_gpu_plan A, dplr_gpu_plan B, void *stream, dplr_gpu_plan *out);
DPLR_API int dplr_gpu_gep2d(dplr_gpu_plan plan, double *D, long long ldd, void *stream);
/* SVD recompression of a device plan (dplr_gpu_reduce_svd without host
 * trees): *out is a new plan in which every low-rank block is its truncated
 * SVD with the singular values >= eps / 4^(depth+1) (dplrreduce's split,
 * src/dplrreduce.c:46); leaves are copied.  Ranks only shrink.  workers as
 * for dplr_gpu_reduce_svd.  DPLR_GPU_ENOTCONV (with *out valid) if an SVD
 * did not converge; that block is kept. */
DPLR_API int dplr_gpu_plan_reduce_svd(dplr_gpu_plan plan, double eps, int workers, void *stream,
                                      dplr_gpu_plan *out);

/* Recompression after the operations that grow ranks, off by default (DPLR
 * never recompresses, quirk Q2).  With eps >= 0, dplraxpy, dplrgeprk,
 * dplrgeinv, dplrgeppmm / dplr_gpu_geppmm run dplr_gpu_reduce_svd(m, out,
 * eps) on their output tree, and dplr_gpu_axpy returns its plan
 * recompressed by dplr_gpu_plan_reduce_svd with eps.  eps < 0 turns it off.
 * Process-wide. */
DPLR_API void dplr_gpu_set_recompress(double eps);

/* Woodbury factorisation of the planned matrix (replaces forming inv(A)
 * with DPLR's dplrgeinv, src/dplrinv.c:93, when the goal is solving):
 * leaf inverses, per-level panels Z = D^-1 W and capacitance inverses
 * (I + S V~^T Z)^-1, all FP64.  Transposed solves reuse these factors
 * (A^-T = D^-T (I - V~ S K^-T Z^T), swept top-down).
 * DPLR_GPU_FACTOR_TRANSPOSED also builds the panels D^-T V~, which only
 * the explicit inverse (dplrgeinv on the device) needs. */
#define DPLR_GPU_FACTOR_TRANSPOSED 1
DPLR_API int dplr_gpu_factor(dplr_gpu_plan plan, int flags, void *stream);
DPLR_API long long dplr_gpu_factor_device_bytes(dplr_gpu_plan plan);

/* X := op(A)^-1 B (device arrays, m x n); B and X must not alias. */
DPLR_API int dplr_gpu_solve(dplr_gpu_plan plan, char trans, int n, const double *B, int ldb,
                            double *X, int ldx, void *stream);

/* Exact-slice copies of the factors for the precise residual: every
 * factor cut into 8 bf16 slices of 7 bits with a power-of-two scale per row
 * or column, so that products run on the tensor cores with exact integer
 * accumulation.  Needs leaf sizes that are multiples of 64. */
DPLR_API int dplr_gpu_prepare_sliced(dplr_gpu_plan plan, void *stream);

/* R := B - A X (device arrays).  flags: DPLR_GPU_RESIDUAL_SLICED computes
 * the products from the exact slices (needs dplr_gpu_prepare_sliced) and
 * sums in double-double, which is more accurate than the FP64 apply; 0
 * uses the FP64 apply. */
#define DPLR_GPU_RESIDUAL_SLICED 1
#define DPLR_GPU_SOLVE_MIXED 2
DPLR_API int dplr_gpu_residual(dplr_gpu_plan plan, int n, const double *X, int ldx, const double *B,
                               int ldb, double *R, int ldr, int flags, void *stream);

/* Low-precision inner solver for refinement: the Woodbury sweep with V,
 * the D^-1 W panels and the leaf inverses cut into `slices` bf16 slices
 * (3 to 7: 22 to 50 bits) on the tensor cores.  The capacitance inverses
 * are formed and stored in FP64; nodes whose two blocks have rank 128 (with
 * 128-row tiles) apply them on the tensor cores from 8 exact slices (57-bit
 * operands, exact products, one rounding: at least FP64 accuracy), the
 * others with FP64 arithmetic.  More slices cost more tensor-core work per
 * solve but keep the refinement convergent on worse-conditioned
 * factorisations.  Needs dplr_gpu_factor first and leaf sizes that are
 * multiples of 64. */
DPLR_API int dplr_gpu_prepare_mixed(dplr_gpu_plan plan, int slices, void *stream);
/* Same, with fp64_capacitance != 0 applying every capacitance inverse with
 * FP64 arithmetic. */
DPLR_API int dplr_gpu_prepare_mixed_caps(dplr_gpu_plan plan, int slices, int fp64_capacitance, void *stream);

/* X := A^-1 B refined until max_j ||B_j - A X_j|| / ||B_j|| <= tol; at
 * most maxiter corrections.  For a batch plan (dplr_gpu_batch_create) the
 * maximum runs over every column of every tree, each with its own rows'
 * norms, so that every matrix of the batch meets tol.  flags: DPLR_GPU_RESIDUAL_SLICED selects the
 * exact-slice residual (as for dplr_gpu_residual); DPLR_GPU_SOLVE_MIXED
 * makes every inner solve the low-precision sweep (needs
 * dplr_gpu_prepare_mixed) instead of the FP64 sweep.  Reports the final relative residual and the number of
 * corrections; returns DPLR_GPU_ENOTCONV if the tolerance was not reached. */
DPLR_API int dplr_gpu_solve_refined(dplr_gpu_plan plan, int n, const double *B, int ldb,
                                    double *X, int ldx, double tol, int maxiter, int flags,
                                    double *rel_resid, int *iters, void *stream);

/* The same refined solve with B and X in host memory (column-major,
 * leading dimensions ldb, ldx >= m): B is copied to the device, solved and
 * X copied back inside the call (pinned host memory makes the copies
 * asynchronous DMA).  Each iterate of X starts back to the host while the
 * refinement checks it, so the last copy overlaps the last residual; X
 * holds the last iterate when the call returns (also on
 * DPLR_GPU_ENOTCONV; after another error it may hold an earlier one). */
DPLR_API int dplr_gpu_solve_refined_host(dplr_gpu_plan plan, int n, const double *B, int ldb,
                                         double *X, int ldx, double tol, int maxiter, int flags,
                                         double *rel_resid, int *iters, void *stream);

/* Y := alpha*op(A)*X + beta*Y like dplr_gpu_apply, but without allocating
 * any device memory.  No counterpart in DPLR (whose routines malloc per
 * block visit).  For callers that cannot allocate when they apply:
 * latency-critical paths that must avoid cudaMalloc/cudaFree and their
 * implicit synchronisation, and hosts that fix the library's device memory
 * in advance.  Scratch is a static 64 MiB
 * device array shared by all calls on a device: calls that may overlap on
 * the GPU race and must be ordered by the caller; a call needing more
 * scratch than that, (sum of ranks + partial panels) * n doubles, fails
 * with DPLR_GPU_EINVAL.  The first call on a device resolves the array's
 * address (cudaGetSymbolAddress).  That address is kept
 * for the life of the process: it assumes one CUDA context per device (the
 * primary context, not reset with cudaDeviceReset in between).  The array's
 * contents are never read before a call writes them, and its 64 MiB are
 * reserved on every device where the library's module is loaded, whether or
 * not this entry point is called. */
DPLR_API int dplr_gpu_apply_noalloc(dplr_gpu_plan plan, char trans, int n, double alpha,
                                    const double *X, int ldx, double beta, double *Y, int ldy,
                                    void *stream);

/* Factor pool.  A plan holds every factor in one device FP64 array of
 * dplr_gpu_pool_size() doubles.  Its blocks are numbered 0 .. nlowrank-1
 * for the low-rank blocks (pre-order over the tree, ne before sw) and
 * nlowrank .. nlowrank+nleaves-1 for the dense leaves (left to right);
 * dplr_gpu_pool_block() gives a block's offsets in the pool (U, V: n x rank
 * column-major, ld n; sig: rank; a leaf's b x b matrix at *u, ld b, with
 * *v = *sig = -1), its size, rank and the rows it writes (row0) and reads
 * (col0) in the op-N product.  No counterpart in DPLR, whose factors live
 * in the host tree. */
DPLR_API long long dplr_gpu_pool_size(dplr_gpu_plan plan);
DPLR_API int dplr_gpu_pool_blocks(dplr_gpu_plan plan, int *nlowrank, int *nleaves);
DPLR_API int dplr_gpu_pool_block(dplr_gpu_plan plan, int i, long long *u, long long *v, long long *sig,
                                 int *n, int *rank, int *row0, int *col0);
/* Device-to-device copies of the pool.  Writing replaces the factor values
 * (same structure) and drops the factorisation and sliced copies built from
 * the old values. */
DPLR_API int dplr_gpu_pool_read(dplr_gpu_plan plan, double *dst, void *stream);
DPLR_API int dplr_gpu_pool_write(dplr_gpu_plan plan, const double *src, void *stream);

/* Adjoint of the product with respect to the factors: G (device, pool
 * layout) += alpha * d<DY, A X>/d(factors), i.e. per low-rank block
 * dU = DY_R (sig o V^T X_C)^T, dV = X_C (sig o U^T DY_R)^T,
 * dsig = rowsum((U^T DY_R) o (V^T X_C)), per leaf dD = DY_R X_R^T (R, C: the
 * block's row and column ranges).  With X = A^-1 B and DY = A^-T G_X,
 * alpha = -1 gives the factor gradient of a solve.  X, DY: m x n device
 * arrays.  No counterpart in DPLR. */
DPLR_API int dplr_gpu_grad_factors(dplr_gpu_plan plan, int n, const double *X, int ldx, const double *DY,
                                   int ldy, double alpha, double *G, void *stream);

/* Batch of independent matrices as one plan: matrix i (size m[i], any
 * depth and ranks) is the diagonal block of rows [off_i, off_i + m[i]) of
 * one block-diagonal matrix, off_i = m[0] + ... + m[i-1]
 * (dplr_gpu_batch_offsets).  Every plan function (apply, factor, solve,
 * refined solve, gradients, pool access) then treats all matrices in the
 * same kernel launches.  Right-hand sides are stacked the same way; a
 * matrix with fewer right-hand sides than n leaves the extra columns
 * unused.  No counterpart in DPLR, which handles one matrix per call.
 * dplr_gpu_plan_refresh does not apply to batches (use dplr_gpu_pool_write). */
DPLR_API int dplr_gpu_batch_create(int count, const int *m, DPlrMtx *const *A, void *stream,
                                   dplr_gpu_plan *plan);
DPLR_API int dplr_gpu_batch_offsets(dplr_gpu_plan plan, int *count, int *row0);

/* CUDA graph of one apply (op 'A': Y = op(A) X), one solve (op 'S':
 * Y = op(A)^-1 X, needs dplr_gpu_factor) or one solve refined by two
 * correction steps (op 'R', trans 'N': Y = A^-1 X, twice R = X - A Y with the
 * exact-slice products if dplr_gpu_prepare_sliced was called, else the FP64
 * apply, Y += A^-1 R; op 'C': the same with one correction step; no host
 * synchronisation inside, so the whole refined solve is one replay;
 * dplr_gpu_residual checks the result) with fixed
 * device arrays: built
 * once (one ordinary run sizes the scratch, a second run is captured on an
 * internal stream), then replayed by dplr_gpu_graph_launch on any stream
 * with one launch call.  Valid while the plan, its factorisation and the
 * arrays live; rebuild it after dplr_gpu_factor or dplr_gpu_autotune. */
DPLR_API int dplr_gpu_graph_create(dplr_gpu_plan plan, char op, char trans, int n, const double *X,
                                   int ldx, double *Y, int ldy, void *stream, dplr_gpu_graph *graph);
DPLR_API int dplr_gpu_graph_launch(dplr_gpu_graph graph, void *stream);
DPLR_API long long dplr_gpu_graph_kernels(dplr_gpu_graph graph);
DPLR_API void dplr_gpu_graph_destroy(dplr_gpu_graph graph);

/* Launch-shape autotuner of the FP64 kernels: times the apply with n
 * right-hand sides for every panel chunk length (256 to 2048 rows),
 * right-hand-side tile (1 to 16 columns) and form (one persistent launch or
 * three launches) and keeps the fastest in the plan.  Call it before
 * dplr_gpu_factor for the solve sweeps to use the tuned chunk length.
 * dplr_gpu_apply_form reports the form kept: 0 persistent, 1 three launches. */
DPLR_API int dplr_gpu_autotune(dplr_gpu_plan plan, int n, void *stream, int *chunk_rows, int *nb_cap,
                               double *best_ms);
DPLR_API int dplr_gpu_apply_form(dplr_gpu_plan plan);

/* Instrumentation.  dplr_gpu_launch_count: kernels launched by this
 * library since load.  Between dplr_gpu_profile_start() and
 * dplr_gpu_profile_stop() the main kernels are bracketed by CUDA events on
 * their launching stream; stop synchronises and returns the number of
 * kernel kinds, whose totals (milliseconds, algorithmic flops and bytes,
 * launches) dplr_gpu_profile_entry() reports. */
DPLR_API long long dplr_gpu_launch_count(void);
/* Fault injection for tests: the next `after` device allocations of plans,
 * factorisations and scratch succeed and the one after fails as if the
 * device were out of memory (then injection is off again); after < 0 turns
 * it off.  DPLR_GB300_FAIL_ALLOC=<after> in the environment arms it when
 * the library loads.  Every entry point then returns DPLR_GPU_ENOMEM (the
 * drop-ins print their message) and leaves its outputs untouched.  No
 * counterpart in DPLR. */
DPLR_API void dplr_gpu_debug_fail_alloc(int after);
/* Fault injection for tests: the bound (in polls) of the waits between the
 * roles of the tensor-core kernels, on the current device, for launches from
 * now on; spins <= 0 restores the default (about 4 million polls).  With a
 * bound of a few polls the waits expire: the kernel stops its work, lets the
 * copies and MMAs in flight land, frees its tensor memory and records the
 * expiry, which the plan's next call returns as DPLR_GPU_ECUDA ("a bounded
 * wait expired"); the call after that runs normally.  No counterpart in
 * DPLR. */
DPLR_API int dplr_gpu_debug_wait_limit(int spins);
DPLR_API int dplr_gpu_profile_start(void);
DPLR_API int dplr_gpu_profile_stop(void);
DPLR_API int dplr_gpu_profile_entry(int i, const char **name, double *ms, double *flops,
                                    double *bytes, int *launches);

/* dplrd2gep with the number of SVD workers chosen (each a host thread with
 * its own stream, cuSOLVER handle and buffers; 0 = 8, fewer where device
 * memory is short).  Blocks of up to 64 rows (DPLR_GB300_SVD_BATCH_RANK
 * lowers the limit) run together in one launch of the library's own SVD
 * kernel instead; a block whose Jacobi sweeps do not converge gives info 1.
 * dplrd2gep is this call with workers = 0.  Returns
 * DPLR_GPU_EINVAL on invalid arguments, DPLR_GPU_ECUDA on a CUDA or
 * cuSOLVER error, else DPLR_GPU_OK with DPLR's info in *info. */
DPLR_API int dplr_gpu_d2gep(int m, const double *A, int lda, DPlrMtx *B, double eps, int nlvl,
                            int workers, int *info);

/* dplrgeppmm with a status: DPLR_GPU_EINVAL (message in
 * dplr_gpu_last_error) when A, B and C differ in structure or are
 * malformed, before C is touched; DPLR_GPU_ECUDA / DPLR_GPU_ENOMEM on a
 * device error.  stream: the CUDA stream of the device work. */
DPLR_API int dplr_gpu_geppmm(char transa, char transb, int m, double alpha, DPlrMtx *A, DPlrMtx *B,
                             double beta, DPlrMtx *C, double eps, void *stream);
/* dplrgeppmm returns its result through a pinned host buffer that is kept
 * (at 1.5x the largest result so far) for later calls; this frees it. */
DPLR_API void dplr_gpu_release_staging(void);

/* SVD-based recompression of every low-rank block of a host tree, the
 * alternative to dplrreduce's Gram-Schmidt (dortlr): each U diag(s) V^T
 * becomes its truncated SVD (QR of U diag(s) and of V, SVD of Ru Rv^T on
 * the GPU), keeping the singular values >= the block's threshold, eps/4
 * per level as dplrreduce splits it.  Ranks only shrink, capacities stay.
 * Blocks of rank r <= min(n, 64) with n r^2 <= 2^22 run together in one
 * launch of the library's own kernel (Householder QR and one-sided Jacobi,
 * one CTA per block); DPLR_GB300_SVD_BATCH_RANK in the environment (0..64,
 * read on every call) lowers that rank limit.  The other blocks use
 * cuSOLVER on `workers` host threads, each with its own stream and handle
 * (0 = 8).  DPLR_GPU_ENOTCONV if an SVD did not converge (that block is
 * kept). */
DPLR_API int dplr_gpu_reduce_svd(int m, DPlrMtx *A, double eps, int workers);

/* Associate the drop-in entry points with a plan for this host tree
 * (they then skip the upload).  dplr_gpu_unregister drops the link.  A
 * registration is found by the tree's address and size only: unregister
 * before freeing or reshaping the tree, or a new tree at the same address
 * would use the old factors.  A drop-in call keeps its registered plan alive
 * until it returns, so (un)registering from another thread is safe; two
 * drop-in calls on the same registered tree must not overlap (they share
 * the plan's device buffers). */
DPLR_API int dplr_gpu_register(int m, DPlrMtx *A);
DPLR_API int dplr_gpu_unregister(DPlrMtx *A);

#ifdef __cplusplus
}
#endif

#endif /* DPLR_GB300_EXT_H */
