// internal.cuh -- shared declarations of libdplr_gb300.so.
//
// Device layout of a PLR matrix ("plan"):
//   * one FP64 factor pool: for every low-rank block its U (n x rank,
//     ld n), V (n x rank, ld n) and sig[rank]; for every dense leaf its
//     b x b matrix (ld b).  Every array starts on a 256-byte boundary.
//   * a block table: LRDesc per low-rank block, LeafDesc per leaf, HDesc
//     per H node, all in pre-order of the host tree.
//   * apply schedules (one per op N / T): "panel" work items that reduce
//     V^T X (U^T X for op T) over row chunks, and "row tiles" that expand
//     every level's U T_b (V T_b) plus the leaf term into one output tile.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dplr.h"
#include "../../include/dplr_gb300.h"

namespace dg {

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
int fail(int code, const char *fmt, ...);
#define DG_CUDA(call)                                                              \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess)                                                     \
            return ::dg::fail(DPLR_GPU_ECUDA, "%s failed: %s (%s:%d)", #call,      \
                              cudaGetErrorString(e_), __FILE__, __LINE__);         \
    } while (0)

// Device allocations of plans, factorisations and scratch go through
// dev_malloc, so that a test can make the k-th of them fail
// (dplr_gpu_debug_fail_alloc, or DPLR_GB300_FAIL_ALLOC=k in the environment
// when the library loads) and check that every caller reports
// DPLR_GPU_ENOMEM and leaves its outputs untouched.
cudaError_t dev_malloc(void **ptr, size_t bytes);
#define DG_ALLOC(ptr, bytes)                                                                     \
    do {                                                                                         \
        cudaError_t e_ = ::dg::dev_malloc((void **)(ptr), (bytes));                             \
        if (e_ != cudaSuccess)                                                                   \
            return ::dg::fail(DPLR_GPU_ENOMEM, "cannot allocate %zu bytes of device memory: %s " \
                              "(%s:%d)", (size_t)(bytes), cudaGetErrorString(e_), __FILE__,      \
                              __LINE__);                                                        \
    } while (0)

// Recompression after rank-growing operations (dplr_gpu_set_recompress):
// the threshold (< 0: off) and the host-tree hook the drop-ins call on their
// output (dplr_gpu_reduce_svd with that threshold).
double recompress_eps();
void recompress_after(int m, DPlrMtx *A);

// NVTX range around an entry point (visible in Nsight tools; a no-op unless
// a tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char *name);
    ~NvtxRange();
};

// ------------------------------------------------------- instrumentation
// Every kernel launch of the library is counted; when profiling is on, the
// main launch sites also bracket their launch with CUDA events on the
// launching stream and record the algorithmic flops and bytes of that
// launch (see prof_begin / prof_end in abi.cu).
void note_launch();
void note_launches(long long k);
struct ProfScope {
    int id = -1;
    cudaStream_t stream_ = nullptr;
    ProfScope(const char *name, cudaStream_t st, double flops, double bytes);
    ~ProfScope();
};

// ---------------------------------------------------------------- tables
struct LRDesc {            // one low-rank block U diag(sig) V^T
    long long u, v, sig;   // pool offsets (doubles)
    int row0;              // first row it writes for op N (rows of U)
    int col0;              // first row of x it reads for op N (rows of V)
    int n, rank;
    int level, node;       // depth of the owning H node, its index
    int toff;              // prefix sum of ranks (T buffer offset / nrhs)
    int is_ne;
};

struct LeafDesc {
    long long d;           // pool offset of the b x b matrix
    int row0, b;
};

struct HDesc {
    int row0, m, level;
    int ne, sw;            // LRDesc indices
    int nw, se;            // child: >= 0 HDesc index, < 0 -> ~leaf index
    int parent;
};

// Work items below are self-contained (offsets, sizes, strides), so the same
// kernels serve the apply (factors U/V of the pool) and the Woodbury solve
// (factors V and the D^-1 W panels of the factorisation).

// Panel item: partial F[r0:r0+len, 0:rank]^T X[in0+r0 : in0+r0+len, :]
// written to partials + p*nrhs + chunk*rank*nrhs (rank x nrhs, ld rank).
struct PanelItem {
    long long f;           // factor offset (column-major, ld n)
    long long p;           // partial block offset / nrhs
    int in0, n, rank, r0, len, chunk;
};

// Reduce item: T[t*nrhs + k + j*rank] = sig[k] * sum_c partial[c][k, j]
// (no scaling when sig < 0).
struct ReduceItem {
    long long p, t, sig;
    int rank, nch;
};

// Term of an output tile: acc += op(A)[tile rows, 0:K] * B[0:K, :]
struct TileTerm {
    long long a;           // offset of A's (tile row 0, k = 0) element
    long long b;           // src 0: T buffer offset / nrhs (ld = ldb)
    int lda, K;
    int trans_a;           // 1: A(i,k) at a + i*lda + k ; 0: a + i + k*lda
    int src;               // 0: B = T + b*nrhs; 1: B = X rows from x_row0; 2: B = T + b
    int ldb, x_row0;
};

// Capacitance item of one H node: W = op(Kinv) [T1; T2] (optionally scaled
// row-wise by [sig1; sig2]); W1, W2 are written at the offsets of T1, T2 in
// the output buffer.
struct CapItem {
    long long k;           // offset of the r x r inverse (r = r1 + r2)
    long long t1, t2;      // T / W offsets / nrhs (ld r1, r2)
    long long s1, s2;      // sig offsets (pool) for the scaled variant
    int r1, r2;
};

struct Schedule {
    std::vector<PanelItem> items;
    std::vector<ReduceItem> reduces;
    long long partial_per_rhs = 0;    // partial doubles / nrhs
    long long t_per_rhs = 0;          // T buffer doubles / nrhs
    std::vector<int> tile_row0, tile_begin;   // tile_begin has ntiles+1 entries
    std::vector<TileTerm> terms;
    std::vector<CapItem> caps;
    int tile_rows = 0;
    int max_rank = 0;
    int nb_cap = 16;                  // largest right-hand-side tile (autotuned)
    int max_len = 0;                  // longest panel item (rows)
    bool has_row_major = false;       // some term reads A row-major (trans_a)
    PanelItem *d_items = nullptr;
    ReduceItem *d_reduces = nullptr;
    int *d_tile_row0 = nullptr, *d_tile_begin = nullptr;
    TileTerm *d_terms = nullptr;
    CapItem *d_caps = nullptr;
    // persistent apply (persist.cu): reduce index of every panel item and
    // of every tile term that reads T (-1: leaf term), built on first use
    int *d_item_red = nullptr, *d_term_red = nullptr;
};

struct Plan {
    int m = 0, levels = 0, max_rank = 0, total_rank = 0;
    int ntrees = 1;                   // > 1: a batch of independent trees (block diagonal)
    std::vector<int> tree_row0;       // first row of every tree
    int *d_tree_row0 = nullptr;       // device copy + m (batch plans, built on first refined solve)
    int nb_cap = 16;                  // largest right-hand-side tile of the FP64 kernels (autotuned)
    long long nnz = 0;
    std::vector<LRDesc> lr;
    std::vector<LeafDesc> leaves;
    std::vector<HDesc> nodes;
    long long pool_doubles = 0;
    double *pool = nullptr;
    LRDesc *d_lr = nullptr;
    LeafDesc *d_leaves = nullptr;
    Schedule sched[2];                // [0] op N, [1] op T
    // scratch for applies (grown on demand)
    double *work = nullptr;
    size_t work_doubles = 0;
    double *xbuf = nullptr, *ybuf = nullptr;   // host<->device staging for drop-in
    size_t xbuf_doubles = 0, ybuf_doubles = 0;
    int chunk_rows = 512;
    int apply_launches = 0;           // 1: the autotuner chose the three-launch apply over the persistent one
    long long device_bytes = 0;
    // Woodbury factorisation (filled by factor.cu)
    void *fact = nullptr;
    // exact-slice factor copies (sliced.cu)
    void *sliced = nullptr;
    // low-precision sliced solve (sliced.cu)
    void *mixed = nullptr;
    // error flag of the tensor-core kernels (mapped host memory, sliced.cu)
    int *tc_err_h = nullptr, *tc_err_d = nullptr;
    // float-pair copy of the factors for the 1-RHS apply (pairs.cu)
    void *pairs = nullptr;
    // factor gradients (grad.cu): work lists and scratch
    void *grad = nullptr;
    double *gbuf = nullptr;
    size_t gbuf_doubles = 0;
};

// plan.cu
int plan_build(int m, const DPlrMtx *A, cudaStream_t st, Plan **out);
int plan_build_forest(int count, const int *ms, const DPlrMtx *const *As, cudaStream_t st, Plan **out);
int plan_reschedule(Plan *p);
int plan_upload_values(Plan *p, const DPlrMtx *A, cudaStream_t st);
void plan_free(Plan *p);
int ensure_buffer(double **buf, size_t *have, size_t need);
int validate_tree(int m, const DPlrMtx *A, const char *fn);

// schedule helpers (plan.cu)
int tile_rows_for(const Plan *p);
void build_tiles(const Plan *p, int trans, int R, std::vector<int> &row0, std::vector<int> &begin,
                 std::vector<TileTerm> &terms, int lmin = 0);
// Apply schedule (op N: trans 0, op T: trans 1) of the blocks of H nodes at
// depth >= lmin and every leaf.
void build_schedule(const Plan *p, int trans, Schedule &S, int lmin = 0);
int upload_schedule(Schedule &S, long long *bytes);
void free_schedule(Schedule &S);

// apply.cu: generic launches over a schedule
int run_panel(const Schedule &S, const double *fbase, const double *X, int ldx, int nrhs,
              double *partials, cudaStream_t st);
int run_reduce(const Schedule &S, const double *sigbase, const double *partials, int nrhs,
               double *T, cudaStream_t st);
int run_expand(const Schedule &S, const double *abase, const double *T, const double *X, int ldx,
               double *Y, int ldy, int nrhs, double alpha, double beta, cudaStream_t st);
int run_caps(const Schedule &S, const double *kbase, const double *sigbase, int trans,
             const double *T, double *W, int nrhs, cudaStream_t st);
int run_cap_list(const std::vector<CapItem> &caps, const CapItem *d_caps, const double *kbase, const double *sigbase,
                 int trans, const double *T, double *W, int nrhs, cudaStream_t st);
int apply_device(Plan *p, int trans, int nrhs, double alpha, const double *X, int ldx,
                 double beta, double *Y, int ldy, cudaStream_t st, bool alpha0_squares_beta);
int scale_device(double *Y, int rows, int cols, int ldy, double beta, cudaStream_t st);

// persist.cu: the whole FP64 apply in one persistent launch
bool persist_usable(const Plan *p, int trans, int nrhs);
int persist_apply(Plan *p, int trans, int nrhs, double alpha, const double *X, int ldx, double beta, double *Y,
                  int ldy, cudaStream_t st);
// sliced.cu: the plan's mapped error flag of kernels with bounded waits
int ensure_err_flag(Plan *p);
int sliced_error(Plan *p);
int set_wait_limit(int spins);

// pairs.cu: FP64-accurate 1-RHS apply on the FP32 pipes
int pairs_prepare(Plan *p, cudaStream_t st);
int pairs_refresh(Plan *p, cudaStream_t st);
void pairs_free(Plan *p);
bool pairs_usable(const Plan *p, int trans, int nrhs);
int pairs_apply(Plan *p, double alpha, const double *X, double beta, double *Y, cudaStream_t st);
long long pairs_bytes(const Plan *p);

// grad.cu
void grad_free(Plan *p);
int grad_factors(Plan *p, int nrhs, const double *X, int ldx, const double *DY, int ldy, double alpha, double *G,
                 cudaStream_t st);
void plan_values_changed(Plan *p);
int transpose_device(const double *src, int rows, int cols, int lds, double *dst, int ldd,
                     cudaStream_t st);

}  // namespace dg
