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

// Work item of the panel kernel: rows [r0, r0+len) of block `blk`.
struct PanelItem {
    int blk, r0, len, chunk;     // chunk index within the block
};

// One term of an output tile: acc += op(A)[tile rows, 0:K] * Bsrc[0:K, :]
struct TileTerm {
    long long a;       // pool offset of A's element (tile row 0, k = 0)
    int lda;           // leading dimension of A
    int K;             // inner size
    int trans_a;       // 1: A element (i,k) at a + i*lda + k ; 0: a + i + k*lda
    int src;           // 0: B = T buffer of block `blk`; 1: B = X rows from x_row0
    int blk, x_row0;
};

struct Schedule {
    std::vector<PanelItem> items;     // host copy
    std::vector<int> chunks_of;       // per block: number of panel chunks
    std::vector<long long> poff;      // per block: prefix of chunks*rank (partials / nrhs)
    long long partial_per_rhs = 0;    // total partial doubles / nrhs
    std::vector<int> tile_row0, tile_begin;   // tile_begin has ntiles+1 entries
    std::vector<TileTerm> terms;
    int tile_rows = 0;
    // device copies
    PanelItem *d_items = nullptr;
    long long *d_poff = nullptr;
    int *d_chunks = nullptr;
    int *d_tile_row0 = nullptr, *d_tile_begin = nullptr;
    TileTerm *d_terms = nullptr;
};

struct Plan {
    int m = 0, levels = 0, max_rank = 0, total_rank = 0;
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
    long long device_bytes = 0;
    // Woodbury factorisation (filled by factor.cu)
    void *fact = nullptr;
};

// plan.cu
int plan_build(int m, const DPlrMtx *A, cudaStream_t st, Plan **out);
int plan_upload_values(Plan *p, const DPlrMtx *A, cudaStream_t st);
void plan_free(Plan *p);
int ensure_buffer(double **buf, size_t *have, size_t need);
int validate_tree(int m, const DPlrMtx *A, const char *fn);

// apply.cu
int apply_device(Plan *p, int trans, int nrhs, double alpha, const double *X, int ldx,
                 double beta, double *Y, int ldy, cudaStream_t st, bool alpha0_squares_beta);
int scale_device(double *Y, int rows, int cols, int ldy, double beta, cudaStream_t st);
int transpose_device(const double *src, int rows, int cols, int lds, double *dst, int ldd,
                     cudaStream_t st);

}  // namespace dg
