// sliced.cuh -- exact-slice tensor-core products (declarations).
//
// An FP64 matrix is stored as NS "slices": integers a_p (|a_1| <= 128,
// |a_p| <= 64 for p > 1, exactly representable in bf16) such that
//     x = 2^e * sum_p a_p 2^(-7p)  (+ a remainder below 2^(e-7 NS-1)),
// with one power-of-two exponent e per row or per column.  A product of two
// sliced operands is sum_{p,q} 2^(-7(p+q)) (A_p B_q): each A_p B_q is a bf16
// tensor-core product of small integers.  Its FP32 accumulation is exact
// while every partial sum stays below 2^24, which holds for 64-row stages
// (products <= 128*128, at most 9 pairs per diagonal): the stage results
// are therefore exact integers, added without rounding into 128-bit
// integers per output.  Only the final conversion to double-double (and
// the truncation of the slices) rounds.  With 8 slices the operands are
// represented to 57 bits and products are accumulated exactly, which is
// more accurate than FP64 dot products; with 3 slices (22 bits) the same
// kernels give the low-precision inner solve.
#pragma once

#include <cuda_bf16.h>

#include "internal.cuh"

namespace dg {

using bf16 = __nv_bfloat16;

// Panel item of a sliced product  P = F[rows]^T X[in0 + rows, :]  where F
// is column-sliced (exponent per column k, column-major, ld n), X is sliced
// with one exponent per column j (global over all rows).
struct SPanelItem {
    long long f;        // element offset of F in the slice pool
    long long p;        // 128-bit partial offset / nrhs
    int n, rank, in0, r0, len, chunk;
};

// Reduce item of one block: T = sig o 2^(fexp + xexp - 7 D) sum_chunks W
// (double-double), then sliced per column into rows [0, rp) of the block's
// T-slice panel (rp = rank rounded up to 8, zero padded).
struct SReduceItem {
    long long p, t, sig;
    int rank, nch, fexp;
    int rp;             // padded rank
    long long tpad;     // offset / nrhs of the block's T-slice panel
    int rsum;           // ranks of the schedule's earlier items (the reduce's element space)
};

// Term of a sliced output tile: acc += A[tile rows, 0:K] * B[0:K, :], A
// row-sliced and stored row-major (row stride lda, zero padded to a
// multiple of 8 columns).
struct STerm {
    long long a;        // element offset of A's tile row 0 in the slice pool
    long long b;        // src 0: T-slice panel offset / nrhs (ld ldb)
    int lda, K, aexp;   // aexp: offset of the tile's first row exponent
    int src;            // 0: B = T slices of reduce item `blk`; 1: B = X slices
    int ldb, x_row0, blk;
};

// Tile-block schedules of the tcgen05 pipeline kernels (tcpipe.cuh).  A
// tile-block is R rows x 16 inner elements of one slice, contiguous, in the
// tensor core's K-major core-matrix order.
struct XTerm {          // term of a 128-row expand tile
    long long a;        // A tile-block of inner block 0 (slice 0); block kb at a + kb * 2048
    long long b;        // src 0: T tile-block base of the block per 64-column rhs tile (times njt);
                        // src 1: first X row-block
    int K;              // inner length (16-element blocks: ceil(K / 16))
    int aexp;           // exponent offset of the tile's row 0
    int src;            // 0: T slices (exponents texp[blk * nrhs + j]), 1: X slices (xexp[j])
    int blk;
};

struct PItem {          // panel work item: one row chunk of a block, one rank tile (<= 64)
    long long v;        // V tile-blocks of (block, rank tile), slice 0: row-block rb at v + rb * nr * 16
    long long p;        // partial offset / nrhs of the block
    int rank, kt, nr;   // block rank, first rank of the tile, padded rows of its tile-blocks
    int xrb0;           // first X row-block ((in0 + r0) / 16)
    int vrb0;           // first V row-block of the chunk (r0 / 16)
    int nkb;            // chunk rows / 16
    int chunk;
};

struct SSchedule {
    int tile_m = 64;                // rows of an expand tile: 64 (mma.sync) or 128 (tcgen05)
    // tcgen05 pipeline (tile_m == 128)
    std::vector<PItem> pitems;
    std::vector<XTerm> xterms;
    long long tpre = 0;             // T tile-block elements of all blocks per 64-column rhs tile
    PItem *d_pitems = nullptr;
    XTerm *d_xterms = nullptr;
    int *d_rmax = nullptr;          // per tile row: max row exponent of the tile's terms (static)
    std::vector<SPanelItem> items;
    std::vector<SReduceItem> reduces;
    long long partial_per_rhs = 0;
    long long t_per_rhs = 0;        // DD T entries / nrhs
    long long tpad_per_rhs = 0;     // T-slice entries / nrhs
    int max_rank = 0;
    int rtotal = 0;                 // sum of the reduce items' ranks
    int *d_rank_item = nullptr;     // per rank position (rsum + k) its reduce item
    std::vector<int> tile_row0, tile_begin;
    std::vector<STerm> terms;
    SPanelItem *d_items = nullptr;
    SReduceItem *d_reduces = nullptr;
    int *d_tile_row0 = nullptr, *d_tile_begin = nullptr;
    STerm *d_terms = nullptr;
};

struct Sliced {
    int ns = 0;                    // slices of the factors
    long long stride = 0;          // elements per slice
    bf16 *pool = nullptr;          // ns x stride
    int *exps = nullptr;           // exponents (per V column, U row, leaf row)
    long long nexp = 0;
    SSchedule apply;               // op N
    // scratch
    bf16 *xs = nullptr;            // sliced right-hand sides
    size_t xs_elems = 0;
    int *xexp = nullptr;
    size_t xexp_n = 0;
    void *work = nullptr;          // 128-bit partials, DD T, T slices, T exponents
    size_t work_bytes = 0;
    long long bytes = 0;
};

// Low-precision inner solve of the refinement: the Woodbury sweep of the
// FP64 factorisation with V, the D^-1 W panels and the leaf inverses cut
// into ns slices (1 + 7 ns bits; pairs p + q <= ns + 1) and every product
// on the tensor cores; the capacitance inverses are applied in FP64.
struct MixedSliced {
    int ns = 4;
    long long stride = 0;
    bf16 *pool = nullptr;
    int *exps = nullptr;
    std::vector<SSchedule> level;  // panel on V + update with Z, per H level
    SSchedule leaf;                // leaf step
    long long tpad_per_rhs = 0;    // T / W slice entries per rhs (all blocks)
    long long t_per_rhs = 0;
    int nblocks = 0;
    // scratch
    bf16 *xs = nullptr;
    size_t xs_elems = 0;
    int *xexp = nullptr;
    size_t xexp_n = 0;
    int *xexp2 = nullptr;          // exponents of the X being written (swapped with xexp)
    size_t xexp2_n = 0;
    // Capacitance on the tensor cores: the K^-1 of every node with two
    // rank-128 blocks in 8 exact slices (row exponents), applied by the
    // multi-term expand; other nodes keep the FP64 kernel.
    bool tc_caps = false;
    bf16 *kslices = nullptr;
    long long kstride = 0;
    int *kexps = nullptr;
    std::vector<SSchedule> capsched;             // per level: output tiles of K^-1 [T1; T2]
    std::vector<std::vector<CapItem>> capfb;     // per level: nodes left to the FP64 kernel
    std::vector<CapItem *> d_capfb;
    void *work = nullptr;
    size_t work_bytes = 0;
    long long bytes = 0;
};

int mixed_build(Plan *p, int ns, cudaStream_t st, bool fp64_caps = false);
void mixed_free(Plan *p);
// X = A^-1 B with the low-precision sweep (B and X must not alias).
int mixed_solve(Plan *p, int nrhs, const double *B, int ldb, double *X, int ldx, cudaStream_t st);

int sliced_build(Plan *p, int ns, cudaStream_t st);
// Error recorded by a tensor-core kernel whose bounded wait expired (the
// flag is cleared); 0 if none.
int sliced_error(Plan *p);
void sliced_free(Plan *p);
// R = B - A X with exact-slice products (8 slices: FP64-or-better accuracy).
int sliced_residual(Plan *p, int nrhs, const double *X, int ldx, const double *B, int ldb,
                    double *R, int ldr, cudaStream_t st);

}  // namespace dg
