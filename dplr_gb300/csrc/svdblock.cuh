// svdblock.cuh -- truncated-SVD recompression of low-rank blocks, shared by
// the host-tree recompression (dplr_gpu_reduce_svd) and the device-plan one
// (dplr_gpu_plan_reduce_svd).  compress.cu runs the blocks.
#pragma once

namespace dg {

// One block U diag(sig) V^T (n x n, rank r): its factors are read from
// u, v, sig (host or device memory) and the truncated SVD (the singular
// values >= eps) is written to du, dv, dsig (host or device; they may be the
// sources).  `rank` receives the new rank.
struct SvdBlock {
    const double *u, *v, *sig;
    double *du, *dv, *dsig;
    int n, r;
    double eps;
    int rank;
};

// Runs every block on up to `workers` host threads (0: 8), each with its own
// stream, cuSOLVER handle and buffers, largest blocks first.  DPLR_GPU_OK,
// DPLR_GPU_ECUDA, or DPLR_GPU_ENOTCONV when an SVD did not converge (that
// block is left with rank = r and its destinations untouched).
int svd_truncate_blocks(SvdBlock *blocks, int count, int workers);

}  // namespace dg
