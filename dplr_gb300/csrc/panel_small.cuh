// panel_small.cuh -- the panel F[r0:r0+len, 0:rank]^T X[rows, j0:j0+nj] of
// one chunk for blocks of rank <= 4, shared by the panel kernel (apply.cu)
// and the persistent apply (persist.cu).
//
// Small ranks leave most of a rank tile idle when threads own rank columns.
// Here every thread owns rows r = t, t + T, ... of the chunk and all of the
// block's (at most 4) rank columns and the tile's right-hand sides, reading
// F and X coalesced straight from memory; the partial sums are reduced with
// warp shuffles, then across warps in shared memory, and written in the
// layout of the other panel paths: P[k + (j0 + j) * rank].
#pragma once

namespace dg {

constexpr int kSmallRank = 4;

// sm: at least (blockDim.x / 32) * kSmallRank * JB doubles.
template <int NB>
__device__ __forceinline__ void panel_small_rank(const double *__restrict__ F, int n, int r0, int len,
                                                 int rank, const double *__restrict__ X, long long ldx,
                                                 int xrow0, int j0, int nj, double *__restrict__ P,
                                                 double *sm)
{
    constexpr int JB = NB < 8 ? NB : 8;        // right-hand sides per register block
    const int t = threadIdx.x, T = blockDim.x, lane = t & 31, warp = t >> 5, nw = T >> 5;
    for (int jb = 0; jb < nj; jb += JB) {
        double acc[kSmallRank][JB];
#pragma unroll
        for (int k = 0; k < kSmallRank; ++k)
#pragma unroll
            for (int j = 0; j < JB; ++j) acc[k][j] = 0.0;
        for (int r = t; r < len; r += T) {
            double x[JB];
#pragma unroll
            for (int j = 0; j < JB; ++j)
                x[j] = jb + j < nj ? __ldg(X + (long long)(j0 + jb + j) * ldx + xrow0 + r0 + r) : 0.0;
#pragma unroll
            for (int k = 0; k < kSmallRank; ++k) {
                if (k < rank) {
                    const double f = __ldg(F + (long long)k * n + r0 + r);
#pragma unroll
                    for (int j = 0; j < JB; ++j) acc[k][j] = fma(f, x[j], acc[k][j]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kSmallRank; ++k)
#pragma unroll
            for (int j = 0; j < JB; ++j) {
                double v = acc[k][j];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                acc[k][j] = v;
            }
        __syncthreads();                       // sm may still be read by an earlier pass
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < kSmallRank; ++k)
#pragma unroll
                for (int j = 0; j < JB; ++j) sm[(warp * kSmallRank + k) * JB + j] = acc[k][j];
        __syncthreads();
        for (int e = t; e < kSmallRank * JB; e += T) {
            const int k = e / JB, j = e % JB;
            if (k < rank && jb + j < nj) {
                double s = 0.0;
                for (int w = 0; w < nw; ++w) s += sm[(w * kSmallRank + k) * JB + j];
                P[k + (long long)(j0 + jb + j) * rank] = s;
            }
        }
    }
    __syncthreads();                           // sm is reused by the caller
}

}  // namespace dg
