// gemm.cuh -- batched FP64 GEMM of the library's structure operations
// (PLR x PLR product, compression): many small and skinny products per
// launch, described by job tables.
//
//   D = alpha op(A) diag(ks) op(B) + beta C
//
// One CTA computes a 64 x 64 output tile (4 x 4 per thread, K staged in
// shared memory 16 at a time).  Long, skinny products (few tiles, K >= 1024)
// are split along K into slices of >= 512 whose raw partial sums a second
// kernel adds in slice order, so results do not depend on scheduling.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

namespace dg {
namespace {

// D = alpha op(A) diag(ks) op(B) + beta C  (C not read when beta == 0; C
// may be D).  op(A) is M x K: a[i + k lda] (ta = 0) or a[k + i lda].
struct GemmJob {
    const double *a, *b, *c, *ks;
    double *d;
    int M, N, K, lda, ldb, ldc, ldd, ta, tb;
    double alpha, beta;
};

// Output tile (i0, j0) of a job over k in [k0, k1); p >= 0: raw partial sums
// to part + p (ld M), summed in slice order by gemm_reduce_kernel (split K
// for long, skinny products).
struct GemmTile {
    int job, i0, j0, k0, k1;
    long long p;
};

struct GemmRed {
    long long p;
    int job, slices;
};

constexpr int kGT = 64;   // output tile edge
constexpr int kGK = 16;   // k step staged in shared memory

__global__ void __launch_bounds__(256) gemm_kernel(const GemmJob *__restrict__ jobs,
                                                   const GemmTile *__restrict__ tiles, double *__restrict__ part)
{
    const GemmTile t = tiles[blockIdx.x];
    const GemmJob J = jobs[t.job];
    __shared__ double As[kGK][kGT + 1];
    __shared__ double Bs[kGK][kGT + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = 0.0;
    // alpha == 0: op(A) op(B) is not read (BLAS semantics, NaN-safe)
    const int kend = J.alpha == 0.0 ? t.k0 : t.k1;
    for (int k0 = t.k0; k0 < kend; k0 += kGK) {
        for (int e = threadIdx.x; e < kGT * kGK; e += 256) {
            // consecutive threads walk the contiguous index of the operand
            const int i = J.ta ? e / kGK : e % kGT;
            const int k = J.ta ? e % kGK : e / kGT;
            const int gi = t.i0 + i, gk = k0 + k;
            double v = 0.0;
            if (gi < J.M && gk < t.k1) {
                v = J.ta ? J.a[gk + (long long)gi * J.lda] : J.a[gi + (long long)gk * J.lda];
                if (J.ks) v *= J.ks[gk];
            }
            As[k][i] = v;
        }
        for (int e = threadIdx.x; e < kGT * kGK; e += 256) {
            const int j = J.tb ? e % kGT : e / kGK;
            const int k = J.tb ? e / kGT : e % kGK;
            const int gj = t.j0 + j, gk = k0 + k;
            double v = 0.0;
            if (gj < J.N && gk < t.k1)
                v = J.tb ? J.b[gj + (long long)gk * J.ldb] : J.b[gk + (long long)gj * J.ldb];
            Bs[k][j] = v;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kGK; ++k) {
            double a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[k][ty + 16 * r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[k][tx + 16 * c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int i = t.i0 + ty + 16 * r, j = t.j0 + tx + 16 * c;
            if (i < J.M && j < J.N && t.p >= 0) {
                part[t.p + i + (long long)j * J.M] = acc[r][c];
            } else if (i < J.M && j < J.N) {
                double v = J.alpha * acc[r][c];
                if (J.beta != 0.0) v = fma(J.beta, J.c[i + (long long)j * J.ldc], v);
                J.d[i + (long long)j * J.ldd] = v;
            }
        }
}

// D = alpha * (sum of a split job's slices, in order) + beta C.
__global__ void gemm_reduce_kernel(const GemmJob *__restrict__ jobs, const GemmRed *__restrict__ reds,
                                   const double *__restrict__ part)
{
    const GemmRed R = reds[blockIdx.y];
    const GemmJob J = jobs[R.job];
    const long long mn = (long long)J.M * J.N;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < mn; e += (long long)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int q = 0; q < R.slices; ++q) acc += part[R.p + q * mn + e];
        const int i = (int)(e % J.M), j = (int)(e / J.M);
        double v = J.alpha * acc;
        if (J.beta != 0.0) v = fma(J.beta, J.c[i + (long long)j * J.ldc], v);
        J.d[i + (long long)j * J.ldd] = v;
    }
}

// Tiles (and split-K reductions) of a job list; ptot = doubles of partial
// sums needed.
inline void plan_gemm_tiles(const std::vector<GemmJob> &jobs, std::vector<GemmTile> &tiles,
                            std::vector<GemmRed> &reds, long long &ptot)
{
    tiles.clear();
    reds.clear();
    ptot = 0;
    for (int j = 0; j < (int)jobs.size(); ++j) {
        const GemmJob &J = jobs[j];
        const int mt = (J.M + kGT - 1) / kGT, nt = (J.N + kGT - 1) / kGT;
        int slices = 1;
        if (mt * nt <= 4 && J.K >= 1024) slices = std::min(64, J.K / 512);
        const int chunk = ((J.K + slices - 1) / slices + kGK - 1) / kGK * kGK;
        slices = J.K > 0 ? (J.K + chunk - 1) / chunk : 1;
        const long long p = slices > 1 ? ptot : -1;
        for (int q = 0; q < slices; ++q)
            for (int i0 = 0; i0 < J.M; i0 += kGT)
                for (int j0 = 0; j0 < J.N; j0 += kGT)
                    tiles.push_back({j, i0, j0, q * chunk, std::min(J.K, (q + 1) * chunk),
                                     p < 0 ? -1 : p + (long long)q * J.M * J.N});
        if (slices > 1) {
            reds.push_back({p, j, slices});
            ptot += (long long)slices * J.M * J.N;
        }
    }
}

// Launch over uploaded tables (tiles in at most 2^30 per grid).
inline void run_gemm_tables(const GemmJob *dj, const GemmTile *dt, size_t ntiles, const GemmRed *dr, size_t nreds,
                            double *part, cudaStream_t st)
{
    for (size_t b0 = 0; b0 < ntiles; b0 += 1u << 30) {
        const unsigned nb = (unsigned)std::min<size_t>(ntiles - b0, 1u << 30);
        gemm_kernel<<<nb, 256, 0, st>>>(dj, dt + b0, part);
    }
    if (nreds) gemm_reduce_kernel<<<dim3(16, (unsigned)nreds), 256, 0, st>>>(dj, dr, part);
}

}  // namespace
}  // namespace dg
