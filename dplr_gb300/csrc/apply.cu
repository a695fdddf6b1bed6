// apply.cu -- FP64 PLR apply  Y := alpha*op(A)*X + beta*Y  on the GPU.
//
// DPLR recurses over the tree and makes two BLAS-2/3 calls per low-rank
// block plus one per leaf (src/dplrpmv.c:19-180, src/dplrpdmm.c:23-241).
// Here the whole tree is applied in three launches over the block table:
//   1. panel:  for every (block, row chunk) item, the partial product
//              F_in[chunk]^T X[chunk rows]  (F_in = V for op N, U for op T)
//   2. reduce: T_b = sig_b o sum_chunks(partials)           (rank x nrhs)
//   3. expand: for every row tile of Y, the sum over levels of
//              F_out[tile] T_b  plus the leaf term  D[tile] X[leaf rows]
//              (D^T for op T), then Y = alpha*acc + beta*Y (beta == 0 does
//              not read Y).
// Every output element is written by exactly one thread (no atomics), so
// results are deterministic.  FP64 on GB300 runs at ~1.2 TFLOP/s, so for
// more than a few right-hand sides the kernels are FP64-issue bound; the
// smem staging only has to keep HBM traffic low, not feed tensor cores.
#include "internal.cuh"

#include <algorithm>

namespace dg {

constexpr int kThreads = 256;
constexpr int kSlab = 32;     // rows of X / factor staged per step
constexpr int kRankTile = 64; // ranks handled per pass of the panel kernel

// ----------------------------------------------------------------- panel
// One CTA per (item, rhs tile).  Thread t owns rank column k = t % 64 of
// the current rank tile and the rows i == t/64 (mod 4) of each slab; the
// four row groups are summed through shared memory at the end.
template <int NB>
__global__ void __launch_bounds__(kThreads) panel_kernel(
    const LRDesc *__restrict__ lr, const PanelItem *__restrict__ items,
    const long long *__restrict__ poff, const double *__restrict__ pool,
    const double *__restrict__ X, int ldx, int nrhs, int trans, double *__restrict__ partials)
{
    constexpr int kStage = kSlab * (kRankTile + 1) + kSlab * NB;
    constexpr int kRed = 4 * kRankTile * NB;
    __shared__ double sm[kStage > kRed ? kStage : kRed];
    double(*Fs)[kRankTile + 1] = reinterpret_cast<double(*)[kRankTile + 1]>(sm);
    double(*Xs)[NB] = reinterpret_cast<double(*)[NB]>(sm + kSlab * (kRankTile + 1));
    double(*red)[kRankTile][NB] = reinterpret_cast<double(*)[kRankTile][NB]>(sm);

    const PanelItem it = items[blockIdx.x];
    const LRDesc L = lr[it.blk];
    const double *F = pool + (trans ? L.u : L.v);
    const int in0 = trans ? L.row0 : L.col0;
    const int j0 = blockIdx.y * NB;
    const int nj = min(NB, nrhs - j0);
    const int t = threadIdx.x;
    const int kk = t % kRankTile, g = t / kRankTile;
    double *P = partials + poff[it.blk] * nrhs + (long long)it.chunk * L.rank * nrhs;

    for (int kt = 0; kt < L.rank; kt += kRankTile) {
        const int nk = min(kRankTile, L.rank - kt);
        double acc[NB];
#pragma unroll
        for (int j = 0; j < NB; ++j) acc[j] = 0.0;
        for (int s0 = 0; s0 < it.len; s0 += kSlab) {
            const int ns = min(kSlab, it.len - s0);
            __syncthreads();
            for (int e = t; e < kSlab * kRankTile; e += kThreads) {
                int r = e % kSlab, c = e / kSlab;
                Fs[r][c] = (r < ns && c < nk) ? F[(long long)(kt + c) * L.n + it.r0 + s0 + r] : 0.0;
            }
            for (int e = t; e < kSlab * NB; e += kThreads) {
                int r = e % kSlab, c = e / kSlab;
                Xs[r][c] = (r < ns && c < nj)
                               ? X[(long long)(j0 + c) * ldx + in0 + it.r0 + s0 + r]
                               : 0.0;
            }
            __syncthreads();
#pragma unroll 4
            for (int r = g; r < kSlab; r += 4) {
                double f = Fs[r][kk];
#pragma unroll
                for (int j = 0; j < NB; ++j) acc[j] = fma(f, Xs[r][j], acc[j]);
            }
        }
        __syncthreads();   // red aliases the staging buffers
#pragma unroll
        for (int j = 0; j < NB; ++j) red[g][kk][j] = acc[j];
        __syncthreads();
        if (g == 0 && kk < nk) {
            for (int j = 0; j < nj; ++j) {
                double s = red[0][kk][j] + red[1][kk][j] + red[2][kk][j] + red[3][kk][j];
                P[(kt + kk) + (long long)(j0 + j) * L.rank] = s;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- reduce
// T_b[k, j] = sig[k] * sum_c P_b[c][k, j]; grid.x = block index.
__global__ void reduce_kernel(const LRDesc *__restrict__ lr, const long long *__restrict__ poff,
                              const int *__restrict__ chunks, const double *__restrict__ pool,
                              const double *__restrict__ partials, int nrhs,
                              double *__restrict__ T)
{
    const int b = blockIdx.x;
    const LRDesc L = lr[b];
    const long long cnt = (long long)L.rank * nrhs;
    const long long e = (long long)blockIdx.y * blockDim.x + threadIdx.x;
    if (e >= cnt) return;
    const int k = (int)(e % L.rank);
    const double *P = partials + poff[b] * nrhs + e;
    double s = 0.0;
    const int nch = chunks[b];
    for (int c = 0; c < nch; ++c) s += P[(long long)c * cnt];
    T[(long long)L.toff * nrhs + e] = pool[L.sig + k] * s;
}

// ---------------------------------------------------------------- expand
// One CTA per (row tile, rhs tile).  Thread t owns tile row i = t % R and
// the inner indices k == t/R (mod G), G = 256/R; partial sums of the G
// groups are combined through shared memory before the write-back.
template <int NB>
__global__ void __launch_bounds__(kThreads) expand_kernel(
    const double *__restrict__ pool, const TileTerm *__restrict__ terms,
    const int *__restrict__ tile_row0, const int *__restrict__ tile_begin,
    const LRDesc *__restrict__ lr, const double *__restrict__ T, const double *__restrict__ X,
    int ldx, double *__restrict__ Y, int ldy, int nrhs, int R, double alpha, double beta)
{
    constexpr int kStage = 64 * (kSlab + 1) + kSlab * NB;
    constexpr int kRed = kThreads * NB;
    __shared__ double sm[kStage > kRed ? kStage : kRed];
    double(*As)[kSlab + 1] = reinterpret_cast<double(*)[kSlab + 1]>(sm);
    double(*Bs)[NB] = reinterpret_cast<double(*)[NB]>(sm + 64 * (kSlab + 1));
    double(*red)[NB] = reinterpret_cast<double(*)[NB]>(sm);

    const int tile = blockIdx.x;
    const int row0 = tile_row0[tile];
    const int j0 = blockIdx.y * NB;
    const int nj = min(NB, nrhs - j0);
    const int t = threadIdx.x;
    const int G = kThreads / R;
    const int i = t % R, g = t / R;

    double acc[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) acc[j] = 0.0;

    for (int q = tile_begin[tile]; q < tile_begin[tile + 1]; ++q) {
        const TileTerm tt = terms[q];
        const double *A = pool + tt.a;
        const double *B;
        long long ldb;
        if (tt.src == 0) {
            const LRDesc L = lr[tt.blk];
            B = T + (long long)L.toff * nrhs + (long long)j0 * L.rank;
            ldb = L.rank;
        } else {
            B = X + tt.x_row0 + (long long)j0 * ldx;
            ldb = ldx;
        }
        for (int k0 = 0; k0 < tt.K; k0 += kSlab) {
            const int nk = min(kSlab, tt.K - k0);
            __syncthreads();
            if (!tt.trans_a) {
                for (int e = t; e < R * kSlab; e += kThreads) {
                    int r = e % R, c = e / R;
                    As[r][c] = c < nk ? A[r + (long long)(k0 + c) * tt.lda] : 0.0;
                }
            } else {
                for (int e = t; e < R * kSlab; e += kThreads) {
                    int c = e % kSlab, r = e / kSlab;
                    As[r][c] = c < nk ? A[(long long)r * tt.lda + k0 + c] : 0.0;
                }
            }
            for (int e = t; e < kSlab * NB; e += kThreads) {
                int r = e % kSlab, c = e / kSlab;
                Bs[r][c] = (r < nk && c < nj) ? B[k0 + r + (long long)c * ldb] : 0.0;
            }
            __syncthreads();
            for (int c = g; c < kSlab; c += G) {
                double a = As[i][c];
#pragma unroll
                for (int j = 0; j < NB; ++j) acc[j] = fma(a, Bs[c][j], acc[j]);
            }
        }
    }
    __syncthreads();   // red aliases the staging buffers
#pragma unroll
    for (int j = 0; j < NB; ++j) red[t][j] = acc[j];
    __syncthreads();
    // Combine the G partial sums of each (row, col) and write back.
    for (int e = t; e < R * NB; e += kThreads) {
        int r = e % R, c = e / R;
        if (c >= nj) continue;
        double s = 0.0;
        for (int gg = 0; gg < G; ++gg) s += red[gg * R + r][c];
        double *y = Y + row0 + r + (long long)(j0 + c) * ldy;
        *y = beta == 0.0 ? alpha * s : fma(alpha, s, beta * *y);
    }
}

// ------------------------------------------------------------- utilities
__global__ void scale_kernel(double *Y, int rows, int cols, int ldy, double beta)
{
    long long n = (long long)rows * cols;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        int r = (int)(e % rows), c = (int)(e / rows);
        double *y = Y + r + (long long)c * ldy;
        *y = beta == 0.0 ? 0.0 : beta * *y;
    }
}

__global__ void transpose_kernel(const double *__restrict__ src, int rows, int cols, int lds,
                                 double *__restrict__ dst, int ldd)
{
    __shared__ double tile[32][33];
    int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        int r = bx + threadIdx.x, c = by + y;
        if (r < rows && c < cols) tile[y][threadIdx.x] = src[r + (long long)c * lds];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        int r = by + threadIdx.x, c = bx + y;   // dst is cols x rows
        if (r < cols && c < rows) dst[r + (long long)c * ldd] = tile[threadIdx.x][y];
    }
}

int scale_device(double *Y, int rows, int cols, int ldy, double beta, cudaStream_t st)
{
    if (rows <= 0 || cols <= 0 || beta == 1.0) return 0;
    long long n = (long long)rows * cols;
    int grid = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
    scale_kernel<<<grid, 256, 0, st>>>(Y, rows, cols, ldy, beta);
    DG_CUDA(cudaGetLastError());
    return 0;
}

// dst (cols x rows, ld ldd) := src^T (src rows x cols, ld lds)
int transpose_device(const double *src, int rows, int cols, int lds, double *dst, int ldd,
                     cudaStream_t st)
{
    if (rows <= 0 || cols <= 0) return 0;
    dim3 grid((rows + 31) / 32, (cols + 31) / 32), block(32, 8);
    transpose_kernel<<<grid, block, 0, st>>>(src, rows, cols, lds, dst, ldd);
    DG_CUDA(cudaGetLastError());
    return 0;
}

template <int NB>
static int launch_apply(Plan *p, const Schedule &S, int trans, int nrhs, double alpha,
                        const double *X, int ldx, double beta, double *Y, int ldy,
                        cudaStream_t st)
{
    double *T = p->work;
    double *partials = p->work + (size_t)p->total_rank * nrhs;
    const int ntile_rhs = (nrhs + NB - 1) / NB;
    if (!S.items.empty()) {
        dim3 g1((unsigned)S.items.size(), ntile_rhs);
        panel_kernel<NB><<<g1, kThreads, 0, st>>>(p->d_lr, S.d_items, S.d_poff, p->pool, X, ldx,
                                                   nrhs, trans, partials);
        DG_CUDA(cudaGetLastError());
        long long maxcnt = (long long)p->max_rank * nrhs;
        dim3 g2((unsigned)p->lr.size(), (unsigned)((maxcnt + 255) / 256));
        reduce_kernel<<<g2, 256, 0, st>>>(p->d_lr, S.d_poff, S.d_chunks, p->pool, partials, nrhs, T);
        DG_CUDA(cudaGetLastError());
    }
    const int ntiles = (int)S.tile_row0.size();
    if (ntiles > 0) {
        dim3 g3(ntiles, ntile_rhs);
        expand_kernel<NB><<<g3, kThreads, 0, st>>>(p->pool, S.d_terms, S.d_tile_row0,
                                                   S.d_tile_begin, p->d_lr, T, X, ldx, Y, ldy,
                                                   nrhs, S.tile_rows, alpha, beta);
        DG_CUDA(cudaGetLastError());
    }
    return 0;
}

int apply_device(Plan *p, int trans, int nrhs, double alpha, const double *X, int ldx,
                 double beta, double *Y, int ldy, cudaStream_t st, bool alpha0_squares_beta)
{
    if (nrhs <= 0 || p->m == 0) return 0;
    if (alpha == 0.0) {
        // Quick path of DPLR: y := beta*y (beta^2 for the vector apply, whose
        // alpha == 0 branch scales twice, src/dplrpmv.c:140-160).
        int rc = scale_device(Y, p->m, nrhs, ldy, beta, st);
        if (!rc && alpha0_squares_beta && beta != 0.0) rc = scale_device(Y, p->m, nrhs, ldy, beta, st);
        return rc;
    }
    const Schedule &S = p->sched[trans ? 1 : 0];
    size_t need = (size_t)(p->total_rank + S.partial_per_rhs) * nrhs;
    int rc = ensure_buffer(&p->work, &p->work_doubles, need);
    if (rc) return rc;
    if (nrhs >= 16) return launch_apply<16>(p, S, trans, nrhs, alpha, X, ldx, beta, Y, ldy, st);
    if (nrhs >= 8) return launch_apply<8>(p, S, trans, nrhs, alpha, X, ldx, beta, Y, ldy, st);
    if (nrhs >= 4) return launch_apply<4>(p, S, trans, nrhs, alpha, X, ldx, beta, Y, ldy, st);
    if (nrhs >= 2) return launch_apply<2>(p, S, trans, nrhs, alpha, X, ldx, beta, Y, ldy, st);
    return launch_apply<1>(p, S, trans, nrhs, alpha, X, ldx, beta, Y, ldy, st);
}

}  // namespace dg
