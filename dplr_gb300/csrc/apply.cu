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
#include "panel_rank4.cuh"

#include <algorithm>
#include <cstdlib>
#include <cstring>

namespace dg {

constexpr int kThreads = 256;
constexpr int kSlab = 32;     // rows of X / factor staged per step
constexpr int kRankTile = 64; // ranks handled per pass of the panel kernel

// ----------------------------------------------------------------- panel
// One CTA per (item, rhs tile).  The rank tile RT (8, 16, 32 or 64 columns)
// follows the item's rank, so blocks of small rank do not pay for 64
// columns: thread t owns rank column k = t % RT and the rows t / RT (mod G),
// G = 256 / RT, of each slab of 4 G rows; the G row groups are summed
// through shared memory at the end.
template <int NB>
__global__ void __launch_bounds__(kThreads) panel_kernel(
    const PanelItem *__restrict__ items, const double *__restrict__ fbase,
    const double *__restrict__ X, int ldx, int nrhs, double *__restrict__ partials)
{
    // staging: at most 4 G (RT + 1) <= 1152 factor doubles and 4 G NB <= 128 NB
    // of X (RT = 8); the reduction: G RT NB = 256 NB
    constexpr int kStage = 1152 + 128 * NB;
    constexpr int kRed = kThreads * NB;
    __shared__ double sm[kStage > kRed ? kStage : kRed];
    static_assert(rank4_smem<NB>(kThreads) <= (kStage > kRed ? kStage : kRed), "rank <= 4 panel scratch");

    const PanelItem it = items[blockIdx.x];
    const double *F = fbase + it.f;
    const int j0 = blockIdx.y * NB;
    const int nj = min(NB, nrhs - j0);
    if (it.rank <= kRank4) {                  // every FMA live: threads own right-hand sides
        panel_rank4<NB>(F, it.n, it.r0, it.len, it.rank, X, ldx, it.in0, j0, nj,
                        partials + it.p * nrhs + (long long)it.chunk * it.rank * nrhs, sm);
        return;
    }
    int RT = 8;
    while (RT < it.rank && RT < kRankTile) RT <<= 1;
    const int G = kThreads / RT, S = 4 * G;
    double *Fs = sm;                     // S x (RT + 1)
    double *Xs = sm + S * (RT + 1);      // S x NB
    const int t = threadIdx.x;
    const int kk = t % RT, g = t / RT;
    double *P = partials + it.p * nrhs + (long long)it.chunk * it.rank * nrhs;

    for (int kt = 0; kt < it.rank; kt += RT) {
        const int nk = min(RT, it.rank - kt);
        double acc[NB];
#pragma unroll
        for (int j = 0; j < NB; ++j) acc[j] = 0.0;
        for (int s0 = 0; s0 < it.len; s0 += S) {
            const int ns = min(S, it.len - s0);
            __syncthreads();
            for (int e = t; e < S * RT; e += kThreads) {
                int r = e % S, c = e / S;
                Fs[r * (RT + 1) + c] = (r < ns && c < nk) ? F[(long long)(kt + c) * it.n + it.r0 + s0 + r] : 0.0;
            }
            for (int e = t; e < S * NB; e += kThreads) {
                int r = e % S, c = e / S;
                Xs[r * NB + c] = (r < ns && c < nj)
                                     ? X[(long long)(j0 + c) * ldx + it.in0 + it.r0 + s0 + r]
                                     : 0.0;
            }
            __syncthreads();
#pragma unroll 4
            for (int r = g; r < ns; r += G) {             // live rows only: short chunks stay cheap
                double f = Fs[r * (RT + 1) + kk];
#pragma unroll
                for (int j = 0; j < NB; ++j) acc[j] = fma(f, Xs[r * NB + j], acc[j]);
            }
        }
        __syncthreads();   // the reduction aliases the staging buffers
#pragma unroll
        for (int j = 0; j < NB; ++j) sm[(g * RT + kk) * NB + j] = acc[j];
        __syncthreads();
        for (int e = t; e < RT * NB; e += kThreads) {
            const int k2 = e % RT, j = e / RT;
            if (k2 < nk && j < nj) {
                double s = 0.0;
                for (int gg = 0; gg < G; ++gg) s += sm[(gg * RT + k2) * NB + j];
                P[(kt + k2) + (long long)(j0 + j) * it.rank] = s;
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------- one right-hand side
// With a single right-hand side the apply is a pair of matrix-vector products
// that stream every factor once: HBM- (and on GB300 FP64-FMA-) bound.  These
// kernels read the factors straight from global memory with 16-byte loads,
// several columns in flight per warp, and keep only x in shared memory.

constexpr int kPanel1MaxLen = 2048;

// Panel, 1 RHS: P[k] = F[r0:r0+len, k]^T x[in0+r0 : ...]; warp w handles
// columns k = w, w+8, ... four at a time; shuffle reduction per column.
__global__ void __launch_bounds__(kThreads) panel1_kernel(const PanelItem *__restrict__ items,
                                                          const double *__restrict__ fbase,
                                                          const double *__restrict__ X,
                                                          double *__restrict__ partials)
{
    __shared__ __align__(16) double xs[kPanel1MaxLen];
    const PanelItem it = items[blockIdx.x];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int r = t; r < it.len; r += kThreads) xs[r] = X[it.in0 + it.r0 + r];
    __syncthreads();
    const double *F = fbase + it.f + it.r0;
    double *P = partials + it.p + (long long)it.chunk * it.rank;
    const bool vec = ((it.n | it.r0 | it.len) & 1) == 0;
    for (int k0 = warp; k0 < it.rank; k0 += 4 * (kThreads / 32)) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        if (vec) {
            for (int r = 2 * lane; r < it.len; r += 64) {
                const double2 xv = *reinterpret_cast<const double2 *>(xs + r);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int k = k0 + c * (kThreads / 32);
                    if (k < it.rank) {
                        const double2 fv = __ldg(reinterpret_cast<const double2 *>(F + (long long)k * it.n + r));
                        acc[c] = fma(fv.x, xv.x, fma(fv.y, xv.y, acc[c]));
                    }
                }
            }
        } else {
            for (int r = lane; r < it.len; r += 32) {
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int k = k0 + c * (kThreads / 32);
                    if (k < it.rank) acc[c] = fma(__ldg(F + (long long)k * it.n + r), xs[r], acc[c]);
                }
            }
        }
        // butterfly reduction of the four column sums: two exchange rounds
        // leave lane l with the partial of column (l >> 3) & 3, three more
        // finish it (6 FP64 adds per lane instead of 20)
        {
            const bool hi16 = lane & 16, hi8 = lane & 8;
            const double s0 = hi16 ? acc[0] : acc[2], s1 = hi16 ? acc[1] : acc[3];
            double a0 = (hi16 ? acc[2] : acc[0]) + __shfl_xor_sync(0xffffffffu, s0, 16);
            double a1 = (hi16 ? acc[3] : acc[1]) + __shfl_xor_sync(0xffffffffu, s1, 16);
            // lanes < 16 now hold columns {0, 1}, lanes >= 16 columns {2, 3}
            const double t = hi8 ? a0 : a1;
            double v = (hi8 ? a1 : a0) + __shfl_xor_sync(0xffffffffu, t, 8);
            // lane l holds column 2*(l >= 16) + (l & 8 ? 1 : 0)
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            const int c = (hi16 ? 2 : 0) + (hi8 ? 1 : 0);
            const int k = k0 + c * (kThreads / 32);
            if ((lane & 7) == 0 && k < it.rank) P[k] = v;
        }
    }
}

// Expand, 1 RHS, column-major terms only: y[tile] = alpha * sum_terms
// A[tile, 0:K] b + beta y.  Thread (i, g) owns row i of the tile and the
// inner indices k == g (mod G); the G partial sums meet in shared memory.
__global__ void __launch_bounds__(kThreads) expand1_kernel(
    const double *__restrict__ abase, const TileTerm *__restrict__ terms, const int *__restrict__ tile_row0,
    const int *__restrict__ tile_begin, const double *__restrict__ T, const double *__restrict__ X,
    double *__restrict__ Y, int R, double alpha, double beta)
{
    __shared__ double red[kThreads];
    const int tile = blockIdx.x, row0 = tile_row0[tile];
    const int t = threadIdx.x, G = kThreads / R, i = t % R, g = t / R;
    double acc = 0.0, acc2 = 0.0;
    for (int q = tile_begin[tile]; q < tile_begin[tile + 1]; ++q) {
        const TileTerm tt = terms[q];
        const double *A = abase + tt.a + i;
        const double *B = tt.src == 0 ? T + tt.b : tt.src == 2 ? T + tt.b : X + tt.x_row0;
        int k = g;
        for (; k + G < tt.K; k += 2 * G) {
            acc = fma(__ldg(A + (long long)k * tt.lda), __ldg(B + k), acc);
            acc2 = fma(__ldg(A + (long long)(k + G) * tt.lda), __ldg(B + k + G), acc2);
        }
        if (k < tt.K) acc = fma(__ldg(A + (long long)k * tt.lda), __ldg(B + k), acc);
    }
    red[t] = acc + acc2;
    __syncthreads();
    if (t < R) {
        double s = 0.0;
        for (int gg = 0; gg < G; ++gg) s += red[gg * R + t];
        double *y = Y + row0 + t;
        *y = beta == 0.0 ? alpha * s : fma(alpha, s, beta * *y);
    }
}

// ---------------------------------------------------------------- reduce
// T[k, j] = sig[k] * sum_c P[c][k, j] (no scaling with a null sigbase);
// grid.x = reduce item.
__global__ void reduce_kernel(const ReduceItem *__restrict__ items,
                              const double *__restrict__ sigbase,
                              const double *__restrict__ partials, int nrhs,
                              double *__restrict__ T)
{
    const ReduceItem R = items[blockIdx.x];
    const long long cnt = (long long)R.rank * nrhs;
    const long long e = (long long)blockIdx.y * blockDim.x + threadIdx.x;
    if (e >= cnt) return;
    const int k = (int)(e % R.rank);
    const double *P = partials + R.p * nrhs + e;
    double s = 0.0;
    for (int c = 0; c < R.nch; ++c) s += P[(long long)c * cnt];
    T[R.t * nrhs + e] = (R.sig >= 0 && sigbase) ? sigbase[R.sig + k] * s : s;
}

// Few right-hand sides: the chunk sums of an element are spread over 8 warps
// (32 elements x 8 chunk groups per CTA) instead of one thread walking all
// chunks, whose dependent loads dominate when a block has hundreds of chunks.
__global__ void reduce_grouped_kernel(const ReduceItem *__restrict__ items, const double *__restrict__ sigbase,
                                      const double *__restrict__ partials, int nrhs, double *__restrict__ T)
{
    __shared__ double red[8][33];
    const ReduceItem R = items[blockIdx.x];
    const long long cnt = (long long)R.rank * nrhs;
    const int el = threadIdx.x & 31, grp = threadIdx.x >> 5;
    const long long e = (long long)blockIdx.y * 32 + el;
    double s = 0.0;
    if (e < cnt) {
        const double *P = partials + R.p * nrhs + e;
        for (int c = grp; c < R.nch; c += 8) s += P[(long long)c * cnt];
    }
    red[grp][el] = s;
    __syncthreads();
    if (grp == 0 && e < cnt) {
        double t = 0.0;
#pragma unroll
        for (int g = 0; g < 8; ++g) t += red[g][el];
        const int k = (int)(e % R.rank);
        T[R.t * nrhs + e] = (R.sig >= 0 && sigbase) ? sigbase[R.sig + k] * t : t;
    }
}

// ---------------------------------------------------------------- expand
// One CTA per (row tile, rhs tile).  Thread t owns tile row i = t % R and
// the inner indices k == t/R (mod G), G = 256/R; partial sums of the G
// groups are combined through shared memory before the write-back.
template <int NB>
__global__ void __launch_bounds__(kThreads) expand_kernel(
    const double *__restrict__ abase, const TileTerm *__restrict__ terms,
    const int *__restrict__ tile_row0, const int *__restrict__ tile_begin,
    const double *__restrict__ T, const double *__restrict__ X, int ldx, double *__restrict__ Y,
    int ldy, int nrhs, int R, double alpha, double beta)
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
        const double *A = abase + tt.a;
        const double *B;
        long long ldb;
        if (tt.src == 0) {
            B = T + tt.b * nrhs + (long long)j0 * tt.ldb;
            ldb = tt.ldb;
        } else if (tt.src == 2) {
            B = T + tt.b + (long long)j0 * tt.ldb;
            ldb = tt.ldb;
        } else {
            B = X + tt.x_row0 + (long long)j0 * ldx;
            ldb = ldx;
        }
        // K slabs of up to kSlab: only the nk live columns are staged and
        // multiplied, so terms of small rank cost what they need
        for (int k0 = 0; k0 < tt.K; k0 += kSlab) {
            const int nk = min(kSlab, tt.K - k0);
            __syncthreads();
            if (!tt.trans_a) {
                for (int e = t; e < R * nk; e += kThreads) {
                    int r = e % R, c = e / R;
                    As[r][c] = A[r + (long long)(k0 + c) * tt.lda];
                }
            } else {
                for (int e = t; e < R * nk; e += kThreads) {
                    int c = e % nk, r = e / nk;
                    As[r][c] = A[(long long)r * tt.lda + k0 + c];
                }
            }
            for (int e = t; e < nk * NB; e += kThreads) {
                int r = e % nk, c = e / nk;
                Bs[r][c] = c < nj ? B[k0 + r + (long long)c * ldb] : 0.0;
            }
            __syncthreads();
            for (int c = g; c < nk; c += G) {
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

// ----------------------------------------------------------- capacitance
// W[i, j] = s_i * sum_k op(Kinv)[i, k] * [T1; T2][k, j] for one H node
// (s_i = 1 unless scaled); grid (node, rhs tile), thread per (i, j-group).
template <int NB>
__global__ void __launch_bounds__(kThreads) cap_kernel(
    const CapItem *__restrict__ items, const double *__restrict__ kbase,
    const double *__restrict__ sigbase, int trans, int scaled, const double *__restrict__ T,
    double *__restrict__ W, int nrhs)
{
    constexpr int KC = 256;            // rows of [T1; T2] staged per pass
    __shared__ double Ts[KC][NB];
    const CapItem c = items[blockIdx.x];
    const int r = c.r1 + c.r2;
    const int j0 = blockIdx.y * NB;
    const int nj = min(NB, nrhs - j0);
    const double *K = kbase + c.k;
    // Each thread owns output rows i = tid, tid + 256, ... (at most 4).
    double acc[4][NB];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int j = 0; j < NB; ++j) acc[q][j] = 0.0;
    for (int k0 = 0; k0 < r; k0 += KC) {
        const int nk = min(KC, r - k0);
        __syncthreads();
        for (int e = threadIdx.x; e < KC * NB; e += blockDim.x) {
            int k = e % KC, j = e / KC;
            double v = 0.0;
            if (j < nj && k < nk) {
                int kk = k0 + k;
                v = kk < c.r1 ? T[c.t1 * nrhs + kk + (long long)(j0 + j) * c.r1]
                              : T[c.t2 * nrhs + (kk - c.r1) + (long long)(j0 + j) * c.r2];
            }
            Ts[k][j] = v;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = threadIdx.x + q * blockDim.x;
            if (i >= r) break;
            for (int k = 0; k < nk; ++k) {
                const int kk = k0 + k;
                double a = trans ? K[kk + (long long)i * r] : K[i + (long long)kk * r];
#pragma unroll
                for (int j = 0; j < NB; ++j) acc[q][j] = fma(a, Ts[k][j], acc[q][j]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = threadIdx.x + q * blockDim.x;
        if (i >= r) break;
        double s = 1.0;
        if (scaled) s = i < c.r1 ? sigbase[c.s1 + i] : sigbase[c.s2 + i - c.r1];
        for (int j = 0; j < nj; ++j) {
            double *w = i < c.r1 ? W + c.t1 * nrhs + i + (long long)(j0 + j) * c.r1
                                 : W + c.t2 * nrhs + (i - c.r1) + (long long)(j0 + j) * c.r2;
            *w = s * acc[q][j];
        }
    }
}

// Capacitance of small nodes (order r <= 64): one CTA per (node, 64
// right-hand sides); thread (i, g) owns row i and the 16 columns of group g,
// [T1; T2] for the 64 columns staged in shared memory.  Same arithmetic as
// cap_kernel (one FMA chain per output over k), with every thread busy.
__global__ void __launch_bounds__(kThreads) cap_small_kernel(
    const CapItem *__restrict__ items, const double *__restrict__ kbase,
    const double *__restrict__ sigbase, int trans, int scaled, const double *__restrict__ T,
    double *__restrict__ W, int nrhs)
{
    __shared__ double Ts[64][65];
    const CapItem c = items[blockIdx.x];
    const int r = c.r1 + c.r2;
    const int j0 = blockIdx.y * 64;
    const int nj = min(64, nrhs - j0);
    const double *K = kbase + c.k;
    for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
        const int k = e % 64, j = e / 64;
        double v = 0.0;
        if (k < r && j < nj)
            v = k < c.r1 ? T[c.t1 * nrhs + k + (long long)(j0 + j) * c.r1]
                         : T[c.t2 * nrhs + (k - c.r1) + (long long)(j0 + j) * c.r2];
        Ts[j][k] = v;
    }
    __syncthreads();
    const int i = threadIdx.x & 63, g = threadIdx.x >> 6;
    if (i >= r) return;
    double acc[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) acc[u] = 0.0;
    for (int k = 0; k < r; ++k) {
        const double a = trans ? K[k + (long long)i * r] : K[i + (long long)k * r];
#pragma unroll
        for (int u = 0; u < 16; ++u) acc[u] = fma(a, Ts[g * 16 + u][k], acc[u]);
    }
    double s = 1.0;
    if (scaled) s = i < c.r1 ? sigbase[c.s1 + i] : sigbase[c.s2 + i - c.r1];
    for (int u = 0; u < 16; ++u) {
        const int j = g * 16 + u;
        if (j >= nj) break;
        double *w = i < c.r1 ? W + c.t1 * nrhs + i + (long long)(j0 + j) * c.r1
                             : W + c.t2 * nrhs + (i - c.r1) + (long long)(j0 + j) * c.r2;
        *w = s * acc[u];
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
    note_launch();
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
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

static int pick_nb(int nrhs, int cap = 16)
{
    const int nb = nrhs >= 16 ? 16 : nrhs >= 8 ? 8 : nrhs >= 4 ? 4 : nrhs >= 2 ? 2 : 1;
    return std::min(nb, std::max(cap, 1));
}

#define DG_DISPATCH_NB(nb, CALL)                                                   \
    switch (nb) {                                                                  \
    case 16: { constexpr int NB = 16; CALL; } break;                               \
    case 8: { constexpr int NB = 8; CALL; } break;                                 \
    case 4: { constexpr int NB = 4; CALL; } break;                                 \
    case 2: { constexpr int NB = 2; CALL; } break;                                 \
    default: { constexpr int NB = 1; CALL; } break;                                \
    }

int run_panel(const Schedule &S, const double *fbase, const double *X, int ldx, int nrhs,
              double *partials, cudaStream_t st)
{
    if (S.items.empty() || nrhs <= 0) return 0;
    const int nb = pick_nb(nrhs, S.nb_cap);
    dim3 g((unsigned)S.items.size(), (unsigned)((nrhs + nb - 1) / nb));
    double fl = 0, by = 0;
    for (const PanelItem &it : S.items) {
        fl += 2.0 * it.len * it.rank * nrhs;
        by += 8.0 * ((double)it.len * it.rank + (double)it.len * nrhs + (double)it.rank * nrhs);
    }
    ProfScope ps("panel", st, fl, by);
    if (nrhs == 1 && S.max_len <= kPanel1MaxLen) {
        panel1_kernel<<<(unsigned)S.items.size(), kThreads, 0, st>>>(S.d_items, fbase, X, partials);
        note_launch();
        DG_CUDA(cudaGetLastError());
        return 0;
    }
    DG_DISPATCH_NB(nb, (panel_kernel<NB><<<g, kThreads, 0, st>>>(S.d_items, fbase, X, ldx, nrhs,
                                                                  partials)));
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

int run_reduce(const Schedule &S, const double *sigbase, const double *partials, int nrhs,
               double *T, cudaStream_t st)
{
    if (S.reduces.empty() || nrhs <= 0 || S.max_rank <= 0) return 0;
    long long maxcnt = (long long)S.max_rank * nrhs;
    dim3 g((unsigned)S.reduces.size(), (unsigned)((maxcnt + 255) / 256));
    double fl = 0, by = 0;
    for (const ReduceItem &r : S.reduces) {
        fl += (double)r.nch * r.rank * nrhs;
        by += 8.0 * (r.nch + 1.0) * r.rank * nrhs;
    }
    ProfScope ps("reduce", st, fl, by);
    if (nrhs < 8) {
        const dim3 g2((unsigned)S.reduces.size(), (unsigned)((maxcnt + 31) / 32));
        reduce_grouped_kernel<<<g2, 256, 0, st>>>(S.d_reduces, sigbase, partials, nrhs, T);
        note_launch();
        DG_CUDA(cudaGetLastError());
        return 0;
    }
    reduce_kernel<<<g, 256, 0, st>>>(S.d_reduces, sigbase, partials, nrhs, T);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

int run_expand(const Schedule &S, const double *abase, const double *T, const double *X, int ldx,
               double *Y, int ldy, int nrhs, double alpha, double beta, cudaStream_t st)
{
    const int ntiles = (int)S.tile_row0.size();
    if (ntiles == 0 || nrhs <= 0) return 0;
    const int nb = pick_nb(nrhs, S.nb_cap);
    dim3 g(ntiles, (unsigned)((nrhs + nb - 1) / nb));
    double fl = 0, by = 8.0 * ntiles * S.tile_rows * nrhs * (beta == 0.0 ? 1.0 : 2.0);
    for (const TileTerm &t : S.terms) {
        fl += 2.0 * S.tile_rows * t.K * nrhs;
        by += 8.0 * ((double)S.tile_rows * t.K + (double)t.K * nrhs);
    }
    ProfScope ps("expand", st, fl, by);
    note_launch();
    if (nrhs == 1 && !S.has_row_major) {
        expand1_kernel<<<ntiles, kThreads, 0, st>>>(abase, S.d_terms, S.d_tile_row0, S.d_tile_begin, T, X, Y,
                                                    S.tile_rows, alpha, beta);
        DG_CUDA(cudaGetLastError());
        return 0;
    }
    DG_DISPATCH_NB(nb, (expand_kernel<NB><<<g, kThreads, 0, st>>>(
                           abase, S.d_terms, S.d_tile_row0, S.d_tile_begin, T, X, ldx, Y, ldy,
                           nrhs, S.tile_rows, alpha, beta)));
    DG_CUDA(cudaGetLastError());
    return 0;
}

int run_cap_list(const std::vector<CapItem> &caps, const CapItem *d_caps, const double *kbase, const double *sigbase,
                 int trans, const double *T, double *W, int nrhs, cudaStream_t st)
{
    if (caps.empty() || nrhs <= 0) return 0;
    for (const CapItem &c : caps)
        if (c.r1 + c.r2 > 4 * kThreads)
            return fail(DPLR_GPU_EINVAL, "capacitance of order %d exceeds %d", c.r1 + c.r2,
                        4 * kThreads);
    const int nb = std::min(pick_nb(nrhs), 8);
    dim3 g((unsigned)caps.size(), (unsigned)((nrhs + nb - 1) / nb));
    const int scaled = sigbase != nullptr;
    int rmax = 0;
    for (const CapItem &c : caps) rmax = std::max(rmax, c.r1 + c.r2);
    double fl = 0, by = 0;
    for (const CapItem &c : caps) {
        double r = c.r1 + c.r2;
        fl += 2.0 * r * r * nrhs;
        by += 8.0 * (r * r + 2.0 * r * nrhs);
    }
    ProfScope ps("capacitance", st, fl, by);
    note_launch();
    if (rmax <= 64 && nrhs >= 16) {
        cap_small_kernel<<<dim3((unsigned)caps.size(), (unsigned)((nrhs + 63) / 64)), kThreads, 0, st>>>(
            d_caps, kbase, sigbase, trans, scaled, T, W, nrhs);
        DG_CUDA(cudaGetLastError());
        return 0;
    }
    switch (nb) {
    case 8: cap_kernel<8><<<g, kThreads, 0, st>>>(d_caps, kbase, sigbase, trans, scaled, T, W, nrhs); break;
    case 4: cap_kernel<4><<<g, kThreads, 0, st>>>(d_caps, kbase, sigbase, trans, scaled, T, W, nrhs); break;
    case 2: cap_kernel<2><<<g, kThreads, 0, st>>>(d_caps, kbase, sigbase, trans, scaled, T, W, nrhs); break;
    default: cap_kernel<1><<<g, kThreads, 0, st>>>(d_caps, kbase, sigbase, trans, scaled, T, W, nrhs); break;
    }
    DG_CUDA(cudaGetLastError());
    return 0;
}

int run_caps(const Schedule &S, const double *kbase, const double *sigbase, int trans, const double *T, double *W,
             int nrhs, cudaStream_t st)
{
    return run_cap_list(S.caps, S.d_caps, kbase, sigbase, trans, T, W, nrhs, st);
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
    if (pairs_usable(p, trans, nrhs)) return pairs_apply(p, alpha, X, beta, Y, st);
    // one persistent launch unless DPLR_GB300_APPLY=launches asks for the
    // three-launch form (panel, reduce, expand)
    // three launches when the autotuner found them faster for this plan
    // (many tiny blocks), or when DPLR_GB300_APPLY=launches asks for them
    const char *mode = getenv("DPLR_GB300_APPLY");
    const bool launches = mode ? !strcmp(mode, "launches") : p->apply_launches != 0;
    if (!launches && persist_usable(p, trans, nrhs))
        return persist_apply(p, trans, nrhs, alpha, X, ldx, beta, Y, ldy, st);
    const Schedule &S = p->sched[trans ? 1 : 0];
    size_t need = (size_t)(S.t_per_rhs + S.partial_per_rhs) * nrhs;
    int rc = ensure_buffer(&p->work, &p->work_doubles, need);
    if (rc) return rc;
    double *T = p->work;
    double *partials = p->work + (size_t)S.t_per_rhs * nrhs;
    if ((rc = run_panel(S, p->pool, X, ldx, nrhs, partials, st))) return rc;
    if ((rc = run_reduce(S, p->pool, partials, nrhs, T, st))) return rc;
    return run_expand(S, p->pool, T, X, ldx, Y, ldy, nrhs, alpha, beta, st);
}

}  // namespace dg
