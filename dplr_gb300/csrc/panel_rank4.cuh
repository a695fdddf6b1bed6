// panel_rank4.cuh -- the FP64 panel P = F[r0:r0+len, 0:rank]^T X[rows, j0:j0+nj]
// of one chunk of a block of rank <= 4, shared by the panel kernel (apply.cu)
// and the persistent apply (persist.cu).
//
// The general panel gives each thread one rank column of a tile of at least
// 8, so a rank-2 block leaves three quarters of the FMAs on zero padding.
// Here thread t owns right-hand side j = t % NB and rows g, g + G, ... of
// each staged slab (G = blockDim / NB), with all of the block's ranks in
// registers: every FMA is live, whatever the rank.  The G row groups are
// summed by shuffles between the lanes of a warp that share j (lane offsets
// NB .. 16), then across warps in shared memory -- a fixed order, so results
// are deterministic.  Output layout as the other panels: P[k + j * rank].
#pragma once

namespace dg {

constexpr int kRank4 = 4;        // largest rank taking this path
constexpr int kRank4Slab = 128;  // rows staged per slab

// Shared memory needed, in doubles: the slab (rows x (4 + NB)) and the
// per-warp sums (warps x 4 x NB).
template <int NB>
__host__ __device__ constexpr int rank4_smem(int threads)
{
    return kRank4Slab * (kRank4 + NB) > (threads / 32) * kRank4 * NB ? kRank4Slab * (kRank4 + NB)
                                                                      : (threads / 32) * kRank4 * NB;
}

template <int NB, int R>
__device__ __forceinline__ void rank4_slab(const double *Fs, const double *Xs, int ns, int g, int G, int j,
                                           double (&acc)[kRank4])
{
#pragma unroll 4
    for (int r = g; r < ns; r += G) {
        const double x = Xs[r * NB + j];
#pragma unroll
        for (int k = 0; k < R; ++k) acc[k] = fma(Fs[r * kRank4 + k], x, acc[k]);
    }
}

// F: the block's factor (column-major, ld n); X column-major (ld ldx), the
// chunk's rows start at xrow0 + r0.  sm: rank4_smem<NB>(blockDim.x) doubles.
// Every thread of the block must call it (it synchronises the block).
template <int NB>
__device__ __forceinline__ void panel_rank4(const double *__restrict__ F, int n, int r0, int len, int rank,
                                            const double *__restrict__ X, long long ldx, int xrow0, int j0,
                                            int nj, double *__restrict__ P, double *sm)
{
    static_assert(NB >= 1 && NB <= 32 && (NB & (NB - 1)) == 0, "NB: a power of two up to 32");
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5, nw = T >> 5;
    const int j = t % NB, g = t / NB, G = T / NB;
    double *Fs = sm;                              // kRank4Slab x 4
    double *Xs = sm + kRank4Slab * kRank4;        // kRank4Slab x NB
    double acc[kRank4] = {0.0, 0.0, 0.0, 0.0};
    for (int s0 = 0; s0 < len; s0 += kRank4Slab) {
        const int ns = min(kRank4Slab, len - s0);
        __syncthreads();                          // the previous slab has been read
        for (int e = t; e < kRank4Slab * kRank4; e += T) {
            const int r = e % kRank4Slab, c = e / kRank4Slab;
            Fs[r * kRank4 + c] = (r < ns && c < rank) ? __ldg(F + (long long)c * n + r0 + s0 + r) : 0.0;
        }
        for (int e = t; e < kRank4Slab * NB; e += T) {
            const int r = e % kRank4Slab, c = e / kRank4Slab;
            Xs[r * NB + c] = (r < ns && c < nj) ? __ldg(X + (long long)(j0 + c) * ldx + xrow0 + r0 + s0 + r) : 0.0;
        }
        __syncthreads();
        switch (rank) {
        case 1: rank4_slab<NB, 1>(Fs, Xs, ns, g, G, j, acc); break;
        case 2: rank4_slab<NB, 2>(Fs, Xs, ns, g, G, j, acc); break;
        case 3: rank4_slab<NB, 3>(Fs, Xs, ns, g, G, j, acc); break;
        default: rank4_slab<NB, 4>(Fs, Xs, ns, g, G, j, acc); break;
        }
    }
    // lanes l and l ^ o (o = NB, 2 NB, ..., 16) hold the same j
#pragma unroll
    for (int k = 0; k < kRank4; ++k)
#pragma unroll
        for (int o = NB; o < 32; o <<= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    __syncthreads();                              // the sums alias the slab
    if (lane < NB)
#pragma unroll
        for (int k = 0; k < kRank4; ++k) sm[(warp * kRank4 + k) * NB + lane] = acc[k];
    __syncthreads();
    for (int e = t; e < rank * nj; e += T) {
        const int k = e % rank, jj = e / rank;
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += sm[(w * kRank4 + k) * NB + jj];
        P[k + (long long)(j0 + jj) * rank] = s;
    }
    __syncthreads();                              // sm is reused by the caller
}

}  // namespace dg
