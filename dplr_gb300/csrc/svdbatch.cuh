// svdbatch.cuh -- truncated SVDs of many small low-rank blocks in one
// launch, one CTA per block, with no library call.
//
// A block U diag(sig) V^T (n x n, rank r <= min(n, kSvdBatchRank)) is
// recompressed as the library path does it (QR of U diag(sig) and of V, SVD
// of the r x r core Ru Rv^T, U' = Qu Uc, V' = Qv Vc), with the dense steps
// written here:
//   * Householder QR (the LAPACK dgeqrf / dlarfg convention: beta =
//     -sign(alpha) ||x||, v(0) = 1, tau = (beta - alpha) / beta), in place in
//     the block's staging copy; each column's reflector is applied by warps
//     over the remaining columns;
//   * one-sided (Hestenes) Jacobi on the core: columns p, q are rotated until
//     |c_p . c_q| <= tol ||c_p|| ||c_q|| for every pair (round-robin order,
//     rp / 2 disjoint pairs per round, at most kSvdSweeps sweeps); the
//     column norms are the singular values, the normalised columns the left
//     singular vectors of the core and the accumulated rotations its right
//     ones (Demmel and Veselic, "Jacobi's method is more accurate than QR",
//     SIAM J. Matrix Anal. Appl. 13 (1992));
//   * the reflectors applied to [Uc; 0] and [Vc; 0] (Q times the core's
//     vectors, reflectors in reverse order).
// Every loop is bounded; a core that has not converged after kSvdSweeps
// sweeps (random and appended cores of rank 64 took at most 23) is
// reported (info 1) and the block is left as it was.
#pragma once

namespace dg {

constexpr int kSvdBatchRank = 64;     // largest rank taking the batched path
constexpr int kSvdThreads = 256;
constexpr int kSvdWarps = kSvdThreads / 32;
constexpr int kSvdSweeps = 60;

// One block's staging area at `off` (doubles): U (n x r, ld n), V (n x r),
// Y (n x r, scratch), sig (r).  On return U holds U' (n x rank), Y holds V'
// and sig the singular values, largest first.
struct SvdBatchJob {
    long long off;
    int n, r;
    double eps;                       // singular values below it are dropped
};

// Shared memory of a CTA for ranks up to r, in bytes.
__host__ __device__ constexpr int svd_batch_smem(int r)
{
    return (3 * r * r + 4 * r + kSvdWarps) * 8 + (r + 2) * 4;
}

__device__ __forceinline__ double svd_warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum (max) over the CTA, the same value in every thread.  red: kSvdWarps
// doubles; the leading barrier keeps a previous call's readers ahead of
// this call's writers.
__device__ __forceinline__ double svd_block_sum(double v, double *red)
{
    v = svd_warp_sum(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kSvdWarps; ++w) s += red[w];
    return s;
}

__device__ __forceinline__ double svd_block_max(double v, double *red)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kSvdWarps; ++w) s = fmax(s, red[w]);
    return s;
}

// In-place Householder QR of A (n x r, ld n, r <= n): R on and above the
// diagonal, the reflectors' tails below it, their factors in tau.  A column
// whose remaining norm is below 2^-60 ||A||_F is left as it is (tau = 0):
// its tail is far below rounding, and reflecting it would cascade towards
// underflow when the columns repeat (as appended blocks do).
__device__ void svd_house_qr(double *A, int n, int r, double *tau, double *red)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    double fro = 0.0;
    for (long long e = t; e < (long long)n * r; e += kSvdThreads) fro = fma(A[e], A[e], fro);
    fro = sqrt(svd_block_sum(fro, red));
    const double negligible = 0x1p-60 * fro;
    for (int j = 0; j < r; ++j) {
        double *a = A + (long long)j * n;
        double amax = 0.0;
        for (int i = j + 1 + t; i < n; i += kSvdThreads) amax = fmax(amax, fabs(a[i]));
        amax = svd_block_max(amax, red);
        double ss = 0.0;
        if (amax > 0.0) {
            const double inv = 1.0 / amax;
            for (int i = j + 1 + t; i < n; i += kSvdThreads) {
                const double y = a[i] * inv;
                ss = fma(y, y, ss);
            }
        }
        ss = svd_block_sum(ss, red);
        const double alpha = a[j];
        const double nrm = hypot(alpha, amax * sqrt(ss));
        const bool reflect = amax > 0.0 && nrm > negligible;
        double tj = 0.0, scale = 0.0, beta = alpha;
        if (reflect) {
            beta = -copysign(nrm, alpha);
            tj = (beta - alpha) / beta;
            scale = 1.0 / (alpha - beta);
        }
        __syncthreads();                          // every thread has read a[j]
        if (reflect) {
            for (int i = j + 1 + t; i < n; i += kSvdThreads) a[i] *= scale;
            if (t == 0) a[j] = beta;
        }
        if (t == 0) tau[j] = tj;
        __syncthreads();
        if (tj != 0.0) {
            // H_j = I - tau v v^T on columns j+1 .. r-1, one warp per column
            for (int c = j + 1 + warp; c < r; c += kSvdWarps) {
                double *ac = A + (long long)c * n;
                double w = 0.0;
                for (int i = j + lane; i < n; i += 32) w = fma(i == j ? 1.0 : a[i], ac[i], w);
                w = svd_warp_sum(w) * tj;
                for (int i = j + lane; i < n; i += 32) ac[i] = fma(-w, i == j ? 1.0 : a[i], ac[i]);
            }
        }
        __syncthreads();
    }
}

// Y (n x nc, ld n) <- H_0 H_1 ... H_{r-1} Y with the reflectors of
// svd_house_qr.  A warp owns its columns for every reflector, so only the
// warp's own lanes need ordering between reflectors.
__device__ void svd_house_apply(const double *A, int n, int r, const double *tau, double *Y, int nc)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = warp; c < nc; c += kSvdWarps) {
        double *y = Y + (long long)c * n;
        for (int j = r - 1; j >= 0; --j) {
            const double tj = tau[j];
            if (tj == 0.0) continue;
            const double *a = A + (long long)j * n;
            double w = 0.0;
            for (int i = j + lane; i < n; i += 32) w = fma(i == j ? 1.0 : a[i], y[i], w);
            w = svd_warp_sum(w) * tj;
            for (int i = j + lane; i < n; i += 32) y[i] = fma(-w, i == j ? 1.0 : a[i], y[i]);
            __syncwarp();
        }
    }
}

// Pair pi of round k of a round-robin over rp (even) columns: element rp-1
// meets k, and k + i meets k - i (mod rp - 1).  Over rp - 1 rounds every
// pair meets once.
__device__ __forceinline__ void svd_pair(int pi, int k, int rp, int &p, int &q)
{
    const int m = rp - 1;
    if (pi == 0) {
        p = k;
        q = m;
    } else {
        p = (k + pi) % m;
        q = (k - pi + m) % m;
    }
}

__global__ void __launch_bounds__(kSvdThreads) svd_batch_kernel(const SvdBatchJob *__restrict__ jobs, int count,
                                                               double *__restrict__ stage, int *__restrict__ out)
{
    if ((int)blockIdx.x >= count) return;
    const SvdBatchJob jb = jobs[blockIdx.x];
    const int n = jb.n, r = jb.r, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    double *U = stage + jb.off, *V = U + (long long)n * r, *Y = V + (long long)n * r, *sig = Y + (long long)n * r;
    extern __shared__ double sm[];
    double *Jm = sm;                              // r x r: Ru, then the rotations
    double *Rv = Jm + r * r;                      // r x r
    double *C = Rv + r * r;                       // r x r: the core, then its rotated columns
    double *tau_u = C + r * r, *tau_v = tau_u + r, *sv = tau_v + r, *inv = sv + r, *red = inv + r;
    int *order = reinterpret_cast<int *>(red + kSvdWarps), *flag = order + r;

    // U diag(sig)
    for (long long e = t; e < (long long)n * r; e += kSvdThreads) U[e] *= sig[e / n];
    __syncthreads();
    svd_house_qr(U, n, r, tau_u, red);
    svd_house_qr(V, n, r, tau_v, red);
    for (int e = t; e < r * r; e += kSvdThreads) {
        const int i = e % r, l = e / r;
        Jm[e] = i <= l ? U[i + (long long)l * n] : 0.0;
        Rv[e] = i <= l ? V[i + (long long)l * n] : 0.0;
    }
    __syncthreads();
    // C = Ru Rv^T (both upper triangular)
    for (int e = t; e < r * r; e += kSvdThreads) {
        const int i = e % r, k = e / r;
        double s = 0.0;
        for (int l = max(i, k); l < r; ++l) s = fma(Jm[i + l * r], Rv[k + l * r], s);
        C[e] = s;
    }
    __syncthreads();
    for (int e = t; e < r * r; e += kSvdThreads) Jm[e] = (e % r) == (e / r) ? 1.0 : 0.0;
    __syncthreads();

    // one-sided Jacobi: C J -> columns orthogonal to tol.  Columns of norm
    // below r u ||C||_F are negligible (singular values at rounding level)
    // and take no rotation: the product C J stays exact, and rotations of
    // rounding noise would only slow the convergence.
    constexpr double u = 1.1102230246251565e-16;
    const double tol = 4.0 * r * u;
    double z2 = 0.0;
    for (int e = t; e < r * r; e += kSvdThreads) z2 = fma(C[e], C[e], z2);
    z2 = svd_block_sum(z2, red) * ((double)r * u) * ((double)r * u);
    const int rp = r + (r & 1);
    bool converged = false;
    for (int sweep = 0; sweep < kSvdSweeps && !converged; ++sweep) {
        if (t == 0) *flag = 0;
        __syncthreads();
        for (int k = 0; k < rp - 1; ++k) {
            for (int pi = warp; pi < rp / 2; pi += kSvdWarps) {
                int p, q;
                svd_pair(pi, k, rp, p, q);
                if (p >= r || q >= r) continue;
                double a = 0.0, b = 0.0, g = 0.0;
                for (int i = lane; i < r; i += 32) {
                    const double x = C[i + p * r], y = C[i + q * r];
                    a = fma(x, x, a);
                    b = fma(y, y, b);
                    g = fma(x, y, g);
                }
                a = svd_warp_sum(a);
                b = svd_warp_sum(b);
                g = svd_warp_sum(g);
                if (a <= z2 || b <= z2 || !(fabs(g) > tol * sqrt(a) * sqrt(b))) continue;
                const double zeta = (b - a) / (2.0 * g);
                const double tt = fabs(zeta) > 1e150 ? 0.5 / zeta
                                                     : copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double cs = 1.0 / sqrt(1.0 + tt * tt), sn = cs * tt;
                for (int i = lane; i < r; i += 32) {
                    const double x = C[i + p * r], y = C[i + q * r];
                    C[i + p * r] = cs * x - sn * y;
                    C[i + q * r] = sn * x + cs * y;
                    const double jp = Jm[i + p * r], jq = Jm[i + q * r];
                    Jm[i + p * r] = cs * jp - sn * jq;
                    Jm[i + q * r] = sn * jp + cs * jq;
                }
                if (lane == 0) *flag = 1;
            }
            __syncthreads();
        }
        converged = *flag == 0;
        __syncthreads();                          // every thread has read the flag
    }
    if (!converged) {
        if (t == 0) {
            out[2 * blockIdx.x] = r;
            out[2 * blockIdx.x + 1] = 1;
        }
        return;
    }
    // singular values (column norms), largest first (ties by column)
    for (int c = warp; c < r; c += kSvdWarps) {
        double s = 0.0;
        for (int i = lane; i < r; i += 32) s = fma(C[i + c * r], C[i + c * r], s);
        s = svd_warp_sum(s);
        if (lane == 0) sv[c] = sqrt(s);
    }
    __syncthreads();
    // a total order (NaN last), so that the positions are a permutation
    for (int c = t; c < r; c += kSvdThreads) {
        const double kc = isnan(sv[c]) ? -1.0 : sv[c];
        int pos = 0;
        for (int d = 0; d < r; ++d) {
            const double kd = isnan(sv[d]) ? -1.0 : sv[d];
            pos += kd > kc || (kd == kc && d < c);
        }
        order[pos] = c;
    }
    __syncthreads();
    int rank = 0;
    while (rank < r && !(sv[order[rank]] < jb.eps)) ++rank;
    for (int c = t; c < rank; c += kSvdThreads) inv[c] = sv[order[c]] > 0.0 ? 1.0 / sv[order[c]] : 0.0;
    __syncthreads();
    // U' = Qu [Uc; 0] in Y, then into U
    for (long long e = t; e < (long long)n * rank; e += kSvdThreads) {
        const int i = (int)(e % n), c = (int)(e / n);
        Y[e] = i < r ? C[i + order[c] * r] * inv[c] : 0.0;
    }
    __syncthreads();
    svd_house_apply(U, n, r, tau_u, Y, rank);
    __syncthreads();
    for (long long e = t; e < (long long)n * rank; e += kSvdThreads) U[e] = Y[e];
    __syncthreads();
    // V' = Qv [Vc; 0] in Y
    for (long long e = t; e < (long long)n * rank; e += kSvdThreads) {
        const int i = (int)(e % n), c = (int)(e / n);
        Y[e] = i < r ? Jm[i + order[c] * r] : 0.0;
    }
    __syncthreads();
    svd_house_apply(V, n, r, tau_v, Y, rank);
    for (int c = t; c < rank; c += kSvdThreads) sig[c] = sv[order[c]];
    if (t == 0) {
        out[2 * blockIdx.x] = rank;
        out[2 * blockIdx.x + 1] = 0;
    }
}

}  // namespace dg
