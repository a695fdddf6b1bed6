// factor.cu -- recursive Woodbury factorisation and FP64 solves.
//
// For an H node with diagonal children A1, A2 and off-diagonal blocks
// ne = U1 S1 V1^T, sw = U2 S2 V2^T, DPLR's inverse (src/dplrinv.c:93-450)
// uses  A^-1 = D^-1 - D^-1 W (S^-1 + V~^T D^-1 W)^-1 V~^T D^-1  with
// D = diag(A1, A2), W = diag(U1, U2), V~^T = [[0, V1^T], [V2^T, 0]].
// Here the same identity is kept in factored form, without 1/sig:
//   Z  = D^-1 W          (panels Z1 = A1^-1 U1, Z2 = A2^-1 U2)
//   K  = I + S V~^T Z = [[I, S1 V1^T Z2], [S2 V2^T Z1, I]]
//   A^-1 b = z - Z K^-1 S V~^T z,       z = D^-1 b
// Its transpose A^-T = D^-T (I - V~ S K^-T Z^T) reuses the same factors:
// the transposed solve sweeps top-down, g -= V~ S K^-T Z^T g per level
// (root first, every node of a level at once), then applies the leaf
// inverses transposed; nothing per level is stored.  The explicit inverse
// also needs Zt = D^-T V~ (Zt1 = A2^-T V1, Zt2 = A1^-T V2, built with
// DPLR_GPU_FACTOR_TRANSPOSED by the same top-down sweep truncated to the
// deeper levels).
//
// Device layout: per H level l one m x r_l matrix Z_l (ld m; rows of the
// ne block of node p hold Z1(p), rows of its sw block hold Z2(p)), the
// same for Zt_l, one (r1+r2)^2 inverse K^-1 per node, and the explicit
// inverses of the dense leaves.  Solves sweep bottom-up: leaves, then the
// deepest H level to the root, each level as one panel / reduce /
// capacitance / update launch sequence over all of its nodes at once.
#include "factor.cuh"

#include <algorithm>
#include <cmath>

namespace dg {

static long long align32(long long x) { return (x + 31) & ~31LL; }

// ------------------------------------------------------------- kernels

// Batched explicit inverse by LU with partial pivoting (the algorithm of
// LAPACK dgetrf + dgetri that DPLR's dplrdinv calls, src/dplrinv.c:20-84),
// one CTA per matrix, in place in global memory; `work` holds an n x n
// row-major scratch per matrix at the same offset.  info[id] = 0 or the
// 1-based index of the first zero pivot.
__global__ void __launch_bounds__(256) lu_inverse_kernel(double *base, const long long *off,
                                                         const int *size, double *work, int *info)
{
    __shared__ int piv[1024];
    __shared__ double rv[256];
    __shared__ int ri[256];
    __shared__ int singular;
    const int id = blockIdx.x, tid = threadIdx.x, bs = blockDim.x;
    double *A = base + off[id];
    double *Wk = work + off[id];
    const int n = size[id];
    if (tid == 0) singular = 0;
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        double best = -1.0;
        int bi = j;
        for (int i = j + tid; i < n; i += bs) {
            double v = fabs(A[i + (long long)j * n]);
            if (v > best) { best = v; bi = i; }
        }
        rv[tid] = best;
        ri[tid] = bi;
        __syncthreads();
        for (int s = bs / 2; s > 0; s >>= 1) {
            if (tid < s) {
                double o = rv[tid + s];
                int oi = ri[tid + s];
                if (o > rv[tid] || (o == rv[tid] && oi < ri[tid])) { rv[tid] = o; ri[tid] = oi; }
            }
            __syncthreads();
        }
        if (tid == 0) {
            piv[j] = ri[0];
            if (rv[0] == 0.0 && singular == 0) singular = j + 1;
        }
        __syncthreads();
        const int p = piv[j];
        if (p != j)
            for (int c = tid; c < n; c += bs) {
                double t = A[j + (long long)c * n];
                A[j + (long long)c * n] = A[p + (long long)c * n];
                A[p + (long long)c * n] = t;
            }
        __syncthreads();
        const double d = A[j + (long long)j * n];
        if (d != 0.0) {
            const double inv = 1.0 / d;
            for (int i = j + 1 + tid; i < n; i += bs) A[i + (long long)j * n] *= inv;
        }
        __syncthreads();
        const int w = n - j - 1;
        const long long cnt = (long long)w * w;
        for (long long e = tid; e < cnt; e += bs) {
            int i = j + 1 + (int)(e % w), c = j + 1 + (int)(e / w);
            A[i + (long long)c * n] -= A[i + (long long)j * n] * A[j + (long long)c * n];
        }
        __syncthreads();
    }
    if (singular) {
        if (tid == 0) info[id] = singular;
        return;
    }
    // Column c of the inverse: solve L U x = P e_c; x kept row-major in Wk.
    for (int c = tid; c < n; c += bs) {
        for (int r = 0; r < n; ++r) Wk[c + (long long)r * n] = r == c ? 1.0 : 0.0;
        for (int j = 0; j < n; ++j) {
            int p = piv[j];
            if (p != j) {
                double t = Wk[c + (long long)j * n];
                Wk[c + (long long)j * n] = Wk[c + (long long)p * n];
                Wk[c + (long long)p * n] = t;
            }
        }
        for (int i = 0; i < n; ++i) {
            double xi = Wk[c + (long long)i * n];
            if (xi != 0.0)
                for (int r = i + 1; r < n; ++r) Wk[c + (long long)r * n] -= A[r + (long long)i * n] * xi;
        }
        for (int i = n - 1; i >= 0; --i) {
            double xi = Wk[c + (long long)i * n] / A[i + (long long)i * n];
            Wk[c + (long long)i * n] = xi;
            for (int r = 0; r < i; ++r) Wk[c + (long long)r * n] -= A[r + (long long)i * n] * xi;
        }
    }
    __syncthreads();
    for (long long e = tid; e < (long long)n * n; e += bs) {
        int r = (int)(e % n), c = (int)(e / n);
        A[r + (long long)c * n] = Wk[c + (long long)r * n];
    }
    if (tid == 0) info[id] = 0;
}

// The same inverse with the matrix in shared memory, for n <= kSmemInvMax
// (at most 206 KB): the LU is the same right-looking elimination, in the
// same order, as lu_inverse_kernel's; the inverse follows LAPACK dgetri's
// unblocked algorithm -- inv(U) in place column by column (dtrti2), then
// inv(A) = inv(U) inv(L) column by column from the last, then the pivots'
// column interchanges in reverse order -- with each column's dot products
// split over the threads.  The matrix goes back to global memory once.
constexpr int kSmemInvMax = 160;

__global__ void __launch_bounds__(256) lu_inverse_smem_kernel(double *base, const long long *off,
                                                              const int *size, int *info)
{
    extern __shared__ double S[];        // n x n (ld n), then n doubles of work
    __shared__ int piv[kSmemInvMax];
    __shared__ double rv[256];
    __shared__ int ri[256];
    __shared__ int singular;
    const int id = blockIdx.x, tid = threadIdx.x, bs = blockDim.x;
    double *A = base + off[id];
    const int n = size[id];
    double *wk = S + n * n;
    for (int e = tid; e < n * n; e += bs) S[e] = A[e];
    if (tid == 0) singular = 0;
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        double best = -1.0;
        int bi = j;
        for (int i = j + tid; i < n; i += bs) {
            const double v = fabs(S[i + j * n]);
            if (v > best) { best = v; bi = i; }
        }
        rv[tid] = best;
        ri[tid] = bi;
        __syncthreads();
        for (int s = bs / 2; s > 0; s >>= 1) {
            if (tid < s) {
                const double o = rv[tid + s];
                const int oi = ri[tid + s];
                if (o > rv[tid] || (o == rv[tid] && oi < ri[tid])) { rv[tid] = o; ri[tid] = oi; }
            }
            __syncthreads();
        }
        if (tid == 0) {
            piv[j] = ri[0];
            if (rv[0] == 0.0 && singular == 0) singular = j + 1;
        }
        __syncthreads();
        const int p = piv[j];
        if (p != j)
            for (int c = tid; c < n; c += bs) {
                const double t = S[j + c * n];
                S[j + c * n] = S[p + c * n];
                S[p + c * n] = t;
            }
        __syncthreads();
        const double d = S[j + j * n];
        if (d != 0.0) {
            const double inv = 1.0 / d;
            for (int i = j + 1 + tid; i < n; i += bs) S[i + j * n] *= inv;
        }
        __syncthreads();
        // trailing update: warps over columns, lanes over rows (no integer
        // division per element); every element gets the same updates, in the
        // same order, as in lu_inverse_kernel
        {
            const int lane = tid & 31, warp = tid >> 5, nwarp = bs >> 5;
            for (int c = j + 1 + warp; c < n; c += nwarp) {
                const double u = S[j + c * n];
                for (int i = j + 1 + lane; i < n; i += 32) S[i + c * n] -= S[i + j * n] * u;
            }
        }
        __syncthreads();
    }
    if (singular) {
        if (tid == 0) info[id] = singular;
        return;
    }
    // inv(U) in place: column j = -inv(U)[0:j, 0:j] U[0:j, j] / U[j, j]
    for (int j = 0; j < n; ++j) {
        for (int i = tid; i < j; i += bs) wk[i] = S[i + j * n];
        __syncthreads();
        const double ujj = 1.0 / S[j + j * n];
        for (int i = tid; i < j; i += bs) {
            double t = 0.0;
            for (int k = i; k < j; ++k) t = fma(S[i + k * n], wk[k], t);
            S[i + j * n] = -ujj * t;
        }
        __syncthreads();
        if (tid == 0) S[j + j * n] = ujj;
        __syncthreads();
    }
    // inv(A) inv(P)^T-free part: column j -= columns j+1.. times L's column j
    for (int j = n - 2; j >= 0; --j) {
        for (int i = j + 1 + tid; i < n; i += bs) {
            wk[i] = S[i + j * n];
            S[i + j * n] = 0.0;
        }
        __syncthreads();
        for (int r = tid; r < n; r += bs) {
            double t = S[r + j * n];
            for (int k = j + 1; k < n; ++k) t = fma(-S[r + k * n], wk[k], t);
            S[r + j * n] = t;
        }
        __syncthreads();
    }
    // the row interchanges of the LU become column interchanges
    for (int j = n - 2; j >= 0; --j) {
        const int p = piv[j];
        if (p != j)
            for (int r = tid; r < n; r += bs) {
                const double t = S[r + j * n];
                S[r + j * n] = S[r + p * n];
                S[r + p * n] = t;
            }
        __syncthreads();
    }
    for (int e = tid; e < n * n; e += bs) A[e] = S[e];
    if (tid == 0) info[id] = 0;
}

// Copy of every leaf into the inverse pool: one CTA per leaf.
__global__ void copy_leaves_kernel(const LeafDesc *__restrict__ leaves, const double *__restrict__ pool,
                                   const long long *__restrict__ dst_off, double *__restrict__ dst)
{
    const LeafDesc L = leaves[blockIdx.x];
    const double *src = pool + L.d;
    double *out = dst + dst_off[blockIdx.x];
    const long long cnt = (long long)L.b * L.b;
    for (long long e = threadIdx.x; e < cnt; e += blockDim.x) out[e] = src[e];
}

// Place one factor per block into the rows of a level right-hand side:
// dst[row0 + i, k] = src[i + k*n] for i < n, k < rank (ld of dst = m).
struct ScatterItem {
    long long src;
    int row0, n, rank;
};

__global__ void scatter_kernel(const ScatterItem *items, const double *src, double *dst, int ldd)
{
    const ScatterItem it = items[blockIdx.y];
    const long long cnt = (long long)it.n * it.rank;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < cnt;
         e += (long long)gridDim.x * blockDim.x) {
        int i = (int)(e % it.n), k = (int)(e / it.n);
        dst[it.row0 + i + (long long)k * ldd] = src[it.src + e];
    }
}

// K = I with off-diagonal blocks from T_ne (r1 x width) and T_sw (r2 x width):
// K[0:r1, r1:r] = T_ne[:, 0:r2],  K[r1:r, 0:r1] = T_sw[:, 0:r1].
__global__ void assemble_k_kernel(const CapItem *items, const double *T, int width, double *kbase)
{
    const CapItem c = items[blockIdx.x];
    const int r = c.r1 + c.r2;
    double *K = kbase + c.k;
    for (long long e = threadIdx.x; e < (long long)r * r; e += blockDim.x) {
        int i = (int)(e % r), j = (int)(e / r);
        double v = i == j ? 1.0 : 0.0;
        if (i < c.r1 && j >= c.r1) v = T[c.t1 * width + i + (long long)(j - c.r1) * c.r1];
        else if (i >= c.r1 && j < c.r1) v = T[c.t2 * width + (i - c.r1) + (long long)j * c.r2];
        K[e] = v;
    }
}

__global__ void zero_kernel(double *p, long long n)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x)
        p[e] = 0.0;
}

// ------------------------------------------------------------- helpers

template <class T>
static int to_device(const std::vector<T> &v, T **dst, long long *bytes)
{
    size_t n = std::max<size_t>(v.size(), 1);
    DG_ALLOC(dst, n * sizeof(T));
    *bytes += (long long)(n * sizeof(T));
    if (!v.empty()) DG_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

static int zero_device(double *p, long long n, cudaStream_t st)
{
    if (n <= 0) return 0;
    int grid = (int)std::min<long long>((n + 255) / 256, 152LL * 32);
    zero_kernel<<<grid, 256, 0, st>>>(p, n);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

// Inverts `count` matrices (offsets d_off, orders d_size; nmax the largest,
// host side) and writes each one's info to d_info[i]; asynchronous: the
// caller reads the infos back once the whole factorisation has run.  Up to
// kSmemInvMax the matrices are inverted in shared memory, else in place in
// global memory with a scratch of `span` doubles (freed in stream order).
static int batched_inverse(double *base, long long *d_off, int *d_size, int count, int nmax, int *d_info,
                           long long span, cudaStream_t st, double flops)
{
    if (count == 0) return 0;
    ProfScope ps("inverse", st, flops, 0.0);       // LU + inverse: 2 n^3 per matrix
    if (nmax <= kSmemInvMax) {
        const int smem = (nmax * nmax + nmax) * (int)sizeof(double);
        DG_CUDA(cudaFuncSetAttribute(lu_inverse_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        lu_inverse_smem_kernel<<<count, 256, smem, st>>>(base, d_off, d_size, d_info);
    } else {
        double *work = nullptr;
        if (cudaMallocAsync((void **)&work, std::max<long long>(span, 1) * sizeof(double), st) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "inverse: cannot allocate %lld doubles of scratch", span);
        lu_inverse_kernel<<<count, 256, 0, st>>>(base, d_off, d_size, work, d_info);
        cudaFreeAsync(work, st);
    }
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

static int ensure_work(Fact *F, const Plan *p, int nrhs)
{
    // T, W and partials for the widest level schedule.
    long long part = 0;
    for (const LevelOps &L : F->lv) part = std::max({part, L.n.partial_per_rhs, L.t.partial_per_rhs});
    size_t need = (size_t)(2 * p->total_rank + part) * std::max(nrhs, 1);
    return ensure_buffer(&F->work, &F->work_doubles, need);
}

// One sweep over the leaves and the H levels from `lowest` to the deepest
// (all of them for lowest = 0).  op N, bottom-up: Xo = leaf^-1 B, then per
// level from the deepest up: Xo -= Z K^-1 S V~^T Xo.  op T, top-down: a
// copy G of B takes G -= V~ S K^-T Z^T G per level from `lowest` down to
// the deepest, then Xo = leaf^-T G.  B and Xo are m x nrhs (ld ldb / ldx)
// and must not alias.
static int sweep(Plan *p, Fact *F, int trans, int lowest, const double *B, int ldb, double *Xo,
                 int ldx, int nrhs, cudaStream_t st)
{
    int rc = ensure_work(F, p, nrhs);
    if (rc) return rc;
    double *T = F->work;
    double *W = F->work + (size_t)p->total_rank * nrhs;
    double *partials = W + (size_t)p->total_rank * nrhs;
    if (!trans) {
        if ((rc = run_expand(F->leafN, F->leafinv, nullptr, B, ldb, Xo, ldx, nrhs, 1.0, 0.0, st))) return rc;
        for (int l = (int)F->lv.size() - 1; l >= lowest; --l) {
            const LevelOps &L = F->lv[l];
            if (L.width == 0) continue;
            if ((rc = run_panel(L.n, p->pool, Xo, ldx, nrhs, partials, st))) return rc;
            if ((rc = run_reduce(L.n, p->pool, partials, nrhs, T, st))) return rc;
            if ((rc = run_caps(L.n, F->kpool, nullptr, 0, T, W, nrhs, st))) return rc;
            if ((rc = run_expand(L.n, F->zpool, W, nullptr, 0, Xo, ldx, nrhs, -1.0, 1.0, st))) return rc;
        }
        return 0;
    }
    const int m = p->m;
    if ((rc = ensure_buffer(&F->gtr, &F->gtr_doubles, (size_t)m * nrhs))) return rc;
    double *G = F->gtr;
    DG_CUDA(cudaMemcpy2DAsync(G, (size_t)m * sizeof(double), B, (size_t)ldb * sizeof(double),
                              (size_t)m * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, st));
    for (int l = lowest; l < (int)F->lv.size(); ++l) {
        const LevelOps &L = F->lv[l];
        if (L.width == 0) continue;
        if ((rc = run_panel(L.t, F->zpool, G, m, nrhs, partials, st))) return rc;       // Z^T G
        if ((rc = run_reduce(L.t, nullptr, partials, nrhs, T, st))) return rc;
        if ((rc = run_caps(L.t, F->kpool, p->pool, 1, T, W, nrhs, st))) return rc;     // S K^-T
        if ((rc = run_expand(L.t, p->pool, W, nullptr, 0, G, m, nrhs, -1.0, 1.0, st))) return rc;   // V~
    }
    return run_expand(F->leafT, F->leafinv, nullptr, G, m, Xo, ldx, nrhs, 1.0, 0.0, st);
}

// ------------------------------------------------------------- schedules

static void build_level_schedules(Plan *p, Fact *F)
{
    const int CH = p->chunk_rows;
    const int R = tile_rows_for(p);
    const int m = p->m;
    for (size_t l = 0; l < F->lv.size(); ++l) {
        LevelOps &L = F->lv[l];
        for (int trans = 0; trans < 2; ++trans) {
            Schedule &S = trans ? L.t : L.n;
            long long poff = 0;
            int maxr = 0;
            for (int b : L.blocks) {
                const LRDesc &D = p->lr[b];
                if (D.rank == 0) continue;
                maxr = std::max(maxr, D.rank);
                int nch = (D.n + CH - 1) / CH;
                for (int c = 0; c < nch; ++c) {
                    PanelItem it;
                    if (!trans) {          // V_b^T x[col0 rows]
                        it.f = D.v;
                        it.n = D.n;
                        it.in0 = D.col0;
                    } else {               // Z_l[row0 rows]^T g[row0 rows] (Z_l: ld m, in zpool)
                        it.f = F->zoff[l] + D.row0;
                        it.n = m;
                        it.in0 = D.row0;
                    }
                    it.p = poff;
                    it.rank = D.rank;
                    it.r0 = c * CH;
                    it.len = std::min(CH, D.n - c * CH);
                    it.chunk = c;
                    S.items.push_back(it);
                }
                ReduceItem r;
                r.p = poff;
                r.t = D.toff;
                r.sig = trans ? -1 : D.sig;
                r.rank = D.rank;
                r.nch = nch;
                S.reduces.push_back(r);
                poff += (long long)nch * D.rank;
                // update tiles: op N, rows of the block with Z_l (ld m, in
                // zpool); op T, the block's column rows with its V (ld n,
                // in the factor pool)
                int out0 = trans ? D.col0 : D.row0;
                for (int t0 = out0; t0 < out0 + D.n; t0 += R) {
                    TileTerm tt;
                    tt.a = trans ? D.v + (t0 - D.col0) : F->zoff[l] + t0;
                    tt.b = D.toff;
                    tt.lda = trans ? D.n : m;
                    tt.K = D.rank;
                    tt.trans_a = 0;
                    tt.src = 0;
                    tt.ldb = D.rank;
                    tt.x_row0 = 0;
                    S.tile_row0.push_back(t0);
                    S.tile_begin.push_back((int)S.terms.size());
                    S.terms.push_back(tt);
                }
            }
            S.tile_begin.push_back((int)S.terms.size());
            S.partial_per_rhs = poff;
            S.t_per_rhs = p->total_rank;
            S.max_rank = maxr;
            S.tile_rows = R;
            S.nb_cap = p->nb_cap;
            for (int nd : L.nodes) {
                const HDesc &H = p->nodes[nd];
                const LRDesc &ne = p->lr[H.ne], &sw = p->lr[H.sw];
                if (ne.rank + sw.rank == 0) continue;
                CapItem c;
                c.k = F->koff[nd];
                c.t1 = ne.toff;
                c.t2 = sw.toff;
                c.s1 = ne.sig;
                c.s2 = sw.sig;
                c.r1 = ne.rank;
                c.r2 = sw.rank;
                S.caps.push_back(c);
            }
        }
    }
    // Leaf step: x[leaf rows] = op(Leaf^-1) b[leaf rows].
    for (int trans = 0; trans < 2; ++trans) {
        Schedule &S = trans ? F->leafT : F->leafN;
        S.tile_rows = R;
        S.nb_cap = p->nb_cap;
        for (size_t i = 0; i < p->leaves.size(); ++i) {
            const LeafDesc &Lf = p->leaves[i];
            for (int t0 = Lf.row0; t0 < Lf.row0 + Lf.b; t0 += R) {
                TileTerm tt;
                tt.b = 0;
                tt.lda = Lf.b;
                tt.K = Lf.b;
                tt.src = 1;
                tt.ldb = 0;
                tt.x_row0 = Lf.row0;
                tt.trans_a = trans;
                tt.a = F->leafoff[i] + (trans ? (long long)(t0 - Lf.row0) * Lf.b : (t0 - Lf.row0));
                S.tile_row0.push_back(t0);
                S.tile_begin.push_back((int)S.terms.size());
                S.terms.push_back(tt);
            }
        }
        S.tile_begin.push_back((int)S.terms.size());
    }
}

void factor_free(Plan *p)
{
    Fact *F = (Fact *)p->fact;
    if (!F) return;
    for (LevelOps &L : F->lv) {
        free_schedule(L.n);
        free_schedule(L.t);
    }
    free_schedule(F->leafN);
    free_schedule(F->leafT);
    cudaFree(F->zpool);
    cudaFree(F->ztpool);
    cudaFree(F->kpool);
    cudaFree(F->leafinv);
    cudaFree(F->d_koff);
    cudaFree(F->d_leafoff);
    cudaFree(F->d_ksize);
    cudaFree(F->d_leafsize);
    cudaFree(F->d_info);
    cudaFree(F->d_scat);
    cudaFree(F->d_inv_off);
    cudaFree(F->d_inv_size);
    cudaFree(F->work);
    cudaFree(F->gtr);
    cudaFree(F->rhs);
    cudaFree(F->vec);
    delete F;
    p->fact = nullptr;
}

// Build the level-r right-hand side: factor `which` (0: U, 1: V) of every
// block at level l placed at the block's rows (U: row0, V: col0).
static int level_rhs(Plan *p, Fact *F, int l, int which, cudaStream_t st)
{
    const int width = F->lv[l].width;
    int rc;
    if ((rc = zero_device(F->rhs, (long long)p->m * width, st))) return rc;
    const int cnt = F->scat_count[which][l];
    if (cnt == 0) return 0;
    dim3 g((unsigned)std::min(64, (F->scat_max[which][l] + 255) / 256), (unsigned)cnt);
    scatter_kernel<<<g, 256, 0, st>>>(F->d_scat + F->scat_begin[which][l], p->pool, F->rhs, p->m);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

// Everything of a factorisation that depends on the plan's structure only:
// offsets, device pools, the level schedules, the levels' scatter items and
// capacitance inverse lists.  Built once; refactorisations after a change
// of the values (the adjoint's every step) reuse it.
static int factor_layout(Plan *p, Fact *F, int flags)
{
    F->flags = flags;
    F->transposed = (flags & 1) != 0;
    F->key_chunk = p->chunk_rows;
    F->key_nb = p->nb_cap;
    const int nlev = p->levels;
    F->lv.resize(nlev);
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &D = p->lr[b];
        LevelOps &L = F->lv[D.level];
        L.blocks.push_back((int)b);
        L.width = std::max(L.width, D.rank);
    }
    for (size_t nd = 0; nd < p->nodes.size(); ++nd) F->lv[p->nodes[nd].level].nodes.push_back((int)nd);
    long long z = 0;
    int wmax = 1;
    for (int l = 0; l < nlev; ++l) {
        F->zoff.push_back(z);
        z += align32((long long)p->m * F->lv[l].width);
        wmax = std::max(wmax, F->lv[l].width);
    }
    F->zdoubles = z;
    std::vector<int> ksize(p->nodes.size());
    long long k = 0;
    for (size_t nd = 0; nd < p->nodes.size(); ++nd) {
        int r = p->lr[p->nodes[nd].ne].rank + p->lr[p->nodes[nd].sw].rank;
        F->koff.push_back(k);
        ksize[nd] = r;
        k += align32((long long)r * r);
    }
    F->kdoubles = k;
    std::vector<int> lsize(p->leaves.size());
    long long lo = 0;
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        F->leafoff.push_back(lo);
        lsize[i] = p->leaves[i].b;
        lo += align32((long long)lsize[i] * lsize[i]);
    }
    F->leafdoubles = lo;
    for (int r : ksize)
        if (r > 1024) return fail(DPLR_GPU_EINVAL, "capacitance order %d exceeds 1024", r);
    for (int b : lsize)
        if (b > 1024) return fail(DPLR_GPU_EINVAL, "leaf size %d exceeds 1024", b);

    int rc;
    auto alloc = [&](double **ptr, long long n) -> int {
        cudaError_t e = dev_malloc((void **)ptr, std::max<long long>(n, 1) * sizeof(double));
        if (e != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "factorisation: cannot allocate %lld doubles", n);
        F->bytes += std::max<long long>(n, 1) * 8;
        return 0;
    };
    if ((rc = alloc(&F->zpool, F->zdoubles))) return rc;
    if (F->transposed && (rc = alloc(&F->ztpool, F->zdoubles))) return rc;
    if ((rc = alloc(&F->kpool, F->kdoubles))) return rc;
    if ((rc = alloc(&F->leafinv, F->leafdoubles))) return rc;
    if ((rc = to_device(F->koff, &F->d_koff, &F->bytes)) || (rc = to_device(ksize, &F->d_ksize, &F->bytes)) ||
        (rc = to_device(F->leafoff, &F->d_leafoff, &F->bytes)) ||
        (rc = to_device(lsize, &F->d_leafsize, &F->bytes)))
        return rc;
    // one info slot per leaf, then one per node (each inverse writes its own)
    std::vector<int> zeros(p->leaves.size() + p->nodes.size() + 1, 0);
    if ((rc = to_device(zeros, &F->d_info, &F->bytes))) return rc;

    build_level_schedules(p, F);
    for (LevelOps &L : F->lv) {
        if ((rc = upload_schedule(L.n, &F->bytes)) || (rc = upload_schedule(L.t, &F->bytes))) return rc;
    }
    if ((rc = upload_schedule(F->leafN, &F->bytes)) || (rc = upload_schedule(F->leafT, &F->bytes)))
        return rc;

    // scatter items of every level (U, and V for the transposed panels)
    std::vector<ScatterItem> scat;
    for (int which = 0; which < 2; ++which) {
        F->scat_begin[which].assign(nlev, 0);
        F->scat_count[which].assign(nlev, 0);
        F->scat_max[which].assign(nlev, 0);
        for (int l = 0; l < nlev; ++l) {
            F->scat_begin[which][l] = (int)scat.size();
            for (int b : F->lv[l].blocks) {
                const LRDesc &D = p->lr[b];
                if (D.rank == 0) continue;
                ScatterItem it;
                it.src = which == 0 ? D.u : D.v;
                it.row0 = which == 0 ? D.row0 : D.col0;
                it.n = D.n;
                it.rank = D.rank;
                scat.push_back(it);
                F->scat_max[which][l] = std::max(F->scat_max[which][l], D.n * D.rank);
            }
            F->scat_count[which][l] = (int)scat.size() - F->scat_begin[which][l];
        }
    }
    if ((rc = to_device(scat, &F->d_scat, &F->bytes))) return rc;
    // capacitance inverses of every level
    std::vector<long long> ioff;
    std::vector<int> isize;
    F->inv_begin.assign(nlev, 0);
    F->inv_count.assign(nlev, 0);
    F->inv_max.assign(nlev, 0);
    for (int l = 0; l < nlev; ++l) {
        F->inv_begin[l] = (int)ioff.size();
        for (int nd : F->lv[l].nodes) {
            const HDesc &H = p->nodes[nd];
            int r = p->lr[H.ne].rank + p->lr[H.sw].rank;
            if (r == 0) continue;
            ioff.push_back(F->koff[nd]);
            isize.push_back(r);
            F->inv_ids.push_back(nd);
            F->inv_max[l] = std::max(F->inv_max[l], r);
        }
        F->inv_count[l] = (int)ioff.size() - F->inv_begin[l];
    }
    if ((rc = to_device(ioff, &F->d_inv_off, &F->bytes)) || (rc = to_device(isize, &F->d_inv_size, &F->bytes)))
        return rc;
    // scratch for the widest level, so that the numeric pass allocates nothing
    if ((rc = ensure_buffer(&F->rhs, &F->rhs_doubles, (size_t)p->m * wmax))) return rc;
    return ensure_work(F, p, wmax);
}

// The first nonzero info of the last numeric pass (leaves first, then the
// nodes in factorisation order), reported as DPLR does.
static int factor_check(Plan *p, Fact *F)
{
    const size_t nl = p->leaves.size();
    std::vector<int> info(nl + F->inv_ids.size());
    if (!info.empty())
        DG_CUDA(cudaMemcpy(info.data(), F->d_info, info.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < nl; ++i)
        if (info[i] != 0) {
            F->sing_kind = 1;
            F->sing_index = (int)i;
            F->sing_info = info[i];
            return fail(DPLR_GPU_ESINGULAR, "leaf %d is singular (zero pivot %d)", (int)i, info[i]);
        }
    for (int l = (int)F->lv.size() - 1; l >= 0; --l)
        for (int q = F->inv_begin[l]; q < F->inv_begin[l] + F->inv_count[l]; ++q)
            if (info[nl + q] != 0) {
                F->sing_kind = 2;
                F->sing_index = F->inv_ids[q];
                F->sing_info = info[nl + q];
                return fail(DPLR_GPU_ESINGULAR, "capacitance %d is singular (zero pivot %d)", q - F->inv_begin[l],
                            info[nl + q]);
            }
    return 0;
}

void factor_invalidate(Plan *p)
{
    if (p->fact) ((Fact *)p->fact)->valid = false;
}

Fact *factor_of(const Plan *p)
{
    Fact *F = (Fact *)p->fact;
    return F && F->valid ? F : nullptr;
}

int factor_build(Plan *p, int flags, cudaStream_t st)
{
    Fact *F = (Fact *)p->fact;
    if (!F || F->flags != flags || F->key_chunk != p->chunk_rows || F->key_nb != p->nb_cap) {
        factor_free(p);
        F = new Fact();
        p->fact = F;
        int rc0 = factor_layout(p, F, flags);
        if (rc0) {
            factor_free(p);
            return rc0;
        }
    }
    F->valid = false;
    F->sing_kind = 0;
    F->sing_index = -1;
    F->sing_info = 0;
    int rc;
    const int nlev = (int)F->lv.size();
    int lmax = 0;
    for (const LeafDesc &Lf : p->leaves) lmax = std::max(lmax, Lf.b);

    // Leaf inverses.
    if (!p->leaves.empty()) {
        copy_leaves_kernel<<<(unsigned)p->leaves.size(), 256, 0, st>>>(p->d_leaves, p->pool, F->d_leafoff,
                                                                      F->leafinv);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }
    double lfl = 0.0;
    for (const LeafDesc &Lf : p->leaves) lfl += 2.0 * Lf.b * Lf.b * (double)Lf.b;
    if ((rc = batched_inverse(F->leafinv, F->d_leafoff, F->d_leafsize, (int)p->leaves.size(), lmax,
                              F->d_info, F->leafdoubles, st, lfl)))
        return rc;

    // Levels bottom-up: Z_l (and Zt_l) through the already factored
    // deeper levels, then the capacitance matrices of level l.
    for (int l = nlev - 1; l >= 0; --l) {
        LevelOps &L = F->lv[l];
        if (L.width == 0) continue;
        if ((rc = level_rhs(p, F, l, 0, st))) return rc;
        if ((rc = sweep(p, F, 0, l + 1, F->rhs, p->m, F->zpool + F->zoff[l], p->m, L.width, st)))
            return rc;
        if (F->transposed) {
            if ((rc = level_rhs(p, F, l, 1, st))) return rc;
            if ((rc = sweep(p, F, 1, l + 1, F->rhs, p->m, F->ztpool + F->zoff[l], p->m, L.width, st)))
                return rc;
        }
        // S V^T Z_l for the level's blocks, then K per node.
        double *T = F->work;
        double *partials = F->work + (size_t)2 * p->total_rank * L.width;
        if ((rc = run_panel(L.n, p->pool, F->zpool + F->zoff[l], p->m, L.width, partials, st))) return rc;
        if ((rc = run_reduce(L.n, p->pool, partials, L.width, T, st))) return rc;
        if (!L.n.caps.empty()) {
            assemble_k_kernel<<<(unsigned)L.n.caps.size(), 256, 0, st>>>(L.n.d_caps, T, L.width,
                                                                         F->kpool);
            note_launch();
            DG_CUDA(cudaGetLastError());
            // invert this level's capacitance matrices (info slots after the leaves')
            const int b0 = F->inv_begin[l];
            double kfl = 0.0;
            for (int q = b0; q < b0 + F->inv_count[l]; ++q) {
                const HDesc &H = p->nodes[F->inv_ids[q]];
                const double r = p->lr[H.ne].rank + p->lr[H.sw].rank;
                kfl += 2.0 * r * r * r;
            }
            if ((rc = batched_inverse(F->kpool, F->d_inv_off + b0, F->d_inv_size + b0, F->inv_count[l],
                                      F->inv_max[l], F->d_info + p->leaves.size() + b0, F->kdoubles, st, kfl)))
                return rc;
        }
    }
    DG_CUDA(cudaStreamSynchronize(st));
    if ((rc = factor_check(p, F))) return rc;
    F->valid = true;
    return 0;
}

int factor_solve(Plan *p, int trans, int nrhs, const double *B, int ldb, double *X, int ldx,
                 cudaStream_t st)
{
    Fact *F = factor_of(p);
    if (!F) return fail(DPLR_GPU_ESTATE, "solve: plan is not factored");
    if (nrhs <= 0 || p->m == 0) return 0;
    return sweep(p, F, trans, 0, B, ldb, X, ldx, nrhs, st);
}

long long factor_bytes(const Plan *p)
{
    const Fact *F = (const Fact *)p->fact;
    if (!F) return 0;
    return F->bytes + (long long)(F->work_doubles + F->rhs_doubles + F->vec_doubles + F->gtr_doubles) * 8;
}

}  // namespace dg
