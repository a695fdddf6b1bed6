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

static int batched_inverse(double *base, long long *d_off, int *d_size, int count, int *d_info,
                           long long span, cudaStream_t st, const char *what, Fact *F = nullptr,
                           int kind = 0, const std::vector<int> *ids = nullptr)
{
    if (count == 0) return 0;
    double *work = nullptr;
    DG_ALLOC(&work, std::max<long long>(span, 1) * sizeof(double));
    lu_inverse_kernel<<<count, 256, 0, st>>>(base, d_off, d_size, work, d_info);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(work);
    if (e != cudaSuccess) return fail(DPLR_GPU_ECUDA, "%s inverse: %s", what, cudaGetErrorString(e));
    std::vector<int> info(count);
    DG_CUDA(cudaMemcpy(info.data(), d_info, count * sizeof(int), cudaMemcpyDeviceToHost));
    for (int i = 0; i < count; ++i)
        if (info[i] != 0) {
            if (F) {
                F->sing_kind = kind;
                F->sing_index = ids ? (*ids)[i] : i;
                F->sing_info = info[i];
            }
            return fail(DPLR_GPU_ESINGULAR, "%s %d is singular (zero pivot %d)", what, i, info[i]);
        }
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
    const LevelOps &L = F->lv[l];
    const int width = L.width;
    int rc;
    if ((rc = ensure_buffer(&F->rhs, &F->rhs_doubles, (size_t)p->m * width))) return rc;
    if ((rc = zero_device(F->rhs, (long long)p->m * width, st))) return rc;
    std::vector<ScatterItem> items;
    int maxcnt = 0;
    for (int b : L.blocks) {
        const LRDesc &D = p->lr[b];
        if (D.rank == 0) continue;
        ScatterItem it;
        it.src = which == 0 ? D.u : D.v;
        it.row0 = which == 0 ? D.row0 : D.col0;
        it.n = D.n;
        it.rank = D.rank;
        items.push_back(it);
        maxcnt = std::max(maxcnt, D.n * D.rank);
    }
    if (items.empty()) return 0;
    ScatterItem *d_items = nullptr;
    long long dummy = 0;
    if ((rc = to_device(items, &d_items, &dummy))) return rc;
    dim3 g((unsigned)std::min(64, (maxcnt + 255) / 256), (unsigned)items.size());
    scatter_kernel<<<g, 256, 0, st>>>(d_items, p->pool, F->rhs, p->m);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_items);
    if (e != cudaSuccess) return fail(DPLR_GPU_ECUDA, "level rhs: %s", cudaGetErrorString(e));
    return 0;
}

int factor_build(Plan *p, int flags, cudaStream_t st)
{
    factor_free(p);
    Fact *F = new Fact();
    p->fact = F;
    F->flags = flags;
    F->transposed = (flags & 1) != 0;
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
    for (int l = 0; l < nlev; ++l) {
        F->zoff.push_back(z);
        z += align32((long long)p->m * F->lv[l].width);
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
    std::vector<int> zeros(std::max(p->nodes.size(), p->leaves.size()) + 1, 0);
    if ((rc = to_device(zeros, &F->d_info, &F->bytes))) return rc;

    build_level_schedules(p, F);
    for (LevelOps &L : F->lv) {
        if ((rc = upload_schedule(L.n, &F->bytes)) || (rc = upload_schedule(L.t, &F->bytes))) return rc;
    }
    if ((rc = upload_schedule(F->leafN, &F->bytes)) || (rc = upload_schedule(F->leafT, &F->bytes)))
        return rc;

    // Leaf inverses.
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        const LeafDesc &Lf = p->leaves[i];
        DG_CUDA(cudaMemcpyAsync(F->leafinv + F->leafoff[i], p->pool + Lf.d,
                                sizeof(double) * Lf.b * Lf.b, cudaMemcpyDeviceToDevice, st));
    }
    if ((rc = batched_inverse(F->leafinv, F->d_leafoff, F->d_leafsize, (int)p->leaves.size(),
                              F->d_info, F->leafdoubles, st, "leaf", F, 1)))
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
        if ((rc = ensure_work(F, p, L.width))) return rc;
        double *T = F->work;
        double *partials = F->work + (size_t)2 * p->total_rank * L.width;
        if ((rc = run_panel(L.n, p->pool, F->zpool + F->zoff[l], p->m, L.width, partials, st))) return rc;
        if ((rc = run_reduce(L.n, p->pool, partials, L.width, T, st))) return rc;
        if (!L.n.caps.empty()) {
            assemble_k_kernel<<<(unsigned)L.n.caps.size(), 256, 0, st>>>(L.n.d_caps, T, L.width,
                                                                         F->kpool);
            note_launch();
            DG_CUDA(cudaGetLastError());
            // invert only this level's capacitance matrices
            std::vector<long long> offs;
            std::vector<int> sizes, ids;
            for (int nd : L.nodes) {
                const HDesc &H = p->nodes[nd];
                int r = p->lr[H.ne].rank + p->lr[H.sw].rank;
                if (r == 0) continue;
                offs.push_back(F->koff[nd]);
                sizes.push_back(r);
                ids.push_back(nd);
            }
            long long *d_o = nullptr;
            int *d_s = nullptr;
            long long dummy = 0;
            if ((rc = to_device(offs, &d_o, &dummy)) || (rc = to_device(sizes, &d_s, &dummy))) return rc;
            rc = batched_inverse(F->kpool, d_o, d_s, (int)offs.size(), F->d_info, F->kdoubles, st,
                                 "capacitance", F, 2, &ids);
            cudaFree(d_o);
            cudaFree(d_s);
            if (rc) return rc;
        }
    }
    DG_CUDA(cudaStreamSynchronize(st));
    return 0;
}

int factor_solve(Plan *p, int trans, int nrhs, const double *B, int ldb, double *X, int ldx,
                 cudaStream_t st)
{
    Fact *F = (Fact *)p->fact;
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
