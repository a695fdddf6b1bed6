// grad.cu -- adjoint of the PLR product with respect to the stored factors,
// and access to the plan's factor pool.
//
// For a product Y = A X (op N) and an output cotangent DY, the derivative
// of <DY, A X> with respect to the factors of a low-rank block
// A_b = U diag(sig) V^T (rows R, columns C of the block) is
//     dU   = DY_R (sig o V^T X_C)^T,       dV = X_C (sig o U^T DY_R)^T,
//     dsig = sum_j (U^T DY_R)_kj (V^T X_C)_kj,
// and for a dense leaf D (rows and columns R): dD = DY_R X_R^T.  For the
// solve X = A^-1 B with cotangent G, the same projection applies to
// dA = -(A^-T G) X^T.  The panels V^T X_C and U^T DY_R are the apply's own
// panel/reduce phases (op N and op T schedules) without the sig scaling;
// one outer-product kernel then writes every block's gradient, in the
// layout of the factor pool, in one launch.
#include "internal.cuh"
#include "sliced.cuh"
#include "factor.cuh"

#include <algorithm>
#include <vector>

namespace dg {

namespace {

// One output chunk: G[out + i + k ldo] += alpha * sum_j A[a_row0 + i, j] B(k, j)
// (times sig[k] when sig >= 0), i < rows, k < cols.
struct GradItem {
    long long out;
    long long b_off;       // b_src 0/2: T offset / nrhs (ld cols); 1: first X row
    long long sig;         // pool offset of sig, or -1
    int ldo, rows, cols;
    int a_row0;
    int a_src;             // 0: DY, 1: X
    int b_src;             // 0: V^T X panels, 1: X rows, 2: U^T DY panels
};

struct Grad {
    std::vector<GradItem> items;
    GradItem *d_items = nullptr;
    std::vector<int> sig_blocks;     // LR blocks with rank > 0
    int *d_sig_blocks = nullptr;
};

__global__ void grad_outer_kernel(const GradItem *__restrict__ items, const double *__restrict__ X, int ldx,
                                  const double *__restrict__ DY, int ldy, const double *__restrict__ TN,
                                  const double *__restrict__ TT, const double *__restrict__ pool, int nrhs,
                                  double alpha, double *__restrict__ G)
{
    const GradItem it = items[blockIdx.x];
    const double *A = it.a_src == 0 ? DY : X;
    const int lda = it.a_src == 0 ? ldy : ldx;
    const long long cnt = (long long)it.rows * it.cols;
    for (long long e = threadIdx.x; e < cnt; e += blockDim.x) {
        const int i = (int)(e % it.rows), k = (int)(e / it.rows);
        double acc = 0.0;
        if (it.b_src == 1) {
            for (int j = 0; j < nrhs; ++j)
                acc = fma(A[it.a_row0 + i + (long long)j * lda], X[it.b_off + k + (long long)j * ldx], acc);
        } else {
            const double *T = (it.b_src == 0 ? TN : TT) + it.b_off * nrhs + k;
            for (int j = 0; j < nrhs; ++j)
                acc = fma(A[it.a_row0 + i + (long long)j * lda], T[(long long)j * it.cols], acc);
        }
        if (it.sig >= 0) acc *= pool[it.sig + k];
        G[it.out + i + (long long)k * it.ldo] += alpha * acc;
    }
}

// dsig[k] += alpha * sum_j TT[k, j] TN[k, j]; one thread per (block, k).
__global__ void grad_sig_kernel(const int *__restrict__ blocks, int nblocks, const LRDesc *__restrict__ lr,
                                const double *__restrict__ TN, const double *__restrict__ TT, int nrhs,
                                double alpha, double *__restrict__ G)
{
    const int b = blockIdx.x;
    if (b >= nblocks) return;
    const LRDesc L = lr[blocks[b]];
    for (int k = threadIdx.x; k < L.rank; k += blockDim.x) {
        const double *tn = TN + (long long)L.toff * nrhs + k, *tt = TT + (long long)L.toff * nrhs + k;
        double acc = 0.0;
        for (int j = 0; j < nrhs; ++j) acc = fma(tn[(long long)j * L.rank], tt[(long long)j * L.rank], acc);
        G[L.sig + k] += alpha * acc;
    }
}

int grad_build(Plan *p, Grad **out)
{
    Grad *g = new Grad();
    const int CH = 1024;
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        if (L.rank == 0 || L.n == 0) continue;
        g->sig_blocks.push_back((int)b);
        for (int r0 = 0; r0 < L.n; r0 += CH) {
            const int rows = std::min(CH, L.n - r0);
            // dU rows R: DY_R times (sig o V^T X_C)
            g->items.push_back(GradItem{L.u + r0, L.toff, L.sig, L.n, rows, L.rank, L.row0 + r0, 0, 0});
            // dV rows C: X_C times (sig o U^T DY_R)
            g->items.push_back(GradItem{L.v + r0, L.toff, L.sig, L.n, rows, L.rank, L.col0 + r0, 1, 2});
        }
    }
    for (const LeafDesc &L : p->leaves) {
        for (int r0 = 0; r0 < L.b; r0 += CH) {
            const int rows = std::min(CH, L.b - r0);
            g->items.push_back(GradItem{L.d + r0, L.row0, -1, L.b, rows, L.b, L.row0 + r0, 0, 1});
        }
    }
    const size_t ib = std::max<size_t>(g->items.size(), 1) * sizeof(GradItem);
    const size_t sb = std::max<size_t>(g->sig_blocks.size(), 1) * sizeof(int);
    if (cudaMalloc((void **)&g->d_items, ib) != cudaSuccess ||
        cudaMalloc((void **)&g->d_sig_blocks, sb) != cudaSuccess) {
        cudaFree(g->d_items);
        delete g;
        return fail(DPLR_GPU_ENOMEM, "gradient: cannot allocate work lists");
    }
    if (!g->items.empty())
        DG_CUDA(cudaMemcpy(g->d_items, g->items.data(), g->items.size() * sizeof(GradItem),
                           cudaMemcpyHostToDevice));
    if (!g->sig_blocks.empty())
        DG_CUDA(cudaMemcpy(g->d_sig_blocks, g->sig_blocks.data(), g->sig_blocks.size() * sizeof(int),
                           cudaMemcpyHostToDevice));
    *out = g;
    return 0;
}

}  // namespace

void grad_free(Plan *p)
{
    Grad *g = (Grad *)p->grad;
    if (!g) return;
    cudaFree(g->d_items);
    cudaFree(g->d_sig_blocks);
    delete g;
    p->grad = nullptr;
}

// G += alpha * d<DY, A X>/d(factors), pool layout.
int grad_factors(Plan *p, int nrhs, const double *X, int ldx, const double *DY, int ldy, double alpha, double *G,
                 cudaStream_t st)
{
    if (nrhs <= 0 || p->m == 0 || alpha == 0.0) return 0;
    int rc;
    if (!p->grad) {
        Grad *g = nullptr;
        if ((rc = grad_build(p, &g))) return rc;
        p->grad = g;
    }
    Grad *g = (Grad *)p->grad;
    const Schedule &SN = p->sched[0], &STr = p->sched[1];
    // scratch: TN, TT (total_rank x nrhs each) + partials of the larger schedule
    const size_t t = (size_t)p->total_rank * nrhs;
    const size_t part = (size_t)std::max(SN.partial_per_rhs, STr.partial_per_rhs) * nrhs;
    if ((rc = ensure_buffer(&p->gbuf, &p->gbuf_doubles, 2 * t + part))) return rc;
    double *TN = p->gbuf, *TT = p->gbuf + t, *partials = p->gbuf + 2 * t;
    if (t > 0) {
        if ((rc = run_panel(SN, p->pool, X, ldx, nrhs, partials, st))) return rc;
        if ((rc = run_reduce(SN, nullptr, partials, nrhs, TN, st))) return rc;
        if ((rc = run_panel(STr, p->pool, DY, ldy, nrhs, partials, st))) return rc;
        if ((rc = run_reduce(STr, nullptr, partials, nrhs, TT, st))) return rc;
    }
    if (!g->items.empty()) {
        double fl = 0;
        for (const GradItem &it : g->items) fl += 2.0 * it.rows * it.cols * nrhs;
        ProfScope ps("grad_outer", st, fl, 8.0 * (double)p->pool_doubles);
        grad_outer_kernel<<<(unsigned)g->items.size(), 256, 0, st>>>(g->d_items, X, ldx, DY, ldy, TN, TT, p->pool,
                                                                    nrhs, alpha, G);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }
    if (!g->sig_blocks.empty()) {
        grad_sig_kernel<<<(unsigned)g->sig_blocks.size(), 128, 0, st>>>(
            g->d_sig_blocks, (int)g->sig_blocks.size(), p->d_lr, TN, TT, nrhs, alpha, G);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }
    return 0;
}

// The factor values changed on the device: drop everything derived from
// them (the factorisation keeps its layout for the next factor_build).
void plan_values_changed(Plan *p)
{
    mixed_free(p);
    sliced_free(p);
    factor_invalidate(p);
}

}  // namespace dg

using namespace dg;

extern "C" {

long long dplr_gpu_pool_size(dplr_gpu_plan plan)
{
    return plan ? ((Plan *)plan)->pool_doubles : 0;
}

int dplr_gpu_pool_blocks(dplr_gpu_plan plan, int *nlowrank, int *nleaves)
{
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_pool_blocks: null plan");
    if (nlowrank) *nlowrank = (int)p->lr.size();
    if (nleaves) *nleaves = (int)p->leaves.size();
    return 0;
}

int dplr_gpu_pool_block(dplr_gpu_plan plan, int i, long long *u, long long *v, long long *sig, int *n, int *rank,
                        int *row0, int *col0)
{
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_pool_block: null plan");
    const int nlr = (int)p->lr.size();
    if (i < 0 || i >= nlr + (int)p->leaves.size()) return fail(DPLR_GPU_EINVAL, "dplr_gpu_pool_block: bad index");
    if (i < nlr) {
        const LRDesc &L = p->lr[i];
        if (u) *u = L.u;
        if (v) *v = L.v;
        if (sig) *sig = L.sig;
        if (n) *n = L.n;
        if (rank) *rank = L.rank;
        if (row0) *row0 = L.row0;
        if (col0) *col0 = L.col0;
    } else {
        const LeafDesc &L = p->leaves[i - nlr];
        if (u) *u = L.d;
        if (v) *v = -1;
        if (sig) *sig = -1;
        if (n) *n = L.b;
        if (rank) *rank = L.b;
        if (row0) *row0 = L.row0;
        if (col0) *col0 = L.row0;
    }
    return 0;
}

int dplr_gpu_pool_read(dplr_gpu_plan plan, double *dst, void *stream)
{
    Plan *p = (Plan *)plan;
    if (!p || (!dst && p->pool_doubles > 0)) return fail(DPLR_GPU_EINVAL, "dplr_gpu_pool_read: null argument");
    DG_CUDA(cudaMemcpyAsync(dst, p->pool, (size_t)p->pool_doubles * sizeof(double), cudaMemcpyDeviceToDevice,
                            (cudaStream_t)stream));
    return 0;
}

int dplr_gpu_pool_write(dplr_gpu_plan plan, const double *src, void *stream)
{
    Plan *p = (Plan *)plan;
    if (!p || (!src && p->pool_doubles > 0)) return fail(DPLR_GPU_EINVAL, "dplr_gpu_pool_write: null argument");
    plan_values_changed(p);
    DG_CUDA(cudaMemcpyAsync(p->pool, src, (size_t)p->pool_doubles * sizeof(double), cudaMemcpyDeviceToDevice,
                            (cudaStream_t)stream));
    return pairs_refresh(p, (cudaStream_t)stream);    // the pair copy follows the new values
}

int dplr_gpu_grad_factors(dplr_gpu_plan plan, int n, const double *X, int ldx, const double *DY, int ldy,
                          double alpha, double *G, void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_grad_factors");
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_grad_factors: null plan");
    const int mm = std::max(p->m, 1);
    if (n < 0 || ldx < mm || ldy < mm || (n > 0 && (!X || !DY || !G)))
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_grad_factors: invalid arguments");
    return grad_factors(p, n, X, ldx, DY, ldy, alpha, G, (cudaStream_t)stream);
}

}  // extern "C"
