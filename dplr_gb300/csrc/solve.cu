// solve.cu -- factor / solve / refined-solve entry points.
//
// DPLR solves by forming B = inv(A) explicitly (dplrgeinv,
// src/dplrinv.c:93) and applying it with dplrgepdmm.  The GPU library keeps
// the Woodbury factorisation instead (factor.cu) and offers
//   dplr_gpu_factor        build Z = D^-1 W, capacitance inverses, leaf inverses
//   dplr_gpu_solve         X = op(A)^-1 B, one bottom-up sweep
//   dplr_gpu_solve_refined X with ||B - A X|| / ||B|| <= tol per column,
//                          by iterative refinement whose residual is the
//                          FP64 PLR apply of the original matrix.
#include "sliced.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace dg {

int factor_build(Plan *p, int flags, cudaStream_t st);
int factor_solve(Plan *p, int trans, int nrhs, const double *B, int ldb, double *X, int ldx,
                 cudaStream_t st);
long long factor_bytes(const Plan *p);
struct Fact;
Fact *factor_of(const Plan *p);

// Column 2-norms of an m x n matrix: one CTA of kNormThreads per column,
// four independent sums per thread so that four loads are in flight (one
// CTA per SM pair covers a 256-column block in one wave).
constexpr int kNormThreads = 1024;

__global__ void __launch_bounds__(kNormThreads) colnorm_kernel(const double *A, int m, int lda, double *out)
{
    __shared__ double red[kNormThreads];
    const double *a = A + (long long)blockIdx.x * lda;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int i = threadIdx.x;
    for (; i + 3 * kNormThreads < m; i += 4 * kNormThreads) {
        const double x0 = a[i], x1 = a[i + kNormThreads], x2 = a[i + 2 * kNormThreads], x3 = a[i + 3 * kNormThreads];
        s0 = fma(x0, x0, s0);
        s1 = fma(x1, x1, s1);
        s2 = fma(x2, x2, s2);
        s3 = fma(x3, x3, s3);
    }
    for (; i < m; i += kNormThreads) s0 = fma(a[i], a[i], s0);
    red[threadIdx.x] = (s0 + s1) + (s2 + s3);
    __syncthreads();
    for (int k = kNormThreads / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sqrt(red[0]);
}

// Column 2-norms per tree of a batch: out[j * nseg + t] over the rows
// [row0[t], row0[t + 1]) of column j; one CTA per (tree, column).
__global__ void segnorm_kernel(const double *A, int lda, int n, const int *row0, int nseg, double *out)
{
    __shared__ double red[256];
    const int t = blockIdx.x;
    const int r0 = row0[t], r1 = row0[t + 1];
    for (int j = blockIdx.y; j < n; j += gridDim.y) {
        const double *a = A + (long long)j * lda;
        double s = 0.0;
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) s = fma(a[i], a[i], s);
        __syncthreads();                 // red is reused across columns
        red[threadIdx.x] = s;
        __syncthreads();
        for (int k = blockDim.x / 2; k > 0; k >>= 1) {
            if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[(long long)j * nseg + t] = sqrt(red[0]);
    }
}

// Y (m x n) := X + alpha*Y  or plain copies, column-major with leading dims.
__global__ void axpby_kernel(int m, int n, double a, const double *X, int ldx, double b, double *Y,
                             int ldy)
{
    long long cnt = (long long)m * n;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < cnt;
         e += (long long)gridDim.x * blockDim.x) {
        int i = (int)(e % m), j = (int)(e / m);
        double *y = Y + i + (long long)j * ldy;
        double x = X[i + (long long)j * ldx];
        *y = b == 0.0 ? a * x : fma(a, x, b * *y);
    }
}

int axpby_device(int m, int n, double a, const double *X, int ldx, double b, double *Y, int ldy,
                 cudaStream_t st)
{
    long long cnt = (long long)m * n;
    if (cnt <= 0) return 0;
    int grid = (int)std::min<long long>((cnt + 255) / 256, 152LL * 16);
    axpby_kernel<<<grid, 256, 0, st>>>(m, n, a, X, ldx, b, Y, ldy);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

// X := A^-1 B refined by `corrections` fixed steps (R = B - A X, X += A^-1 R
// with the FP64 sweep), with no host synchronisation, so that the whole
// refined solve can be captured in a CUDA graph.  The residual uses the
// exact-slice products when the plan has them (dplr_gpu_prepare_sliced),
// else the FP64 apply.  Scratch: p->ybuf (2 m n doubles) and the sliced
// scratch, sized by an ordinary call before any capture.
int refine_fixed(Plan *p, int n, const double *B, int ldb, double *X, int ldx, int corrections, cudaStream_t st)
{
    const int m = p->m;
    int rc = ensure_buffer(&p->ybuf, &p->ybuf_doubles, (size_t)2 * m * n);
    if (rc) return rc;
    double *R = p->ybuf, *D = p->ybuf + (size_t)m * n;
    if ((rc = factor_solve(p, 0, n, B, ldb, X, ldx, st))) return rc;
    for (int it = 0; it < corrections; ++it) {
        if (p->sliced) {
            if ((rc = sliced_residual(p, n, X, ldx, B, ldb, R, m, st))) return rc;
        } else {
            if ((rc = axpby_device(m, n, 1.0, B, ldb, 0.0, R, m, st))) return rc;
            if ((rc = apply_device(p, 0, n, -1.0, X, ldx, 1.0, R, m, st, false))) return rc;
        }
        if ((rc = factor_solve(p, 0, n, R, m, D, m, st))) return rc;
        if ((rc = axpby_device(m, n, 1.0, D, m, 1.0, X, ldx, st))) return rc;
    }
    return 0;
}

int colnorms_device(const double *A, int m, int n, int lda, double *out, cudaStream_t st)
{
    if (n <= 0) return 0;
    colnorm_kernel<<<n, kNormThreads, 0, st>>>(A, m, lda, out);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

// Norms of every column of every tree: nseg = 1 for one tree (plain column
// norms), else per tree of the batch, out[j * nseg + t].
static int segnorms_device(Plan *p, const double *A, int n, int lda, double *out, cudaStream_t st)
{
    if (p->ntrees <= 1) return colnorms_device(A, p->m, n, lda, out, st);
    if (n <= 0) return 0;
    if (!p->d_tree_row0) {
        std::vector<int> rows(p->tree_row0);
        rows.push_back(p->m);
        DG_ALLOC(&p->d_tree_row0, rows.size() * sizeof(int));
        DG_CUDA(cudaMemcpy(p->d_tree_row0, rows.data(), rows.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    segnorm_kernel<<<dim3((unsigned)p->ntrees, (unsigned)std::min(n, 65535)), 256, 0, st>>>(
        A, lda, n, p->d_tree_row0, p->ntrees, out);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

// X's copy to a host array on a side stream, while the refinement goes
// on: the copy of each iterate starts as soon as it exists and overlaps the
// residual that checks it; the next update of X waits for it.  The stream
// is drained (and destroyed) on every way out, so no copy lands after the
// call has returned.
struct HostCopy {
    double *hX = nullptr;
    int ldhx = 0;
    cudaStream_t cs = nullptr;
    cudaEvent_t ready = nullptr, done = nullptr;
    bool pending = false;
    ~HostCopy()
    {
        if (cs) cudaStreamSynchronize(cs);
        if (ready) cudaEventDestroy(ready);
        if (done) cudaEventDestroy(done);
        if (cs) cudaStreamDestroy(cs);
    }
    int init(double *h, int ld)
    {
        hX = h;
        ldhx = ld;
        if (!hX) return 0;
        if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&done, cudaEventDisableTiming) != cudaSuccess)
            return fail(DPLR_GPU_ECUDA, "refined solve: cannot create the copy stream");
        return 0;
    }
    // X (m x n, ld ldx on the device) is final for now: copy it out
    int start(const double *X, int ldx, int m, int n, cudaStream_t st)
    {
        if (!hX) return 0;
        DG_CUDA(cudaEventRecord(ready, st));
        DG_CUDA(cudaStreamWaitEvent(cs, ready, 0));
        DG_CUDA(cudaMemcpy2DAsync(hX, sizeof(double) * ldhx, X, sizeof(double) * ldx, sizeof(double) * m, n,
                                  cudaMemcpyDeviceToHost, cs));
        DG_CUDA(cudaEventRecord(done, cs));
        pending = true;
        return 0;
    }
    // X is about to change on st: wait for its copy
    int before_write(cudaStream_t st)
    {
        if (!hX || !pending) return 0;
        DG_CUDA(cudaStreamWaitEvent(st, done, 0));
        return 0;
    }
    int finish()
    {
        if (!hX) return 0;
        DG_CUDA(cudaStreamSynchronize(cs));
        return 0;
    }
};

// The refinement loop of dplr_gpu_solve_refined; with hX, every iterate of
// X is also copied to the host array hX (ld ldhx), and the last one is there
// when it returns.
static int refine(Plan *p, int n, const double *B, int ldb, double *X, int ldx, double tol, int maxiter, int flags,
                  double *rel_resid, int *iters, cudaStream_t st, double *hX, int ldhx)
{
    if (n == 0 || p->m == 0) {
        if (rel_resid) *rel_resid = 0.0;
        if (iters) *iters = 0;
        return 0;
    }
    const int m = p->m;
    // Scratch: residual R, correction D (m x n each), the norms of B and R
    // per column and tree: a batch converges when every tree's every column
    // does, not on the norms of the stacked columns.
    const size_t nn = (size_t)n * std::max(p->ntrees, 1);
    size_t need = (size_t)2 * m * n + 2 * nn;
    int rc = ensure_buffer(&p->ybuf, &p->ybuf_doubles, need);
    if (rc) return rc;
    double *R = p->ybuf, *D = p->ybuf + (size_t)m * n;
    double *bn = D + (size_t)m * n, *rn = bn + nn;
    std::vector<double> hb(nn), hr(nn);
    const bool mixed = (flags & DPLR_GPU_SOLVE_MIXED) != 0;
    if (mixed && !p->mixed) return fail(DPLR_GPU_ESTATE, "solve: mixed solve not prepared");
    if ((flags & DPLR_GPU_RESIDUAL_SLICED) && !p->sliced)
        return fail(DPLR_GPU_ESTATE, "solve: sliced residual not prepared");
    HostCopy hc;
    if ((rc = hc.init(hX, ldhx))) return rc;
    auto inner = [&](const double *rhs, int ld, double *out, int ldo) -> int {
        return mixed ? mixed_solve(p, n, rhs, ld, out, ldo, st) : factor_solve(p, 0, n, rhs, ld, out, ldo, st);
    };
    if ((rc = segnorms_device(p, B, n, ldb, bn, st))) return rc;
    DG_CUDA(cudaMemcpyAsync(hb.data(), bn, nn * sizeof(double), cudaMemcpyDeviceToHost, st));
    if ((rc = inner(B, ldb, X, ldx))) return rc;
    if ((rc = hc.start(X, ldx, m, n, st))) return rc;
    double worst = INFINITY;
    int it = 0;
    for (;;) {
        // R = B - A X with the original matrix (FP64 apply, or exact-slice products)
        if (flags & DPLR_GPU_RESIDUAL_SLICED) {
            if ((rc = sliced_residual(p, n, X, ldx, B, ldb, R, m, st))) return rc;
        } else {
            if ((rc = axpby_device(m, n, 1.0, B, ldb, 0.0, R, m, st))) return rc;
            if ((rc = apply_device(p, 0, n, -1.0, X, ldx, 1.0, R, m, st, false))) return rc;
        }
        {
            ProfScope ps("refine_norms", st, 0.0, 8.0 * m * n);
            if ((rc = segnorms_device(p, R, n, m, rn, st))) return rc;
        }
        DG_CUDA(cudaMemcpyAsync(hr.data(), rn, nn * sizeof(double), cudaMemcpyDeviceToHost, st));
        DG_CUDA(cudaStreamSynchronize(st));
        if ((rc = sliced_error(p))) return rc;
        worst = 0.0;
        for (size_t j = 0; j < nn; ++j) worst = std::max(worst, hb[j] > 0 ? hr[j] / hb[j] : hr[j]);
        if (worst <= tol || it >= maxiter) break;
        if ((rc = inner(R, m, D, m))) return rc;
        {
            ProfScope ps("refine_update", st, 0.0, 24.0 * m * n);
            if ((rc = hc.before_write(st))) return rc;
            if ((rc = axpby_device(m, n, 1.0, D, m, 1.0, X, ldx, st))) return rc;
        }
        if ((rc = hc.start(X, ldx, m, n, st))) return rc;
        ++it;
    }
    if ((rc = hc.finish())) return rc;
    if (rel_resid) *rel_resid = worst;
    if (iters) *iters = it;
    if (!(worst <= tol))
        return fail(DPLR_GPU_ENOTCONV, "refinement stopped at relative residual %.3e after %d steps",
                    worst, it);
    return 0;
}

}  // namespace dg

using namespace dg;

extern "C" {

int dplr_gpu_factor(dplr_gpu_plan plan, int flags, void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_factor");
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_factor: null plan");
    return factor_build(p, flags, (cudaStream_t)stream);
}

int dplr_gpu_solve(dplr_gpu_plan plan, char trans, int n, const double *B, int ldb, double *X,
                   int ldx, void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_solve");
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_solve: null plan");
    if (n < 0 || ldb < std::max(p->m, 1) || ldx < std::max(p->m, 1))
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_solve: invalid n/ldb/ldx");
    if (B == X) return fail(DPLR_GPU_EINVAL, "dplr_gpu_solve: B and X must not alias");
    int tr = !(trans == 'N' || trans == 'n');
    return factor_solve(p, tr, n, B, ldb, X, ldx, (cudaStream_t)stream);
}

int dplr_gpu_prepare_sliced(dplr_gpu_plan plan, void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_prepare_sliced");
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_prepare_sliced: null plan");
    return sliced_build(p, 8, (cudaStream_t)stream);
}

int dplr_gpu_prepare_mixed(dplr_gpu_plan plan, int slices, void *stream)
{
    return dplr_gpu_prepare_mixed_caps(plan, slices, 0, stream);
}

int dplr_gpu_prepare_mixed_caps(dplr_gpu_plan plan, int slices, int fp64_capacitance, void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_prepare_mixed_caps");
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_prepare_mixed: null plan");
    return mixed_build(p, slices, (cudaStream_t)stream, fp64_capacitance != 0);
}

int dplr_gpu_residual(dplr_gpu_plan plan, int n, const double *X, int ldx, const double *B, int ldb,
                      double *R, int ldr, int flags, void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_residual");
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_residual: null plan");
    const int mm = std::max(p->m, 1);
    if (n < 0 || ldx < mm || ldb < mm || ldr < mm)
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_residual: invalid n or leading dimension");
    cudaStream_t st = (cudaStream_t)stream;
    int rc0 = sliced_error(p);          // reported by an earlier asynchronous call
    if (rc0) return rc0;
    if (flags & DPLR_GPU_RESIDUAL_SLICED) return sliced_residual(p, n, X, ldx, B, ldb, R, ldr, st);
    int rc = axpby_device(p->m, n, 1.0, B, ldb, 0.0, R, ldr, st);
    if (rc) return rc;
    return apply_device(p, 0, n, -1.0, X, ldx, 1.0, R, ldr, st, false);
}

int dplr_gpu_solve_refined(dplr_gpu_plan plan, int n, const double *B, int ldb, double *X, int ldx,
                           double tol, int maxiter, int flags, double *rel_resid, int *iters,
                           void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_solve_refined");
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_solve_refined: null plan");
    if (!factor_of(p)) return fail(DPLR_GPU_ESTATE, "dplr_gpu_solve_refined: plan is not factored");
    if (n < 0 || ldb < std::max(p->m, 1) || ldx < std::max(p->m, 1) || maxiter < 0)
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_solve_refined: invalid arguments");
    return refine(p, n, B, ldb, X, ldx, tol, maxiter, flags, rel_resid, iters, (cudaStream_t)stream, nullptr, 0);
}

int dplr_gpu_solve_refined_host(dplr_gpu_plan plan, int n, const double *B, int ldb, double *X,
                                int ldx, double tol, int maxiter, int flags, double *rel_resid,
                                int *iters, void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_solve_refined_host");
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_solve_refined_host: null plan");
    if (n < 0 || ldb < std::max(p->m, 1) || ldx < std::max(p->m, 1))
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_solve_refined_host: invalid arguments");
    if (n == 0 || p->m == 0) return dplr_gpu_solve_refined(plan, n, nullptr, 1, nullptr, 1, tol,
                                                          maxiter, flags, rel_resid, iters, stream);
    if (!factor_of(p)) return fail(DPLR_GPU_ESTATE, "dplr_gpu_solve_refined_host: plan is not factored");
    if (maxiter < 0) return fail(DPLR_GPU_EINVAL, "dplr_gpu_solve_refined_host: invalid arguments");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t cnt = (size_t)p->m * n;
    int rc = ensure_buffer(&p->xbuf, &p->xbuf_doubles, 2 * cnt);
    if (rc) return rc;
    double *dB = p->xbuf, *dX = p->xbuf + cnt;
    // one copy each way: measured on the GB300, pinned copies run at the
    // link's 210 GB/s (host to device) and 193 GB/s (device to host) whether
    // issued on one stream or split over four.  X goes back while the
    // refinement checks it (see refine).
    DG_CUDA(cudaMemcpy2DAsync(dB, sizeof(double) * p->m, B, sizeof(double) * ldb,
                              sizeof(double) * p->m, n, cudaMemcpyHostToDevice, st));
    return refine(p, n, dB, p->m, dX, p->m, tol, maxiter, flags, rel_resid, iters, st, X, ldx);
}

long long dplr_gpu_factor_device_bytes(dplr_gpu_plan plan)
{
    return plan ? factor_bytes((Plan *)plan) : 0;
}

}  // extern "C"
