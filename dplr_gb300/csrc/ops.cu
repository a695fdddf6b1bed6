// ops.cu -- structure-level arithmetic on a plan's device factors, so that
// pipelines (scale, shift the diagonal, apply, factor, solve) stay on the
// device without a host round trip:
//   dplr_gpu_scal  A := alpha A            (dplrscal, src/dplrscal.c:17)
//   dplr_gpu_adpy  A := alpha diag(D) + A  (dplradpy, src/dplraxpy.c:141)
// Both keep DPLR's conventions (sig >= 0; a negative scale negates the u
// vectors) and run over the plan's device block tables: one CTA per
// low-rank block or leaf.  The factorisation and the sliced copies describe
// the old values afterwards and are dropped, as after dplr_gpu_pool_write;
// the float-pair copy is rebuilt.
#include "internal.cuh"

#include <cmath>

namespace dg {

namespace {

__global__ void scal_lr_kernel(const LRDesc *__restrict__ lr, int nlr, double *pool, double alpha)
{
    if (blockIdx.x >= nlr) return;
    const LRDesc L = lr[blockIdx.x];
    if (L.rank == 0) return;
    const double a = fabs(alpha);
    for (int k = threadIdx.x; k < L.rank; k += blockDim.x) pool[L.sig + k] *= a;
    if (alpha < 0.0) {
        const long long n = (long long)L.n * L.rank;
        for (long long i = threadIdx.x; i < n; i += blockDim.x) pool[L.u + i] = -pool[L.u + i];
    }
}

__global__ void scal_leaf_kernel(const LeafDesc *__restrict__ lv, int nl, double *pool, double alpha)
{
    if (blockIdx.x >= nl) return;
    const LeafDesc L = lv[blockIdx.x];
    const long long n = (long long)L.b * L.b;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) pool[L.d + i] *= alpha;
}

__global__ void adpy_leaf_kernel(const LeafDesc *__restrict__ lv, int nl, double *pool, double alpha,
                                 const double *__restrict__ D)
{
    if (blockIdx.x >= nl) return;
    const LeafDesc L = lv[blockIdx.x];
    for (int i = threadIdx.x; i < L.b; i += blockDim.x) pool[L.d + (long long)i * L.b + i] += alpha * D[L.row0 + i];
}

}  // namespace

}  // namespace dg

using namespace dg;

extern "C" {

int dplr_gpu_scal(dplr_gpu_plan plan, double alpha, void *stream)
{
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_scal: null plan");
    if (!std::isfinite(alpha)) return fail(DPLR_GPU_EINVAL, "dplr_gpu_scal: alpha must be finite");
    cudaStream_t st = (cudaStream_t)stream;
    plan_values_changed(p);
    if (!p->lr.empty()) {
        scal_lr_kernel<<<(unsigned)p->lr.size(), 256, 0, st>>>(p->d_lr, (int)p->lr.size(), p->pool, alpha);
        note_launch();
    }
    if (!p->leaves.empty()) {
        scal_leaf_kernel<<<(unsigned)p->leaves.size(), 256, 0, st>>>(p->d_leaves, (int)p->leaves.size(), p->pool,
                                                                     alpha);
        note_launch();
    }
    DG_CUDA(cudaGetLastError());
    return pairs_refresh(p, st);
}

int dplr_gpu_adpy(dplr_gpu_plan plan, double alpha, const double *D, void *stream)
{
    Plan *p = (Plan *)plan;
    if (!p || (!D && p->m > 0)) return fail(DPLR_GPU_EINVAL, "dplr_gpu_adpy: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    plan_values_changed(p);
    if (!p->leaves.empty() && alpha != 0.0) {
        adpy_leaf_kernel<<<(unsigned)p->leaves.size(), 256, 0, st>>>(p->d_leaves, (int)p->leaves.size(), p->pool,
                                                                     alpha, D);
        note_launch();
    }
    DG_CUDA(cudaGetLastError());
    return pairs_refresh(p, st);
}

}  // extern "C"
