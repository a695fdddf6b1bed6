// noalloc.cu -- a PLR apply that allocates no device memory.
//
// Some callers of this library cannot allocate device memory at the moment
// they need an apply:
//   * latency-critical serving paths that must never pay for cudaMalloc or
//     the device-wide synchronisation cudaFree can imply;
//   * host frameworks that hand the library a fixed device-memory budget up
//     front and forbid allocations afterwards.
// dplr_gpu_apply_noalloc serves them.  It runs the same panel / reduce /
// expand kernels as dplr_gpu_apply, but its scratch (the per-block V^T X
// panels and their partial sums) is one statically sized array in device
// memory that belongs to the library, instead of a buffer grown with
// cudaMalloc.  The caller still passes the plan, X and Y.
//
// Limits and sharing:
//   * the array holds kNoAllocScratchDoubles doubles (64 MiB), and every GPU
//     that loads the library keeps it until the process exits;
//   * a call needs (sum of the block ranks + partial panels) * n doubles; a
//     call that needs more is rejected with DPLR_GPU_EINVAL and a message
//     giving both numbers;
//   * all calls on a device share the one array, so calls that can overlap
//     on the GPU (unordered streams, concurrent host threads) race on it and
//     must be ordered by the caller;
//   * the array keeps whatever the previous call left; every element a call
//     reads is written earlier in the same call, so nothing is cleared;
//   * the first call on each device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current) and keeps it.
#include "internal.cuh"

#include <mutex>

namespace dg {

constexpr size_t kNoAllocScratchDoubles = (size_t)8 << 20;   // 64 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[kMaxDevices];

// Device address of the static scratch on the current device (set up once
// per device; host code must not use the symbol itself as an address).
static int noalloc_scratch(double **out)
{
    int dev = 0;
    DG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_apply_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(DPLR_GPU_ECUDA, "dplr_gpu_apply_noalloc: scratch address lookup failed: %s",
                        cudaGetErrorString(e));
        g_noalloc_ptr[dev] = (double *)p;
    }
    *out = g_noalloc_ptr[dev];
    return 0;
}

}  // namespace dg

using namespace dg;

extern "C" int dplr_gpu_apply_noalloc(dplr_gpu_plan plan, char trans, int n, double alpha,
                                      const double *X, int ldx, double beta, double *Y, int ldy,
                                      void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_apply_noalloc");
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_apply_noalloc: null plan");
    if (n < 0 || ldx < (p->m > 0 ? p->m : 1) || ldy < (p->m > 0 ? p->m : 1))
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_apply_noalloc: invalid n/ldx/ldy");
    if (n == 0 || p->m == 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    if (alpha == 0.0) return scale_device(Y, p->m, n, ldy, beta, st);
    const int tr = !(trans == 'N' || trans == 'n');
    const Schedule &S = p->sched[tr];
    const size_t need = (size_t)(S.t_per_rhs + S.partial_per_rhs) * (size_t)n;
    if (need > kNoAllocScratchDoubles) {
        const size_t per = (size_t)(S.t_per_rhs + S.partial_per_rhs);
        return fail(DPLR_GPU_EINVAL,
                    "dplr_gpu_apply_noalloc: needs %zu doubles of scratch, the static scratch "
                    "holds %zu (at most %zu right-hand sides for this matrix)",
                    need, kNoAllocScratchDoubles, per ? kNoAllocScratchDoubles / per : (size_t)0);
    }
    double *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    double *T = scratch;
    double *partials = scratch + (size_t)S.t_per_rhs * n;
    if ((rc = run_panel(S, p->pool, X, ldx, n, partials, st))) return rc;
    if ((rc = run_reduce(S, p->pool, partials, n, T, st))) return rc;
    return run_expand(S, p->pool, T, X, ldx, Y, ldy, n, alpha, beta, st);
}
