// abi.cu -- extern "C" entry points: the DPLR drop-ins and the plan API.
//
// The drop-ins keep DPLR's observable contract:
//   * void return, errors reported as "<function>: <reason>" on stderr and
//     the outputs left untouched (DPLR src/dplrpmv.c:22-36,
//     src/dplrpdmm.c:180-199); the reason is also kept for
//     dplr_gpu_last_error();
//   * scalars by pointer, column-major host arrays, BLAS-style strides;
//   * alpha == 0 scales y by beta twice in dplrgepmv (src/dplrpmv.c:140-160)
//     and once in dplrgepdmm;  beta == 0 never reads the output.
// Deliberate tightening: non-positive increments and ldb smaller than the
// rows of op(B) are rejected (DPLR reads out of bounds for them).
#include "internal.cuh"

#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

namespace dg {
const char *last_error_c();
}

using namespace dg;

namespace {

// Registered plans are shared: a drop-in call holds its own reference for
// the whole call, so dplr_gpu_register / dplr_gpu_unregister on the same
// tree from another thread never frees a plan that is still in use (the
// plan goes when its last user lets go).
std::mutex g_reg_mu;
std::map<const DPlrMtx *, std::shared_ptr<Plan>> g_registered;

std::shared_ptr<Plan> shared_plan(Plan *p)
{
    return std::shared_ptr<Plan>(p, [](Plan *q) { plan_free(q); });
}

std::shared_ptr<Plan> lookup_registered(const DPlrMtx *A, int m)
{
    std::lock_guard<std::mutex> lk(g_reg_mu);
    auto it = g_registered.find(A);
    if (it == g_registered.end() || it->second->m != m) return nullptr;
    return it->second;
}

void report(const char *fn)
{
    fprintf(stderr, "%s: %s\n", fn, dg::last_error_c());
}

// Plan for a drop-in call: the registered one, or a temporary upload.
struct CallPlan {
    Plan *p = nullptr;
    std::shared_ptr<Plan> keep;
    bool owned = false;
    ~CallPlan()
    {
        if (owned) plan_free(p);
    }
    int get(int m, const DPlrMtx *A)
    {
        keep = lookup_registered(A, m);
        if (keep) {
            p = keep.get();
            return 0;
        }
        owned = true;
        return plan_build(m, A, 0, &p);
    }
};

// Host <-> device staging of strided vectors / matrices.
int upload_matrix(Plan *p, double **buf, size_t *have, const double *src, long long row_stride,
                  long long col_stride, int rows, int cols)
{
    int rc = ensure_buffer(buf, have, (size_t)rows * cols);
    if (rc) return rc;
    if (row_stride == 1) {
        DG_CUDA(cudaMemcpy2D(*buf, sizeof(double) * rows, src, sizeof(double) * col_stride,
                             sizeof(double) * rows, cols, cudaMemcpyHostToDevice));
    } else {
        // rows strided by row_stride, one column (vector case)
        DG_CUDA(cudaMemcpy2D(*buf, sizeof(double), src, sizeof(double) * row_stride,
                             sizeof(double), rows, cudaMemcpyHostToDevice));
    }
    (void)p;
    return 0;
}

int download_matrix(double *dst, long long row_stride, long long col_stride, const double *buf,
                    int rows, int cols)
{
    if (row_stride == 1) {
        DG_CUDA(cudaMemcpy2D(dst, sizeof(double) * col_stride, buf, sizeof(double) * rows,
                             sizeof(double) * rows, cols, cudaMemcpyDeviceToHost));
    } else {
        DG_CUDA(cudaMemcpy2D(dst, sizeof(double) * row_stride, buf, sizeof(double),
                             sizeof(double), rows, cudaMemcpyDeviceToHost));
    }
    return 0;
}

void scale_host_vector(int m, double beta, double *y, int incy)
{
    for (int i = 0; i < m; ++i) y[(size_t)i * incy] = beta == 0.0 ? 0.0 : beta * y[(size_t)i * incy];
}

}  // namespace

extern "C" {

const char *dplr_gpu_last_error(void) { return dg::last_error_c(); }

int dplr_gpu_plan_create(int m, const DPlrMtx *A, void *stream, dplr_gpu_plan *plan)
{
    dg::NvtxRange nvtx_("dplr_gpu_plan_create");
    if (!plan) return fail(DPLR_GPU_EINVAL, "dplr_gpu_plan_create: null output");
    Plan *p = nullptr;
    int rc = plan_build(m, A, (cudaStream_t)stream, &p);
    if (rc) return rc;
    *plan = (dplr_gpu_plan)p;
    return 0;
}

void dplr_gpu_plan_destroy(dplr_gpu_plan plan) { plan_free((Plan *)plan); }

int dplr_gpu_plan_refresh(dplr_gpu_plan plan, const DPlrMtx *A, void *stream)
{
    if (!plan) return fail(DPLR_GPU_EINVAL, "dplr_gpu_plan_refresh: null plan");
    return plan_upload_values((Plan *)plan, A, (cudaStream_t)stream);
}

int dplr_gpu_plan_info(dplr_gpu_plan plan, int *m, long long *nnz, int *levels, int *max_rank)
{
    if (!plan) return fail(DPLR_GPU_EINVAL, "dplr_gpu_plan_info: null plan");
    Plan *p = (Plan *)plan;
    if (m) *m = p->m;
    if (nnz) *nnz = p->nnz;
    if (levels) *levels = p->levels;
    if (max_rank) *max_rank = p->max_rank;
    return 0;
}

long long dplr_gpu_plan_device_bytes(dplr_gpu_plan plan)
{
    Plan *p = (Plan *)plan;
    if (!p) return 0;
    return p->device_bytes + (long long)p->work_doubles * 8 + (long long)p->xbuf_doubles * 8 +
           (long long)p->ybuf_doubles * 8 + pairs_bytes(p);
}

int dplr_gpu_prepare_pairs(dplr_gpu_plan plan, void *stream)
{
    if (!plan) return fail(DPLR_GPU_EINVAL, "dplr_gpu_prepare_pairs: null plan");
    return pairs_prepare((Plan *)plan, (cudaStream_t)stream);
}

int dplr_gpu_apply(dplr_gpu_plan plan, char trans, int n, double alpha, const double *X, int ldx,
                   double beta, double *Y, int ldy, void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_apply");
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_apply: null plan");
    if (n < 0 || ldx < (p->m > 0 ? p->m : 1) || ldy < (p->m > 0 ? p->m : 1))
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_apply: invalid n/ldx/ldy");
    int tr = !(trans == 'N' || trans == 'n');
    return apply_device(p, tr, n, alpha, X, ldx, beta, Y, ldy, (cudaStream_t)stream, false);
}

int dplr_gpu_register(int m, DPlrMtx *A)
{
    Plan *p = nullptr;
    int rc = plan_build(m, A, 0, &p);
    if (rc) return rc;
    std::shared_ptr<Plan> fresh = shared_plan(p), old;
    {
        std::lock_guard<std::mutex> lk(g_reg_mu);
        old.swap(g_registered[A]);
        g_registered[A] = fresh;
    }
    return 0;       // `old` is released here, or by the last call still using it
}

int dplr_gpu_unregister(DPlrMtx *A)
{
    std::shared_ptr<Plan> old;
    {
        std::lock_guard<std::mutex> lk(g_reg_mu);
        auto it = g_registered.find(A);
        if (it == g_registered.end())
            return fail(DPLR_GPU_EINVAL, "dplr_gpu_unregister: not registered");
        old.swap(it->second);
        g_registered.erase(it);
    }
    return 0;
}

// y := alpha*op(A)*x + beta*y  (DPLR src/dplrpmv.c:262)
void dplrgepmv(char trans, int m, double *alpha, DPlrMtx *A, double *x, int incx, double *beta,
               double *y, int incy)
{
    dg::NvtxRange nvtx_("dplrgepmv");
    const char *fn = "dplrgepmv";
    if (m < 0) {
        fail(DPLR_GPU_EINVAL, "invalid matrix size %d", m);
        return report(fn);
    }
    if (validate_tree(m, A, fn)) return report(fn);
    if (incx <= 0 || incy <= 0) {
        fail(DPLR_GPU_EINVAL, "non-positive increment (incx=%d, incy=%d)", incx, incy);
        return report(fn);
    }
    if (m == 0) return;
    if (*alpha == 0.0) {
        // y := beta*y applied twice (DPLR's alpha == 0 branch does not return).
        scale_host_vector(m, *beta, y, incy);
        if (*beta != 0.0) scale_host_vector(m, *beta, y, incy);
        return;
    }
    CallPlan cp;
    if (cp.get(m, A)) return report(fn);
    Plan *p = cp.p;
    int tr = !(trans == 'N' || trans == 'n');
    if (upload_matrix(p, &p->xbuf, &p->xbuf_doubles, x, incx, m, m, 1)) return report(fn);
    if (ensure_buffer(&p->ybuf, &p->ybuf_doubles, m)) return report(fn);
    if (*beta != 0.0 && upload_matrix(p, &p->ybuf, &p->ybuf_doubles, y, incy, m, m, 1))
        return report(fn);
    if (apply_device(p, tr, 1, *alpha, p->xbuf, m, *beta, p->ybuf, m, 0, true)) return report(fn);
    if (download_matrix(y, incy, m, p->ybuf, m, 1)) return report(fn);
}

// C := alpha*op(A)*op(B) + beta*C  (DPLR src/dplrpdmm.c:454)
void dplrgepdmm(char transa, char transb, int m, int n, double *alpha, DPlrMtx *A, double *B,
                int ldb, double *beta, double *C, int ldc)
{
    dg::NvtxRange nvtx_("dplrgepdmm");
    const char *fn = "dplrgepdmm";
    int ta = !(transa == 'N' || transa == 'n');
    int tb = !(transb == 'N' || transb == 'n');
    if (m < 0) {
        fail(DPLR_GPU_EINVAL, "invalid matrix size %d", m);
        return report(fn);
    }
    if (validate_tree(m, A, fn)) return report(fn);
    if (ldc < m) {
        fail(DPLR_GPU_EINVAL, "invalid leading dimensions");
        return report(fn);
    }
    if (n < 0 || ldb < (tb ? (n > 0 ? n : 1) : (m > 0 ? m : 1))) {
        fail(DPLR_GPU_EINVAL, "invalid n or ldb (n=%d, ldb=%d)", n, ldb);
        return report(fn);
    }
    if (m == 0 || n == 0) return;
    if (*alpha == 0.0) {
        for (int j = 0; j < n; ++j) scale_host_vector(m, *beta, C + (size_t)j * ldc, 1);
        return;
    }
    CallPlan cp;
    if (cp.get(m, A)) return report(fn);
    Plan *p = cp.p;
    if (!tb) {
        if (upload_matrix(p, &p->xbuf, &p->xbuf_doubles, B, 1, ldb, m, n)) return report(fn);
    } else {
        // op(B) = B^T with B n x m: stage B, then transpose on the device.
        if (ensure_buffer(&p->xbuf, &p->xbuf_doubles, (size_t)2 * m * n)) return report(fn);
        double *raw = p->xbuf + (size_t)m * n;
        if (cudaMemcpy2D(raw, sizeof(double) * n, B, sizeof(double) * ldb, sizeof(double) * n, m,
                         cudaMemcpyHostToDevice) != cudaSuccess) {
            fail(DPLR_GPU_ECUDA, "copy of B failed");
            return report(fn);
        }
        if (transpose_device(raw, n, m, n, p->xbuf, m, 0)) return report(fn);
    }
    if (ensure_buffer(&p->ybuf, &p->ybuf_doubles, (size_t)m * n)) return report(fn);
    if (*beta != 0.0 && upload_matrix(p, &p->ybuf, &p->ybuf_doubles, C, 1, ldc, m, n))
        return report(fn);
    if (apply_device(p, ta, n, *alpha, p->xbuf, m, *beta, p->ybuf, m, 0, false)) return report(fn);
    if (download_matrix(C, 1, ldc, p->ybuf, m, n)) return report(fn);
}

}  // extern "C"

// ---------------------------------------------------------- instrumentation
namespace dg {

static std::atomic<long long> g_launches{0};
static std::atomic<int> g_prof_on{0};
struct ProfRec {
    const char *name;
    cudaEvent_t e0, e1;
    double flops, bytes;
};
static std::mutex g_prof_mu;
static std::vector<ProfRec> g_prof;
struct ProfAgg {
    std::string name;
    double ms = 0, flops = 0, bytes = 0;
    int launches = 0;
};
static std::vector<ProfAgg> g_prof_out;

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_launches(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

// Allocation-failure injection: countdown of allocations that still
// succeed; -1 = off.  Armed from DPLR_GB300_FAIL_ALLOC at load, or by
// dplr_gpu_debug_fail_alloc.  The failing allocation makes no CUDA call.
static std::atomic<long long> g_fail_countdown{[] {
    const char *v = getenv("DPLR_GB300_FAIL_ALLOC");
    return v && *v ? atoll(v) : -1LL;
}()};

cudaError_t dev_malloc(void **ptr, size_t bytes)
{
    long long c = g_fail_countdown.load();
    while (c >= 0) {
        if (g_fail_countdown.compare_exchange_weak(c, c - 1)) {
            if (c == 0) {
                *ptr = nullptr;
                return cudaErrorMemoryAllocation;
            }
            break;
        }
    }
    return cudaMalloc(ptr, bytes);
}

// Recompression after the operations that grow ranks (off unless a caller
// sets a threshold with dplr_gpu_set_recompress).
static std::atomic<double> g_recompress_eps{-1.0};

double recompress_eps() { return g_recompress_eps.load(); }

void recompress_after(int m, DPlrMtx *A)
{
    const double e = g_recompress_eps.load();
    if (!(e >= 0.0) || !A) return;
    if (dplr_gpu_reduce_svd(m, A, e, 0) != DPLR_GPU_OK)
        fprintf(stderr, "dplr_gpu_reduce_svd: %s\n", last_error_c());
}

NvtxRange::NvtxRange(const char *name) { nvtxRangePushA(name); }
NvtxRange::~NvtxRange() { nvtxRangePop(); }

ProfScope::ProfScope(const char *name, cudaStream_t st, double flops, double bytes)
{
    if (!g_prof_on.load()) return;
    ProfRec r{name, nullptr, nullptr, flops, bytes};
    if (cudaEventCreate(&r.e0) != cudaSuccess || cudaEventCreate(&r.e1) != cudaSuccess) return;
    cudaEventRecord(r.e0, st);
    std::lock_guard<std::mutex> lk(g_prof_mu);
    id = (int)g_prof.size();
    g_prof.push_back(r);
    stream_ = st;
}

ProfScope::~ProfScope()
{
    if (id < 0) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEventRecord(g_prof[id].e1, stream_);
}

}  // namespace dg

extern "C" {

long long dplr_gpu_launch_count(void) { return dg::g_launches.load(); }

void dplr_gpu_debug_fail_alloc(int after) { dg::g_fail_countdown.store(after < 0 ? -1 : after); }

int dplr_gpu_debug_wait_limit(int spins) { return dg::set_wait_limit(spins); }

void dplr_gpu_set_recompress(double eps) { dg::g_recompress_eps.store(eps >= 0.0 ? eps : -1.0); }

int dplr_gpu_profile_start(void)
{
    std::lock_guard<std::mutex> lk(dg::g_prof_mu);
    for (auto &r : dg::g_prof) {
        cudaEventDestroy(r.e0);
        cudaEventDestroy(r.e1);
    }
    dg::g_prof.clear();
    dg::g_prof_out.clear();
    dg::g_prof_on.store(1);
    return 0;
}

int dplr_gpu_profile_stop(void)
{
    dg::g_prof_on.store(0);
    std::lock_guard<std::mutex> lk(dg::g_prof_mu);
    dg::g_prof_out.clear();
    for (auto &r : dg::g_prof) {
        float ms = 0.0f;
        if (cudaEventSynchronize(r.e1) != cudaSuccess || cudaEventElapsedTime(&ms, r.e0, r.e1) != cudaSuccess)
            return fail(DPLR_GPU_ECUDA, "profile: event timing failed");
        dg::ProfAgg *a = nullptr;
        for (auto &x : dg::g_prof_out)
            if (x.name == r.name) a = &x;
        if (!a) {
            dg::g_prof_out.push_back(dg::ProfAgg());
            a = &dg::g_prof_out.back();
            a->name = r.name;
        }
        a->ms += ms;
        a->flops += r.flops;
        a->bytes += r.bytes;
        a->launches += 1;
        cudaEventDestroy(r.e0);
        cudaEventDestroy(r.e1);
    }
    dg::g_prof.clear();
    return (int)dg::g_prof_out.size();
}

int dplr_gpu_profile_entry(int i, const char **name, double *ms, double *flops, double *bytes,
                           int *launches)
{
    std::lock_guard<std::mutex> lk(dg::g_prof_mu);
    if (i < 0 || i >= (int)dg::g_prof_out.size()) return fail(DPLR_GPU_EINVAL, "profile: no entry %d", i);
    const dg::ProfAgg &a = dg::g_prof_out[i];
    if (name) *name = a.name.c_str();
    if (ms) *ms = a.ms;
    if (flops) *flops = a.flops;
    if (bytes) *bytes = a.bytes;
    if (launches) *launches = a.launches;
    return 0;
}

}  // extern "C"
