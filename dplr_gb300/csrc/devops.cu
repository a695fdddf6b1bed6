// devops.cu -- DPLR's structure arithmetic on device-resident plans:
//   dplr_gpu_plan_copy  B := A             (dplrcpy,   src/dplrcpy.c:19)
//   dplr_gpu_axpy       C := alpha A + B   (dplraxpy,  src/dplraxpy.c:81)
//   dplr_gpu_gep2d      D := dense(A)      (dplrgep2d, src/dplrp2d.c:98)
// so that a pipeline of scale / add / factor / solve never returns to host
// trees.  dplraxpy appends A's columns to every low-rank block of B
// (src/dplraxpy.c:17-71: rank r_A + r_B, sig of A scaled by |alpha|, u of A
// negated for alpha < 0) and adds the leaves; on the device the result is a
// new plan whose factor pool has room for the summed ranks, filled by one
// copy launch.  Low-rank columns are kept in DPLR's order: B's first, then
// A's.
#include "internal.cuh"
#include "svdblock.cuh"

#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

namespace dg {

namespace {

long long align32(long long x) { return (x + 31) & ~31LL; }

// dst[i] = sa * a[i] (+ b[i] when b != null), i < n
struct CopyJob {
    double *dst;
    const double *a, *b;
    long long n;
    double sa;
};

constexpr long long kJobChunk = 1 << 16;

__global__ void copy_jobs_kernel(const CopyJob *__restrict__ jobs)
{
    const CopyJob j = jobs[blockIdx.x];
    for (long long i = threadIdx.x; i < j.n; i += blockDim.x) {
        const double a = __ldg(j.a + i);
        j.dst[i] = j.b ? fma(j.sa, a, __ldg(j.b + i)) : j.sa * a;
    }
}

void add_job(std::vector<CopyJob> &v, double *dst, const double *a, const double *b, long long n, double sa)
{
    for (long long o = 0; o < n; o += kJobChunk)
        v.push_back(CopyJob{dst + o, a + o, b ? b + o : nullptr, std::min(kJobChunk, n - o), sa});
}

int run_jobs(const std::vector<CopyJob> &jobs, cudaStream_t st)
{
    if (jobs.empty()) return 0;
    CopyJob *d = nullptr;
    DG_ALLOC(&d, jobs.size() * sizeof(CopyJob));
    cudaError_t e = cudaMemcpyAsync(d, jobs.data(), jobs.size() * sizeof(CopyJob), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        copy_jobs_kernel<<<(unsigned)jobs.size(), 256, 0, st>>>(d);
        note_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e != cudaSuccess) return fail(DPLR_GPU_ECUDA, "device structure arithmetic: %s", cudaGetErrorString(e));
    return 0;
}

template <class T>
int upload(const std::vector<T> &v, T **dst, long long *bytes)
{
    const size_t n = std::max<size_t>(v.size(), 1);
    DG_ALLOC(dst, n * sizeof(T));
    *bytes += (long long)(n * sizeof(T));
    if (!v.empty()) DG_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

// A plan with ref's tree(s) and the low-rank ranks `ranks` (one per block of
// ref->lr): pool offsets are assigned in the walk order of plan.cu's builder
// (pre-order; at an H node ne, sw, then the nw and se subtrees), the tables
// and schedules uploaded and the pool allocated, uninitialised.
int clone_layout(const Plan *ref, const std::vector<int> &ranks, Plan **out)
{
    Plan *p = new Plan();
    p->m = ref->m;
    p->ntrees = ref->ntrees;
    p->tree_row0 = ref->tree_row0;
    p->nb_cap = ref->nb_cap;
    p->chunk_rows = ref->chunk_rows;
    p->levels = ref->levels;
    p->nodes = ref->nodes;
    p->lr = ref->lr;
    p->leaves = ref->leaves;
    struct Walk {
        Plan *p;
        const std::vector<int> &ranks;
        void leaf(int li)
        {
            LeafDesc &L = p->leaves[li];
            L.d = p->pool_doubles;
            p->pool_doubles += align32((long long)L.b * L.b);
            p->nnz += (long long)L.b * L.b;
        }
        void node(int hi)
        {
            const HDesc h = p->nodes[hi];
            for (int b : {h.ne, h.sw}) {
                LRDesc &d = p->lr[b];
                d.rank = ranks[b];
                d.u = p->pool_doubles;
                p->pool_doubles += align32((long long)d.n * d.rank);
                d.v = p->pool_doubles;
                p->pool_doubles += align32((long long)d.n * d.rank);
                d.sig = p->pool_doubles;
                p->pool_doubles += align32(d.rank);
                d.toff = p->total_rank;
                p->total_rank += d.rank;
                p->max_rank = std::max(p->max_rank, d.rank);
                p->nnz += 2LL * d.n * d.rank;
            }
            visit(h.nw);
            visit(h.se);
        }
        void visit(int c) { c >= 0 ? node(c) : leaf(~c); }
    } w{p, ranks};
    // roots in tree order: the parentless H node starting at the tree's first
    // row, or the tree's only leaf
    std::map<int, int> hroot, lroot;
    for (size_t i = 0; i < p->nodes.size(); ++i)
        if (p->nodes[i].parent < 0) hroot[p->nodes[i].row0] = (int)i;
    for (size_t i = 0; i < p->leaves.size(); ++i) lroot.emplace(p->leaves[i].row0, (int)i);
    for (int r0 : p->tree_row0) {
        auto h = hroot.find(r0);
        if (h != hroot.end())
            w.node(h->second);
        else
            w.leaf(lroot.at(r0));
    }
    build_schedule(p, 0, p->sched[0]);
    build_schedule(p, 1, p->sched[1]);
    long long bytes = 0;
    int rc = 0;
    const size_t pool_bytes = (size_t)std::max<long long>(p->pool_doubles, 1) * sizeof(double);
    if (dev_malloc((void **)&p->pool, pool_bytes) != cudaSuccess)
        rc = fail(DPLR_GPU_ENOMEM, "cannot allocate %zu bytes of factor pool", pool_bytes);
    else if (cudaMemset(p->pool, 0, pool_bytes) != cudaSuccess)     // alignment gaps stay zero
        rc = fail(DPLR_GPU_ECUDA, "cannot clear the factor pool");
    bytes += (long long)pool_bytes;
    if (!rc) rc = upload(p->lr, &p->d_lr, &bytes);
    if (!rc) rc = upload(p->leaves, &p->d_leaves, &bytes);
    if (!rc) rc = upload_schedule(p->sched[0], &bytes);
    if (!rc) rc = upload_schedule(p->sched[1], &bytes);
    if (rc) {
        plan_free(p);
        return rc;
    }
    p->device_bytes = bytes;
    *out = p;
    return 0;
}

bool same_structure(const Plan *a, const Plan *b)
{
    if (a->m != b->m || a->ntrees != b->ntrees || a->tree_row0 != b->tree_row0 || a->lr.size() != b->lr.size() ||
        a->leaves.size() != b->leaves.size() || a->nodes.size() != b->nodes.size())
        return false;
    for (size_t i = 0; i < a->lr.size(); ++i)
        if (a->lr[i].n != b->lr[i].n || a->lr[i].row0 != b->lr[i].row0 || a->lr[i].col0 != b->lr[i].col0)
            return false;
    for (size_t i = 0; i < a->leaves.size(); ++i)
        if (a->leaves[i].b != b->leaves[i].b || a->leaves[i].row0 != b->leaves[i].row0) return false;
    return true;
}

// dense expansion: one CTA per 32 x 32 output tile of one block or leaf
struct DenseTile {
    int kind;             // 0: low-rank block, 1: leaf
    int idx, i0, j0;
};

__global__ void gep2d_kernel(const DenseTile *__restrict__ tiles, const LRDesc *__restrict__ lr,
                             const LeafDesc *__restrict__ leaves, const double *__restrict__ pool,
                             double *__restrict__ D, long long ldd)
{
    const DenseTile t = tiles[blockIdx.x];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;       // 32 x 8 threads, 4 rows each
    if (t.kind == 1) {
        const LeafDesc L = leaves[t.idx];
        for (int r = ty; r < 32; r += 8) {
            const int i = t.i0 + tx, j = t.j0 + r;
            if (i < L.b && j < L.b)
                D[(long long)(L.row0 + i) + (long long)(L.row0 + j) * ldd] = __ldg(pool + L.d + i + (long long)j * L.b);
        }
        return;
    }
    const LRDesc B = lr[t.idx];
    for (int r = ty; r < 32; r += 8) {
        const int i = t.i0 + tx, j = t.j0 + r;
        if (i >= B.n || j >= B.n) continue;
        double s = 0.0;
        for (int k = 0; k < B.rank; ++k)
            s = fma(__ldg(pool + B.u + i + (long long)k * B.n) * __ldg(pool + B.sig + k),
                    __ldg(pool + B.v + j + (long long)k * B.n), s);
        D[(long long)(B.row0 + i) + (long long)(B.col0 + j) * ldd] = s;
    }
}

// SVD recompression of every low-rank block of a plan into a new plan
// (dplrreduce's thresholds: eps / 4^(depth + 1), src/dplrreduce.c:46): the
// factors are read from the pool, each block's truncated SVD is written into
// a scratch copy of the pool at the block's own offsets (ranks only
// shrink), then the new plan with the new ranks is filled from it.
int plan_reduce(Plan *p, double eps, int workers, cudaStream_t st, Plan **out)
{
    *out = nullptr;
    DG_CUDA(cudaStreamSynchronize(st));       // the workers read the pool on their own streams
    const size_t bytes = (size_t)std::max<long long>(p->pool_doubles, 1) * sizeof(double);
    double *scratch = nullptr;
    DG_ALLOC(&scratch, bytes);
    // a block whose SVD does not converge keeps its factors: start from a copy
    cudaError_t e = cudaMemcpy(scratch, p->pool, bytes, cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);   // done before other streams write the scratch
    if (e != cudaSuccess) {
        cudaFree(scratch);
        return fail(DPLR_GPU_ECUDA, "plan recompression: %s", cudaGetErrorString(e));
    }
    std::vector<SvdBlock> blocks;
    for (const LRDesc &L : p->lr) {
        double thr = eps;
        for (int l = 0; l <= L.level; ++l) thr /= 4.0;
        blocks.push_back({p->pool + L.u, p->pool + L.v, p->pool + L.sig, scratch + L.u, scratch + L.v,
                          scratch + L.sig, L.n, L.rank, thr, L.rank});
    }
    int rc = svd_truncate_blocks(blocks.data(), (int)blocks.size(), workers);
    if (rc && rc != DPLR_GPU_ENOTCONV) {
        cudaFree(scratch);
        return rc;
    }
    std::vector<int> ranks;
    for (const SvdBlock &b : blocks) ranks.push_back(b.rank);
    Plan *c = nullptr;
    int rc2 = clone_layout(p, ranks, &c);
    if (rc2) {
        cudaFree(scratch);
        return rc2;
    }
    std::vector<CopyJob> jobs;
    for (size_t i = 0; i < c->lr.size(); ++i) {
        const LRDesc &dc = c->lr[i], &ds = p->lr[i];
        const long long n = (long long)dc.n * dc.rank;
        add_job(jobs, c->pool + dc.u, scratch + ds.u, nullptr, n, 1.0);
        add_job(jobs, c->pool + dc.v, scratch + ds.v, nullptr, n, 1.0);
        add_job(jobs, c->pool + dc.sig, scratch + ds.sig, nullptr, dc.rank, 1.0);
    }
    for (size_t i = 0; i < c->leaves.size(); ++i)
        add_job(jobs, c->pool + c->leaves[i].d, p->pool + p->leaves[i].d, nullptr,
                (long long)c->leaves[i].b * c->leaves[i].b, 1.0);
    rc2 = run_jobs(jobs, st);
    cudaFree(scratch);
    if (rc2) {
        plan_free(c);
        return rc2;
    }
    *out = c;
    return rc;        // DPLR_GPU_ENOTCONV reports the kept blocks, the plan is valid
}

}  // namespace

}  // namespace dg

using namespace dg;

extern "C" {

int dplr_gpu_plan_copy(dplr_gpu_plan plan, void *stream, dplr_gpu_plan *out)
{
    dg::NvtxRange nvtx_("dplr_gpu_plan_copy");
    Plan *a = (Plan *)plan;
    if (!a || !out) return fail(DPLR_GPU_EINVAL, "dplr_gpu_plan_copy: null argument");
    *out = nullptr;
    std::vector<int> ranks;
    for (const LRDesc &d : a->lr) ranks.push_back(d.rank);
    Plan *c = nullptr;
    int rc = clone_layout(a, ranks, &c);
    if (rc) return rc;
    // same layout: the pool is one device-to-device copy
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(c->pool, a->pool, (size_t)a->pool_doubles * sizeof(double),
                                    cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        plan_free(c);
        return fail(DPLR_GPU_ECUDA, "dplr_gpu_plan_copy: %s", cudaGetErrorString(e));
    }
    *out = (dplr_gpu_plan)c;
    return 0;
}

int dplr_gpu_axpy(double alpha, dplr_gpu_plan A, dplr_gpu_plan B, void *stream, dplr_gpu_plan *out)
{
    dg::NvtxRange nvtx_("dplr_gpu_axpy");
    Plan *a = (Plan *)A, *b = (Plan *)B;
    if (!a || !b || !out) return fail(DPLR_GPU_EINVAL, "dplr_gpu_axpy: null argument");
    *out = nullptr;
    if (!same_structure(a, b)) return fail(DPLR_GPU_EINVAL, "dplr_gpu_axpy: A and B differ in structure");
    const bool add = alpha != 0.0;        // alpha == 0: C = B (dplraxpy returns early)
    std::vector<int> ranks;
    for (size_t i = 0; i < b->lr.size(); ++i) ranks.push_back(b->lr[i].rank + (add ? a->lr[i].rank : 0));
    Plan *c = nullptr;
    int rc = clone_layout(b, ranks, &c);
    if (rc) return rc;
    std::vector<CopyJob> jobs;
    const double aa = std::fabs(alpha), su = alpha < 0.0 ? -1.0 : 1.0;
    for (size_t i = 0; i < c->lr.size(); ++i) {
        const LRDesc &dc = c->lr[i], &db = b->lr[i], &da = a->lr[i];
        const long long nb = (long long)db.n * db.rank, na = (long long)da.n * da.rank;
        add_job(jobs, c->pool + dc.u, b->pool + db.u, nullptr, nb, 1.0);
        add_job(jobs, c->pool + dc.v, b->pool + db.v, nullptr, nb, 1.0);
        add_job(jobs, c->pool + dc.sig, b->pool + db.sig, nullptr, db.rank, 1.0);
        if (add && da.rank) {
            add_job(jobs, c->pool + dc.u + nb, a->pool + da.u, nullptr, na, su);
            add_job(jobs, c->pool + dc.v + nb, a->pool + da.v, nullptr, na, 1.0);
            add_job(jobs, c->pool + dc.sig + db.rank, a->pool + da.sig, nullptr, da.rank, aa);
        }
    }
    for (size_t i = 0; i < c->leaves.size(); ++i) {
        const long long n = (long long)c->leaves[i].b * c->leaves[i].b;
        double *dst = c->pool + c->leaves[i].d;
        if (add)          // B + alpha A, one fused multiply-add per entry
            add_job(jobs, dst, a->pool + a->leaves[i].d, b->pool + b->leaves[i].d, n, alpha);
        else
            add_job(jobs, dst, b->pool + b->leaves[i].d, nullptr, n, 1.0);
    }
    if ((rc = run_jobs(jobs, (cudaStream_t)stream))) {
        plan_free(c);
        return rc;
    }
    // the ranks grew: recompress when dplr_gpu_set_recompress asked for it
    const double reps = recompress_eps();
    if (add && reps >= 0.0) {
        Plan *r = nullptr;
        rc = plan_reduce(c, reps, 0, (cudaStream_t)stream, &r);
        plan_free(c);
        if (!r) return rc;
        c = r;
    }
    *out = (dplr_gpu_plan)c;
    return 0;
}

int dplr_gpu_plan_reduce_svd(dplr_gpu_plan plan, double eps, int workers, void *stream, dplr_gpu_plan *out)
{
    dg::NvtxRange nvtx_("dplr_gpu_plan_reduce_svd");
    Plan *p = (Plan *)plan;
    if (!p || !out) return fail(DPLR_GPU_EINVAL, "dplr_gpu_plan_reduce_svd: null argument");
    *out = nullptr;
    if (!(eps >= 0.0)) return fail(DPLR_GPU_EINVAL, "dplr_gpu_plan_reduce_svd: eps must be nonnegative");
    Plan *r = nullptr;
    const int rc = plan_reduce(p, eps, workers, (cudaStream_t)stream, &r);
    *out = (dplr_gpu_plan)r;
    return rc;
}

int dplr_gpu_gep2d(dplr_gpu_plan plan, double *D, long long ldd, void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_gep2d");
    Plan *p = (Plan *)plan;
    if (!p || (!D && p->m > 0)) return fail(DPLR_GPU_EINVAL, "dplr_gpu_gep2d: null argument");
    if (ldd < std::max(p->m, 1)) return fail(DPLR_GPU_EINVAL, "dplr_gpu_gep2d: ldd smaller than the matrix");
    if (p->m == 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<DenseTile> tiles;
    for (size_t i = 0; i < p->lr.size(); ++i)
        for (int i0 = 0; i0 < p->lr[i].n; i0 += 32)
            for (int j0 = 0; j0 < p->lr[i].n; j0 += 32) tiles.push_back(DenseTile{0, (int)i, i0, j0});
    for (size_t i = 0; i < p->leaves.size(); ++i)
        for (int i0 = 0; i0 < p->leaves[i].b; i0 += 32)
            for (int j0 = 0; j0 < p->leaves[i].b; j0 += 32) tiles.push_back(DenseTile{1, (int)i, i0, j0});
    // blocks of a batch outside its diagonal trees are zero
    DG_CUDA(cudaMemset2DAsync(D, (size_t)ldd * sizeof(double), 0, (size_t)p->m * sizeof(double), (size_t)p->m, st));
    if (tiles.empty()) return 0;
    DenseTile *d = nullptr;
    DG_ALLOC(&d, tiles.size() * sizeof(DenseTile));
    cudaError_t e = cudaMemcpyAsync(d, tiles.data(), tiles.size() * sizeof(DenseTile), cudaMemcpyHostToDevice, st);
    for (size_t o = 0; e == cudaSuccess && o < tiles.size(); o += 1u << 30) {
        const unsigned n = (unsigned)std::min<size_t>(tiles.size() - o, 1u << 30);
        gep2d_kernel<<<n, 256, 0, st>>>(d + o, p->d_lr, p->d_leaves, p->pool, D, ldd);
        note_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e != cudaSuccess) return fail(DPLR_GPU_ECUDA, "dplr_gpu_gep2d: %s", cudaGetErrorString(e));
    return 0;
}

}  // extern "C"
