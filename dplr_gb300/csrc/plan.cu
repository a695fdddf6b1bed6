// plan.cu -- flatten a host PLR tree into the device block table.
//
// The tree walk visits nodes in the order of DPLR's recursions
// (src/dplrpmv.c:166-173: ne, sw, then nw, se), records one LRDesc per
// low-rank block and one LeafDesc per dense leaf, assigns every factor
// array a 256-byte aligned slot in one FP64 pool, and builds the apply
// schedules for op N and op T.
#include "internal.cuh"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>

namespace dg {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

int fail(int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

const char *last_error_c() { return g_last_error.c_str(); }

static long long align32(long long x) { return (x + 31) & ~31LL; }

// Structural checks performed by DPLR's recursions before they touch any
// output (src/dplrpmv.c:22-36, :116-130); here they run over the whole
// tree up front so that a malformed tree never produces partial output.
static int check_node(const DPlrMtx *A, int m, const char *fn, int depth)
{
    if (!A) return fail(DPLR_GPU_EINVAL, "%s: null node", fn);
    if (depth > 60) return fail(DPLR_GPU_EINVAL, "%s: tree too deep", fn);
    if (A->type != PLR_DMTX && A->type != PLR_HMTX)
        return fail(DPLR_GPU_EINVAL, "%s: invalid A type", fn);
    if (A->size != m) return fail(DPLR_GPU_EINVAL, "%s: invalid A size", fn);
    if (A->type == PLR_DMTX) {
        if (m > 0 && !A->dd.d) return fail(DPLR_GPU_EINVAL, "%s: dense leaf without data", fn);
        if ((long long)m * m > (1LL << 31))
            return fail(DPLR_GPU_EINVAL, "%s: dense leaf too large", fn);
        return 0;
    }
    if (m % 2 != 0) return fail(DPLR_GPU_EINVAL, "%s: H node of odd size %d", fn, m);
    int h = m / 2;
    const DPlrMtx *lr[2] = {A->dh.ne, A->dh.sw};
    for (const DPlrMtx *L : lr) {
        if (!L) return fail(DPLR_GPU_EINVAL, "%s: null low-rank block", fn);
        if (L->type != PLR_LRMTX) return fail(DPLR_GPU_EINVAL, "%s: invalid A type", fn);
        if (L->size != h) return fail(DPLR_GPU_EINVAL, "%s: invalid A size", fn);
        if (L->dlr.rank < 0 || L->dlr.rank > L->dlr.capacity)
            return fail(DPLR_GPU_EINVAL, "%s: rank %d outside [0, capacity %d]", fn,
                        L->dlr.rank, L->dlr.capacity);
        if (L->dlr.rank > 0 && (!L->dlr.u || !L->dlr.v || !L->dlr.sig))
            return fail(DPLR_GPU_EINVAL, "%s: low-rank block without data", fn);
    }
    int rc = check_node(A->dh.nw, h, fn, depth + 1);
    if (rc) return rc;
    return check_node(A->dh.se, h, fn, depth + 1);
}

int validate_tree(int m, const DPlrMtx *A, const char *fn)
{
    if (m < 0) return fail(DPLR_GPU_EINVAL, "%s: invalid matrix size %d", fn, m);
    return check_node(A, m, fn, 0);
}

// ------------------------------------------------------------- flattening
struct Builder {
    Plan *p;
    int walk(const DPlrMtx *A, int row0, int level)
    {
        if (A->type == PLR_DMTX) {
            LeafDesc L;
            L.d = p->pool_doubles;
            L.row0 = row0;
            L.b = A->size;
            p->pool_doubles += align32((long long)L.b * L.b);
            p->leaves.push_back(L);
            p->nnz += (long long)L.b * L.b;
            return ~(int)(p->leaves.size() - 1);
        }
        int idx = (int)p->nodes.size();
        p->nodes.push_back(HDesc{});
        int h = A->size / 2;
        p->levels = std::max(p->levels, level + 1);
        int ids[2];
        for (int s = 0; s < 2; ++s) {
            const DPlrMtx *B = s == 0 ? A->dh.ne : A->dh.sw;
            LRDesc d;
            d.n = h;
            d.rank = B->dlr.rank;
            d.row0 = s == 0 ? row0 : row0 + h;
            d.col0 = s == 0 ? row0 + h : row0;
            d.level = level;
            d.node = idx;
            d.is_ne = s == 0;
            d.u = p->pool_doubles;
            p->pool_doubles += align32((long long)h * d.rank);
            d.v = p->pool_doubles;
            p->pool_doubles += align32((long long)h * d.rank);
            d.sig = p->pool_doubles;
            p->pool_doubles += align32(d.rank);
            d.toff = p->total_rank;
            p->total_rank += d.rank;
            p->max_rank = std::max(p->max_rank, d.rank);
            p->nnz += 2LL * h * d.rank;          // U and V, as src/dplrnz.c:45 counts
            ids[s] = (int)p->lr.size();
            p->lr.push_back(d);
        }
        HDesc hd;
        hd.row0 = row0;
        hd.m = A->size;
        hd.level = level;
        hd.ne = ids[0];
        hd.sw = ids[1];
        hd.parent = -1;
        hd.nw = walk(A->dh.nw, row0, level + 1);
        hd.se = walk(A->dh.se, row0 + h, level + 1);
        if (hd.nw >= 0) p->nodes[hd.nw].parent = idx;
        if (hd.se >= 0) p->nodes[hd.se].parent = idx;
        p->nodes[idx] = hd;
        return idx;
    }
};

static int gcd_int(int a, int b) { return b == 0 ? a : gcd_int(b, a % b); }

// Tile height: a power of two (<= 64) dividing every leaf size, so every
// block and leaf boundary falls on a tile boundary.
int tile_rows_for(const Plan *p)
{
    int g = 0;
    for (const LeafDesc &L : p->leaves) g = gcd_int(g, L.b);
    int R = 64;
    while (R > 1 && g > 0 && (g % R) != 0) R >>= 1;
    return R;
}

// Apply schedule for op N (trans = 0) or op T (trans = 1): panels contract
// V (U) with x over the block's input rows, tiles expand U (V) T_b over the
// block's output rows plus the leaf term.
// Output tiles of R rows (R divides every leaf) and their terms: every
// low-rank block whose output rows cover the tile, then the leaf term.
// Blocks of H nodes shallower than lmin are left out: the schedule then
// applies the block-diagonal part of the matrix made of its subtrees at
// depth lmin (and the leaves above them).
void build_tiles(const Plan *p, int trans, int R, std::vector<int> &row0, std::vector<int> &begin,
                 std::vector<TileTerm> &terms, int lmin)
{
    int ntiles = p->m / R;
    std::vector<std::vector<TileTerm>> per(ntiles);
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        if (L.rank == 0 || L.level < lmin) continue;
        int out0 = trans ? L.col0 : L.row0;
        long long base = trans ? L.v : L.u;
        for (int t0 = out0; t0 < out0 + L.n; t0 += R) {
            TileTerm tt;
            tt.a = base + (t0 - out0);
            tt.b = L.toff;
            tt.lda = L.n;
            tt.K = L.rank;
            tt.trans_a = 0;
            tt.src = 0;
            tt.ldb = L.rank;
            tt.x_row0 = 0;
            per[t0 / R].push_back(tt);
        }
    }
    for (const LeafDesc &L : p->leaves) {
        for (int t0 = L.row0; t0 < L.row0 + L.b; t0 += R) {
            TileTerm tt;
            tt.b = 0;
            tt.lda = L.b;
            tt.K = L.b;
            tt.src = 1;
            tt.ldb = 0;
            tt.x_row0 = L.row0;
            if (!trans) {
                tt.a = L.d + (t0 - L.row0);
                tt.trans_a = 0;
            } else {
                tt.a = L.d + (long long)(t0 - L.row0) * L.b;
                tt.trans_a = 1;
            }
            per[t0 / R].push_back(tt);
        }
    }
    row0.clear();
    begin.clear();
    terms.clear();
    for (int t = 0; t < ntiles; ++t) {
        row0.push_back(t * R);
        begin.push_back((int)terms.size());
        terms.insert(terms.end(), per[t].begin(), per[t].end());
    }
    begin.push_back((int)terms.size());
}

void build_schedule(const Plan *p, int trans, Schedule &S, int lmin)
{
    const int CH = p->chunk_rows;
    S.items.clear();
    S.reduces.clear();
    long long poff = 0;
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        if (L.rank == 0 || L.n == 0 || L.level < lmin) continue;
        int nch = (L.n + CH - 1) / CH;
        for (int c = 0; c < nch; ++c) {
            PanelItem it;
            it.f = trans ? L.u : L.v;
            it.p = poff;
            it.in0 = trans ? L.row0 : L.col0;
            it.n = L.n;
            it.rank = L.rank;
            it.r0 = c * CH;
            it.len = std::min(CH, L.n - c * CH);
            it.chunk = c;
            S.items.push_back(it);
        }
        ReduceItem r;
        r.p = poff;
        r.t = L.toff;
        r.sig = L.sig;
        r.rank = L.rank;
        r.nch = nch;
        S.reduces.push_back(r);
        poff += (long long)nch * L.rank;
    }
    S.partial_per_rhs = poff;
    S.t_per_rhs = p->total_rank;
    S.max_rank = p->max_rank;

    S.tile_rows = tile_rows_for(p);
    build_tiles(p, trans, S.tile_rows, S.tile_row0, S.tile_begin, S.terms, lmin);
}

template <class T>
static int upload_vec(const std::vector<T> &v, T **dst, long long *bytes)
{
    size_t n = std::max<size_t>(v.size(), 1);
    DG_ALLOC(dst, n * sizeof(T));
    *bytes += (long long)(n * sizeof(T));
    if (!v.empty()) DG_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

int upload_schedule(Schedule &S, long long *bytes)
{
    S.max_len = 0;
    for (const PanelItem &it : S.items) S.max_len = std::max(S.max_len, it.len);
    S.has_row_major = false;
    for (const TileTerm &t : S.terms) S.has_row_major = S.has_row_major || t.trans_a;
    int rc;
    if ((rc = upload_vec(S.items, &S.d_items, bytes))) return rc;
    if ((rc = upload_vec(S.reduces, &S.d_reduces, bytes))) return rc;
    if ((rc = upload_vec(S.tile_row0, &S.d_tile_row0, bytes))) return rc;
    if ((rc = upload_vec(S.tile_begin, &S.d_tile_begin, bytes))) return rc;
    if ((rc = upload_vec(S.terms, &S.d_terms, bytes))) return rc;
    return upload_vec(S.caps, &S.d_caps, bytes);
}

// Copy live factor values from the host tree into the pool, in the same
// pre-order as Builder::walk.
struct Uploader {
    Plan *p;
    cudaStream_t st;
    size_t lr_i = 0, leaf_i = 0;
    int walk(const DPlrMtx *A)
    {
        if (A->type == PLR_DMTX) {
            const LeafDesc &L = p->leaves[leaf_i++];
            if (L.b > 0)
                DG_CUDA(cudaMemcpyAsync(p->pool + L.d, A->dd.d, sizeof(double) * L.b * L.b,
                                        cudaMemcpyHostToDevice, st));
            return 0;
        }
        for (int s = 0; s < 2; ++s) {
            const DPlrMtx *B = s == 0 ? A->dh.ne : A->dh.sw;
            const LRDesc &L = p->lr[lr_i++];
            if (B->dlr.rank != L.rank || B->size != L.n)
                return fail(DPLR_GPU_EINVAL, "plan refresh: structure or rank changed");
            size_t cnt = (size_t)L.n * L.rank;
            if (cnt) {
                DG_CUDA(cudaMemcpyAsync(p->pool + L.u, B->dlr.u, cnt * sizeof(double),
                                        cudaMemcpyHostToDevice, st));
                DG_CUDA(cudaMemcpyAsync(p->pool + L.v, B->dlr.v, cnt * sizeof(double),
                                        cudaMemcpyHostToDevice, st));
                DG_CUDA(cudaMemcpyAsync(p->pool + L.sig, B->dlr.sig, L.rank * sizeof(double),
                                        cudaMemcpyHostToDevice, st));
            }
        }
        int rc = walk(A->dh.nw);
        if (rc) return rc;
        return walk(A->dh.se);
    }
};

int plan_upload_values(Plan *p, const DPlrMtx *A, cudaStream_t st)
{
    if (p->ntrees != 1) return fail(DPLR_GPU_EINVAL, "plan refresh: batched plans are refreshed through the pool");
    if (!A || A->size != p->m) return fail(DPLR_GPU_EINVAL, "plan refresh: size mismatch");
    int rc = validate_tree(p->m, A, "dplr_gpu_plan_refresh");
    if (rc) return rc;
    Uploader up{p, st};
    rc = up.walk(A);
    if (rc) return rc;
    if (up.lr_i != p->lr.size() || up.leaf_i != p->leaves.size())
        return fail(DPLR_GPU_EINVAL, "plan refresh: structure changed");
    if ((rc = pairs_refresh(p, st))) return rc;
    DG_CUDA(cudaStreamSynchronize(st));
    return 0;
}

int plan_build(int m, const DPlrMtx *A, cudaStream_t st, Plan **out)
{
    return plan_build_forest(1, &m, &A, st, out);
}

// A forest of independent trees as one block-diagonal matrix: tree i owns
// rows [sum_{k<i} m_k, sum_{k<=i} m_k).  Blocks and leaves of all trees go
// into the same tables, so every phase covers all trees in one launch.
int plan_build_forest(int count, const int *ms, const DPlrMtx *const *As, cudaStream_t st, Plan **out)
{
    int rc;
    long long total = 0;
    for (int i = 0; i < count; ++i) {
        if ((rc = validate_tree(ms[i], As[i], count == 1 ? "dplr_gpu_plan_create" : "dplr_gpu_batch_create")))
            return rc;
        total += ms[i];
    }
    if (total > (1LL << 31) - 1) return fail(DPLR_GPU_EINVAL, "plan: %lld rows exceed the int range", total);
    Plan *p = new Plan();
    p->m = (int)total;
    p->ntrees = count;
    Builder b{p};
    int row0 = 0;
    for (int i = 0; i < count; ++i) {
        p->tree_row0.push_back(row0);
        b.walk(As[i], row0, 0);
        row0 += ms[i];
    }
    build_schedule(p, 0, p->sched[0]);
    build_schedule(p, 1, p->sched[1]);
    long long bytes = 0;
    size_t pool_bytes = (size_t)std::max<long long>(p->pool_doubles, 1) * sizeof(double);
    cudaError_t e = dev_malloc((void **)&p->pool, pool_bytes);
    if (e != cudaSuccess) {
        plan_free(p);
        return fail(DPLR_GPU_ENOMEM, "plan: cannot allocate %zu bytes of factor pool: %s",
                    pool_bytes, cudaGetErrorString(e));
    }
    bytes += (long long)pool_bytes;
    // the 256-byte alignment gaps between arrays are zero, so that two plans
    // of equal factors have equal pools
    if (cudaMemsetAsync(p->pool, 0, pool_bytes, st) != cudaSuccess) {
        plan_free(p);
        return fail(DPLR_GPU_ECUDA, "plan: cannot clear the factor pool");
    }
    if ((rc = upload_vec(p->lr, &p->d_lr, &bytes)) || (rc = upload_vec(p->leaves, &p->d_leaves, &bytes)) ||
        (rc = upload_schedule(p->sched[0], &bytes)) || (rc = upload_schedule(p->sched[1], &bytes))) {
        plan_free(p);
        return rc;
    }
    p->device_bytes = bytes;
    Uploader up{p, st};
    for (int i = 0; i < count && !rc; ++i) rc = up.walk(As[i]);
    if (!rc) {
        cudaError_t e2 = cudaStreamSynchronize(st);
        if (e2 != cudaSuccess) rc = fail(DPLR_GPU_ECUDA, "plan upload: %s", cudaGetErrorString(e2));
    }
    if (rc) {
        plan_free(p);
        return rc;
    }
    *out = p;
    return 0;
}

// Rebuild the apply schedules (after a change of the panel chunk length).
int plan_reschedule(Plan *p)
{
    long long bytes = 0;
    free_schedule(p->sched[0]);
    free_schedule(p->sched[1]);
    build_schedule(p, 0, p->sched[0]);
    build_schedule(p, 1, p->sched[1]);
    int rc;
    if ((rc = upload_schedule(p->sched[0], &bytes)) || (rc = upload_schedule(p->sched[1], &bytes))) return rc;
    return 0;
}

void free_schedule(Schedule &S)
{
    cudaFree(S.d_items);
    cudaFree(S.d_reduces);
    cudaFree(S.d_tile_row0);
    cudaFree(S.d_tile_begin);
    cudaFree(S.d_terms);
    cudaFree(S.d_caps);
    cudaFree(S.d_item_red);
    cudaFree(S.d_term_red);
    S.d_item_red = S.d_term_red = nullptr;
    S.d_items = nullptr;
    S.d_reduces = nullptr;
    S.d_tile_row0 = S.d_tile_begin = nullptr;
    S.d_terms = nullptr;
    S.d_caps = nullptr;
}

void factor_free(Plan *p);   // factor.cu
void sliced_free(Plan *p);   // sliced.cu
void mixed_free(Plan *p);    // sliced.cu

void plan_free(Plan *p)
{
    if (!p) return;
    mixed_free(p);
    factor_free(p);
    sliced_free(p);
    pairs_free(p);
    cudaFree(p->pool);
    cudaFree(p->d_lr);
    cudaFree(p->d_leaves);
    cudaFree(p->d_tree_row0);
    free_schedule(p->sched[0]);
    free_schedule(p->sched[1]);
    cudaFree(p->work);
    cudaFree(p->xbuf);
    cudaFree(p->ybuf);
    if (p->tc_err_h) cudaFreeHost(p->tc_err_h);
    grad_free(p);
    cudaFree(p->gbuf);
    delete p;
}

int ensure_buffer(double **buf, size_t *have, size_t need)
{
    if (need <= *have && *buf) return 0;
    if (*buf) cudaFree(*buf);
    *buf = nullptr;
    *have = 0;
    size_t n = std::max<size_t>(need, 1);
    cudaError_t e = dev_malloc((void **)buf, n * sizeof(double));
    if (e != cudaSuccess)
        return fail(DPLR_GPU_ENOMEM, "cannot allocate %zu bytes of device scratch: %s",
                    n * sizeof(double), cudaGetErrorString(e));
    *have = n;
    return 0;
}

}  // namespace dg
