// batch.cu -- many independent PLR matrices in one plan, CUDA-graph replay
// of the apply and solve, and the launch-shape autotuner.
//
// A batch is a forest: tree i is the diagonal block of rows
// [off_i, off_i + m_i) of one block-diagonal matrix.  The block tables,
// work lists and factor pool of all trees are merged, so an apply, a
// Woodbury factorisation or a solve of the batch is the same handful of
// launches as for one matrix (each launch's grid spans every tree's work
// items); trees of different depth simply contribute nothing to levels they
// do not have.  Right-hand sides are stacked the same way ((sum m_i) x n);
// a matrix with fewer right-hand sides leaves its extra columns unused.
#include "internal.cuh"
#include "factor.cuh"

#include <algorithm>
#include <vector>

namespace dg {

namespace {

struct GraphH {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
    long long kernels = 0;
};

int run_op(Plan *p, char op, int trans, int n, const double *X, int ldx, double *Y, int ldy, cudaStream_t st)
{
    if (op == 'A' || op == 'a') return apply_device(p, trans, n, 1.0, X, ldx, 0.0, Y, ldy, st, false);
    if (op == 'R' || op == 'r') return refine_fixed(p, n, X, ldx, Y, ldy, 2, st);
    if (op == 'C' || op == 'c') return refine_fixed(p, n, X, ldx, Y, ldy, 1, st);
    return factor_solve(p, trans, n, X, ldx, Y, ldy, st);
}

void set_nb_cap(Plan *p, int cap)
{
    p->nb_cap = cap;
    p->sched[0].nb_cap = p->sched[1].nb_cap = cap;
}

}  // namespace

}  // namespace dg

using namespace dg;

extern "C" {

int dplr_gpu_batch_create(int count, const int *m, DPlrMtx *const *A, void *stream, dplr_gpu_plan *plan)
{
    dg::NvtxRange nvtx_("dplr_gpu_batch_create");
    if (!plan || count <= 0 || !m || !A) return fail(DPLR_GPU_EINVAL, "dplr_gpu_batch_create: invalid arguments");
    *plan = nullptr;
    for (int i = 0; i < count; ++i)
        if (!A[i] || m[i] < 0) return fail(DPLR_GPU_EINVAL, "dplr_gpu_batch_create: matrix %d is invalid", i);
    std::vector<const DPlrMtx *> trees(A, A + count);
    Plan *p = nullptr;
    int rc = plan_build_forest(count, m, trees.data(), (cudaStream_t)stream, &p);
    if (rc) return rc;
    *plan = (dplr_gpu_plan)p;
    return 0;
}

int dplr_gpu_batch_offsets(dplr_gpu_plan plan, int *count, int *row0)
{
    Plan *p = (Plan *)plan;
    if (!p) return fail(DPLR_GPU_EINVAL, "dplr_gpu_batch_offsets: null plan");
    if (count) *count = p->ntrees;
    if (row0) std::copy(p->tree_row0.begin(), p->tree_row0.end(), row0);
    return 0;
}

int dplr_gpu_graph_create(dplr_gpu_plan plan, char op, char trans, int n, const double *X, int ldx, double *Y,
                          int ldy, void *stream, dplr_gpu_graph *graph)
{
    dg::NvtxRange nvtx_("dplr_gpu_graph_create");
    Plan *p = (Plan *)plan;
    if (!p || !graph) return fail(DPLR_GPU_EINVAL, "dplr_gpu_graph_create: null argument");
    *graph = nullptr;
    const int mm = std::max(p->m, 1);
    if (n <= 0 || ldx < mm || ldy < mm || !X || !Y || X == Y)
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_graph_create: invalid n, leading dimension or pointers");
    if (!(op == 'A' || op == 'a' || op == 'S' || op == 's' || op == 'R' || op == 'r' || op == 'C' || op == 'c'))
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_graph_create: op must be 'A' (apply), 'S' (solve), 'C' (solve "
                                     "with one refinement step) or 'R' (two refinement steps)");
    const int tr = !(trans == 'N' || trans == 'n');
    if ((op == 'R' || op == 'r' || op == 'C' || op == 'c') && tr)
        return fail(DPLR_GPU_EINVAL, "dplr_gpu_graph_create: the refined solve is op N only");
    GraphH *g = new GraphH();
    auto bail = [&](int rc) {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        if (g->graph) cudaGraphDestroy(g->graph);
        if (g->cs) cudaStreamDestroy(g->cs);
        delete g;
        return rc;
    };
    if (cudaStreamCreateWithFlags(&g->cs, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(DPLR_GPU_ECUDA, "dplr_gpu_graph_create: cannot create a stream"));
    // order after the caller's prior work, then size every scratch buffer
    // with one ordinary run so that the captured run allocates nothing
    cudaEvent_t ev;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(DPLR_GPU_ECUDA, "dplr_gpu_graph_create: cannot create an event"));
    cudaEventRecord(ev, (cudaStream_t)stream);
    cudaStreamWaitEvent(g->cs, ev, 0);
    cudaEventDestroy(ev);
    int rc = run_op(p, op, tr, n, X, ldx, Y, ldy, g->cs);
    if (rc) return bail(rc);
    if (cudaStreamSynchronize(g->cs) != cudaSuccess)
        return bail(fail(DPLR_GPU_ECUDA, "dplr_gpu_graph_create: warm-up run failed"));
    const long long l0 = dplr_gpu_launch_count();
    if (cudaStreamBeginCapture(g->cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return bail(fail(DPLR_GPU_ECUDA, "dplr_gpu_graph_create: cannot begin capture"));
    rc = run_op(p, op, tr, n, X, ldx, Y, ldy, g->cs);
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamEndCapture(g->cs, &gr);
    g->graph = gr;
    if (rc) return bail(rc);
    if (e != cudaSuccess)
        return bail(fail(DPLR_GPU_ECUDA, "dplr_gpu_graph_create: capture failed: %s", cudaGetErrorString(e)));
    g->kernels = dplr_gpu_launch_count() - l0;
    if (cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess)
        return bail(fail(DPLR_GPU_ECUDA, "dplr_gpu_graph_create: cannot instantiate the graph"));
    *graph = (dplr_gpu_graph)g;
    return 0;
}

int dplr_gpu_graph_launch(dplr_gpu_graph graph, void *stream)
{
    GraphH *g = (GraphH *)graph;
    if (!g) return fail(DPLR_GPU_EINVAL, "dplr_gpu_graph_launch: null graph");
    DG_CUDA(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    note_launches(g->kernels);
    return 0;
}

int dplr_gpu_apply_form(dplr_gpu_plan plan)
{
    const Plan *p = (const Plan *)plan;
    return p ? p->apply_launches : fail(DPLR_GPU_EINVAL, "dplr_gpu_apply_form: null plan");
}

long long dplr_gpu_graph_kernels(dplr_gpu_graph graph)
{
    return graph ? ((GraphH *)graph)->kernels : 0;
}

void dplr_gpu_graph_destroy(dplr_gpu_graph graph)
{
    GraphH *g = (GraphH *)graph;
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->cs) cudaStreamDestroy(g->cs);
    delete g;
}

int dplr_gpu_autotune(dplr_gpu_plan plan, int n, void *stream, int *chunk_rows, int *nb_cap, double *best_ms)
{
    Plan *p = (Plan *)plan;
    if (!p || n <= 0) return fail(DPLR_GPU_EINVAL, "dplr_gpu_autotune: invalid arguments");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t cnt = (size_t)std::max(p->m, 1) * n;
    double *buf = nullptr;
    if (cudaMalloc((void **)&buf, 2 * cnt * sizeof(double)) != cudaSuccess)
        return fail(DPLR_GPU_ENOMEM, "dplr_gpu_autotune: cannot allocate test vectors");
    double *X = buf, *Y = buf + cnt;
    int rc = 0;
    if (cudaMemsetAsync(X, 0, cnt * sizeof(double), st) != cudaSuccess)   // values do not matter
        rc = fail(DPLR_GPU_ECUDA, "dplr_gpu_autotune: cannot clear test vectors");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int chunks[] = {256, 512, 1024, 2048};
    const int caps[] = {1, 2, 4, 8, 16};
    int best_c = p->chunk_rows, best_nb = p->nb_cap, best_form = p->apply_launches;
    float best = 1e30f;
    for (int c : chunks) {
        if (rc) break;
        p->chunk_rows = c;
        if ((rc = plan_reschedule(p))) break;
        for (int nb : caps) {
            if (nb > 1 && nb > n) break;
            set_nb_cap(p, nb);
            // both forms of the apply: one persistent launch, three launches
            for (int form = 0; form < 2 && !rc; ++form) {
                p->apply_launches = form;
                if ((rc = apply_device(p, 0, n, 1.0, X, p->m, 0.0, Y, p->m, st, false))) break;
                cudaEventRecord(e0, st);
                for (int r = 0; r < 3 && !rc; ++r)
                    rc = apply_device(p, 0, n, 1.0, X, p->m, 0.0, Y, p->m, st, false);
                cudaEventRecord(e1, st);
                if (rc) break;
                if (cudaEventSynchronize(e1) != cudaSuccess) {
                    rc = fail(DPLR_GPU_ECUDA, "dplr_gpu_autotune: timing failed");
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                ms /= 3.f;
                if (ms < best) {
                    best = ms;
                    best_c = c;
                    best_nb = nb;
                    best_form = form;
                }
            }
            if (rc) break;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    p->chunk_rows = best_c;
    p->apply_launches = best_form;
    int rc2 = plan_reschedule(p);
    set_nb_cap(p, best_nb);
    if (rc) return rc;
    if (rc2) return rc2;
    if (chunk_rows) *chunk_rows = best_c;
    if (nb_cap) *nb_cap = best_nb;
    if (best_ms) *best_ms = best;
    return 0;
}

}  // extern "C"
