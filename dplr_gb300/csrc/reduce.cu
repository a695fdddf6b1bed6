// reduce.cu -- dplrreduce on the GPU: re-orthogonalise and truncate every
// low-rank block with the pivoted, sval-weighted Gram-Schmidt of DPLR's
// dortlr (src/dortlr.f90:12-207), called as DPLR's dplrreduce intends
// (src/dplrreduce.c:25-82: eps/4 per level, one iteration) but with the
// interface fixed: pivots start as the identity (src/ortlrini.f90) and the
// new rank is returned.  The shipped C caller passes its arguments in the
// wrong order and a 32-bit pivot buffer to a 64-bit routine, so the
// algorithm is taken from the Fortran source, not from that call.
//
// One CTA per low-rank block; the pivot loop is inherently sequential,
// every dot product and update inside it is spread over the CTA.  Columns
// are RMS-normalised (|x|/sqrt(n)) exactly as the Fortran does.
#include "internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace dg {

struct ReduceJob {
    long long u, v, sig;   // pool offsets
    int n, rank;
    double eps;
};

constexpr int kRT = 256;

__device__ double block_sum(double x, double *red)
{
    __syncthreads();
    red[threadIdx.x] = x;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    return red[0];
}

// One pass of dortlr over factor `a` (partner `b`), see oracle gs_pass.
__device__ int gs_pass_dev(int na, int nb, double *a, double *b, int *piv, int rank, double *sval,
                           double eps, double eps2, double *red, int *sh)
{
    for (int j = 0; j < rank; ++j) {
        if (threadIdx.x == 0) {
            int kmax = j;
            double smax = -111.0;
            for (int k = j; k < rank; ++k)
                if (smax < sval[piv[k]]) { kmax = k; smax = sval[piv[k]]; }
            int t = piv[j];
            piv[j] = piv[kmax];
            piv[kmax] = t;
            sh[0] = piv[j];
            sh[1] = sval[piv[j]] <= eps;
        }
        __syncthreads();
        const int mm = sh[0];
        if (sh[1]) return j;
        double *am = a + (long long)mm * na, *bm = b + (long long)mm * nb;
        for (int l = j + 1; l < rank; ++l) {
            const int ll = piv[l];
            __syncthreads();
            if (sval[ll] <= eps) {
                __syncthreads();
                if (threadIdx.x == 0) sval[ll] = 0.0;
                __syncthreads();
                continue;
            }
            double *al = a + (long long)ll * na, *bl = b + (long long)ll * nb;
            double d = 0.0;
            for (int i = threadIdx.x; i < na; i += blockDim.x) d = fma(am[i], al[i], d);
            const double proj = block_sum(d, red) / na;
            double q = 0.0;
            for (int i = threadIdx.x; i < na; i += blockDim.x) {
                double x = fma(-proj, am[i], al[i]);
                al[i] = x;
                q = fma(x, x, q);
            }
            const double f1 = sqrt(block_sum(q, red) / na);
            const double svl = sval[ll];
            if (f1 * svl > eps2) {
                const double g = 1.0 / f1;
                for (int i = threadIdx.x; i < na; i += blockDim.x) al[i] *= g;
            }
            const double p2 = proj * svl / sval[mm];
            for (int i = threadIdx.x; i < nb; i += blockDim.x) bm[i] = fma(p2, bl[i], bm[i]);
            __syncthreads();
            if (threadIdx.x == 0) sval[ll] = svl * f1;
            __syncthreads();
        }
        double q = 0.0;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) q = fma(bm[i], bm[i], q);
        const double f2 = sqrt(block_sum(q, red) / nb);
        const double svm = sval[mm];
        if (f2 * svm > eps2) {
            const double g = 1.0 / f2;
            for (int i = threadIdx.x; i < nb; i += blockDim.x) bm[i] *= g;
        }
        __syncthreads();
        if (threadIdx.x == 0) sval[mm] = svm * f2;
        __syncthreads();
    }
    return rank;
}

__global__ void __launch_bounds__(kRT) dortlr_kernel(const ReduceJob *jobs, double *pool,
                                                     int *new_rank)
{
    extern __shared__ double dyn[];
    __shared__ double red[kRT];
    __shared__ int sh[2];
    const ReduceJob J = jobs[blockIdx.x];
    double *sval = dyn;                             // rank doubles
    int *piv = (int *)(dyn + J.rank);               // rank ints
    int *hole = piv + J.rank;                       // rank ints
    double *u = pool + J.u, *v = pool + J.v;
    for (int k = threadIdx.x; k < J.rank; k += blockDim.x) {
        sval[k] = pool[J.sig + k];
        piv[k] = k;
    }
    __syncthreads();
    const double eps2 = J.eps * J.eps;
    int rank = gs_pass_dev(J.n, J.n, u, v, piv, J.rank, sval, J.eps, eps2, red, sh);
    rank = gs_pass_dev(J.n, J.n, v, u, piv, rank, sval, J.eps, eps2, red, sh);
    __syncthreads();
    // Gap fill (src/dortlr.f90:177-200): survivors into slots 0..rank-1.
    if (threadIdx.x == 0) {
        int nh = 0;
        for (int l = rank; l < J.rank; ++l)
            if (piv[l] < rank) hole[nh++] = piv[l];
        sh[0] = nh;
    }
    __syncthreads();
    int used = 0;
    for (int l = 0; l < rank; ++l) {
        const int src = piv[l];
        if (src < rank) continue;
        const int dst = hole[used++];
        for (int i = threadIdx.x; i < J.n; i += blockDim.x) {
            u[(long long)dst * J.n + i] = u[(long long)src * J.n + i];
            v[(long long)dst * J.n + i] = v[(long long)src * J.n + i];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            sval[dst] = sval[src];
            piv[l] = dst;
        }
        __syncthreads();
    }
    for (int k = threadIdx.x; k < J.rank; k += blockDim.x) pool[J.sig + k] = sval[k];
    if (threadIdx.x == 0) new_rank[blockIdx.x] = rank;
}

}  // namespace dg

using namespace dg;

extern "C" void dplrreduce(int m, DPlrMtx *A, double eps)
{
    dg::NvtxRange nvtx_("dplrreduce");
    const char *fn = "dplrreduce";
    if (m < 0) {
        fprintf(stderr, "%s: invalid matrix size %d\n", fn, m);
        return;
    }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) {
        fprintf(stderr, "%s: invalid A type\n", fn);
        return;
    }
    if (A->size != m) {
        fprintf(stderr, "%s: invalid A size\n", fn);
        return;
    }
    if (A->type == PLR_DMTX) return;
    if (validate_tree(m, A, fn)) {
        fprintf(stderr, "%s: %s\n", fn, dplr_gpu_last_error());
        return;
    }
    Plan *p = nullptr;
    if (plan_build(m, A, 0, &p)) {
        fprintf(stderr, "%s: %s\n", fn, dplr_gpu_last_error());
        return;
    }
    // eps/4 at every level (src/dplrreduce.c:46).
    std::vector<double> epsn(p->nodes.size());
    for (size_t nd = 0; nd < p->nodes.size(); ++nd) {
        const HDesc &H = p->nodes[nd];
        epsn[nd] = (H.parent < 0 ? eps : epsn[H.parent]) / 4.0;
    }
    std::vector<ReduceJob> jobs;
    std::vector<int> blk;
    int maxr = 0;
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        if (L.rank == 0) continue;
        ReduceJob j{L.u, L.v, L.sig, L.n, L.rank, epsn[L.node]};
        jobs.push_back(j);
        blk.push_back((int)b);
        maxr = std::max(maxr, L.rank);
    }
    std::vector<int> ranks(jobs.size());
    int ok = 1;
    if (!jobs.empty()) {
        ReduceJob *d_j = nullptr;
        int *d_r = nullptr;
        size_t smem = (size_t)maxr * (sizeof(double) + 2 * sizeof(int));
        ok = cudaMalloc((void **)&d_j, jobs.size() * sizeof(ReduceJob)) == cudaSuccess &&
             cudaMalloc((void **)&d_r, jobs.size() * sizeof(int)) == cudaSuccess &&
             cudaMemcpy(d_j, jobs.data(), jobs.size() * sizeof(ReduceJob), cudaMemcpyHostToDevice) ==
                 cudaSuccess &&
             cudaFuncSetAttribute(dortlr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem) == cudaSuccess;
        if (ok) {
            dortlr_kernel<<<(unsigned)jobs.size(), kRT, smem>>>(d_j, p->pool, d_r);
            note_launch();
            ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
                 cudaMemcpy(ranks.data(), d_r, ranks.size() * sizeof(int), cudaMemcpyDeviceToHost) ==
                     cudaSuccess;
        }
        cudaFree(d_j);
        cudaFree(d_r);
    }
    if (!ok) {
        fprintf(stderr, "%s: GPU Gram-Schmidt failed: %s\n", fn, cudaGetErrorString(cudaGetLastError()));
        plan_free(p);
        return;
    }
    // Copy the re-orthogonalised factors back (all former live columns) and
    // set the new ranks, walking the tree in plan order.
    std::vector<int> newrank(p->lr.size(), 0);
    for (size_t q = 0; q < jobs.size(); ++q) newrank[blk[q]] = ranks[q];
    struct Walk {
        Plan *p;
        const std::vector<int> &nr;
        size_t b = 0;
        int fail = 0;
        void go(DPlrMtx *A)
        {
            if (A->type == PLR_DMTX) return;
            DPlrMtx *bl[2] = {A->dh.ne, A->dh.sw};
            for (DPlrMtx *L : bl) {
                const LRDesc &D = p->lr[b];
                size_t cnt = (size_t)D.n * D.rank;
                if (cnt) {
                    fail |= cudaMemcpy(L->dlr.u, p->pool + D.u, cnt * 8, cudaMemcpyDeviceToHost) != cudaSuccess;
                    fail |= cudaMemcpy(L->dlr.v, p->pool + D.v, cnt * 8, cudaMemcpyDeviceToHost) != cudaSuccess;
                    fail |= cudaMemcpy(L->dlr.sig, p->pool + D.sig, D.rank * 8, cudaMemcpyDeviceToHost) != cudaSuccess;
                }
                L->dlr.rank = nr[b];
                ++b;
            }
            go(A->dh.nw);
            go(A->dh.se);
        }
    } w{p, newrank};
    w.go(A);
    if (w.fail) fprintf(stderr, "%s: download failed\n", fn);
    plan_free(p);
}
