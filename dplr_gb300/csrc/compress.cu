// compress.cu -- dense -> PLR compression with the SVDs on the GPU.
//
// Replaces dplrd2gep (src/dplrd2p.c:186) with the same tree and the same
// results up to the sign choices of the singular vectors:
//   * nlvl == 0: B is a dense copy of A;
//   * otherwise B is an H node whose off-diagonal blocks are truncated SVDs
//     of A's off-diagonal blocks (rank = number of singular values >= the
//     block's absolute threshold, src/dplrd2p.c:22-178: U kept, sig, V = the
//     rows of V^T), the threshold being eps/2 when the children are leaves
//     and eps/4 otherwise, passed down to the diagonal blocks.
// B is reshaped first, with DPLR's rule (a node whose type or size differs
// is cleared and rebuilt), and every off-diagonal block becomes one SVD job.
// A is copied to the device once; the jobs, largest first, are spread over
// worker threads, each with its own stream, cuSOLVER handle and buffers:
// the SVD (cuSOLVER's gesvd, the QR-iteration SVD LAPACK's dgesvd is) of a
// small block is a long chain of small launches, so independent blocks run
// side by side.  The tree B stays on the host, as DPLR's callers expect.
// Argument checks, messages and info codes are DPLR's: info = -1 on invalid
// arguments, the SVD's info if one does not converge.
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/dplr.h"
#include "../../include/dplr_gb300.h"

namespace dg {
int fail(int code, const char *fmt, ...);
}

namespace {

// DPLR's message on stderr, and the same text as the library's last error.
int report(int code, const char *msg)
{
    fprintf(stderr, "%s\n", msg);
    return dg::fail(code, "%s", msg);
}

// cuSOLVER is opened on the first call, so that the apply and solve paths
// (everything else in this library) load without it.
struct Solver {
    decltype(&cusolverDnCreate) create = nullptr;
    decltype(&cusolverDnDestroy) destroy = nullptr;
    decltype(&cusolverDnSetStream) set_stream = nullptr;
    decltype(&cusolverDnDgesvd_bufferSize) gesvd_size = nullptr;
    decltype(&cusolverDnDgesvd) gesvd = nullptr;
    bool ok = false;

    Solver()
    {
        void *so = dlopen("libcusolver.so.12", RTLD_NOW | RTLD_LOCAL);
        if (!so) so = dlopen("libcusolver.so", RTLD_NOW | RTLD_LOCAL);
        if (!so) so = dlopen("/usr/local/cuda/lib64/libcusolver.so.12", RTLD_NOW | RTLD_LOCAL);
        if (!so) return;
        create = (decltype(create))dlsym(so, "cusolverDnCreate");
        destroy = (decltype(destroy))dlsym(so, "cusolverDnDestroy");
        set_stream = (decltype(set_stream))dlsym(so, "cusolverDnSetStream");
        gesvd_size = (decltype(gesvd_size))dlsym(so, "cusolverDnDgesvd_bufferSize");
        gesvd = (decltype(gesvd))dlsym(so, "cusolverDnDgesvd");
        ok = create && destroy && set_stream && gesvd_size && gesvd;
    }
};

const Solver &solver()
{
    static const Solver s;
    return s;
}

// One off-diagonal block: rows r0.., columns c0.. of A, order n.
struct Job {
    int n, r0, c0;
    double eps;
    DPlrMtx *L;
    int order;      // position in DPLR's depth-first NE, SW, NW, SE order
    int devinfo;    // the SVD's info
};

// Reshape B as dplrd2gep does (src/dplrd2p.c:231-291), copy the leaves from
// the host and list the off-diagonal jobs.
void plan_tree(int n, int r0, const double *hA, int lda, DPlrMtx *B, double eps, int nlvl, std::vector<Job> &jobs)
{
    if (nlvl == 0) {
        if (B->type != PLR_DMTX || B->size != n) {
            dplrclr(B);
            dplrinid(n, B);
        }
        for (int j = 0; j < n; ++j)
            memcpy(B->dd.d + (size_t)j * n, hA + r0 + (size_t)(r0 + j) * lda, (size_t)n * sizeof(double));
        return;
    }
    const double eps2 = nlvl == 1 ? eps / 2.0 : eps / 4.0;
    const int h = n / 2;
    if (B->type != PLR_HMTX || B->size != n) {
        dplrclr(B);
        dplrinih(n, B);
        dplrinilr(h, B->dh.ne, 0);
        dplrinilr(h, B->dh.sw, 0);
    }
    jobs.push_back({h, r0, r0 + h, eps2, B->dh.ne, (int)jobs.size(), 0});
    jobs.push_back({h, r0 + h, r0, eps2, B->dh.sw, (int)jobs.size(), 0});
    plan_tree(h, r0, hA, lda, B->dh.nw, eps2, nlvl - 1, jobs);
    plan_tree(h, r0 + h, hA, lda, B->dh.se, eps2, nlvl - 1, jobs);
}

struct Worker {
    cudaStream_t st = nullptr;
    cusolverDnHandle_t h = nullptr;
    double *W = nullptr, *U = nullptr, *VT = nullptr, *S = nullptr, *work = nullptr, *rwork = nullptr;
    int *info = nullptr;
    int lwork = 0;
    std::vector<double> hS, hVT;

    bool init(int nmax)
    {
        const size_t nn = (size_t)nmax * nmax;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return false;
        if (solver().create(&h) != CUSOLVER_STATUS_SUCCESS) return false;
        if (solver().set_stream(h, st) != CUSOLVER_STATUS_SUCCESS) return false;
        if (solver().gesvd_size(h, nmax, nmax, &lwork) != CUSOLVER_STATUS_SUCCESS) return false;
        return cudaMalloc((void **)&W, nn * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&U, nn * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&VT, nn * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&S, (size_t)nmax * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&rwork, (size_t)nmax * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&work, (size_t)std::max(lwork, 1) * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&info, sizeof(int)) == cudaSuccess;
    }

    void release()
    {
        cudaFree(W);
        cudaFree(U);
        cudaFree(VT);
        cudaFree(S);
        cudaFree(work);
        cudaFree(rwork);
        cudaFree(info);
        if (h) solver().destroy(h);
        if (st) cudaStreamDestroy(st);
    }

    // Truncated SVD of one block (dplrlrappx, src/dplrd2p.c:22): 0, the
    // SVD's nonzero info (> 0), or -1 on a CUDA / cuSOLVER error.
    int run(const double *dA, int m, Job &jb)
    {
        const int n = jb.n;
        DPlrMtx *L = jb.L;
        if (n == 0) {
            L->dlr.rank = 0;
            return 0;
        }
        if (cudaMemcpy2DAsync(W, (size_t)n * sizeof(double), dA + jb.r0 + (size_t)jb.c0 * m, (size_t)m * sizeof(double),
                              (size_t)n * sizeof(double), n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            return -1;
        if (solver().gesvd(h, 'S', 'S', n, n, W, n, S, U, n, VT, n, work, lwork, rwork, info) !=
            CUSOLVER_STATUS_SUCCESS)
            return -1;
        hS.resize(n);
        if (cudaMemcpyAsync(&jb.devinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(hS.data(), S, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return -1;
        if (jb.devinfo != 0) return 1;
        int rank = 0;
        while (rank < n && !(hS[rank] < jb.eps)) ++rank;
        if (L->dlr.capacity < rank) dplrresizelr(L, rank);
        L->dlr.rank = rank;
        if (rank == 0) return 0;
        memcpy(L->dlr.sig, hS.data(), (size_t)rank * sizeof(double));
        // V: column j is row j of V^T (the first rank rows, ld n)
        hVT.resize((size_t)rank * n);
        if (cudaMemcpyAsync(L->dlr.u, U, (size_t)n * rank * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpy2DAsync(hVT.data(), (size_t)rank * sizeof(double), VT, (size_t)n * sizeof(double),
                              (size_t)rank * sizeof(double), n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return -1;
        for (int j = 0; j < rank; ++j)
            for (int i = 0; i < n; ++i) L->dlr.v[(size_t)j * n + i] = hVT[(size_t)i * rank + j];
        return 0;
    }
};

const char *block_name(const Job &jb) { return jb.r0 < jb.c0 ? "NE" : "SW"; }

}  // namespace

extern "C" {

int dplr_gpu_d2gep(int m, const double *A, int lda, DPlrMtx *B, double eps, int nlvl, int workers, int *info)
{
    *info = -1;
    if (m < 0) {
        fprintf(stderr, "dplrd2gep: invalid matrix size %d\n", m);
        return dg::fail(DPLR_GPU_EINVAL, "dplrd2gep: invalid matrix size %d", m);
    }
    if (lda < m)
        return report(DPLR_GPU_EINVAL, "dplrd2gep: invalid leading dimension");
    if (eps < 0.0)
        return report(DPLR_GPU_EINVAL, "dplrd2gep: eps must be nonnegative");
    if (nlvl < 0 || nlvl > 30 || m % (1 << nlvl) != 0)
        return report(DPLR_GPU_EINVAL, "dplrd2gep: m not divisible by 2**nlvl");
    if (!B || (!A && m > 0))
        return report(DPLR_GPU_EINVAL, "dplrd2gep: null argument");
    std::vector<Job> jobs;
    plan_tree(m, 0, A, lda, B, eps, nlvl, jobs);
    if (jobs.empty() || m == 0) {
        for (Job &jb : jobs) jb.L->dlr.rank = 0;
        *info = 0;
        return DPLR_GPU_OK;
    }
    // a reused B must hold low-rank nodes where the blocks go
    for (const Job &jb : jobs)
        if (jb.L->type != PLR_LRMTX || jb.L->size != jb.n) {
            fprintf(stderr, "dplrlrappx: invalid B type or size\n");
            fprintf(stderr, "dplrd2gep: failed to approximate %s block\n", block_name(jb));
            return DPLR_GPU_OK;
        }
    if (!solver().ok)
        return report(DPLR_GPU_ECUDA, "dplrd2gep: cannot load cuSOLVER (libcusolver.so.12)");

    // device copy of A, ld m
    double *dA = nullptr;
    if (cudaMalloc((void **)&dA, (size_t)m * m * sizeof(double)) != cudaSuccess ||
        cudaMemcpy2D(dA, (size_t)m * sizeof(double), A, (size_t)lda * sizeof(double), (size_t)m * sizeof(double), m,
                     cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(dA);
        return report(DPLR_GPU_ECUDA, "dplrd2gep: device copy of A failed");
    }

    // workers: 8 unless asked otherwise, no more than there are blocks, and
    // their buffers within a quarter of the free device memory
    const int nmax = m / 2;
    const size_t per = (3 * (size_t)nmax * nmax + 8 * (size_t)nmax) * sizeof(double);
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    int nw = workers > 0 ? workers : 8;
    nw = std::min<int>(nw, (int)jobs.size());
    nw = (int)std::max<size_t>(1, std::min<size_t>((size_t)nw, fr / 4 / std::max<size_t>(per, 1)));
    std::vector<Worker> pool(nw);
    bool ok = true;
    for (Worker &w : pool) ok = ok && w.init(nmax);

    std::vector<int> rc(jobs.size(), 0);
    if (ok) {
        // largest blocks first; ties in DPLR's order
        std::vector<int> idx(jobs.size());
        for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int)i;
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return jobs[a].n > jobs[b].n; });
        std::atomic<int> next{0};
        std::atomic<bool> failed{false};
        auto body = [&](Worker &w) {
            for (;;) {
                if (failed.load()) return;
                const int k = next.fetch_add(1);
                if (k >= (int)idx.size()) return;
                Job &jb = jobs[idx[k]];
                rc[idx[k]] = w.run(dA, m, jb);
                if (rc[idx[k]] != 0) failed.store(true);
            }
        };
        std::vector<std::thread> th;
        for (int t = 1; t < nw; ++t) th.emplace_back(body, std::ref(pool[t]));
        body(pool[0]);
        for (std::thread &t : th) t.join();
    }
    for (Worker &w : pool) w.release();
    cudaFree(dA);
    if (!ok)
        return report(DPLR_GPU_ECUDA, "dplrd2gep: device setup failed");

    // the first failure in DPLR's order decides info
    for (const Job &jb : jobs) {
        if (rc[jb.order] < 0)
            return report(DPLR_GPU_ECUDA, "dplrd2gep: CUDA or cuSOLVER call failed");
        if (rc[jb.order] > 0) {
            fprintf(stderr, "dplrlrappx: dgesvd() failed: %d\n", jb.devinfo);
            fprintf(stderr, "dplrd2gep: failed to approximate %s block\n", block_name(jb));
            *info = jb.devinfo;
            return DPLR_GPU_OK;
        }
    }
    *info = 0;
    return DPLR_GPU_OK;
}

void dplrd2gep(int m, double *A, int lda, DPlrMtx *B, double eps, int nlvl, int *info)
{
    dplr_gpu_d2gep(m, A, lda, B, eps, nlvl, 0, info);
}

}  // extern "C"
