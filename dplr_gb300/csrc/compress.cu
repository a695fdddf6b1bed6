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
// A is copied to the device once.  Blocks of up to 64 rows run together in
// one launch of the batched SVD kernel (svdbatch.cuh: Householder QR and
// one-sided Jacobi, one CTA per block).  The other jobs, largest first,
// are spread over worker threads, each with its own stream, cuSOLVER
// handle and buffers:
// the SVD (cuSOLVER's gesvd, the QR-iteration SVD LAPACK's dgesvd is) of a
// small block is a long chain of small launches, so independent blocks run
// side by side.  Blocks of 512 and more first try a sketch: Q = orth(A
// Omega) (own Gaussian and FP64 GEMM kernels, cuSOLVER QR), B = Q^T A and
// the residual ||A - Q B||_F; when the residual proves that no singular
// value at or above the threshold is missed and the kept ones are as
// accurate as a full SVD's, the SVD of the n x l matrix B^T gives the
// block's factors, otherwise the full SVD runs.  The tree B stays on the
// host, as DPLR's callers expect.
// The SVD-based recompression (dplr_gpu_reduce_svd) shares the batched
// kernel for its blocks of rank <= 64 and the library for the others.
// Argument checks, messages and info codes are DPLR's: info = -1 on invalid
// arguments, the SVD's info if one does not converge (1 for the batched
// kernel).
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/dplr.h"
#include "../../include/dplr_gb300.h"
#include "gemm.cuh"
#include "svdblock.cuh"
#include "svdbatch.cuh"

namespace dg {
int fail(int code, const char *fmt, ...);
struct NvtxRange {
    explicit NvtxRange(const char *name);
    ~NvtxRange();
};
void note_launch();
void note_launches(long long k);
int validate_tree(int m, const DPlrMtx *A, const char *fn);
}
using dg::GemmJob;
using dg::GemmRed;
using dg::GemmTile;

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
    decltype(&cusolverDnDgeqrf_bufferSize) geqrf_size = nullptr;
    decltype(&cusolverDnDgeqrf) geqrf = nullptr;
    decltype(&cusolverDnDorgqr_bufferSize) orgqr_size = nullptr;
    decltype(&cusolverDnDorgqr) orgqr = nullptr;
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
        geqrf_size = (decltype(geqrf_size))dlsym(so, "cusolverDnDgeqrf_bufferSize");
        geqrf = (decltype(geqrf))dlsym(so, "cusolverDnDgeqrf");
        orgqr_size = (decltype(orgqr_size))dlsym(so, "cusolverDnDorgqr_bufferSize");
        orgqr = (decltype(orgqr))dlsym(so, "cusolverDnDorgqr");
        ok = create && destroy && set_stream && gesvd_size && gesvd && geqrf_size && geqrf && orgqr_size && orgqr;
    }
};

const Solver &solver()
{
    static const Solver s;
    return s;
}

// Standard normal sketch entries from a counter-based hash (SplitMix64
// finaliser) and the Box-Muller transform: deterministic per (seed, index).
__device__ inline unsigned long long mix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void gauss_kernel(double *out, long long count, unsigned long long seed)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h = mix64(seed ^ mix64((unsigned long long)i));
        const double u1 = ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);        // (0, 1)
        const double u2 = (double)(mix64(h) >> 11) * (1.0 / 9007199254740992.0);         // [0, 1)
        out[i] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    }
}

// Sum of squares of a rows x cols block (ld lda): one partial per CTA.
__global__ void fro2_kernel(const double *a, int lda, int rows, int cols, double *part)
{
    __shared__ double red[8];
    double q = 0.0;
    const long long cnt = (long long)rows * cols;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < cnt;
         e += (long long)gridDim.x * blockDim.x) {
        const double x = a[(e % rows) + (e / rows) * (long long)lda];
        q = fma(x, x, q);
    }
    for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = q;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        part[blockIdx.x] = t;
    }
}

constexpr int kFroBlocks = 128;   // partials of fro2_kernel
constexpr int kRandMin = 512;     // blocks at least this large try the sketch first

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
    // sketch path: Omega / U of A, Q, B^T, U of B^T (n x lmax), V^T of B^T
    // (lmax x lmax), Householder scalars, norm partials
    double *Om = nullptr, *Q = nullptr, *Bt = nullptr, *Ub = nullptr, *Vbt = nullptr, *tau = nullptr, *fro = nullptr;
    int *info = nullptr;
    int lwork = 0, lmax = 0;
    std::vector<double> hS, hVT;

    bool init(int nmax)
    {
        const size_t nn = (size_t)nmax * nmax;
        lmax = nmax >= kRandMin ? nmax / 3 : 0;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return false;
        if (solver().create(&h) != CUSOLVER_STATUS_SUCCESS) return false;
        if (solver().set_stream(h, st) != CUSOLVER_STATUS_SUCCESS) return false;
        if (solver().gesvd_size(h, nmax, nmax, &lwork) != CUSOLVER_STATUS_SUCCESS) return false;
        if (lmax > 0) {
            int a = 0, b = 0, c = 0;
            if (solver().geqrf_size(h, nmax, lmax, W, nmax, &a) != CUSOLVER_STATUS_SUCCESS ||
                solver().orgqr_size(h, nmax, lmax, lmax, W, nmax, S, &b) != CUSOLVER_STATUS_SUCCESS ||
                solver().gesvd_size(h, nmax, lmax, &c) != CUSOLVER_STATUS_SUCCESS)
                return false;
            lwork = std::max({lwork, a, b, c});
        }
        const size_t nl = (size_t)nmax * std::max(lmax, 1), ll = (size_t)std::max(lmax, 1) * std::max(lmax, 1);
        return cudaMalloc((void **)&W, nn * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&U, nn * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&VT, nn * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&S, (size_t)nmax * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&rwork, (size_t)nmax * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&work, (size_t)std::max(lwork, 1) * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&info, sizeof(int)) == cudaSuccess &&
               cudaMalloc((void **)&Om, nl * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&Q, nl * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&Bt, nl * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&Ub, nl * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&Vbt, ll * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&tau, (size_t)std::max(lmax, 1) * sizeof(double)) == cudaSuccess &&
               cudaMalloc((void **)&fro, 2 * kFroBlocks * sizeof(double)) == cudaSuccess;
    }

    void release()
    {
        for (double *p : {W, U, VT, S, work, rwork, Om, Q, Bt, Ub, Vbt, tau, fro}) cudaFree(p);
        cudaFree(info);
        if (h) solver().destroy(h);
        if (st) cudaStreamDestroy(st);
    }

    // One GEMM on the worker's stream (tables staged in stream-ordered memory).
    bool gemm(const GemmJob &J)
    {
        std::vector<GemmJob> jobs{J};
        std::vector<GemmTile> tiles;
        std::vector<GemmRed> reds;
        long long ptot = 0;
        plan_gemm_tiles(jobs, tiles, reds, ptot);
        if (tiles.empty()) return true;
        GemmJob *dj = nullptr;
        GemmTile *dt = nullptr;
        GemmRed *dr = nullptr;
        double *part = nullptr;
        bool ok = cudaMallocAsync((void **)&dj, sizeof(GemmJob), st) == cudaSuccess &&
                  cudaMallocAsync((void **)&dt, sizeof(GemmTile) * tiles.size(), st) == cudaSuccess &&
                  cudaMemcpyAsync(dj, jobs.data(), sizeof(GemmJob), cudaMemcpyHostToDevice, st) == cudaSuccess &&
                  cudaMemcpyAsync(dt, tiles.data(), sizeof(GemmTile) * tiles.size(), cudaMemcpyHostToDevice, st) ==
                      cudaSuccess;
        if (ok && !reds.empty())
            ok = cudaMallocAsync((void **)&dr, sizeof(GemmRed) * reds.size(), st) == cudaSuccess &&
                 cudaMallocAsync((void **)&part, sizeof(double) * ptot, st) == cudaSuccess &&
                 cudaMemcpyAsync(dr, reds.data(), sizeof(GemmRed) * reds.size(), cudaMemcpyHostToDevice, st) ==
                     cudaSuccess;
        if (ok) {
            run_gemm_tables(dj, dt, tiles.size(), dr, reds.size(), part, st);
            dg::note_launches((long long)((tiles.size() + (1u << 30) - 1) >> 30) + (reds.empty() ? 0 : 1));
            ok = cudaGetLastError() == cudaSuccess;
        }
        for (void *q : {(void *)dj, (void *)dt, (void *)dr, (void *)part})
            if (q) cudaFreeAsync(q, st);
        return ok;
    }

    // Frobenius norm of a rows x cols block (ld lda); < 0 on error.
    double fro_norm(const double *a, int lda, int rows, int cols)
    {
        fro2_kernel<<<kFroBlocks, 256, 0, st>>>(a, lda, rows, cols, fro);
        dg::note_launch();
        double hp[kFroBlocks];
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(hp, fro, sizeof(hp), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return -1.0;
        double t = 0.0;
        for (double x : hp) t += x;
        return sqrt(t);
    }

    // Sketch path for a large block: Q = orth(A Omega), B^T = A^T Q, checked
    // by the residual ||A - Q B||_F; on success the SVD of B^T (n x l) gives
    // A's leading singular triplets (A ~ (Q V_b) S U_b^T).  Accepted only when
    // the residual is below 1e-3 of the threshold, or at rounding level
    // (32 eps ||A||_F) and below half the threshold: then no singular value
    // at or above the threshold is missed (sigma_{l+1}(A) <= ||A - Q B||) and
    // the kept ones are as accurate as a full SVD's.  Returns 0 (done), 2 (not
    // accepted: use the full SVD), -1 on an error.
    int run_sketch(const double *dA, int m, Job &jb)
    {
        const int n = jb.n;
        const double *Ab = dA + jb.r0 + (size_t)jb.c0 * m;
        const double fa = fro_norm(Ab, m, n, n);
        if (fa < 0) return -1;
        const unsigned long long seed = ((unsigned long long)jb.r0 << 32) ^ (unsigned long long)jb.c0;
        const int lcap = std::min(lmax, n / 3);   // beyond n/3 columns the full SVD is as cheap
        for (int l = std::min(192, lcap); l >= 32 && l <= lcap; l = (l == lcap ? lcap + 1 : std::min(2 * l, lcap))) {
            gauss_kernel<<<256, 256, 0, st>>>(Om, (long long)n * l, seed + (unsigned long long)l);
            dg::note_launch();
            if (cudaGetLastError() != cudaSuccess) return -1;
            // Q = orth(A Omega)
            if (!gemm({Ab, Om, nullptr, nullptr, Q, n, l, n, m, n, 0, n, 0, 0, 1.0, 0.0})) return -1;
            if (solver().geqrf(h, n, l, Q, n, tau, work, lwork, info) != CUSOLVER_STATUS_SUCCESS ||
                solver().orgqr(h, n, l, l, Q, n, tau, work, lwork, info) != CUSOLVER_STATUS_SUCCESS)
                return -1;
            // B^T = A^T Q ; W = A - Q B
            if (!gemm({Ab, Q, nullptr, nullptr, Bt, n, l, n, m, n, 0, n, 1, 0, 1.0, 0.0})) return -1;
            if (cudaMemcpy2DAsync(W, (size_t)n * sizeof(double), Ab, (size_t)m * sizeof(double),
                                  (size_t)n * sizeof(double), n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
                return -1;
            if (!gemm({Q, Bt, W, nullptr, W, n, n, l, n, n, n, n, 0, 1, -1.0, 1.0})) return -1;
            const double fe = fro_norm(W, n, n, n);
            if (fe < 0) return -1;
            const double eps64 = 2.220446049250313e-16;
            const bool accept = fe <= 1e-3 * jb.eps || (fe <= 32.0 * eps64 * fa && fe < 0.5 * jb.eps);
            if (!accept) continue;
            // B^T = U_b S V_b^T
            if (solver().gesvd(h, 'S', 'S', n, l, Bt, n, S, Ub, n, Vbt, l, work, lwork, rwork, info) !=
                CUSOLVER_STATUS_SUCCESS)
                return -1;
            int devinfo = 0;
            hS.resize(l);
            if (cudaMemcpyAsync(&devinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaMemcpyAsync(hS.data(), S, (size_t)l * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)
                return -1;
            if (devinfo != 0) return 2;
            int rank = 0;
            while (rank < l && !(hS[rank] < jb.eps)) ++rank;
            DPlrMtx *L = jb.L;
            if (L->dlr.capacity < rank) dplrresizelr(L, rank);
            L->dlr.rank = rank;
            if (rank == 0) return 0;
            memcpy(L->dlr.sig, hS.data(), (size_t)rank * sizeof(double));
            // U = Q V_b (first rank columns) into Om ; V = U_b
            if (!gemm({Q, Vbt, nullptr, nullptr, Om, n, rank, l, n, l, 0, n, 0, 1, 1.0, 0.0})) return -1;
            if (cudaMemcpyAsync(L->dlr.u, Om, (size_t)n * rank * sizeof(double), cudaMemcpyDeviceToHost, st) !=
                    cudaSuccess ||
                cudaMemcpyAsync(L->dlr.v, Ub, (size_t)n * rank * sizeof(double), cudaMemcpyDeviceToHost, st) !=
                    cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)
                return -1;
            return 0;
        }
        return 2;
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
        if (n >= kRandMin && lmax >= 32) {
            const int rs = run_sketch(dA, m, jb);
            if (rs != 2) return rs;
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

// Staging of dense blocks for svd_batch_kernel: V = I and sig = 1 (the
// block itself is copied into U), one CTA per block.
__global__ void svd_stage_dense_kernel(const dg::SvdBatchJob *__restrict__ jobs, int count, double *__restrict__ stage)
{
    if ((int)blockIdx.x >= count) return;
    const dg::SvdBatchJob jb = jobs[blockIdx.x];
    const long long nn = (long long)jb.n * jb.n;
    double *v = stage + jb.off + nn, *sig = v + 2 * nn;
    for (long long e = threadIdx.x; e < nn; e += blockDim.x) v[e] = (e % jb.n) == (e / jb.n) ? 1.0 : 0.0;
    for (int e = threadIdx.x; e < jb.n; e += blockDim.x) sig[e] = 1.0;
}

// Truncated SVDs of the blocks of order n <= the batched kernel's rank limit
// (dplrlrappx, src/dplrd2p.c:22) in one launch: each block is the rank-n
// product A I^T.  rc[order]: 0, 1 (the Jacobi sweeps did not converge,
// devinfo 1); returns -1 on a CUDA error.
int run_dense_batch(const double *dA, int m, std::vector<Job> &jobs, const std::vector<int> &ids, std::vector<int> &rc)
{
    if (ids.empty()) return 0;
    std::vector<dg::SvdBatchJob> bj;
    long long tot = 0;
    int nmax = 0;
    for (int id : ids) {
        const Job &jb = jobs[id];
        bj.push_back({tot, jb.n, jb.n, jb.eps});
        tot += (3LL * jb.n * jb.n + jb.n + 3) & ~3LL;
        nmax = std::max(nmax, jb.n);
    }
    const int cnt = (int)bj.size();
    cudaStream_t st = nullptr;
    double *stage = nullptr;
    dg::SvdBatchJob *dj = nullptr;
    int *dout = nullptr;
    std::vector<int> hout((size_t)cnt * 2, 0);
    bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc((void **)&stage, (size_t)tot * sizeof(double)) == cudaSuccess &&
              cudaMalloc((void **)&dj, (size_t)cnt * sizeof(dg::SvdBatchJob)) == cudaSuccess &&
              cudaMalloc((void **)&dout, (size_t)cnt * 2 * sizeof(int)) == cudaSuccess &&
              cudaMemcpyAsync(dj, bj.data(), (size_t)cnt * sizeof(dg::SvdBatchJob), cudaMemcpyHostToDevice, st) ==
                  cudaSuccess;
    for (int k = 0; ok && k < cnt; ++k) {
        const Job &jb = jobs[ids[k]];
        ok = cudaMemcpy2DAsync(stage + bj[k].off, (size_t)jb.n * sizeof(double), dA + jb.r0 + (size_t)jb.c0 * m,
                               (size_t)m * sizeof(double), (size_t)jb.n * sizeof(double), jb.n,
                               cudaMemcpyDeviceToDevice, st) == cudaSuccess;
    }
    if (ok) {
        svd_stage_dense_kernel<<<cnt, 256, 0, st>>>(dj, cnt, stage);
        dg::note_launch();
        const int smem = dg::svd_batch_smem(nmax);
        ok = cudaGetLastError() == cudaSuccess &&
             cudaFuncSetAttribute(dg::svd_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) ==
                 cudaSuccess;
        if (ok) {
            dg::svd_batch_kernel<<<cnt, dg::kSvdThreads, smem, st>>>(dj, cnt, stage, dout);
            dg::note_launch();
            ok = cudaGetLastError() == cudaSuccess &&
                 cudaMemcpyAsync(hout.data(), dout, (size_t)cnt * 2 * sizeof(int), cudaMemcpyDeviceToHost, st) ==
                     cudaSuccess &&
                 cudaStreamSynchronize(st) == cudaSuccess;
        }
    }
    for (int k = 0; ok && k < cnt; ++k) {
        Job &jb = jobs[ids[k]];
        DPlrMtx *L = jb.L;
        if (hout[2 * k + 1] != 0) {
            jb.devinfo = 1;
            rc[jb.order] = 1;
            continue;
        }
        const int n = jb.n, rank = std::min(std::max(hout[2 * k], 0), n);
        if (L->dlr.capacity < rank) dplrresizelr(L, rank);
        L->dlr.rank = rank;
        if (rank == 0) continue;
        const double *u = stage + bj[k].off;
        const size_t nn = (size_t)n * n, nk = (size_t)n * rank;
        ok = cudaMemcpyAsync(L->dlr.u, u, nk * sizeof(double), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaMemcpyAsync(L->dlr.v, u + 2 * nn, nk * sizeof(double), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaMemcpyAsync(L->dlr.sig, u + 3 * nn, (size_t)rank * sizeof(double), cudaMemcpyDeviceToHost, st) ==
                 cudaSuccess;
    }
    ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
    cudaFree(stage);
    cudaFree(dj);
    cudaFree(dout);
    if (st) cudaStreamDestroy(st);
    return ok ? 0 : -1;
}

// ------------------------------------------------ SVD-based recompression

// R (k x r, ld k) = the upper triangle of the first k rows of a geqrf result
// (ld lda), zeros below the diagonal.
__global__ void triu_kernel(const double *__restrict__ a, int lda, int k, int r, double *__restrict__ R)
{
    const long long cnt = (long long)k * r;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < cnt;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % k), j = (int)(e / k);
        R[e] = i <= j ? a[i + (long long)j * lda] : 0.0;
    }
}

// u := u diag(s): column j of an n x r block scaled by s[j].
__global__ void scale_cols_kernel(double *__restrict__ u, const double *__restrict__ s, int n, int r)
{
    const long long cnt = (long long)n * r;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < cnt;
         e += (long long)gridDim.x * blockDim.x)
        u[e] *= s[e / n];
}


// The batched path (svdbatch.cuh) takes blocks of rank r <= min(n, limit)
// with n r^2 <= 2^22, for which one CTA's QRs stay within milliseconds;
// larger blocks go to the library workers below.  The limit is
// kSvdBatchRank, or DPLR_GB300_SVD_BATCH_RANK from the environment (read on
// every call; 0 sends every block to the library).
int batch_rank_limit()
{
    const char *v = getenv("DPLR_GB300_SVD_BATCH_RANK");
    if (!v || !*v) return dg::kSvdBatchRank;
    return std::max(0, std::min(atoi(v), dg::kSvdBatchRank));
}

bool batch_takes(const dg::SvdBlock &b, int limit)
{
    return b.r > 0 && b.r <= limit && b.r <= b.n && (long long)b.n * b.r * b.r <= (1LL << 22);
}

// Truncated SVDs of blocks[ids[..]] by svd_batch_kernel, in launches of at
// most 2^25 staged doubles.  res[id]: 0 done, 1 not converged (block left
// as it was, rank = r); returns -1 on a CUDA error.
int run_svd_batch(dg::SvdBlock *blocks, const std::vector<int> &ids, std::vector<int> &res)
{
    if (ids.empty()) return 0;
    for (int id : ids) blocks[id].rank = blocks[id].r;
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return -1;
    const long long cap = 1LL << 25;
    bool ok = true;
    for (size_t g0 = 0; ok && g0 < ids.size();) {
        std::vector<dg::SvdBatchJob> jobs;
        long long tot = 0;
        int rmax = 0;
        size_t g1 = g0;
        for (; g1 < ids.size(); ++g1) {
            const dg::SvdBlock &b = blocks[ids[g1]];
            const long long need = (3LL * b.n * b.r + b.r + 3) & ~3LL;
            if (!jobs.empty() && tot + need > cap) break;
            jobs.push_back({tot, b.n, b.r, b.eps});
            tot += need;
            rmax = std::max(rmax, b.r);
        }
        const int cnt = (int)jobs.size();
        double *stage = nullptr;
        dg::SvdBatchJob *dj = nullptr;
        int *dout = nullptr;
        ok = cudaMalloc((void **)&stage, (size_t)tot * sizeof(double)) == cudaSuccess &&
             cudaMalloc((void **)&dj, (size_t)cnt * sizeof(dg::SvdBatchJob)) == cudaSuccess &&
             cudaMalloc((void **)&dout, (size_t)cnt * 2 * sizeof(int)) == cudaSuccess &&
             cudaMemcpyAsync(dj, jobs.data(), (size_t)cnt * sizeof(dg::SvdBatchJob), cudaMemcpyHostToDevice, st) ==
                 cudaSuccess;
        for (int k = 0; ok && k < cnt; ++k) {
            const dg::SvdBlock &b = blocks[ids[g0 + k]];
            const size_t nr = (size_t)b.n * b.r;
            double *u = stage + jobs[k].off;
            ok = cudaMemcpyAsync(u, b.u, nr * sizeof(double), cudaMemcpyDefault, st) == cudaSuccess &&
                 cudaMemcpyAsync(u + nr, b.v, nr * sizeof(double), cudaMemcpyDefault, st) == cudaSuccess &&
                 cudaMemcpyAsync(u + 3 * nr, b.sig, (size_t)b.r * sizeof(double), cudaMemcpyDefault, st) ==
                     cudaSuccess;
        }
        std::vector<int> hout((size_t)cnt * 2, 0);
        if (ok) {
            const int smem = dg::svd_batch_smem(rmax);
            ok = cudaFuncSetAttribute(dg::svd_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) ==
                 cudaSuccess;
            if (ok) {
                dg::svd_batch_kernel<<<cnt, dg::kSvdThreads, smem, st>>>(dj, cnt, stage, dout);
                dg::note_launch();
                ok = cudaGetLastError() == cudaSuccess &&
                     cudaMemcpyAsync(hout.data(), dout, (size_t)cnt * 2 * sizeof(int), cudaMemcpyDeviceToHost, st) ==
                         cudaSuccess &&
                     cudaStreamSynchronize(st) == cudaSuccess;
            }
        }
        for (int k = 0; ok && k < cnt; ++k) {
            dg::SvdBlock &b = blocks[ids[g0 + k]];
            if (hout[2 * k + 1] != 0) {
                res[ids[g0 + k]] = 1;
                continue;
            }
            const int rank = std::min(std::max(hout[2 * k], 0), b.r);
            const size_t nr = (size_t)b.n * b.r, nk = (size_t)b.n * rank;
            const double *u = stage + jobs[k].off;
            if (rank > 0)
                ok = cudaMemcpyAsync(b.du, u, nk * sizeof(double), cudaMemcpyDefault, st) == cudaSuccess &&
                     cudaMemcpyAsync(b.dv, u + 2 * nr, nk * sizeof(double), cudaMemcpyDefault, st) == cudaSuccess &&
                     cudaMemcpyAsync(b.dsig, u + 3 * nr, (size_t)rank * sizeof(double), cudaMemcpyDefault, st) ==
                         cudaSuccess;
            b.rank = rank;
        }
        ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
        cudaFree(stage);
        cudaFree(dj);
        cudaFree(dout);
        g0 = g1;
    }
    cudaStreamDestroy(st);
    return ok ? 0 : -1;
}

// Buffers of one recompression worker, sized for the largest block.
struct RWorker {
    cudaStream_t st = nullptr;
    cusolverDnHandle_t h = nullptr;
    double *U = nullptr, *V = nullptr, *Ru = nullptr, *Rv = nullptr, *M = nullptr, *Um = nullptr, *Vmt = nullptr,
           *S = nullptr, *sg = nullptr, *tau = nullptr, *work = nullptr, *rwork = nullptr, *Un = nullptr,
           *Vn = nullptr;
    int *info = nullptr;
    int lwork = 0;
    std::vector<double> hS;

    bool init(int nmax, int rmax)
    {
        const int kmax = std::max(1, std::min(nmax, rmax));
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return false;
        if (solver().create(&h) != CUSOLVER_STATUS_SUCCESS || solver().set_stream(h, st) != CUSOLVER_STATUS_SUCCESS)
            return false;
        int a = 0, b = 0, c = 0;
        if (solver().geqrf_size(h, nmax, rmax, U, nmax, &a) != CUSOLVER_STATUS_SUCCESS ||
            solver().orgqr_size(h, nmax, kmax, kmax, U, nmax, S, &b) != CUSOLVER_STATUS_SUCCESS ||
            solver().gesvd_size(h, kmax, kmax, &c) != CUSOLVER_STATUS_SUCCESS)
            return false;
        lwork = std::max({a, b, c, 1});
        const size_t nr = (size_t)nmax * rmax, kr = (size_t)kmax * rmax, kk = (size_t)kmax * kmax,
                     nk = (size_t)nmax * kmax;
        bool ok = true;
        for (auto pr : {std::make_pair(&U, nr), std::make_pair(&V, nr), std::make_pair(&Ru, kr), std::make_pair(&Rv, kr),
                        std::make_pair(&M, kk), std::make_pair(&Um, kk), std::make_pair(&Vmt, kk),
                        std::make_pair(&S, (size_t)kmax), std::make_pair(&sg, (size_t)rmax),
                        std::make_pair(&tau, (size_t)kmax),
                        std::make_pair(&work, (size_t)lwork), std::make_pair(&rwork, (size_t)kmax),
                        std::make_pair(&Un, nk), std::make_pair(&Vn, nk)})
            ok = ok && cudaMalloc((void **)pr.first, std::max<size_t>(pr.second, 1) * sizeof(double)) == cudaSuccess;
        return ok && cudaMalloc((void **)&info, sizeof(int)) == cudaSuccess;
    }

    void release()
    {
        for (double *q : {U, V, Ru, Rv, M, Um, Vmt, S, sg, tau, work, rwork, Un, Vn}) cudaFree(q);
        cudaFree(info);
        if (h) solver().destroy(h);
        if (st) cudaStreamDestroy(st);
    }

    bool gemm(const GemmJob &J)
    {
        std::vector<GemmJob> jobs{J};
        std::vector<GemmTile> tiles;
        std::vector<GemmRed> reds;
        long long ptot = 0;
        plan_gemm_tiles(jobs, tiles, reds, ptot);
        if (tiles.empty()) return true;
        GemmJob *dj = nullptr;
        GemmTile *dt = nullptr;
        GemmRed *dr = nullptr;
        double *part = nullptr;
        bool ok = cudaMallocAsync((void **)&dj, sizeof(GemmJob), st) == cudaSuccess &&
                  cudaMallocAsync((void **)&dt, sizeof(GemmTile) * tiles.size(), st) == cudaSuccess &&
                  cudaMemcpyAsync(dj, jobs.data(), sizeof(GemmJob), cudaMemcpyHostToDevice, st) == cudaSuccess &&
                  cudaMemcpyAsync(dt, tiles.data(), sizeof(GemmTile) * tiles.size(), cudaMemcpyHostToDevice, st) ==
                      cudaSuccess;
        if (ok && !reds.empty())
            ok = cudaMallocAsync((void **)&dr, sizeof(GemmRed) * reds.size(), st) == cudaSuccess &&
                 cudaMallocAsync((void **)&part, sizeof(double) * ptot, st) == cudaSuccess &&
                 cudaMemcpyAsync(dr, reds.data(), sizeof(GemmRed) * reds.size(), cudaMemcpyHostToDevice, st) ==
                     cudaSuccess;
        if (ok) {
            run_gemm_tables(dj, dt, tiles.size(), dr, reds.size(), part, st);
            dg::note_launches((long long)((tiles.size() + (1u << 30) - 1) >> 30) + (reds.empty() ? 0 : 1));
            ok = cudaGetLastError() == cudaSuccess;
        }
        for (void *q : {(void *)dj, (void *)dt, (void *)dr, (void *)part})
            if (q) cudaFreeAsync(q, st);
        return ok;
    }

    // U diag(s) V^T (n x n, rank r) -> its SVD truncated where sigma < eps:
    // QR of U diag(s) and of V, SVD of Ru Rv^T (k x k, k = min(n, r)).
    // Sources and destinations may be host or device memory (UVA copies).
    // 0 done, 1 the SVD did not converge (block left as it was), -1 error.
    int run(dg::SvdBlock &jb)
    {
        const int n = jb.n, r = jb.r;
        jb.rank = r;
        if (r == 0 || n == 0) return 0;
        const int k = std::min(n, r);
        const size_t nr = (size_t)n * r;
        if (cudaMemcpyAsync(U, jb.u, nr * sizeof(double), cudaMemcpyDefault, st) != cudaSuccess ||
            cudaMemcpyAsync(V, jb.v, nr * sizeof(double), cudaMemcpyDefault, st) != cudaSuccess ||
            cudaMemcpyAsync(sg, jb.sig, (size_t)r * sizeof(double), cudaMemcpyDefault, st) != cudaSuccess)
            return -1;
        scale_cols_kernel<<<128, 256, 0, st>>>(U, sg, n, r);
        dg::note_launch();
        if (solver().geqrf(h, n, r, U, n, tau, work, lwork, info) != CUSOLVER_STATUS_SUCCESS) return -1;
        triu_kernel<<<64, 256, 0, st>>>(U, n, k, r, Ru);
        dg::note_launch();
        if (solver().orgqr(h, n, k, k, U, n, tau, work, lwork, info) != CUSOLVER_STATUS_SUCCESS) return -1;
        if (solver().geqrf(h, n, r, V, n, tau, work, lwork, info) != CUSOLVER_STATUS_SUCCESS) return -1;
        triu_kernel<<<64, 256, 0, st>>>(V, n, k, r, Rv);
        dg::note_launch();
        if (solver().orgqr(h, n, k, k, V, n, tau, work, lwork, info) != CUSOLVER_STATUS_SUCCESS) return -1;
        if (cudaGetLastError() != cudaSuccess) return -1;
        // M = Ru Rv^T (k x k)
        if (!gemm({Ru, Rv, nullptr, nullptr, M, k, k, r, k, k, 0, k, 0, 1, 1.0, 0.0})) return -1;
        if (solver().gesvd(h, 'S', 'S', k, k, M, k, S, Um, k, Vmt, k, work, lwork, rwork, info) !=
            CUSOLVER_STATUS_SUCCESS)
            return -1;
        int devinfo = 0;
        hS.resize(k);
        if (cudaMemcpyAsync(&devinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(hS.data(), S, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return -1;
        if (devinfo != 0) return 1;
        int rank = 0;
        while (rank < k && !(hS[rank] < jb.eps)) ++rank;
        if (rank > 0) {
            // U_new = Qu Um[:, :rank], V_new = Qv Vm[:, :rank] = Qv (Vm^T)^T
            if (!gemm({U, Um, nullptr, nullptr, Un, n, rank, k, n, k, 0, n, 0, 0, 1.0, 0.0}) ||
                !gemm({V, Vmt, nullptr, nullptr, Vn, n, rank, k, n, k, 0, n, 0, 1, 1.0, 0.0}))
                return -1;
            if (cudaMemcpyAsync(jb.du, Un, (size_t)n * rank * sizeof(double), cudaMemcpyDefault, st) != cudaSuccess ||
                cudaMemcpyAsync(jb.dv, Vn, (size_t)n * rank * sizeof(double), cudaMemcpyDefault, st) != cudaSuccess ||
                cudaMemcpyAsync(jb.dsig, hS.data(), (size_t)rank * sizeof(double), cudaMemcpyDefault, st) !=
                    cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)
                return -1;
        }
        jb.rank = rank;
        return 0;
    }
};

// Blocks of a host tree with dplrreduce's thresholds (eps/4 per level,
// src/dplrreduce.c:46); `nodes` keeps each block's node for its new rank.
void collect_rjobs(DPlrMtx *A, double eps, std::vector<dg::SvdBlock> &jobs, std::vector<DPlrMtx *> &nodes)
{
    if (A->type != PLR_HMTX) return;
    const double e2 = eps / 4.0;
    for (DPlrMtx *L : {A->dh.ne, A->dh.sw}) {
        jobs.push_back({L->dlr.u, L->dlr.v, L->dlr.sig, L->dlr.u, L->dlr.v, L->dlr.sig, L->size, L->dlr.rank, e2,
                        L->dlr.rank});
        nodes.push_back(L);
    }
    collect_rjobs(A->dh.nw, e2, jobs, nodes);
    collect_rjobs(A->dh.se, e2, jobs, nodes);
}

}  // namespace

namespace dg {

int svd_truncate_blocks(SvdBlock *blocks, int count, int workers)
{
    // small blocks: one batched launch; the others: the library workers
    const int limit = batch_rank_limit();
    std::vector<int> batched, order;
    int nmax = 0, rmax = 0;
    for (int i = 0; i < count; ++i) {
        blocks[i].rank = blocks[i].r;
        if (blocks[i].r == 0 || blocks[i].n == 0) continue;
        if (batch_takes(blocks[i], limit)) {
            batched.push_back(i);
        } else {
            order.push_back(i);
            nmax = std::max(nmax, blocks[i].n);
            rmax = std::max(rmax, blocks[i].r);
        }
    }
    std::vector<int> res(count, 0);
    if (run_svd_batch(blocks, batched, res) < 0)
        return report(DPLR_GPU_ECUDA, "SVD recompression: CUDA call of the batched SVD failed");
    const int nbig = (int)order.size();
    if (nbig > 0) {
        if (!solver().ok)
            return report(DPLR_GPU_ECUDA, "SVD recompression: cannot load cuSOLVER (libcusolver.so.12)");
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            return (long long)blocks[a].n * blocks[a].r > (long long)blocks[b].n * blocks[b].r;
        });
        int nw = workers > 0 ? workers : 8;
        nw = std::max(1, std::min(nw, nbig));
        std::vector<RWorker> pool(nw);
        bool ok = true;
        for (RWorker &w : pool) ok = ok && w.init(nmax, rmax);
        if (ok) {
            std::atomic<int> next{0};
            auto body = [&](RWorker &w) {
                for (int k = next.fetch_add(1); k < nbig; k = next.fetch_add(1))
                    res[order[k]] = w.run(blocks[order[k]]);
            };
            std::vector<std::thread> th;
            for (int t = 1; t < nw; ++t) th.emplace_back(body, std::ref(pool[t]));
            body(pool[0]);
            for (std::thread &t : th) t.join();
        }
        for (RWorker &w : pool) w.release();
        if (!ok) return report(DPLR_GPU_ECUDA, "SVD recompression: device setup failed");
    }
    for (int r : res)
        if (r < 0) return report(DPLR_GPU_ECUDA, "SVD recompression: CUDA or cuSOLVER call failed");
    for (int r : res)
        if (r > 0) return report(DPLR_GPU_ENOTCONV, "SVD recompression: an SVD did not converge (block kept)");
    return 0;
}

}  // namespace dg

extern "C" {

int dplr_gpu_d2gep(int m, const double *A, int lda, DPlrMtx *B, double eps, int nlvl, int workers, int *info)
{
    dg::NvtxRange nvtx_("dplr_gpu_d2gep");
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
    // blocks of order <= the batched kernel's limit run together on it; the
    // others on the library workers
    const int limit = batch_rank_limit();
    std::vector<int> batched, big;
    for (size_t i = 0; i < jobs.size(); ++i) (jobs[i].n > 0 && jobs[i].n <= limit ? batched : big).push_back((int)i);
    if (!big.empty() && !solver().ok)
        return report(DPLR_GPU_ECUDA, "dplrd2gep: cannot load cuSOLVER (libcusolver.so.12)");

    // device copy of A, ld m
    double *dA = nullptr;
    if (cudaMalloc((void **)&dA, (size_t)m * m * sizeof(double)) != cudaSuccess ||
        cudaMemcpy2D(dA, (size_t)m * sizeof(double), A, (size_t)lda * sizeof(double), (size_t)m * sizeof(double), m,
                     cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaStreamSynchronize(nullptr) != cudaSuccess) {   // the blocks read dA on streams of their own
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
    nw = std::min<int>(nw, (int)big.size());
    nw = big.empty() ? 0 : (int)std::max<size_t>(1, std::min<size_t>((size_t)nw, fr / 4 / std::max<size_t>(per, 1)));
    std::vector<Worker> pool(nw);
    bool ok = true;
    for (Worker &w : pool) ok = ok && w.init(nmax);

    std::vector<int> rc(jobs.size(), 0);
    if (ok && run_dense_batch(dA, m, jobs, batched, rc) < 0) {
        for (Worker &w : pool) w.release();
        cudaFree(dA);
        return report(DPLR_GPU_ECUDA, "dplrd2gep: CUDA call of the batched SVD failed");
    }
    if (ok && !big.empty()) {
        // largest blocks first; ties in DPLR's order
        std::vector<int> idx(big);
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

int dplr_gpu_reduce_svd(int m, DPlrMtx *A, double eps, int workers)
{
    dg::NvtxRange nvtx_("dplr_gpu_reduce_svd");
    const char *fn = "dplr_gpu_reduce_svd";
    if (m < 0) return dg::fail(DPLR_GPU_EINVAL, "%s: invalid matrix size %d", fn, m);
    if (!A) return dg::fail(DPLR_GPU_EINVAL, "%s: null argument", fn);
    if (!(eps >= 0.0)) return dg::fail(DPLR_GPU_EINVAL, "%s: eps must be nonnegative", fn);
    int rc = dg::validate_tree(m, A, fn);
    if (rc) return rc;
    std::vector<dg::SvdBlock> jobs;
    std::vector<DPlrMtx *> nodes;
    collect_rjobs(A, eps, jobs, nodes);
    rc = dg::svd_truncate_blocks(jobs.data(), (int)jobs.size(), workers);
    // ranks only shrink; a block whose SVD failed keeps its rank
    for (size_t i = 0; i < jobs.size(); ++i) nodes[i]->dlr.rank = jobs[i].rank;
    return rc;
}

void dplrd2gep(int m, double *A, int lda, DPlrMtx *B, double eps, int nlvl, int *info)
{
    dg::NvtxRange nvtx_("dplrd2gep");
    dplr_gpu_d2gep(m, A, lda, B, eps, nlvl, 0, info);
}

}  // extern "C"
