// persist.cu -- the whole FP64 apply  Y := alpha*op(A)*X + beta*Y  in ONE
// persistent launch over the device-resident block table.
//
// DPLR recurses over the tree, two BLAS calls per low-rank block and one per
// leaf (src/dplrpmv.c:113-180, src/dplrpdmm.c:177-241).  Here one grid of
// (SM count x resident CTAs) pulls work units from a device queue:
//   1. panel units (block, row chunk, right-hand-side tile): the partial
//      F[chunk]^T X[chunk rows] of one chunk (F = V for op N, U for op T),
//      written to its own slot;  the LAST chunk of a block to finish (found
//      with a counter) sums the block's partials in chunk order, scales by
//      sig and publishes T_b with a release flag -- the reduce is fused, in
//      a fixed order, so results are deterministic;
//   2. expand units (row tile, right-hand-side tile): wait (bounded) for the
//      T_b of every level that covers the tile, then
//      y = alpha * (sum_levels F_out[tile] T_b + D[tile] x[leaf]) + beta y.
// Every panel unit is dequeued before any expand unit, and panel units never
// wait, so an expand unit only ever waits for work that a running CTA holds:
// no deadlock, whatever the residency.  A wait that still expires sets the
// plan's error flag (read by the host on its next call) and the kernel runs
// to completion.
//
// The rank tile of a panel unit follows the block's rank (8, 16, 32 or 64
// columns), so blocks of rank 1-4 do not pay for 64 columns.  One
// right-hand side uses warp-per-column panels with 16-byte loads and
// shuffle reductions; more use shared-memory staged tiles of NB columns.
#include "internal.cuh"
#include "panel_rank4.cuh"

#include <algorithm>

namespace dg {

namespace {

constexpr int kPT = 256;                 // threads per CTA
constexpr int kExpSlab = 32;             // K slab of the expand staging
constexpr int kX1Max = 2048;             // longest chunk of the 1-RHS panel (x in smem)
constexpr int kWaitSpins = 1 << 22;      // bound of one readiness wait (~0.5 s with backoff)

struct Args {
    const PanelItem *items;
    const int *item_red;
    const ReduceItem *reduces;
    const int *tile_row0, *tile_begin;
    const TileTerm *terms;
    const int *term_red;
    const double *pool;
    const double *X;
    double *Y;
    double *partials, *T;
    int *ctl;                            // [0] queue, then cnt[nred*njt], ready[nred*njt]
    int *err;                            // mapped host flag
    int nitems, nred, ntiles, R, ldx, ldy, nrhs, njt;
    double alpha, beta;
};

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ------------------------------------------------------------- panel units
// Partial F[r0:r0+len, :]^T X[rows, j0:j0+nj] of one chunk; rank tile RT
// (8..64) follows the block's rank: thread t owns rank column t % RT and
// rows t / RT (mod G) of each slab of 8 G rows; the G partial sums meet in
// shared memory.
template <int NB>
__device__ void panel_unit(const Args &a, const PanelItem &it, int jt, double *sm)
{
    const int j0 = jt * NB, nj = min(NB, a.nrhs - j0);
    if (it.rank <= kRank4) {                  // every FMA live: threads own right-hand sides
        panel_rank4<NB>(a.pool + it.f, it.n, it.r0, it.len, it.rank, a.X, a.ldx, it.in0, j0, nj,
                        a.partials + it.p * a.nrhs + (long long)it.chunk * it.rank * a.nrhs, sm);
        return;
    }
    int RT = 8;
    while (RT < it.rank && RT < 64) RT <<= 1;
    const int G = kPT / RT, S = 8 * G;
    double *Fs = sm;                     // S x (RT + 1)
    double *Xs = sm + S * (RT + 1);      // S x NB
    const int t = threadIdx.x, kk = t % RT, g = t / RT;
    const double *F = a.pool + it.f;
    double *P = a.partials + it.p * a.nrhs + (long long)it.chunk * it.rank * a.nrhs;
    for (int kt = 0; kt < it.rank; kt += RT) {
        const int nk = min(RT, it.rank - kt);
        double acc[NB];
#pragma unroll
        for (int j = 0; j < NB; ++j) acc[j] = 0.0;
        for (int s0 = 0; s0 < it.len; s0 += S) {
            const int ns = min(S, it.len - s0);
            __syncthreads();
            for (int e = t; e < S * RT; e += kPT) {
                const int r = e % S, c = e / S;
                Fs[r * (RT + 1) + c] =
                    (r < ns && c < nk) ? __ldg(F + (long long)(kt + c) * it.n + it.r0 + s0 + r) : 0.0;
            }
            for (int e = t; e < S * NB; e += kPT) {
                const int r = e % S, c = e / S;
                Xs[r * NB + c] = (r < ns && c < nj)
                                     ? __ldg(a.X + (long long)(j0 + c) * a.ldx + it.in0 + it.r0 + s0 + r)
                                     : 0.0;
            }
            __syncthreads();
#pragma unroll 4
            for (int r = g; r < ns; r += G) {             // live rows only: short chunks stay cheap
                const double f = Fs[r * (RT + 1) + kk];
#pragma unroll
                for (int j = 0; j < NB; ++j) acc[j] = fma(f, Xs[r * NB + j], acc[j]);
            }
        }
        __syncthreads();                 // the reduction aliases the staging
#pragma unroll
        for (int j = 0; j < NB; ++j) sm[(g * RT + kk) * NB + j] = acc[j];
        __syncthreads();
        for (int e = t; e < RT * NB; e += kPT) {
            const int k2 = e % RT, j = e / RT;
            if (k2 < nk && j < nj) {
                double s = 0.0;
                for (int gg = 0; gg < G; ++gg) s += sm[(gg * RT + k2) * NB + j];
                P[(kt + k2) + (long long)(j0 + j) * it.rank] = s;
            }
        }
        __syncthreads();
    }
}

// One right-hand side: warp w handles columns w, w + 8, ... four at a time,
// 16-byte loads of the factor, x staged in shared memory, butterfly
// reduction of the four column sums.
__device__ void panel_unit1(const Args &a, const PanelItem &it, double *sm)
{
    double *xs = sm;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int r = t; r < it.len; r += kPT) xs[r] = __ldg(a.X + it.in0 + it.r0 + r);
    __syncthreads();
    const double *F = a.pool + it.f + it.r0;
    double *P = a.partials + it.p + (long long)it.chunk * it.rank;
    const bool vec = ((it.n | it.r0 | it.len) & 1) == 0;
    constexpr int W = kPT / 32;
    for (int k0 = warp; k0 < it.rank; k0 += 4 * W) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        if (vec) {
            for (int r = 2 * lane; r < it.len; r += 64) {
                const double2 xv = *reinterpret_cast<const double2 *>(xs + r);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int k = k0 + c * W;
                    if (k < it.rank) {
                        const double2 fv = __ldg(reinterpret_cast<const double2 *>(F + (long long)k * it.n + r));
                        acc[c] = fma(fv.x, xv.x, fma(fv.y, xv.y, acc[c]));
                    }
                }
            }
        } else {
            for (int r = lane; r < it.len; r += 32) {
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int k = k0 + c * W;
                    if (k < it.rank) acc[c] = fma(__ldg(F + (long long)k * it.n + r), xs[r], acc[c]);
                }
            }
        }
        const bool hi16 = lane & 16, hi8 = lane & 8;
        const double s0 = hi16 ? acc[0] : acc[2], s1 = hi16 ? acc[1] : acc[3];
        const double a0 = (hi16 ? acc[2] : acc[0]) + __shfl_xor_sync(0xffffffffu, s0, 16);
        const double a1 = (hi16 ? acc[3] : acc[1]) + __shfl_xor_sync(0xffffffffu, s1, 16);
        const double tt = hi8 ? a0 : a1;
        double v = (hi8 ? a1 : a0) + __shfl_xor_sync(0xffffffffu, tt, 8);
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        const int k = k0 + ((hi16 ? 2 : 0) + (hi8 ? 1 : 0)) * W;
        if ((lane & 7) == 0 && k < it.rank) P[k] = v;
    }
    __syncthreads();                     // xs is reused by the next unit
}

// Reduce of block R for one right-hand-side tile (run by the CTA that
// finished the block's last chunk): T = sig o sum_chunks partials, chunks
// summed by 8 warps in a fixed order.
template <int NB>
__device__ void reduce_unit(const Args &a, const ReduceItem &R, int jt, double *sm)
{
    const int j0 = jt * NB, nj = min(NB, a.nrhs - j0);
    const int cnt = R.rank * nj;
    const long long blk = (long long)R.rank * a.nrhs;
    const int el = threadIdx.x & 31, grp = threadIdx.x >> 5;
    double(*red)[33] = reinterpret_cast<double(*)[33]>(sm);
    for (int e0 = 0; e0 < cnt; e0 += 32) {
        const int e = e0 + el;
        const long long off = (long long)j0 * R.rank + e;   // k + j * rank
        double s = 0.0;
        if (e < cnt) {
            const double *P = a.partials + R.p * a.nrhs + off;
            for (int c = grp; c < R.nch; c += 8) s += __ldcg(P + (long long)c * blk);
        }
        red[grp][el] = s;
        __syncthreads();
        if (grp == 0 && e < cnt) {
            double tot = 0.0;
#pragma unroll
            for (int g = 0; g < 8; ++g) tot += red[g][el];
            const int k = e % R.rank;
            a.T[R.t * a.nrhs + off] = R.sig >= 0 ? __ldg(a.pool + R.sig + k) * tot : tot;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ expand units
// Wait (bounded) until the T blocks of every term of the tile are published.
__device__ void wait_terms(const Args &a, int tile, int jt, int *sflag)
{
    if (threadIdx.x == 0) {
        bool ok = true;
        for (int q = a.tile_begin[tile]; q < a.tile_begin[tile + 1] && ok; ++q) {
            const int r = a.term_red[q];
            if (r < 0) continue;
            const int *flag = a.ctl + 1 + a.nred * a.njt + r * a.njt + jt;
            int it = 0;
            while (ld_acquire(flag) == 0) {
                if (++it > kWaitSpins) {
                    ok = false;
                    break;
                }
                __nanosleep(64);
            }
        }
        if (!ok) atomicExch(a.err, 3);
        *sflag = ok;
    }
    __syncthreads();
}

template <int NB>
__device__ void expand_unit(const Args &a, int tile, int jt, double *sm)
{
    double(*As)[kExpSlab + 1] = reinterpret_cast<double(*)[kExpSlab + 1]>(sm);
    double(*Bs)[NB] = reinterpret_cast<double(*)[NB]>(sm + 64 * (kExpSlab + 1));
    double(*red)[NB] = reinterpret_cast<double(*)[NB]>(sm);
    const int row0 = a.tile_row0[tile];
    const int j0 = jt * NB, nj = min(NB, a.nrhs - j0);
    const int t = threadIdx.x, R = a.R, G = kPT / R, i = t % R, g = t / R;
    double acc[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) acc[j] = 0.0;
    for (int q = a.tile_begin[tile]; q < a.tile_begin[tile + 1]; ++q) {
        const TileTerm tt = a.terms[q];
        const double *A = a.pool + tt.a;
        const bool fromT = tt.src == 0;
        const double *B = fromT ? a.T + tt.b * a.nrhs + (long long)j0 * tt.ldb
                                : a.X + tt.x_row0 + (long long)j0 * a.ldx;
        const long long ldb = fromT ? tt.ldb : a.ldx;
        // only the nk live columns of a slab are staged and multiplied
        for (int k0 = 0; k0 < tt.K; k0 += kExpSlab) {
            const int nk = min(kExpSlab, tt.K - k0);
            __syncthreads();
            if (!tt.trans_a) {
                for (int e = t; e < R * nk; e += kPT) {
                    const int r = e % R, c = e / R;
                    As[r][c] = __ldg(A + r + (long long)(k0 + c) * tt.lda);
                }
            } else {
                for (int e = t; e < R * nk; e += kPT) {
                    const int c = e % nk, r = e / nk;
                    As[r][c] = __ldg(A + (long long)r * tt.lda + k0 + c);
                }
            }
            for (int e = t; e < nk * NB; e += kPT) {
                const int r = e % nk, c = e / nk;
                double v = 0.0;
                if (c < nj) {
                    const double *src = B + k0 + r + (long long)c * ldb;
                    v = fromT ? __ldcg(src) : __ldg(src);
                }
                Bs[r][c] = v;
            }
            __syncthreads();
            for (int c = g; c < nk; c += G) {
                const double av = As[i][c];
#pragma unroll
                for (int j = 0; j < NB; ++j) acc[j] = fma(av, Bs[c][j], acc[j]);
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NB; ++j) red[t][j] = acc[j];
    __syncthreads();
    for (int e = t; e < R * NB; e += kPT) {
        const int r = e % R, c = e / R;
        if (c >= nj) continue;
        double s = 0.0;
        for (int gg = 0; gg < G; ++gg) s += red[gg * R + r][c];
        double *y = a.Y + row0 + r + (long long)(j0 + c) * a.ldy;
        *y = a.beta == 0.0 ? a.alpha * s : fma(a.alpha, s, a.beta * *y);
    }
    __syncthreads();
}

// One right-hand side, column-major terms: thread (i, g) owns row i and the
// inner indices k == g (mod G).
__device__ void expand_unit1(const Args &a, int tile, double *sm)
{
    const int row0 = a.tile_row0[tile];
    const int t = threadIdx.x, R = a.R, G = kPT / R, i = t % R, g = t / R;
    double acc = 0.0, acc2 = 0.0;
    for (int q = a.tile_begin[tile]; q < a.tile_begin[tile + 1]; ++q) {
        const TileTerm tt = a.terms[q];
        const double *A = a.pool + tt.a + i;
        if (tt.src == 0) {
            const double *B = a.T + tt.b;
            int k = g;
            for (; k + G < tt.K; k += 2 * G) {
                acc = fma(__ldg(A + (long long)k * tt.lda), __ldcg(B + k), acc);
                acc2 = fma(__ldg(A + (long long)(k + G) * tt.lda), __ldcg(B + k + G), acc2);
            }
            if (k < tt.K) acc = fma(__ldg(A + (long long)k * tt.lda), __ldcg(B + k), acc);
        } else {
            const double *B = a.X + tt.x_row0;
            int k = g;
            for (; k + G < tt.K; k += 2 * G) {
                acc = fma(__ldg(A + (long long)k * tt.lda), __ldg(B + k), acc);
                acc2 = fma(__ldg(A + (long long)(k + G) * tt.lda), __ldg(B + k + G), acc2);
            }
            if (k < tt.K) acc = fma(__ldg(A + (long long)k * tt.lda), __ldg(B + k), acc);
        }
    }
    sm[t] = acc + acc2;
    __syncthreads();
    if (t < R) {
        double s = 0.0;
        for (int gg = 0; gg < G; ++gg) s += sm[gg * R + t];
        double *y = a.Y + row0 + t;
        *y = a.beta == 0.0 ? a.alpha * s : fma(a.alpha, s, a.beta * *y);
    }
    __syncthreads();
}

// --------------------------------------------------------------- the kernel
template <int NB>
__global__ void __launch_bounds__(kPT) persist_apply_kernel(const Args a)
{
    extern __shared__ __align__(16) double sm[];
    __shared__ int s_unit, s_flag;
    const int npanel = a.nitems * a.njt, total = npanel + a.ntiles * a.njt;
    int *cnt = a.ctl + 1, *ready = a.ctl + 1 + a.nred * a.njt;
    for (;;) {
        if (threadIdx.x == 0) s_unit = atomicAdd(a.ctl, 1);
        __syncthreads();
        const int u = s_unit;
        __syncthreads();
        if (u >= total) break;
        if (u < npanel) {
            const int i = u / a.njt, jt = u % a.njt;
            const PanelItem it = a.items[i];
            if (NB == 1)
                panel_unit1(a, it, sm);
            else
                panel_unit<NB>(a, it, jt, sm);
            // publish the chunk; the last chunk of the block runs its reduce
            const int r = a.item_red[i];
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                const int old = atomicAdd(cnt + r * a.njt + jt, 1);
                s_flag = old == a.reduces[r].nch - 1;
                if (s_flag) __threadfence();
            }
            __syncthreads();
            if (s_flag) {
                reduce_unit<NB>(a, a.reduces[r], jt, sm);
                __syncthreads();
                if (threadIdx.x == 0) {
                    __threadfence();
                    st_release(ready + r * a.njt + jt, 1);
                }
            }
        } else {
            const int v = u - npanel, tile = v / a.njt, jt = v % a.njt;
            wait_terms(a, tile, jt, &s_flag);
            if (NB == 1)
                expand_unit1(a, tile, sm);
            else
                expand_unit<NB>(a, tile, jt, sm);
        }
    }
}

template <int NB>
constexpr size_t smem_bytes()
{
    // panel: worst rank tile (8): 256 x 9 + 256 x NB; expand: 64 x 33 + 32 x NB;
    // reductions: 256 x NB (panel, expand) and 8 x 33 (reduce)
    constexpr size_t p = 256 * 9 + 256 * NB, e = 64 * (kExpSlab + 1) + kExpSlab * NB, r = kPT * NB;
    constexpr size_t m1 = p > e ? p : e, m2 = m1 > r ? m1 : r;
    static_assert((size_t)rank4_smem<NB>(kPT) <= m2, "rank <= 4 panel scratch");
    return (NB == 1 ? (size_t)kX1Max > m2 ? (size_t)kX1Max : m2 : m2) * sizeof(double);
}

// Reduce index of every panel item (by partial offset) and of every tile
// term that reads T (by T offset); built once per schedule.
int persist_prepare(Schedule &S)
{
    if (S.d_item_red) return 0;
    std::vector<int> ired(S.items.size()), tred(S.terms.size(), -1);
    std::vector<std::pair<long long, int>> byp, byt;
    for (size_t r = 0; r < S.reduces.size(); ++r) {
        byp.push_back({S.reduces[r].p, (int)r});
        byt.push_back({S.reduces[r].t, (int)r});
    }
    std::sort(byp.begin(), byp.end());
    std::sort(byt.begin(), byt.end());
    auto find = [](const std::vector<std::pair<long long, int>> &v, long long key) {
        auto it = std::lower_bound(v.begin(), v.end(), std::make_pair(key, -1));
        return (it != v.end() && it->first == key) ? it->second : -1;
    };
    for (size_t i = 0; i < S.items.size(); ++i) {
        ired[i] = find(byp, S.items[i].p);
        if (ired[i] < 0) return fail(DPLR_GPU_ESTATE, "persistent apply: panel item without reduce");
    }
    for (size_t q = 0; q < S.terms.size(); ++q) {
        if (S.terms[q].src == 2) return fail(DPLR_GPU_ESTATE, "persistent apply: unsupported term");
        if (S.terms[q].src == 0) {
            tred[q] = find(byt, S.terms[q].b);
            if (tred[q] < 0) return fail(DPLR_GPU_ESTATE, "persistent apply: term without reduce");
        }
    }
    DG_ALLOC(&S.d_item_red, std::max<size_t>(ired.size(), 1) * sizeof(int));
    DG_ALLOC(&S.d_term_red, std::max<size_t>(tred.size(), 1) * sizeof(int));
    if (!ired.empty())
        DG_CUDA(cudaMemcpy(S.d_item_red, ired.data(), ired.size() * sizeof(int), cudaMemcpyHostToDevice));
    if (!tred.empty())
        DG_CUDA(cudaMemcpy(S.d_term_red, tred.data(), tred.size() * sizeof(int), cudaMemcpyHostToDevice));
    return 0;
}

// Resident CTAs of one instantiation on the current device (SM count x
// CTAs per SM), found once per device: the first call on a device sets the
// kernel's shared-memory limit and queries the occupancy, so it should come
// before any stream capture (the library's graph builder makes an ordinary
// run first).
template <int NB>
int resident_ctas(int *out)
{
    constexpr int kMaxDev = 64;
    static int cache[kMaxDev];
    int dev = 0;
    DG_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < kMaxDev && cache[dev] > 0) {
        *out = cache[dev];
        return 0;
    }
    auto *kern = persist_apply_kernel<NB>;
    const size_t smem = smem_bytes<NB>();
    DG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0, sms = 0;
    DG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPT, smem));
    DG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    *out = std::max(1, per_sm) * std::max(1, sms);
    if (dev >= 0 && dev < kMaxDev) cache[dev] = *out;
    return 0;
}

template <int NB>
int launch(const Args &a, cudaStream_t st)
{
    auto *kern = persist_apply_kernel<NB>;
    const size_t smem = smem_bytes<NB>();
    int resident = 0;
    int rc = resident_ctas<NB>(&resident);
    if (rc) return rc;
    const int units = (a.nitems + a.ntiles) * a.njt;
    const int grid = std::max(1, std::min(units, resident));
    kern<<<grid, kPT, smem, st>>>(a);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

}  // namespace

bool persist_usable(const Plan *p, int trans, int nrhs)
{
    const Schedule &S = p->sched[trans ? 1 : 0];
    if (S.tile_rows <= 0 || 256 % S.tile_rows) return false;
    if (nrhs == 1) return S.max_len <= kX1Max && !S.has_row_major;
    return true;
}

int persist_apply(Plan *p, int trans, int nrhs, double alpha, const double *X, int ldx, double beta, double *Y,
                  int ldy, cudaStream_t st)
{
    Schedule &S = p->sched[trans ? 1 : 0];
    int rc = persist_prepare(S);
    if (rc) return rc;
    if ((rc = ensure_err_flag(p))) return rc;
    if ((rc = sliced_error(p))) return rc;     // a wait of an earlier launch expired
    const int nb = nrhs == 1 ? 1 : nrhs >= 16 ? std::min(16, std::max(p->nb_cap, 2)) : nrhs >= 8 ? 8
                                                                                       : nrhs >= 4 ? 4 : 2;
    const int njt = (nrhs + nb - 1) / nb;
    const int nred = (int)S.reduces.size();
    const size_t ctl_ints = 1 + 2 * (size_t)nred * njt;
    const size_t need = (size_t)(S.t_per_rhs + S.partial_per_rhs) * nrhs + (ctl_ints + 1) / 2;
    if ((rc = ensure_buffer(&p->work, &p->work_doubles, need))) return rc;
    Args a;
    a.T = p->work;
    a.partials = p->work + (size_t)S.t_per_rhs * nrhs;
    a.ctl = reinterpret_cast<int *>(a.partials + (size_t)S.partial_per_rhs * nrhs);
    DG_CUDA(cudaMemsetAsync(a.ctl, 0, ctl_ints * sizeof(int), st));
    a.items = S.d_items;
    a.item_red = S.d_item_red;
    a.reduces = S.d_reduces;
    a.tile_row0 = S.d_tile_row0;
    a.tile_begin = S.d_tile_begin;
    a.terms = S.d_terms;
    a.term_red = S.d_term_red;
    a.pool = p->pool;
    a.X = X;
    a.Y = Y;
    a.err = p->tc_err_d;
    a.nitems = (int)S.items.size();
    a.nred = nred;
    a.ntiles = (int)S.tile_row0.size();
    a.R = S.tile_rows;
    a.ldx = ldx;
    a.ldy = ldy;
    a.nrhs = nrhs;
    a.njt = njt;
    a.alpha = alpha;
    a.beta = beta;
    double fl = 2.0 * (double)p->nnz * nrhs, by = 8.0 * (double)p->nnz + 16.0 * p->m * (double)nrhs;
    ProfScope ps("apply_persistent", st, fl, by);
    switch (nb) {
    case 1: return launch<1>(a, st);
    case 2: return launch<2>(a, st);
    case 4: return launch<4>(a, st);
    case 8: return launch<8>(a, st);
    default: return launch<16>(a, st);
    }
}

}  // namespace dg
