// pairs.cu -- FP64-accurate single-right-hand-side apply on the FP32 pipes.
//
// With one right-hand side the apply (src/dplrpmv.c:113-180) streams every
// factor element once for one multiply-add: 0.25 flop per byte.  GB300
// issues FP64 FMAs at 1.19 TFLOP/s, which caps FP64 kernels at 4.76 TB/s
// (70 % of the measured copy rate) before any other instruction.  These
// kernels move the arithmetic to the FP32 pipes, about 60x wider:
//   * the factor pool is copied once as float pairs, hi = rn(d),
//     lo = rn(d - hi): the leading 48 bits of every double, still 8 bytes
//     per element;
//   * x (scaled by a power of two so its largest entry is below 1) and the
//     panel results T are split the same way per call;
//   * a product (ah + al)(bh + bl) is p + e with p = rn(ah bh) and
//     e = fma(ah, bh, -p) + ah bl + al bh (exact high part, al bl dropped);
//   * sums are compensated: (sh, sl) += (p, e) by TwoSum on sh.
// One element costs 12 FP32 operations, so the kernels stream the factors
// at HBM speed.  Every operation is written with the _rn intrinsics, which
// the compiler never contracts into FMAs (TwoSum needs its exact steps).
// Relative error of a product ~2^-47; of a sum of K terms ~2^-46 |sum of
// |terms|| (compensated), i.e. about 1e-14 of |A||x| -- far inside the
// 1e-12 parity bar of the FP64 path.  Panel partials, the sig scaling and
// the outputs stay FP64.
#include "internal.cuh"

#include <algorithm>
#include <climits>
#include <numeric>
#include <type_traits>
#include <vector>

namespace dg {

namespace {

constexpr int kPThreads = 256;
constexpr int kPMaxLen = 2048;   // longest panel item staged in shared memory
constexpr int kPairMaxExp = 50;  // largest pool exponent accepted (no FP32 overflow)

struct PairScratch {
    float2 *pool = nullptr;      // the factor pool as float pairs
    float2 *x = nullptr;         // scaled x as pairs (m)
    float2 *t = nullptr;         // scaled T as pairs (t_per_rhs of the op-N schedule)
    double *w = nullptr;         // partials and T (FP64)
    int *ex = nullptr;           // exponent of max |x| (device)
    size_t t_n = 0, w_n = 0;     // capacities of t and w (the schedule may change after prepare)
    // output tiles of the expand: R rows (64, or the largest power of two
    // dividing every leaf); 256 threads = R rows x 256/R inner-index groups
    int R = 0;
    std::vector<int> row0, begin;
    std::vector<TileTerm> terms;
    int *d_row0 = nullptr, *d_begin = nullptr;
    TileTerm *d_terms = nullptr;
    long long bytes = 0;
};

__device__ __forceinline__ float2 split_pair(double v)
{
    const float h = __double2float_rn(v);
    const float l = __double2float_rn(v - (double)h);
    return make_float2(h, l);
}

// (sh, sl) += a * b in compensated FP32 pair arithmetic.
__device__ __forceinline__ void pair_fma(float &sh, float &sl, float2 a, float2 b)
{
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// (ah, al) += (bh, bl).
__device__ __forceinline__ void pair_add(float &ah, float &al, float bh, float bl)
{
    const float s = __fadd_rn(ah, bh);
    const float bb = __fsub_rn(s, ah);
    const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    ah = s;
    al = __fadd_rn(al, __fadd_rn(err, bl));
}

__device__ __forceinline__ int scale_of(const int *ex)
{
    const int e = *ex;
    return (e < -1100 || e > 1100) ? 0 : e;      // all-zero (or empty) x: any scale
}

// Largest exponent (ilogb) of the finite nonzero entries.
__global__ void max_exp_kernel(const double *__restrict__ v, long long n, int *out)
{
    int e = INT_MIN;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double a = fabs(v[i]);
        if (a > 0.0 && a <= 1.7976931348623157e308) e = max(e, ilogb(a));
    }
    e = __reduce_max_sync(0xffffffffu, e);
    if ((threadIdx.x & 31) == 0 && e != INT_MIN) atomicMax(out, e);
}

__global__ void split_kernel(const double *__restrict__ v, long long n, int shift, float2 *__restrict__ out)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = split_pair(ldexp(v[i], shift));
}

// x / 2^(ex+1) as pairs (largest entry below 1).
__global__ void xsplit_kernel(const double *__restrict__ x, int m, const int *ex, float2 *__restrict__ out)
{
    const int s = -(scale_of(ex) + 1);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        out[i] = split_pair(ldexp(x[i], s));
}

// Panel, 1 RHS: P[k] = 2^(ex+1) sum_r F[r, k] xs[r] (F column-major, ld n)
// for one item; warp w handles columns k = w, w + 8, ... four at a time,
// every lane two rows per step (16-byte loads), pair butterfly at the end.
__global__ void __launch_bounds__(kPThreads) panel_pairs_kernel(const PanelItem *__restrict__ items,
                                                                const float2 *__restrict__ fbase,
                                                                const float2 *__restrict__ xp, const int *ex,
                                                                double *__restrict__ partials)
{
    __shared__ __align__(16) float2 xs[kPMaxLen];
    const PanelItem it = items[blockIdx.x];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int r = t; r < it.len; r += kPThreads) xs[r] = xp[it.in0 + it.r0 + r];
    __syncthreads();
    const double sc = ldexp(1.0, scale_of(ex) + 1);
    const float2 *F = fbase + it.f + it.r0;
    double *P = partials + it.p + (long long)it.chunk * it.rank;
    const bool vec = ((it.n | it.r0 | it.len) & 1) == 0 && ((it.f & 1) == 0);
    for (int k0 = warp; k0 < it.rank; k0 += 4 * (kPThreads / 32)) {
        float sh[4] = {0.f, 0.f, 0.f, 0.f}, sl[4] = {0.f, 0.f, 0.f, 0.f};
        if (vec) {
            // two 64-row steps per iteration: eight 16-byte loads in flight per lane
            int r = 2 * lane;
            for (; r + 64 < it.len; r += 128) {
                float4 fv[2][4];
#pragma unroll
                for (int u = 0; u < 2; ++u)
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const int k = min(k0 + c * (kPThreads / 32), it.rank - 1);
                        fv[u][c] = __ldg(reinterpret_cast<const float4 *>(F + (long long)k * it.n + r + 64 * u));
                    }
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const float4 xv = *reinterpret_cast<const float4 *>(xs + r + 64 * u);
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        pair_fma(sh[c], sl[c], make_float2(fv[u][c].x, fv[u][c].y), make_float2(xv.x, xv.y));
                        pair_fma(sh[c], sl[c], make_float2(fv[u][c].z, fv[u][c].w), make_float2(xv.z, xv.w));
                    }
                }
            }
            if (r < it.len) {
                const float4 xv = *reinterpret_cast<const float4 *>(xs + r);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int k = min(k0 + c * (kPThreads / 32), it.rank - 1);
                    const float4 fv = __ldg(reinterpret_cast<const float4 *>(F + (long long)k * it.n + r));
                    pair_fma(sh[c], sl[c], make_float2(fv.x, fv.y), make_float2(xv.x, xv.y));
                    pair_fma(sh[c], sl[c], make_float2(fv.z, fv.w), make_float2(xv.z, xv.w));
                }
            }
        } else {
            for (int r = lane; r < it.len; r += 32) {
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int k = k0 + c * (kPThreads / 32);
                    if (k < it.rank) pair_fma(sh[c], sl[c], __ldg(F + (long long)k * it.n + r), xs[r]);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                pair_add(sh[c], sl[c], __shfl_xor_sync(0xffffffffu, sh[c], o), __shfl_xor_sync(0xffffffffu, sl[c], o));
        if (lane < 4) {
            const int k = k0 + lane * (kPThreads / 32);
            float h = sh[0], l = sl[0];
#pragma unroll
            for (int c = 1; c < 4; ++c)
                if (lane == c) {
                    h = sh[c];
                    l = sl[c];
                }
            if (k < it.rank) P[k] = ((double)h + (double)l) * sc;
        }
    }
}

// T / 2^(ex+1) as pairs.
__global__ void tsplit_kernel(const double *__restrict__ T, long long n, const int *ex, float2 *__restrict__ out)
{
    const int s = -(scale_of(ex) + 1);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = split_pair(ldexp(T[i], s));
}

// Expand, 1 RHS, column-major terms: y[tile] = alpha 2^(ex+1) sum_terms
// A[tile, 0:K] b + beta y; thread (i, g) owns row i and inner indices
// k == g (mod G), the G pair sums meet in shared memory.
__global__ void __launch_bounds__(kPThreads, 8) expand_pairs_kernel(
    const float2 *__restrict__ abase, const TileTerm *__restrict__ terms, const int *__restrict__ tile_row0,
    const int *__restrict__ tile_begin, const float2 *__restrict__ tp, const float2 *__restrict__ xp, const int *ex,
    double *__restrict__ Y, int R, double alpha, double beta)
{
    __shared__ float red_h[kPThreads], red_l[kPThreads];
    const int tile = blockIdx.x, row0 = tile_row0[tile];
    const int t = threadIdx.x, G = kPThreads / R, i = t % R, g = t / R;
    // two accumulator chains, four loads of A in flight per thread; 32
    // registers keep 8 CTAs per SM, so a tile grid of ~1000 CTAs is one wave
    float h[2] = {0.f, 0.f}, l[2] = {0.f, 0.f};
    for (int q = tile_begin[tile]; q < tile_begin[tile + 1]; ++q) {
        const TileTerm tt = terms[q];
        const float2 *A = abase + tt.a + i;
        const float2 *B = tt.src == 1 ? xp + tt.x_row0 : tp + tt.b;
        int k = g;
        for (; k + 3 * G < tt.K; k += 4 * G) {
            float2 a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = __ldg(A + (long long)(k + u * G) * tt.lda);
                b[u] = __ldg(B + k + u * G);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) pair_fma(h[u & 1], l[u & 1], a[u], b[u]);
        }
        for (; k < tt.K; k += G) pair_fma(h[0], l[0], __ldg(A + (long long)k * tt.lda), __ldg(B + k));
    }
    float h0 = h[0], l0 = l[0];
    pair_add(h0, l0, h[1], l[1]);
    red_h[t] = h0;
    red_l[t] = l0;
    __syncthreads();
    if (t < R) {
        float h = red_h[t], l = red_l[t];
        for (int gg = 1; gg < G; ++gg) pair_add(h, l, red_h[gg * R + t], red_l[gg * R + t]);
        const double s = ((double)h + (double)l) * ldexp(1.0, scale_of(ex) + 1);
        double *y = Y + row0 + t;
        *y = beta == 0.0 ? alpha * s : fma(alpha, s, beta * *y);
    }
}

// Partials / T (FP64) and T pairs for the schedule as it is now.
int pairs_scratch(PairScratch *P, const Schedule &S)
{
    const size_t nt = (size_t)std::max<long long>(S.t_per_rhs, 1);
    const size_t nw = (size_t)std::max<long long>(S.t_per_rhs + S.partial_per_rhs, 1);
    if (P->t_n < nt) {
        cudaFree(P->t);
        P->t = nullptr;
        P->bytes -= (long long)P->t_n * sizeof(float2);
        P->t_n = 0;
        if (cudaMalloc((void **)&P->t, nt * sizeof(float2)) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "pair apply: cannot allocate scratch");
        P->t_n = nt;
        P->bytes += (long long)nt * sizeof(float2);
    }
    if (P->w_n < nw) {
        cudaFree(P->w);
        P->w = nullptr;
        P->bytes -= (long long)P->w_n * sizeof(double);
        P->w_n = 0;
        if (cudaMalloc((void **)&P->w, nw * sizeof(double)) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "pair apply: cannot allocate scratch");
        P->w_n = nw;
        P->bytes += (long long)nw * sizeof(double);
    }
    return 0;
}

}  // namespace

void pairs_free(Plan *p)
{
    PairScratch *P = (PairScratch *)p->pairs;
    if (!P) return;
    cudaFree(P->pool);
    cudaFree(P->x);
    cudaFree(P->t);
    cudaFree(P->w);
    cudaFree(P->ex);
    cudaFree(P->d_row0);
    cudaFree(P->d_begin);
    cudaFree(P->d_terms);
    delete P;
    p->pairs = nullptr;
}

bool pairs_usable(const Plan *p, int trans, int nrhs)
{
    if (!p->pairs || trans != 0 || nrhs != 1) return false;
    const PairScratch *P = (const PairScratch *)p->pairs;
    return p->sched[0].max_len <= kPMaxLen && P->R > 0 && kPThreads % P->R == 0;
}

int pairs_prepare(Plan *p, cudaStream_t st)
{
    pairs_free(p);
    if (p->pool_doubles == 0) return 0;
    PairScratch *P = new PairScratch();
    p->pairs = P;
    auto bail = [&](int rc) {
        pairs_free(p);
        return rc;
    };
    const Schedule &S = p->sched[0];
    if (cudaMalloc((void **)&P->ex, sizeof(int)) != cudaSuccess)
        return bail(fail(DPLR_GPU_ENOMEM, "pair apply: cannot allocate"));
    // largest exponent of the pool: products and sums must stay in FP32 range
    int h_ex = INT_MIN;
    DG_CUDA(cudaMemcpyAsync(P->ex, &h_ex, sizeof(int), cudaMemcpyHostToDevice, st));
    const int grid = (int)std::min<long long>((p->pool_doubles + 255) / 256, 152LL * 32);
    max_exp_kernel<<<grid, 256, 0, st>>>(p->pool, p->pool_doubles, P->ex);
    note_launch();
    DG_CUDA(cudaMemcpyAsync(&h_ex, P->ex, sizeof(int), cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    if (h_ex != INT_MIN && (h_ex > kPairMaxExp || h_ex < -kPairMaxExp))
        return bail(fail(DPLR_GPU_EINVAL, "pair apply: factor magnitudes 2^%d outside the supported 2^+-%d", h_ex,
                         kPairMaxExp));
    const size_t np = (size_t)p->pool_doubles;
    if (cudaMalloc((void **)&P->pool, np * sizeof(float2)) != cudaSuccess ||
        cudaMalloc((void **)&P->x, (size_t)std::max(p->m, 1) * sizeof(float2)) != cudaSuccess)
        return bail(fail(DPLR_GPU_ENOMEM, "pair apply: cannot allocate the pair copy of the factors"));
    P->bytes = (long long)(np * sizeof(float2) + p->m * sizeof(float2));
    int rc = pairs_scratch(P, S);
    if (rc) return bail(rc);
    int g = 0;
    for (const LeafDesc &L : p->leaves) g = std::gcd(g, L.b);
    P->R = 64;            // 64-row tiles: 4x the CTAs of 256-row ones, same bandwidth at full size
    while (P->R > 1 && g > 0 && g % P->R != 0) P->R >>= 1;
    build_tiles(p, 0, P->R, P->row0, P->begin, P->terms);
    auto up = [&](auto &v, auto **d) -> int {
        using T = typename std::remove_reference<decltype(v)>::type::value_type;
        const size_t n = std::max<size_t>(v.size(), 1);
        if (cudaMalloc((void **)d, n * sizeof(T)) != cudaSuccess) return fail(DPLR_GPU_ENOMEM, "pair apply: tiles");
        P->bytes += (long long)(n * sizeof(T));
        if (!v.empty() && cudaMemcpy(*d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(DPLR_GPU_ECUDA, "pair apply: tile upload");
        return 0;
    };
    if ((rc = up(P->row0, &P->d_row0)) || (rc = up(P->begin, &P->d_begin)) || (rc = up(P->terms, &P->d_terms)))
        return bail(rc);
    split_kernel<<<grid, 256, 0, st>>>(p->pool, p->pool_doubles, 0, P->pool);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

// Rebuild the pair copy after new factor values; values outside the FP32
// range drop it (applies fall back to the FP64 kernels).
int pairs_refresh(Plan *p, cudaStream_t st)
{
    if (!p->pairs) return 0;
    const int rc = pairs_prepare(p, st);
    return rc == DPLR_GPU_EINVAL ? 0 : rc;
}

long long pairs_bytes(const Plan *p)
{
    return p->pairs ? ((PairScratch *)p->pairs)->bytes : 0;
}

int pairs_apply(Plan *p, double alpha, const double *X, double beta, double *Y, cudaStream_t st)
{
    PairScratch *P = (PairScratch *)p->pairs;
    const Schedule &S = p->sched[0];
    const int m = p->m;
    int rc0 = pairs_scratch(P, S);
    if (rc0) return rc0;
    double *T = P->w, *partials = P->w + S.t_per_rhs;
    const int ninit = INT_MIN;
    DG_CUDA(cudaMemcpyAsync(P->ex, &ninit, sizeof(int), cudaMemcpyHostToDevice, st));
    {
        ProfScope ps("pair_split_x", st, 0.0, 16.0 * m);
        const int g = std::max(1, std::min((m + 255) / 256, 152 * 8));
        max_exp_kernel<<<g, 256, 0, st>>>(X, m, P->ex);
        note_launch();
        xsplit_kernel<<<g, 256, 0, st>>>(X, m, P->ex, P->x);
        note_launch();
    }
    if (!S.items.empty()) {
        double fl = 0, by = 0;
        for (const PanelItem &it : S.items) {
            fl += 2.0 * it.len * it.rank;
            by += 8.0 * ((double)it.len * it.rank + it.len + it.rank);
        }
        {
            ProfScope ps("pair_panel", st, fl, by);
            panel_pairs_kernel<<<(unsigned)S.items.size(), kPThreads, 0, st>>>(S.d_items, P->pool, P->x, P->ex,
                                                                               partials);
            note_launch();
        }
        int rc = run_reduce(S, p->pool, partials, 1, T, st);
        if (rc) return rc;
        ProfScope ps("pair_split_t", st, 0.0, 16.0 * S.t_per_rhs);
        const int g = (int)std::max<long long>(1, std::min<long long>((S.t_per_rhs + 255) / 256, 152 * 8));
        tsplit_kernel<<<g, 256, 0, st>>>(T, S.t_per_rhs, P->ex, P->t);
        note_launch();
    }
    const int ntiles = (int)P->row0.size();
    if (ntiles > 0) {
        double fl = 0, by = 8.0 * ntiles * P->R * (beta == 0.0 ? 1.0 : 2.0);
        for (const TileTerm &t : P->terms) {
            fl += 2.0 * P->R * t.K;
            by += 8.0 * ((double)P->R * t.K + t.K);
        }
        ProfScope ps("pair_expand", st, fl, by);
        expand_pairs_kernel<<<ntiles, kPThreads, 0, st>>>(P->pool, P->d_terms, P->d_row0, P->d_begin, P->t, P->x,
                                                          P->ex, Y, P->R, alpha, beta);
        note_launch();
    }
    DG_CUDA(cudaGetLastError());
    return 0;
}

}  // namespace dg
