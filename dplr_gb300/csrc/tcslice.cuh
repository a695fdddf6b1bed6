// tcslice.cuh -- tcgen05 (5th-generation tensor core) kernels for the
// exact-slice products of sliced.cu.
//
// Same arithmetic as the mma.sync kernels (sliced.cuh explains the slice
// representation), mapped onto tcgen05.mma with the accumulators in tensor
// memory:
//   * a CTA computes one 128 x 64 output tile (128 TMEM lanes = rows, 64
//     columns = right-hand sides); every slice diagonal d = p + q has its own
//     FP32 accumulator of 64 TMEM columns, so D - 1 diagonals use up to 512
//     columns;
//   * operands are staged by all threads with 16-byte cp.async copies into
//     the canonical K-major no-swizzle layout (8 rows x 16 bytes core
//     matrices), KB inner-dimension elements per stage, in a ring of stages;
//     one thread issues the MMAs of a stage and commits them to that stage's
//     mbarrier, which frees the stage for the next copy;
//   * products of 7-bit slices summed over at most 256 inner elements stay
//     below 2^24, so each diagonal's FP32 accumulator holds an exact integer
//     when it is read out (tcgen05.ld) every 256 inner elements and added
//     into 64-bit integers, one group for the diagonals d > D - 4 and one for
//     the rest (shifts of at most 21 bits inside a group);
//   * the panel kernel writes the 128-bit per-chunk partials that the reduce
//     kernel of sliced.cu consumes; the expand kernel adds every term into a
//     128-bit fixed-point accumulator per output, aligned to an exponent
//     bound per row and per column, folds in +-B exactly and rounds once to
//     FP64 with integer arithmetic (GB300's FP64 rate makes per-term
//     double-double arithmetic more expensive than the products).
// Every mbarrier wait is bounded: on expiry the kernel records an error,
// lets its outstanding MMAs drain (again bounded), frees its tensor memory
// and returns.
#pragma once

#include <cstdint>

namespace dg {
namespace tc {

constexpr int M = 128;          // tile rows (TMEM lanes)
constexpr int N = 64;           // tile columns (right-hand sides)
constexpr int KR = 256;         // inner elements between exact read-outs
constexpr int THREADS = 256;
constexpr int kSmemBudget = 200 * 1024;
constexpr int kSpin = 1 << 21;  // mbarrier try_wait rounds before giving up

template <int NS>
struct Cfg {
    static constexpr int KB = NS <= 4 ? 32 : 16;                  // inner elements per stage
    static constexpr int A_SLICE = M * KB * 2;                    // bytes of one A slice tile
    static constexpr int B_SLICE = N * KB * 2;
    static constexpr int STAGE = NS * (A_SLICE + B_SLICE);
    static constexpr int NST = (kSmemBudget / STAGE) > 8 ? 8 : (kSmemBudget / STAGE);
    static constexpr int PF = NST - 2;                            // prefetch distance (blocks)
    static constexpr int SBO = (KB / 8) * 128;                    // row-group stride
    static constexpr int LBO = 128;                               // k-chunk stride
    static constexpr int CH = KB / 8;                             // 16-byte chunks per row
    static constexpr int RANGE = KR / KB;                         // blocks per exact read-out
    static constexpr int SMEM = NST * STAGE;
};

__host__ __device__ constexpr int tmem_cols(int D)
{
    return (D - 1) * N <= 32 ? 32 : (D - 1) * N <= 64 ? 64 : (D - 1) * N <= 128 ? 128
         : (D - 1) * N <= 256 ? 256 : 512;
}

// kind::f16 instruction descriptor: F32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
                            ((uint32_t)(M >> 4) << 24);

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle, sm_100 version bit.
template <int NS>
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(Cfg<NS>::LBO >> 4) << 16) |
           ((uint64_t)(Cfg<NS>::SBO >> 4) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ void cp16z(uint32_t dst, const void *src, bool valid)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int K>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t *b, int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count));
}

// Bounded wait for the phase with the given parity; false on expiry.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity)
{
    const uint32_t a = su32(b);
    for (int it = 0; it < kSpin; ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t acc)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}

__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 32 lanes x 8 consecutive columns (one register per column).
__device__ __forceinline__ void ld8(uint32_t taddr, uint32_t (&r)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr));
}

// Exact FP32 integer (|v| < 2^24) -> int64, shifted.
__device__ __forceinline__ long long fint(uint32_t bits, int sh)
{
    return (long long)__float2int_rn(__uint_as_float(bits)) << sh;
}

// Arithmetic shift of a 128-bit integer by a signed amount (left if >= 0).
__device__ __forceinline__ __int128 ashift(__int128 w, int sh)
{
    if (sh >= 0) return w << sh;
    if (sh <= -127) return w < 0 ? (__int128)-1 : (__int128)0;
    return w >> (-sh);
}

// v * 2^U rounded to nearest (ties to even) with integer arithmetic.
__device__ __forceinline__ double i128_to_double(__int128 v, int U)
{
    if (v == 0) return 0.0;
    const bool neg = v < 0;
    const unsigned __int128 a = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
    const unsigned long long hi = (unsigned long long)(a >> 64), lo = (unsigned long long)a;
    const int msb = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
    unsigned long long mant;
    int e;
    if (msb <= 52) {
        mant = lo << (52 - msb);
        e = U - (52 - msb);
    } else {
        const int sh = msb - 52;
        const unsigned __int128 q = a >> sh;
        mant = (unsigned long long)q;
        const unsigned __int128 rem = a - (q << sh);
        const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        e = U + sh;
        if (rem > half || (rem == half && (mant & 1ULL))) {
            ++mant;
            if (mant == (1ULL << 53)) {
                mant >>= 1;
                ++e;
            }
        }
    }
    const int be = e + 52 + 1023;
    if (be >= 1 && be <= 2046) {
        const unsigned long long bits =
            ((unsigned long long)be << 52) | (mant & ((1ULL << 52) - 1)) | (neg ? (1ULL << 63) : 0ULL);
        return __longlong_as_double((long long)bits);
    }
    const double r = ldexp((double)mant, e);
    return neg ? -r : r;
}

// Stage the MMAs of one stage: all pairs p + q <= D, diagonal d into TMEM
// columns (d - 2) * N.  `first` starts the diagonals' accumulation.
template <int NS, int D>
__device__ __forceinline__ void issue_stage(uint32_t tmem, uint32_t a0, bool first)
{
    using C = Cfg<NS>;
    const uint32_t b0 = a0 + NS * C::A_SLICE;
#pragma unroll
    for (int ks = 0; ks < C::KB / 16; ++ks) {
#pragma unroll
        for (int d = 2; d <= D; ++d) {
            const int plo = d - NS > 1 ? d - NS : 1, phi = d - 1 < NS ? d - 1 : NS;
#pragma unroll
            for (int p = plo; p <= phi; ++p) {
                const uint64_t ad = sdesc<NS>(a0 + (p - 1) * C::A_SLICE + ks * 2 * C::LBO);
                const uint64_t bd = sdesc<NS>(b0 + (d - p - 1) * C::B_SLICE + ks * 2 * C::LBO);
                mma(tmem + (uint32_t)((d - 2) * N), ad, bd, (first && ks == 0 && p == plo) ? 0u : 1u);
            }
        }
    }
}

// Shared control state of a CTA.
struct Ctl {
    uint64_t bar[8];
    uint32_t tmem;
};

__device__ __forceinline__ void record_error(int *err, int code)
{
    if (err) atomicCAS(err, 0, code);
}

// Let committed MMAs drain (bounded) after an abort.
template <int NST>
__device__ __forceinline__ void drain(Ctl &c, int last_block)
{
    if (last_block >= 0) mbar_wait(&c.bar[last_block % NST], (uint32_t)((last_block / NST) & 1));
}

// Read out 8 columns (c8-th group of this warp's 32) of every diagonal and
// combine them exactly: W = ghi * 2^28 + glo in units 2^-7D, where the
// diagonals d > D - 4 shift by 7 (D - d) into glo and the others by
// 7 (D - 4 - d) into ghi.
template <int D>
__device__ __forceinline__ void read_group(uint32_t trow, int c8, __int128 (&W)[8])
{
    constexpr int DH = D >= 6 ? D - 4 : 1;       // diagonals 2..DH go to ghi (none when DH < 2)
    long long ghi[8], glo[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) ghi[u] = glo[u] = 0;
    if (DH >= 2) {
        uint32_t r[DH >= 2 ? DH - 1 : 1][8];
#pragma unroll
        for (int d = 2; d <= DH; ++d) ld8(trow + (uint32_t)((d - 2) * N + c8 * 8), r[d - 2]);
        ld_wait();
#pragma unroll
        for (int d = 2; d <= DH; ++d)
#pragma unroll
            for (int u = 0; u < 8; ++u) ghi[u] += fint(r[d - 2][u], 7 * (D - 4 - d));
    }
    {
        constexpr int D0 = DH + 1;
        uint32_t r[D - D0 + 1][8];
#pragma unroll
        for (int d = D0; d <= D; ++d) ld8(trow + (uint32_t)((d - 2) * N + c8 * 8), r[d - D0]);
        ld_wait();
#pragma unroll
        for (int d = D0; d <= D; ++d)
#pragma unroll
            for (int u = 0; u < 8; ++u) glo[u] += fint(r[d - D0][u], 7 * (D - d));
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) W[u] = (DH >= 2 ? ((__int128)ghi[u] << 28) : (__int128)0) + glo[u];
}

// ------------------------------------------------------------- panel
// P[k, j] = sum over the item's rows of F[row, k] X[row, j] as exact 128-bit
// integers (units 2^-7D), F column-major (ld n), X column-major (ld ldx).
template <int NS, int D>
__global__ void __launch_bounds__(THREADS, 1)
    tc_panel_kernel(const SPanelItem *__restrict__ items, const bf16 *__restrict__ apool, long long astride,
                    const bf16 *__restrict__ xs, long long xstride, int ldx, int nrhs,
                    __int128 *__restrict__ partials, int *err, int items_on_x)
{
    using C = Cfg<NS>;
    constexpr int TC = tmem_cols(D);
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ Ctl ctl;
    // right-hand-side tiles of one item run side by side (grid.x) unless
    // the item count exceeds grid.y's range
    const SPanelItem it = items[items_on_x ? blockIdx.x : blockIdx.y];
    const int j0 = (items_on_x ? blockIdx.y : blockIdx.x) * N;
    const int kt = blockIdx.z * M;          // rank tile
    if (kt >= it.rank) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int lq = warp & 3, ch = warp >> 2;
    const int nkb = it.len / C::KB;
    const int total = nkb;
    if (tid == 0) {
        for (int s = 0; s < C::NST; ++s) mbar_init(&ctl.bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&ctl.tmem)),
                     "r"(TC));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = ctl.tmem;
    const uint32_t sbase = su32(smem);

    auto load = [&](int i) {
        const int kb = i;
        const uint32_t As = sbase + (uint32_t)((i % C::NST) * C::STAGE), Bs = As + NS * C::A_SLICE;
        const long long k0 = it.r0 + (long long)kb * C::KB;
#pragma unroll 2
        for (int e = tid; e < NS * M * C::CH; e += THREADS) {
            const int c = e % C::CH, r = (e / C::CH) % M, p = e / (C::CH * M);
            const bool ok = kt + r < it.rank;
            const bf16 *src = apool + p * astride + it.f + (long long)(ok ? kt + r : 0) * it.n + k0 + c * 8;
            cp16z(As + p * C::A_SLICE + (r >> 3) * C::SBO + c * C::LBO + (r & 7) * 16, src, ok);
        }
#pragma unroll 2
        for (int e = tid; e < NS * N * C::CH; e += THREADS) {
            const int c = e % C::CH, r = (e / C::CH) % N, q = e / (C::CH * N);
            const bool ok = j0 + r < nrhs;
            const bf16 *src = xs + q * xstride + (long long)(ok ? j0 + r : 0) * ldx + it.in0 + k0 + c * 8;
            cp16z(Bs + q * C::B_SLICE + (r >> 3) * C::SBO + c * C::LBO + (r & 7) * 16, src, ok);
        }
        cp_commit();
    };

    __int128 acc[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) acc[c] = 0;
    __int128 *P = partials + it.p * nrhs + (long long)it.chunk * it.rank * nrhs;
    int last = -1;
    bool ab = false;                     // bounded wait expired (made uniform at barriers)
    for (int i = 0; i < C::PF; ++i) {
        if (i < total) load(i); else cp_commit();
    }
    for (int i = 0; i < total; ++i) {
        const int il = i + C::PF;
        if (il < total) {
            const int jb = il - C::NST;          // last block that read the stage being refilled
            if (jb >= 0 && !mbar_wait(&ctl.bar[jb % C::NST], (uint32_t)((jb / C::NST) & 1))) ab = true;
            load(il);
        } else {
            cp_commit();
        }
        cp_wait<C::PF>();
        fence_async_smem();
        if (__syncthreads_or(ab)) { ab = true; break; }
        const int kb = i;
        const bool first = kb % C::RANGE == 0;
        const bool flush = (kb + 1) % C::RANGE == 0 || kb == nkb - 1;
        if (tid == 0) {
            fence_after();
            issue_stage<NS, D>(tmem, sbase + (uint32_t)((i % C::NST) * C::STAGE), first);
            commit(&ctl.bar[i % C::NST]);
        }
        last = i;
        if (flush) {
            if (!mbar_wait(&ctl.bar[i % C::NST], (uint32_t)((i / C::NST) & 1))) {
                ab = true;
            } else {
                fence_after();
                const uint32_t trow = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(ch * 32);
#pragma unroll
                for (int c8 = 0; c8 < 4; ++c8) {
                    __int128 W[8];
                    read_group<D>(trow, c8, W);
#pragma unroll
                    for (int u = 0; u < 8; ++u) acc[c8 * 8 + u] += W[u];
                }
                fence_before();
            }
            if (__syncthreads_or(ab)) { ab = true; break; }
        }
    }
    if (ab) {
        record_error(err, 1);
        cp_wait<0>();
        if (tid == 0) drain<C::NST>(ctl, last);
    } else {
        const int m = kt + lq * 32 + lane;
        if (m < it.rank) {
            __int128 *q = P + m + (long long)(j0 + ch * 32) * it.rank;
#pragma unroll
            for (int c = 0; c < 32; ++c)
                if (j0 + ch * 32 + c < nrhs) q[(long long)c * it.rank] = acc[c];
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC));
}

// ------------------------------------------------------------- expand
// Y[tile] = (-1)^neg sum_terms A_t B_t (+ Bin if addb) for one 128-row tile
// and 64 right-hand sides; A_t row-sliced row-major (stride lda, padded to
// a multiple of 8 columns), B_t the T slices of a block (src 0) or the X
// slices (src 1).  Each term is read out every 256 inner elements.
template <int NS, int D>
__global__ void __launch_bounds__(THREADS, 1)
    tc_expand_kernel(const STerm *__restrict__ terms, const int *__restrict__ tile_row0,
                     const int *__restrict__ tile_begin, const bf16 *__restrict__ apool, long long astride,
                     const int *__restrict__ aexp, const bf16 *__restrict__ ts, long long tstride,
                     const int *__restrict__ texp, const bf16 *__restrict__ xs, long long xstride, int ldx,
                     const int *__restrict__ xexp, int nrhs, int neg, const double *__restrict__ Bin,
                     int ldbin, int addb, double *__restrict__ Y, int ldy, int *err, int tiles_on_x)
{
    using C = Cfg<NS>;
    constexpr int TC = tmem_cols(D);
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ Ctl ctl;
    __shared__ int cmax[N];
    // right-hand-side tiles of one row tile run side by side (grid.x) unless
    // the tile count exceeds grid.y's range
    const int tile = tiles_on_x ? blockIdx.x : blockIdx.y;
    const int row0 = tile_row0[tile];
    const int q0 = tile_begin[tile], q1 = tile_begin[tile + 1];
    const int j0 = (tiles_on_x ? blockIdx.y : blockIdx.x) * N;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int lq = warp & 3, ch = warp >> 2;
    const int row = lq * 32 + lane;

    // exponent bounds: per row (this thread) and per column (shared)
    int rmax = -100000, total = 0;
    for (int q = q0; q < q1; ++q) {
        const STerm &tt = terms[q];
        rmax = max(rmax, aexp[tt.aexp + row]);
        if (tt.K > 0) total += (((tt.K + 7) & ~7) + C::KB - 1) / C::KB;
    }
    if (tid < N) {
        int cm = -100000;
        const int j = j0 + tid;
        if (j < nrhs)
            for (int q = q0; q < q1; ++q) {
                const STerm &tt = terms[q];
                cm = max(cm, tt.src == 0 ? texp[(long long)tt.blk * nrhs + j] : xexp[j]);
            }
        cmax[tid] = cm < -99999 ? 0 : cm;
    }
    if (rmax < -99999) rmax = 0;
    if (tid == 0) {
        for (int s = 0; s < C::NST; ++s) mbar_init(&ctl.bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&ctl.tmem)),
                     "r"(TC));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = ctl.tmem;
    const uint32_t sbase = su32(smem);

    // load cursor (term, block within term)
    int lqt = q0, lkb = 0;
    while (lqt < q1 && terms[lqt].K <= 0) ++lqt;
    auto load = [&](int i) {
        const STerm tt = terms[lqt];
        const int Kp = (tt.K + 7) & ~7;
        const uint32_t As = sbase + (uint32_t)((i % C::NST) * C::STAGE), Bs = As + NS * C::A_SLICE;
        const int k0 = lkb * C::KB;
#pragma unroll 2
        for (int e = tid; e < NS * M * C::CH; e += THREADS) {
            const int c = e % C::CH, r = (e / C::CH) % M, p = e / (C::CH * M);
            const bool ok = k0 + c * 8 < Kp;
            const bf16 *src = apool + p * astride + tt.a + (long long)r * tt.lda + (ok ? k0 + c * 8 : 0);
            cp16z(As + p * C::A_SLICE + (r >> 3) * C::SBO + c * C::LBO + (r & 7) * 16, src, ok);
        }
#pragma unroll 2
        for (int e = tid; e < NS * N * C::CH; e += THREADS) {
            const int c = e % C::CH, r = (e / C::CH) % N, q = e / (C::CH * N);
            const bool ok = j0 + r < nrhs && k0 + c * 8 < Kp;
            const int jj = j0 + (ok ? r : 0), kk = ok ? k0 + c * 8 : 0;
            const bf16 *src = tt.src == 0
                                  ? ts + q * tstride + tt.b * nrhs + (long long)jj * tt.ldb + kk
                                  : xs + q * xstride + (long long)(tt.x_row0 + kk) + (long long)jj * ldx;
            cp16z(Bs + q * C::B_SLICE + (r >> 3) * C::SBO + c * C::LBO + (r & 7) * 16, src, ok);
        }
        cp_commit();
        if (++lkb * C::KB >= Kp) {
            lkb = 0;
            do ++lqt; while (lqt < q1 && terms[lqt].K <= 0);
        }
    };

    __int128 acc[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) acc[c] = 0;
    int cqt = q0, ckb = 0;     // compute cursor
    while (cqt < q1 && terms[cqt].K <= 0) ++cqt;
    int last = -1;
    bool ab = false;
    for (int i = 0; i < C::PF; ++i) {
        if (i < total) load(i); else cp_commit();
    }
    for (int i = 0; i < total; ++i) {
        const int il = i + C::PF;
        if (il < total) {
            const int jb = il - C::NST;
            if (jb >= 0 && !mbar_wait(&ctl.bar[jb % C::NST], (uint32_t)((jb / C::NST) & 1))) ab = true;
            load(il);
        } else {
            cp_commit();
        }
        cp_wait<C::PF>();
        fence_async_smem();
        if (__syncthreads_or(ab)) { ab = true; break; }
        const STerm tt = terms[cqt];
        const int nkb = (((tt.K + 7) & ~7) + C::KB - 1) / C::KB;
        const int kb = ckb;
        const bool first = kb % C::RANGE == 0;
        const bool flush = (kb + 1) % C::RANGE == 0 || kb == nkb - 1;
        if (tid == 0) {
            fence_after();
            issue_stage<NS, D>(tmem, sbase + (uint32_t)((i % C::NST) * C::STAGE), first);
            commit(&ctl.bar[i % C::NST]);
        }
        last = i;
        if (++ckb == nkb) {
            ckb = 0;
            ++cqt;
        }
        if (flush) {
            if (!mbar_wait(&ctl.bar[i % C::NST], (uint32_t)((i / C::NST) & 1))) {
                ab = true;
            } else {
                fence_after();
                const uint32_t trow = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(ch * 32);
                const int rdel = aexp[tt.aexp + row] - rmax + 109 - 7 * D;
#pragma unroll
                for (int c8 = 0; c8 < 4; ++c8) {
                    __int128 W[8];
                    read_group<D>(trow, c8, W);
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int col = ch * 32 + c8 * 8 + u;
                        const int j = j0 + col;
                        if (j < nrhs) {
                            const int ce = tt.src == 0 ? texp[(long long)tt.blk * nrhs + j] : xexp[j];
                            acc[c8 * 8 + u] += ashift(W[u], rdel + ce - cmax[col]);
                        }
                    }
                }
                fence_before();
            }
            if (__syncthreads_or(ab)) { ab = true; break; }
        }
    }
    if (ab) {
        record_error(err, 1);
        cp_wait<0>();
        if (tid == 0) drain<C::NST>(ctl, last);
    } else {
        // epilogue: fold in +-B exactly, round once
        const int gr = row0 + row;
#pragma unroll
        for (int c = 0; c < 32; ++c) {
            const int col = ch * 32 + c, j = j0 + col;
            if (j < nrhs) {
            const int U = rmax + cmax[col] - 109;
            __int128 v = neg ? -acc[c] : acc[c];
            double out;
            if (addb) {
                const double b = Bin[gr + (long long)j * ldbin];
                const long long bits = __double_as_longlong(b);
                int eb = (int)((bits >> 52) & 0x7FF);
                long long mb = bits & ((1LL << 52) - 1);
                if (eb == 0x7FF) {
                    out = b + i128_to_double(v, U);
                } else {
                    if (eb) mb |= 1LL << 52; else eb = 1;
                    const int sb = eb - 1075 - U;
                    if (sb <= 70) {
                        const __int128 bm = ashift((__int128)mb, sb);
                        v += bits < 0 ? -bm : bm;
                        out = i128_to_double(v, U);
                    } else {
                        out = b + i128_to_double(v, U);
                    }
                }
            } else {
                out = i128_to_double(v, U);
            }
            Y[gr + (long long)j * ldy] = out;
            }
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC));
}

}  // namespace tc
}  // namespace dg
