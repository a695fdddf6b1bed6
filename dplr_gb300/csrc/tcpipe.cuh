// tcpipe.cuh -- warp-specialised persistent tcgen05 kernels for the
// exact-slice products: one FP32 TMEM accumulator per slice diagonal, exact
// read-out every 256 inner elements, 64- or 128-bit integer combination.
//
// Operand layout ("tile-blocks"): every slice of every operand is stored as
// tile-blocks of R rows x 16 inner elements (R = 128 or 64, or the padded
// rank of a panel tile), each contiguous and already in the canonical
// K-major no-swizzle order of the tensor core (8-row x 16-byte core
// matrices: element (r, k) at (r/8)*128 + (k/8)*64 + (r%8)*8 + k%8).  One
// pipeline stage is therefore 2*NS contiguous blocks, fetched with one
// cp.async.bulk each into a ring of shared-memory stages.
//
// Roles (320 threads, one CTA per SM, persistent over work items):
//   warp 0, lane 0: producer -- waits for a free stage, posts the stage's
//       byte count on its `full` mbarrier and issues the bulk copies;
//   warp 1, lane 0: MMA issuer -- waits for `full`, issues every slice pair
//       of the stage (tcgen05.mma), commits to the stage's `empty` barrier;
//       at the end of a 256-deep range it commits to `accf`;
//   warps 2..9: epilogue -- wait for `accf`, read the diagonals out of TMEM,
//       combine them exactly, release TMEM through `acce` (the next range's
//       MMAs start while the epilogue finishes its integer work), and write
//       the item's outputs.
// Waits are bounded; an expired wait sets a CTA-wide abort flag that every
// role polls, the kernel records an error, drains and frees TMEM.
#pragma once

#include "tcslice.cuh"

namespace dg {
namespace tc2 {

using tc::ashift;
using tc::commit;
using tc::fence_after;
using tc::fence_before;
using tc::fint;
using tc::ld_wait;
using tc::su32;

constexpr int KB = 16;                 // inner elements per stage
constexpr int M = 128, N = 64;
constexpr int RANGE = 16;              // stages per exact read-out (256 inner elements)
constexpr int TB_A = M * KB;           // elements of a 128-row tile-block
constexpr int TB_B = N * KB;           // elements of a 64-row tile-block
constexpr int EW = 16;                 // epilogue warps: 4 per TMEM lane quadrant
constexpr int CPW = 4 * N / EW;        // TMEM columns per epilogue warp
constexpr int C4N = CPW / 4;           // 4-column read-out groups per epilogue warp
constexpr int THREADS = 64 + 32 * EW;  // producer warp, MMA warp, epilogue warps
// registers per thread of one CTA per SM (warps are allocated in groups of 4)
constexpr int kRegs = (65536 / (((THREADS / 32 + 3) / 4) * 4 * 32)) & ~7;
constexpr int kSmem = 192 * 1024;
constexpr int kColCap = 1024;          // right-hand sides whose output exponents the lean expand gathers
constexpr int kNoExpT = -(1 << 24);    // "no entry" exponent (below every finite one)
constexpr int kSpin = 1 << 22;
// Bound of the role-to-role waits (wait_bar), read once per CTA at set-up.
// dplr_gpu_debug_wait_limit lowers it so that a test can make the waits
// expire and check the error path; the drain waits after an abort keep
// kSpin, so copies and MMAs in flight always land before the CTA exits.
__device__ int g_wait_limit = kSpin;

template <int NS>
struct Cfg {
    static constexpr int STAGE = NS * (TB_A + TB_B) * 2;                    // bytes
    static constexpr int NST = (kSmem / STAGE) > 8 ? 8 : (kSmem / STAGE);
    static constexpr int SMEM = NST * STAGE;
};

// Element offset of (r, k) inside a tile-block.
__host__ __device__ constexpr int tbo(int r, int k)
{
    return (r >> 3) * 128 + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

constexpr uint32_t kIdescM128 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(M >> 4) << 24);
__device__ __forceinline__ uint32_t idesc_n(int n) { return kIdescM128 | ((uint32_t)(n >> 3) << 17); }

// LBO 128 B (next 8 inner elements), SBO 256 B (next 8 rows).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
           ((uint64_t)1 << 46);
}

__device__ __forceinline__ void mma_n(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(su32(bar))
        : "memory");
}

__device__ __forceinline__ void arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}


// 32 lanes x 4 consecutive columns.
__device__ __forceinline__ void ld4(uint32_t taddr, uint32_t (&r)[4])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
}

// Exact read-out of 4 columns (c4-th group of this warp's 32) of every
// diagonal: W = ghi * 2^28 + glo in units 2^-7D (see tcslice.cuh).
template <int D>
__device__ __forceinline__ void read4(uint32_t trow, int c4, __int128 (&W)[4])
{
    constexpr int DH = D >= 6 ? D - 4 : 1;
    long long ghi[4], glo[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) ghi[u] = glo[u] = 0;
    if (DH >= 2) {
        uint32_t r[DH >= 2 ? DH - 1 : 1][4];
#pragma unroll
        for (int d = 2; d <= DH; ++d) ld4(trow + (uint32_t)((d - 2) * N + c4 * 4), r[d - 2]);
        ld_wait();
#pragma unroll
        for (int d = 2; d <= DH; ++d)
#pragma unroll
            for (int u = 0; u < 4; ++u) ghi[u] += fint(r[d - 2][u], 7 * (D - 4 - d));
    }
    {
        constexpr int D0 = DH + 1;
        uint32_t r[D - D0 + 1][4];
#pragma unroll
        for (int d = D0; d <= D; ++d) ld4(trow + (uint32_t)((d - 2) * N + c4 * 4), r[d - D0]);
        ld_wait();
#pragma unroll
        for (int d = D0; d <= D; ++d)
#pragma unroll
            for (int u = 0; u < 4; ++u) glo[u] += fint(r[d - D0][u], 7 * (D - d));
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) W[u] = (DH >= 2 ? ((__int128)ghi[u] << 28) : (__int128)0) + glo[u];
}

// Bits the 64-bit read-out drops: for D = 8 it counts in units 2^-7(D-1)
// and the lowest diagonal is shifted right by 7 (rounded), so every shift
// stays <= 35 bits.
template <int D>
constexpr int kLeanDrop = D > 7 ? 7 * (D - 7) : 0;

// Same read-out for D <= 8 as one 64-bit integer per column, in units
// 2^(kLeanDrop - 7D).  The sum stays below 2^62: at most seven diagonals of
// |I| < 2^24 shifted by at most 35.  For D <= 7 it is exact; for D = 8 the
// dropped 7 bits sit 2^-66 below the leading diagonal, far under the
// truncation of the slice pairs beyond D.
template <int D>
__device__ __forceinline__ void read4_64(uint32_t trow, int c4, long long (&W)[4])
{
    static_assert(D <= 8, "64-bit read-out holds at most seven diagonals");
    constexpr int DROP = kLeanDrop<D>;
    uint32_t r[D - 1][4];
#pragma unroll
    for (int d = 2; d <= D; ++d) ld4(trow + (uint32_t)((d - 2) * N + c4 * 4), r[d - 2]);
    ld_wait();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        long long w = 0;
#pragma unroll
        for (int d = 2; d <= D; ++d) {
            const int sh = 7 * (D - d) - DROP;
            if (sh >= 0)
                w += fint(r[d - 2][u], sh);
            else
                w += (fint(r[d - 2][u], 0) + (1LL << (-sh - 1))) >> (-sh);
        }
        W[u] = w;
    }
}

// v * 2^E rounded to nearest with integer arithmetic (|v| < 2^63).
__device__ __forceinline__ double i64_scaled(long long v, int E)
{
    if (v == 0) return 0.0;
    const bool neg = v < 0;
    unsigned long long a = neg ? (unsigned long long)(-v) : (unsigned long long)v;
    const int msb = 63 - __clzll((long long)a);
    unsigned long long mant;
    int e;
    if (msb <= 52) {
        mant = a << (52 - msb);
        e = E - (52 - msb);
    } else {
        const int sh = msb - 52;
        mant = a >> sh;
        const unsigned long long rem = a & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
        e = E + sh;
        if (rem > half || (rem == half && (mant & 1ULL))) {
            ++mant;
            if (mant == (1ULL << 53)) {
                mant >>= 1;
                ++e;
            }
        }
    }
    const int be = e + 52 + 1023;
    if (be >= 1 && be <= 2046)
        return __longlong_as_double((long long)(((unsigned long long)be << 52) | (mant & ((1ULL << 52) - 1)) |
                                                (neg ? (1ULL << 63) : 0ULL)));
    const double r = ldexp((double)mant, e);
    return neg ? -r : r;
}

struct Ctl {
    uint64_t full[8], empty[8];
    uint64_t accf, acce;
    uint32_t tmem;
    int limit;
    volatile int abort;
};

// Bounded wait; false (and the CTA-wide abort flag set) on expiry or when
// another role aborted.
__device__ __forceinline__ bool wait_bar(Ctl &c, uint64_t *bar, uint32_t parity)
{
    const uint32_t a = su32(bar);
    for (int it = 0; it < c.limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (c.abort) return false;
    }
    c.abort = 1;
    return false;
}

// Bounded wait that ignores the abort flag (draining after an abort).
__device__ __forceinline__ void wait_raw(uint64_t *bar, uint32_t parity)
{
    const uint32_t a = su32(bar);
    for (int it = 0; it < kSpin; ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return;
    }
}

// All slice pairs p + q <= D of one stage (A: NS blocks of 128 rows, B: NS
// blocks of `nb` rows), diagonal d into TMEM columns (d - 2) * 64.  The
// slices of a stage sit at fixed distances, so every descriptor is the
// stage's base descriptor plus a multiple of the distance / 16 (the 14-bit
// address field cannot carry: shared addresses are below 256 KB); fully
// unrolled, one MMA costs the issuing thread a few instructions.  FIRST
// starts each diagonal's accumulation.
template <int NS, int D, bool FIRST>
__device__ __forceinline__ void issue(uint32_t tmem, uint64_t ad0, uint64_t bd0, uint32_t bstep, uint32_t idesc)
{
#pragma unroll
    for (int d = 2; d <= D; ++d) {
#pragma unroll
        for (int p = 1; p <= NS; ++p) {
            const int q = d - p;
            if (q < 1 || q > NS) continue;
            const bool start = FIRST && p == (d - NS > 1 ? d - NS : 1);
            mma_n(tmem + (uint32_t)((d - 2) * N), ad0 + (uint64_t)((p - 1) * (TB_A * 2 / 16)),
                  bd0 + (uint64_t)(q - 1) * bstep, idesc, start ? 0u : 1u);
        }
    }
}

// The same products with 64-row B slices, one MMA per (A slice p, group of
// up to four B slices q0..q0+k-1).  The B slices of a stage are contiguous
// 64-row tile-blocks, so k of them form one operand of N = 64 k rows with
// the same descriptor strides; its output columns j land on TMEM column
// (p + q0 - 2) * 64 + j, which is diagonal d = p + q0 + j / 64, column
// j % 64 -- exactly where the per-pair MMAs put them.  A slice p is read
// from shared memory once per group instead of once per pair (12 MMAs of
// N <= 256 instead of 36 of N = 64 for 8 slices), which takes the MMAs off
// the shared-memory bound.  Needs D <= NS + 1: then every diagonal gets its
// first pair from p = 1, so FIRST overwrites exactly at p == 1.
template <int NS, int D, bool FIRST>
__device__ __forceinline__ void issue_wide(uint32_t tmem, uint64_t ad0, uint64_t bd0, uint32_t bstep)
{
    static_assert(D <= NS + 1, "wide issue needs every diagonal to start at p = 1");
#pragma unroll
    for (int p = 1; p <= NS; ++p) {
        const int qmax = D - p < NS ? D - p : NS;
#pragma unroll
        for (int q0 = 1; q0 <= qmax; q0 += 4) {
            const int k = qmax - q0 + 1 < 4 ? qmax - q0 + 1 : 4;
            mma_n(tmem + (uint32_t)((p + q0 - 2) * N), ad0 + (uint64_t)((p - 1) * (TB_A * 2 / 16)),
                  bd0 + (uint64_t)(q0 - 1) * bstep, idesc_n(N * k), (FIRST && p == 1) ? 0u : 1u);
        }
    }
}

template <int NS, int D>
__device__ __forceinline__ void issue_stage(uint32_t tmem, uint32_t a0, int nb, uint32_t idesc, bool first)
{
    const uint64_t ad0 = sdesc(a0), bd0 = sdesc(a0 + NS * TB_A * 2);
    const uint32_t bstep = (uint32_t)(nb * KB * 2 / 16);
    if constexpr (D <= NS + 1) {
        if (nb == N) {
            if (first)
                issue_wide<NS, D, true>(tmem, ad0, bd0, bstep);
            else
                issue_wide<NS, D, false>(tmem, ad0, bd0, bstep);
            return;
        }
    }
    if (first)
        issue<NS, D, true>(tmem, ad0, bd0, bstep, idesc);
    else
        issue<NS, D, false>(tmem, ad0, bd0, bstep, idesc);
}

template <int NS, int D>
__device__ __forceinline__ void setup(Ctl &ctl, int warp, int lane)
{
    if (warp == 0 && lane == 0) {
        for (int s = 0; s < Cfg<NS>::NST; ++s) {
            tc::mbar_init(&ctl.full[s], 1);
            tc::mbar_init(&ctl.empty[s], 1);
        }
        tc::mbar_init(&ctl.accf, 1);
        tc::mbar_init(&ctl.acce, EW);
        ctl.abort = 0;
        ctl.limit = g_wait_limit;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&ctl.tmem)),
                     "r"(tc::tmem_cols(D)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
}

// Teardown.  After an abort the producer waits (bounded) for the copies
// still in flight (the last fill of each stage) and the MMA lane for its
// last committed MMAs; then TMEM is freed.
template <int NS, int D>
__device__ __forceinline__ void teardown(Ctl &ctl, int warp, int lane, int issued, int consumed, int *err)
{
    if (ctl.abort && lane == 0) {
        if (warp == 0)
            for (int k = issued > Cfg<NS>::NST ? issued - Cfg<NS>::NST : 0; k < issued; ++k)
                wait_raw(&ctl.full[k % Cfg<NS>::NST], (uint32_t)((k / Cfg<NS>::NST) & 1));
        if (warp == 1 && consumed > 0)
            wait_raw(&ctl.empty[(consumed - 1) % Cfg<NS>::NST], (uint32_t)(((consumed - 1) / Cfg<NS>::NST) & 1));
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (ctl.abort && threadIdx.x == 0) tc::record_error(err, 2);
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(ctl.tmem),
                                "r"(tc::tmem_cols(D)));
}

// ------------------------------------------------------------- expand
__device__ __forceinline__ int nkb_of(int K) { return (K + KB - 1) / KB; }


// Y[tile, 64 columns] = (-1)^neg sum_terms A_t B_t (+ Bin).  Work item
// it = tile * njt + jt (right-hand-side tiles of one row tile adjacent).
// Output row i of a tile is Y row tile_row0 * rscale + i (rscale > 1 places
// tiles at offsets that scale with the right-hand-side count).
// LEAN (D <= 8, every tile a single term, as in the inner solve): the
// product of each output is one 64-bit integer, rounded once to FP64 and
// added to Bin in FP64 (accurate far beyond the inner solve's slices); otherwise
// all terms and Bin meet in a 128-bit fixed-point sum rounded once.
template <int NS, int D, bool LEAN>
__global__ void __maxnreg__(kRegs)
    expand_kernel(const XTerm *__restrict__ terms, const int *__restrict__ tile_row0,
                  const int *__restrict__ tile_begin, int ntiles, int njt, const bf16 *__restrict__ apool,
                  long long astride, const int *__restrict__ aexp, const bf16 *__restrict__ ts, long long tstride,
                  const int *__restrict__ texp, const bf16 *__restrict__ xs, long long xstride, int xnjt,
                  const int *__restrict__ xexp, int nrhs, int neg, const double *__restrict__ Bin, int ldbin,
                  int addb, double *__restrict__ Y, int ldy, const int *__restrict__ rmaxt,
                  const int *__restrict__ cmaxt, int *__restrict__ yexp, int rscale, int *err)
{
    using C = Cfg<NS>;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ Ctl ctl;
    // lean expand with yexp: per right-hand side the largest exponent of the
    // outputs written (the next slicing of Y needs it); gathered per CTA here
    __shared__ int colmax[LEAN ? kColCap : 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if constexpr (LEAN)
        if (yexp)
            for (int j = threadIdx.x; j < min(nrhs, kColCap); j += blockDim.x) colmax[j] = kNoExpT;
    setup<NS, D>(ctl, warp, lane);
    const uint32_t sbase = su32(smem);
    const int nitems = ntiles * njt;
    int issued = 0, consumed = 0;

    if (warp == 0) {
        // ---------------------------------------------------- producer
        if (lane == 0) {
            for (int it = blockIdx.x; it < nitems && !ctl.abort; it += gridDim.x) {
                const int tile = it / njt, jt = it % njt;
                for (int q = tile_begin[tile]; q < tile_begin[tile + 1] && !ctl.abort; ++q) {
                    const XTerm tt = terms[q];
                    const int nkb = nkb_of(tt.K);
                    for (int kb = 0; kb < nkb; ++kb) {
                        const int s = issued % C::NST, f = issued / C::NST;
                        if (f > 0 && !wait_bar(ctl, &ctl.empty[s], (uint32_t)((f - 1) & 1))) break;
                        expect_tx(&ctl.full[s], (uint32_t)C::STAGE);
                        const uint32_t da = sbase + (uint32_t)(s * C::STAGE), db = da + NS * TB_A * 2;
#pragma unroll 1
                        for (int p = 0; p < NS; ++p)
                            bulk_g2s(da + p * TB_A * 2, apool + p * astride + tt.a + (long long)kb * TB_A, TB_A * 2,
                                     &ctl.full[s]);
                        const long long boff = tt.src == 0 ? tt.b * njt + ((long long)jt * nkb + kb) * TB_B
                                                           : ((tt.b + kb) * (long long)xnjt + jt) * TB_B;
                        const bf16 *bsrc = tt.src == 0 ? ts : xs;
                        const long long bstr = tt.src == 0 ? tstride : xstride;
#pragma unroll 1
                        for (int p = 0; p < NS; ++p)
                            bulk_g2s(db + p * TB_B * 2, bsrc + p * bstr + boff, TB_B * 2, &ctl.full[s]);
                        ++issued;
                    }
                }
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------- MMA issuer
        if (lane == 0) {
            const uint32_t tmem = ctl.tmem;
            const uint32_t idesc = idesc_n(N);
            int rc = 0;
            for (int it = blockIdx.x; it < nitems && !ctl.abort; it += gridDim.x) {
                const int tile = it / njt;
                for (int q = tile_begin[tile]; q < tile_begin[tile + 1] && !ctl.abort; ++q) {
                    const int nkb = nkb_of(terms[q].K);
                    for (int kb0 = 0; kb0 < nkb && !ctl.abort; kb0 += RANGE) {
                        if (rc > 0 && !wait_bar(ctl, &ctl.acce, (uint32_t)((rc - 1) & 1))) break;
                        const int kb1 = min(nkb, kb0 + RANGE);
                        for (int kb = kb0; kb < kb1; ++kb) {
                            const int s = consumed % C::NST;
                            if (!wait_bar(ctl, &ctl.full[s], (uint32_t)((consumed / C::NST) & 1))) break;
                            fence_after();
                            const uint32_t a0 = sbase + (uint32_t)(s * C::STAGE);
                            issue_stage<NS, D>(tmem, a0, N, idesc, kb == kb0);
                            commit(&ctl.empty[s]);
                            ++consumed;
                        }
                        if (ctl.abort) break;
                        commit(&ctl.accf);
                        ++rc;
                    }
                }
            }
        }
    } else {
        // ---------------------------------------------------- epilogue
        const int lq = warp & 3, ch = (warp - 2) >> 2;
        const int row = lq * 32 + lane;
        const uint32_t trow = ctl.tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(ch * CPW);
        int ec = 0;
        if constexpr (LEAN) {
            // the item's exponents and its CPW values of Bin do not depend on
            // the products: they are loaded before waiting for the MMAs (and
            // the next item's exponents before this item's output pass)
            auto meta = [&](int it, int &re, int &cel, int &nkb) {
                const int tile = it / njt, jt = it % njt;
                const XTerm tt = terms[tile_begin[tile]];
                const int myj = jt * N + ch * CPW + lane;
                nkb = nkb_of(tt.K);
                re = aexp[tt.aexp + row] - 7 * D + kLeanDrop<D>;
                cel = myj < nrhs ? (tt.src == 0 ? texp[(long long)tt.blk * nrhs + myj] : xexp[myj]) : 0;
            };
            int re = 0, cel = 0, nkb = 0;
            if (blockIdx.x < nitems) meta(blockIdx.x, re, cel, nkb);
            for (int it = blockIdx.x; it < nitems && !ctl.abort; it += gridDim.x) {
                const int tile = it / njt, jt = it % njt;
                const int j0 = jt * N + ch * CPW;
                const long long gr = (long long)tile_row0[tile] * rscale + row;
                double bv[CPW];
                if (addb) {
#pragma unroll
                    for (int c = 0; c < CPW; ++c) bv[c] = j0 + c < nrhs ? Bin[gr + (long long)(j0 + c) * ldbin] : 0.0;
                }
                long long acc[CPW];
#pragma unroll
                for (int c = 0; c < CPW; ++c) acc[c] = 0;
                bool ok = true;
                for (int kb0 = 0; kb0 < nkb; kb0 += RANGE) {
                    if (!wait_bar(ctl, &ctl.accf, (uint32_t)(ec & 1))) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    // (every warp reads: skipping the columns past nrhs here
                    // made the full-width inner-solve expand 7 % slower)
#pragma unroll
                    for (int c4 = 0; c4 < C4N; ++c4) {
                        long long W[4];
                        read4_64<D>(trow, c4, W);
#pragma unroll
                        for (int u = 0; u < 4; ++u) acc[c4 * 4 + u] += W[u];
                    }
                    fence_before();
                    __syncwarp();
                    if (lane == 0) arrive(&ctl.acce);
                    ++ec;
                }
                if (!ok) break;
                const int rcur = re, ccur = cel;
                if (it + (int)gridDim.x < nitems) meta(it + gridDim.x, re, cel, nkb);
#pragma unroll
                for (int c = 0; c < CPW; ++c) {
                    const int j = j0 + c;
                    const int ce = __shfl_sync(0xffffffffu, ccur, c);
                    double y = 0.0;
                    if (j < nrhs) {
                        const double t = i64_scaled(neg ? -acc[c] : acc[c], rcur + ce);
                        y = addb ? bv[c] + t : t;
                        Y[gr + (long long)j * ldy] = y;
                    }
                    if (yexp) {
                        // exponent e with |y| < 2^e from the bits (subnormals: ilogb)
                        const int be = (int)((__double_as_longlong(y) >> 52) & 0x7FF);
                        int e = kNoExpT;
                        if (be > 0 && be < 0x7FF) e = be - 1022;
                        else if (be == 0 && y != 0.0) e = ilogb(fabs(y)) + 1;
                        e = __reduce_max_sync(0xffffffffu, e);
                        if (lane == c && j < min(nrhs, kColCap) && e > kNoExpT) atomicMax(&colmax[j], e);
                    }
                }
            }
            if (yexp) {
                // every epilogue warp leaves the item loop exactly once: named
                // barrier over the epilogue threads, then one flush per CTA
                asm volatile("bar.sync 1, %0;" ::"r"(EW * 32) : "memory");
                for (int j = threadIdx.x - 64; j < min(nrhs, kColCap); j += EW * 32)
                    if (colmax[j] > kNoExpT) atomicMax(&yexp[j], colmax[j]);
            }
        } else
        for (int it = blockIdx.x; it < nitems && !ctl.abort; it += gridDim.x) {
            const int tile = it / njt, jt = it % njt;
            const int q0 = tile_begin[tile], q1 = tile_begin[tile + 1];
            const int j0 = jt * N + ch * CPW;        // this warp's first column
            const int myj = j0 + lane;               // column whose exponents this lane holds
            // alignment exponents: the tile's largest row exponent per row and
            // column exponent per column (precomputed, or from the terms)
            int rmax, cmaxl;
            if (rmaxt) {
                rmax = rmaxt[(long long)tile * M + row];
                cmaxl = myj < nrhs ? cmaxt[(long long)tile * nrhs + myj] : 0;
            } else {
                rmax = cmaxl = -100000;
                for (int q = q0; q < q1; ++q) {
                    const XTerm &tt = terms[q];
                    rmax = max(rmax, aexp[tt.aexp + row]);
                    if (myj < nrhs) cmaxl = max(cmaxl, tt.src == 0 ? texp[(long long)tt.blk * nrhs + myj] : xexp[myj]);
                }
                if (rmax < -99999) rmax = 0;
                if (cmaxl < -99999) cmaxl = 0;
            }
            __int128 acc[CPW];
#pragma unroll
            for (int c = 0; c < CPW; ++c) acc[c] = 0;
            bool ok = true;
            // a term's shifts and depth, loaded one term ahead of its read-out
            auto shifts = [&](int q, int &rd, int &cd, int &kbs) {
                const XTerm tt = terms[q];
                kbs = nkb_of(tt.K);
                rd = aexp[tt.aexp + row] - rmax + 109 - 7 * D;
                cd = (myj < nrhs ? (tt.src == 0 ? texp[(long long)tt.blk * nrhs + myj] : xexp[myj]) : 0) - cmaxl;
            };
            int rdel = 0, cdl = 0, nkb = 0;
            if (q0 < q1) shifts(q0, rdel, cdl, nkb);
            for (int q = q0; q < q1 && ok; ++q) {
                int rdn = 0, cdn = 0, nkbn = 0;
                if (q + 1 < q1) shifts(q + 1, rdn, cdn, nkbn);
                for (int kb0 = 0; kb0 < nkb; kb0 += RANGE) {
                    if (!wait_bar(ctl, &ctl.accf, (uint32_t)(ec & 1))) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    if (j0 < nrhs) {             // warps past the last column only release
#pragma unroll
                        for (int c4 = 0; c4 < C4N; ++c4) {
                            __int128 W[4];
                            read4<D>(trow, c4, W);
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                const int sh = rdel + __shfl_sync(0xffffffffu, cdl, c4 * 4 + u);
                                acc[c4 * 4 + u] += ashift(W[u], sh);
                            }
                        }
                    }
                    fence_before();
                    __syncwarp();
                    if (lane == 0) arrive(&ctl.acce);
                    ++ec;
                }
                rdel = rdn;
                cdl = cdn;
                nkb = nkbn;
            }
            if (!ok) break;
            // outputs: fold in +-Bin exactly, round once
            const long long gr = (long long)tile_row0[tile] * rscale + row;
#pragma unroll
            for (int c = 0; c < CPW; ++c) {
                const int j = j0 + c;
                const int cm = __shfl_sync(0xffffffffu, cmaxl, c);
                if (j < nrhs) {
                    const int U = rmax + cm - 109;
                    __int128 v = neg ? -acc[c] : acc[c];
                    double out;
                    if (addb) {
                        const double b = Bin[gr + (long long)j * ldbin];
                        const long long bits = __double_as_longlong(b);
                        int eb = (int)((bits >> 52) & 0x7FF);
                        long long mb = bits & ((1LL << 52) - 1);
                        if (eb == 0x7FF) {
                            out = b + tc::i128_to_double(v, U);
                        } else {
                            if (eb) mb |= 1LL << 52; else eb = 1;
                            const int sb = eb - 1075 - U;
                            if (sb <= 70) {
                                const __int128 bm = ashift((__int128)mb, sb);
                                v += bits < 0 ? -bm : bm;
                                out = tc::i128_to_double(v, U);
                            } else {
                                out = b + tc::i128_to_double(v, U);
                            }
                        }
                    } else {
                        out = tc::i128_to_double(v, U);
                    }
                    Y[gr + (long long)j * ldy] = out;
                }
            }
        }
    }
    teardown<NS, D>(ctl, warp, lane, issued, consumed, err);
}

// ------------------------------------------------------------- panel
// Work unit it = item * njp + jp (pairs of 64-column X tiles adjacent).
template <int NS, int D>
__global__ void __maxnreg__(kRegs)
    panel_kernel(const PItem *__restrict__ items, int nitems, int njp, const bf16 *__restrict__ vpool,
                 long long vstride, const bf16 *__restrict__ xs, long long xstride, int xnjt, int nrhs,
                 __int128 *__restrict__ partials, int *err)
{
    using C = Cfg<NS>;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ Ctl ctl;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    setup<NS, D>(ctl, warp, lane);
    const uint32_t sbase = su32(smem);
    const int nunits = nitems * njp;
    int issued = 0, consumed = 0;

    if (warp == 0) {
        if (lane == 0) {
            for (int u = blockIdx.x; u < nunits && !ctl.abort; u += gridDim.x) {
                const PItem itm = items[u / njp];
                const int jp = u % njp;
                const uint32_t bbytes = (uint32_t)(itm.nr * KB * 2);
                for (int kb = 0; kb < itm.nkb; ++kb) {
                    const int s = issued % C::NST, f = issued / C::NST;
                    if (f > 0 && !wait_bar(ctl, &ctl.empty[s], (uint32_t)((f - 1) & 1))) break;
                    expect_tx(&ctl.full[s], (uint32_t)NS * (TB_A * 2 + bbytes));
                    const uint32_t da = sbase + (uint32_t)(s * C::STAGE), db = da + NS * TB_A * 2;
                    const long long aoff = ((long long)(itm.xrb0 + kb) * xnjt + 2 * jp) * TB_B;   // two 64-row blocks
#pragma unroll 1
                    for (int p = 0; p < NS; ++p) bulk_g2s(da + p * TB_A * 2, xs + p * xstride + aoff, TB_A * 2, &ctl.full[s]);
                    const long long boff = itm.v + (long long)(itm.vrb0 + kb) * itm.nr * KB;
#pragma unroll 1
                    for (int p = 0; p < NS; ++p)
                        bulk_g2s(db + p * bbytes, vpool + p * vstride + boff, bbytes, &ctl.full[s]);
                    ++issued;
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t tmem = ctl.tmem;
            int rc = 0;
            for (int u = blockIdx.x; u < nunits && !ctl.abort; u += gridDim.x) {
                const PItem itm = items[u / njp];
                const uint32_t idesc = idesc_n(itm.nr);
                for (int kb0 = 0; kb0 < itm.nkb && !ctl.abort; kb0 += RANGE) {
                    if (rc > 0 && !wait_bar(ctl, &ctl.acce, (uint32_t)((rc - 1) & 1))) break;
                    const int kb1 = min(itm.nkb, kb0 + RANGE);
                    for (int kb = kb0; kb < kb1; ++kb) {
                        const int s = consumed % C::NST;
                        if (!wait_bar(ctl, &ctl.full[s], (uint32_t)((consumed / C::NST) & 1))) break;
                        fence_after();
                        const uint32_t a0 = sbase + (uint32_t)(s * C::STAGE);
                        issue_stage<NS, D>(tmem, a0, itm.nr, idesc, kb == kb0);
                        commit(&ctl.empty[s]);
                        ++consumed;
                    }
                    if (ctl.abort) break;
                    commit(&ctl.accf);
                    ++rc;
                }
            }
        }
    } else {
        const int lq = warp & 3, ch = (warp - 2) >> 2;
        const uint32_t trow = ctl.tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)(ch * CPW);
        int ec = 0;
        for (int u = blockIdx.x; u < nunits && !ctl.abort; u += gridDim.x) {
            const PItem itm = items[u / njp];
            const int jp = u % njp;
            const int ncol = min(itm.nr, itm.rank - itm.kt);     // live ranks of the tile
            // warps whose right-hand sides or rank columns are all past the
            // live ones only release tensor memory
            const bool live = jp * M + lq * 32 < nrhs && ch * CPW < ncol;
            __int128 acc[CPW];
#pragma unroll
            for (int c = 0; c < CPW; ++c) acc[c] = 0;
            bool ok = true;
            for (int kb0 = 0; kb0 < itm.nkb; kb0 += RANGE) {
                if (!wait_bar(ctl, &ctl.accf, (uint32_t)(ec & 1))) {
                    ok = false;
                    break;
                }
                fence_after();
                // columns past the tile's padded rank hold stale values; they
                // are read (the loads are warp-collective) but never written
                if (live) {
#pragma unroll
                    for (int c4 = 0; c4 < C4N; ++c4) {
                        __int128 W[4];
                        read4<D>(trow, c4, W);
#pragma unroll
                        for (int v = 0; v < 4; ++v) acc[c4 * 4 + v] += W[v];
                    }
                }
                fence_before();
                __syncwarp();
                if (lane == 0) arrive(&ctl.acce);
                ++ec;
            }
            if (!ok) break;
            const int j = jp * M + lq * 32 + lane;                 // right-hand side of this lane
            if (j < nrhs) {
                __int128 *P = partials + itm.p * nrhs + (long long)itm.chunk * itm.rank * nrhs +
                              (long long)j * itm.rank + itm.kt + ch * CPW;
#pragma unroll
                for (int c = 0; c < CPW; ++c)
                    if (ch * CPW + c < ncol) P[c] = acc[c];
            }
        }
    }
    teardown<NS, D>(ctl, warp, lane, issued, consumed, err);
}

}  // namespace tc2
}  // namespace dg
