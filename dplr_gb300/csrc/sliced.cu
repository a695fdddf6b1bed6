// sliced.cu -- exact-slice bf16 tensor-core products for the PLR apply.
//
// R = B - A X computed with every factor and X cut into 8 bf16 slices of
// 7 bits (sliced.cuh explains the representation).  The three phases of
// the FP64 apply (panel, reduce, expand) keep their structure; the inner
// products become sums over slice pairs (p, q), p + q <= D, of bf16 MMAs
// (mma.sync m16n8k16, FP32 accumulate).  Per 64-row stage and per slice
// diagonal d = p + q the FP32 accumulator holds an exact integer, which is
// shifted by 7 (D - d) and added into a 128-bit integer per output.  The
// panel's 128-bit partials are summed exactly, converted to double-double
// and scaled by sig; the expand converts each term to double-double and
// adds terms with error-free two-sums, so the only roundings are the slice
// truncation (below 2^-57 of the row/column scale) and double-double
// arithmetic (2^-106).  That is what lets iterative refinement reach a
// 1e-12 relative residual where an FP64 residual stalls.
#include "sliced.cuh"
#include "factor.cuh"
#include "tcslice.cuh"
#include "tcpipe.cuh"

#include <algorithm>
#include <unordered_map>
#include <climits>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>

namespace dg {

struct Fact;
static int sliced_build_tb(Plan *p, Sliced *S, cudaStream_t st);
template <int NSR>
static int sliced_residual_tb(Plan *p, Sliced *S, int nrhs, const double *X, int ldx, const double *B, int ldb,
                              double *R, int ldr, cudaStream_t st);
template <int NS>
static int mixed_build_tb_t(Plan *p, MixedSliced *M, Fact *F, cudaStream_t st);
template <int NS>
static int mixed_solve_tb(Plan *p, MixedSliced *M, Fact *F, int nrhs, const double *B, int ldb, double *X, int ldx,
                          cudaStream_t st);

constexpr int SK = 64;          // inner-dimension rows per stage
constexpr int SLD = SK + 8;     // padded smem row (bf16 elements)
constexpr int ST = 64;          // output tile (rows x rhs) of one CTA
constexpr int kSThreads = 256;

// ------------------------------------------------------------- helpers

__device__ __forceinline__ uint32_t ld32(const bf16 *p)
{
    return *reinterpret_cast<const uint32_t *>(p);
}

// 16-byte global -> shared copy; zero fill when !valid (src is not read).
__device__ __forceinline__ void cp16(void *smem_dst, const void *gmem_src, bool valid)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    const int sz = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem_src), "r"(sz));
}

__device__ __forceinline__ void cp_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

__device__ __forceinline__ void mma16816(float *c, const uint32_t *a, const uint32_t *b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Exponent e with |x| < 2^e for every x of magnitude <= amax (0 for amax 0).
__device__ __forceinline__ int scale_exp(double amax)
{
    return amax > 0.0 ? ilogb(amax) + 1 : 0;
}

// round(x * 2^sh) as a 64-bit integer, from the bits of x (integer
// arithmetic only; the caller keeps |x| 2^sh below 2^62).
__device__ __forceinline__ long long scaled_int(double x, int sh)
{
    const long long bits = __double_as_longlong(x);
    int ex = (int)((bits >> 52) & 0x7FF);
    long long m = bits & ((1LL << 52) - 1);
    if (ex == 0) {
        if (m == 0) return 0;
        ex = 1;
    } else {
        m |= 1LL << 52;
    }
    const int s = ex - 1075 + sh;        // |x| 2^sh = m 2^s
    long long y;
    if (s >= 0)
        y = m << s;
    else if (s <= -54)
        y = 0;
    else
        y = (m + (1LL << (-s - 1))) >> (-s);
    return bits < 0 ? -y : y;
}

// bf16 bits of a digit a (-128 <= a <= 128, the range of the slices),
// exactly, with full-rate arithmetic: the float 2^23 + 128 + a is built from
// its bit pattern, 2^23 + 128 subtracted, and the float's top 16 bits
// (exact: <= 8 significant bits) kept.
__device__ __forceinline__ uint32_t digit_bits(int a)
{
    const float f = __int_as_float(0x4B000080 + a) - 8388736.0f;
    return __float_as_uint(f) >> 16;
}

// Balanced base-128 digits of y (|y| < 2^(7 NS)): y = sum_p a_p 2^(7 (NS - p)),
// a_p in [-64, 63] for p > 1 and |a_1| <= 128; written as bf16 (exact).
template <int NS>
__device__ __forceinline__ void int_slices(long long y, bf16 *out, long long stride)
{
    int a[NS];
#pragma unroll
    for (int p = NS - 1; p >= 1; --p) {
        const long long d = ((y + 64) & 127) - 64;
        a[p] = (int)d;
        y = (y - d) >> 7;
    }
    a[0] = (int)y;
#pragma unroll
    for (int p = 0; p < NS; ++p) out[p * stride] = __ushort_as_bfloat16((unsigned short)digit_bits(a[p]));
}

// Slices of x with |x| < 2^e: x = 2^e sum_p a_p 2^(-7p) up to 2^(e - 7 NS - 1).
template <int NS>
__device__ __forceinline__ void slice_d(double x, int e, bf16 *out, long long stride)
{
    int_slices<NS>(scaled_int(x, 7 * NS - e), out, stride);
}

// Same for a double-double value hi + lo.
template <int NS>
__device__ __forceinline__ void slice_dd(double hi, double lo, int e, bf16 *out, long long stride)
{
    int_slices<NS>(scaled_int(hi, 7 * NS - e) + scaled_int(lo, 7 * NS - e), out, stride);
}

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e)
{
    s = a + b;
    double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// 128-bit integer -> double-double (exact split of the top 106 bits).
__device__ __forceinline__ void i128_to_dd(__int128 w, double &hi, double &lo)
{
    hi = (double)w;
    lo = (double)(w - (__int128)hi);
}

// w 2^E as double-double with integer arithmetic only: hi = w rounded to 53
// bits (nearest, ties to even), lo = the exact remainder rounded to 53 bits;
// both scaled by 2^E through the exponent field.  GB300's FP64 rate makes
// this much cheaper than the library's 128-bit conversions and ldexp.
__device__ __forceinline__ void i128_to_dd_scaled(__int128 w, int E, double &hi, double &lo)
{
    if (w == 0) {
        hi = lo = 0.0;
        return;
    }
    const bool neg = w < 0;
    const unsigned __int128 a = neg ? (unsigned __int128)(-w) : (unsigned __int128)w;
    const unsigned long long ah = (unsigned long long)(a >> 64), al = (unsigned long long)a;
    const int msb = ah ? 127 - __clzll((long long)ah) : 63 - __clzll((long long)al);
    if (msb <= 52) {
        hi = tc::i128_to_double(w, E);
        lo = 0.0;
        return;
    }
    const int sh = msb - 52;
    unsigned __int128 m = a >> sh;
    const unsigned __int128 rem = a - (m << sh), half = (unsigned __int128)1 << (sh - 1);
    if (rem > half || (rem == half && (m & 1))) ++m;            // may reach 2^53: still exact below
    const __int128 hint = (__int128)(m << sh);                  // |w| rounded, exactly
    const __int128 r = (__int128)a - hint;                      // |r| <= 2^(sh-1)
    hi = tc::i128_to_double(neg ? -hint : hint, E);
    lo = tc::i128_to_double(neg ? -r : r, E);
}

// One warp: 32 x 16 output block (2 x 2 fragments) for one slice pair over
// one SK-row stage; As rows are output rows (m), Bs rows are output columns.
__device__ __forceinline__ void warp_pair(float (&acc)[2][2][4], const bf16 *As, const bf16 *Bs,
                                          int m0, int n0, int lane)
{
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int ks = 0; ks < SK; ks += 16) {
        uint32_t a[2][4], b[2][2];
#pragma unroll
        for (int fm = 0; fm < 2; ++fm) {
            const bf16 *r0 = As + (m0 + fm * 16 + g) * SLD + ks + 2 * t;
            const bf16 *r1 = r0 + 8 * SLD;
            a[fm][0] = ld32(r0);
            a[fm][1] = ld32(r1);
            a[fm][2] = ld32(r0 + 8);
            a[fm][3] = ld32(r1 + 8);
        }
#pragma unroll
        for (int fn = 0; fn < 2; ++fn) {
            const bf16 *c0 = Bs + (n0 + fn * 8 + g) * SLD + ks + 2 * t;
            b[fn][0] = ld32(c0);
            b[fn][1] = ld32(c0 + 8);
        }
#pragma unroll
        for (int fm = 0; fm < 2; ++fm)
#pragma unroll
            for (int fn = 0; fn < 2; ++fn) mma16816(acc[fm][fn], a[fm], b[fn]);
    }
}

// All slice pairs of one stage, diagonal by diagonal, flushed exactly.
template <int NSA, int NSB, int DMAX>
__device__ __forceinline__ void stage_products(__int128 (&W)[2][2][4], const bf16 *As,
                                               const bf16 *Bs, int m0, int n0, int lane)
{
#pragma unroll 1
    for (int d = 2; d <= DMAX; ++d) {
        float acc[2][2][4];
#pragma unroll
        for (int fm = 0; fm < 2; ++fm)
#pragma unroll
            for (int fn = 0; fn < 2; ++fn)
#pragma unroll
                for (int i = 0; i < 4; ++i) acc[fm][fn][i] = 0.0f;
        const int plo = d - NSB > 1 ? d - NSB : 1, phi = d - 1 < NSA ? d - 1 : NSA;
#pragma unroll 1
        for (int p = plo; p <= phi; ++p)
            warp_pair(acc, As + (p - 1) * ST * SLD, Bs + (d - p - 1) * ST * SLD, m0, n0, lane);
        const int sh = 7 * (DMAX - d);
#pragma unroll
        for (int fm = 0; fm < 2; ++fm)
#pragma unroll
            for (int fn = 0; fn < 2; ++fn)
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    W[fm][fn][i] += ((__int128)__float2ll_rn(acc[fm][fn][i])) << sh;
    }
}

// ----------------------------------------------------------- slicing kernels

struct SliceJob {
    long long off;     // source element offset of the matrix (column-major, ld)
    long long doff;    // destination element offset (column-major, same ld)
    int ld, rows, cols;
    int exp;           // offset of the exponents
};

// Column slicing (one exponent per column): one CTA per (job, column).
template <int NS>
__global__ void slice_cols_kernel(const SliceJob *jobs, const int *col_base, int njobs,
                                  const double *src, bf16 *dst, long long stride, int *exps)
{
    __shared__ double red[256];
    // locate job: col_base is the prefix of columns over jobs
    const int gc = blockIdx.x;
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) / 2;
        if (col_base[mid] <= gc) lo = mid; else hi = mid - 1;
    }
    const SliceJob J = jobs[lo];
    const int c = gc - col_base[lo];
    const double *col = src + J.off + (long long)c * J.ld;
    double m = 0.0;
    for (int i = threadIdx.x; i < J.rows; i += blockDim.x) m = fmax(m, fabs(col[i]));
    red[threadIdx.x] = m;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + k]);
        __syncthreads();
    }
    const int e = scale_exp(red[0]);
    if (threadIdx.x == 0) exps[J.exp + c] = e;
    for (int i = threadIdx.x; i < J.rows; i += blockDim.x) {
        long long o = J.doff + (long long)c * J.ld + i;
        slice_d<NS>(col[i], e, dst + o, stride);
    }
}

// Row slicing (one exponent per row): one thread per (job, row); the
// slices are written row-major with row stride `dld` (>= cols, multiple
// of 8, zero padded) starting at element `doff` of the job.
struct RowSliceJob {
    long long off;     // source element offset (column-major, ld)
    long long doff;    // destination element offset (row-major, stride dld)
    int ld, rows, cols, dld;
    int exp;
};

template <int NS>
__global__ void slice_rows_kernel(const RowSliceJob *jobs, const int *row_base, int njobs, int total,
                                  const double *src, bf16 *dst, long long stride, int *exps)
{
    const int gr = blockIdx.x * blockDim.x + threadIdx.x;
    if (gr >= total) return;
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) / 2;
        if (row_base[mid] <= gr) lo = mid; else hi = mid - 1;
    }
    const RowSliceJob J = jobs[lo];
    const int r = gr - row_base[lo];
    double m = 0.0;
    for (int k = 0; k < J.cols; ++k) m = fmax(m, fabs(src[J.off + r + (long long)k * J.ld]));
    const int e = scale_exp(m);
    exps[J.exp + r] = e;
    const bf16 zero = __float2bfloat16(0.0f);
    for (int k = 0; k < J.dld; ++k) {
        bf16 *o = dst + J.doff + (long long)r * J.dld + k;
        if (k < J.cols) {
            slice_d<NS>(src[J.off + r + (long long)k * J.ld], e, o, stride);
        } else {
#pragma unroll
            for (int p = 0; p < NS; ++p) o[p * stride] = zero;
        }
    }
}

// Right-hand sides: one exponent per column over all rows.  Each column is
// split over gridDim.y CTAs whose exponents meet in an integer atomicMax
// (exponent of the maximum = maximum of the exponents); CTAs whose part is
// zero contribute nothing, and a column that stays at the initial value is
// all zero and gets exponent 0.
constexpr int kNoExp = -(1 << 24);

__global__ void xcol_init_kernel(int *xexp, int nrhs)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < nrhs) xexp[j] = kNoExp;
}

__global__ void xcol_exp_kernel(const double *__restrict__ X, int m, int ldx, int *xexp)
{
    __shared__ double red[256];
    const double *col = X + (long long)blockIdx.x * ldx;
    const int per = (m + gridDim.y - 1) / gridDim.y;
    const int r0 = blockIdx.y * per, r1 = min(m, r0 + per);
    double v = 0.0;
    int i = r0 + threadIdx.x;
    for (; i + 7 * 256 < r1; i += 8 * 256) {        // 8 independent loads in flight
        double x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) x[u] = col[i + u * 256];
#pragma unroll
        for (int u = 0; u < 8; ++u) v = fmax(v, fabs(x[u]));
    }
    for (; i < r1; i += 256) v = fmax(v, fabs(col[i]));
    red[threadIdx.x] = v;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + k]);
        __syncthreads();
    }
    if (threadIdx.x == 0 && red[0] > 0.0) atomicMax(xexp + blockIdx.x, scale_exp(red[0]));
}

__global__ void xcol_fix_kernel(int *xexp, int nrhs)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < nrhs && xexp[j] == kNoExp) xexp[j] = 0;       // all-zero column
}

// Column exponents of an m x nrhs block: 16 CTAs per column.
static void xcol_exps(const double *X, int m, int ldx, int nrhs, int *xexp, cudaStream_t st)
{
    xcol_init_kernel<<<(nrhs + 255) / 256, 256, 0, st>>>(xexp, nrhs);
    note_launch();
    const int parts = std::max(1, std::min(16, m / 4096));
    xcol_exp_kernel<<<dim3((unsigned)nrhs, (unsigned)parts), 256, 0, st>>>(X, m, ldx, xexp);
    note_launch();
    xcol_fix_kernel<<<(nrhs + 255) / 256, 256, 0, st>>>(xexp, nrhs);
    note_launch();
}

// One column per blockIdx.y, rows strided over the x-blocks.
template <int NS>
__global__ void xslice_kernel(const double *X, int m, int ldx, int nrhs, const int *xexp, bf16 *xs,
                              long long stride)
{
    for (int j = blockIdx.y; j < nrhs; j += gridDim.y) {
        const int e = xexp[j];
        const double *col = X + (long long)j * ldx;
        bf16 *out = xs + (long long)j * m;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
            slice_d<NS>(col[i], e, out + i, stride);
    }
}

static dim3 xslice_grid(int m, int nrhs)
{
    return dim3((unsigned)std::max(1, std::min((m + 1023) / 1024, 64)), (unsigned)std::min(nrhs, 65535));
}

// ------------------------------------------------------------- products

// Panel: W = F[rows]^T X[rows] for one (item, rhs tile), exact 128-bit sums.
// F slices are column-major (ld n), X slices column-major (ld ldx); rows of
// a stage are contiguous in both, so stages are staged with 16-byte
// cp.async copies.  Block sizes and chunk offsets are multiples of 64.
template <int NSA, int NSB, int DMAX>
__global__ void __launch_bounds__(kSThreads) sp_panel_kernel(
    const SPanelItem *__restrict__ items, const bf16 *__restrict__ apool, long long astride,
    const bf16 *__restrict__ xs, long long xstride, int ldx, int nrhs, __int128 *__restrict__ partials)
{
    extern __shared__ __align__(16) unsigned char smem[];
    bf16 *As = reinterpret_cast<bf16 *>(smem);          // [NSA][ST][SLD]
    bf16 *Bs = As + NSA * ST * SLD;                      // [NSB][ST][SLD]
    const SPanelItem it = items[blockIdx.x];
    const int j0 = blockIdx.y * ST;
    const int nj = min(ST, nrhs - j0);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m0 = (warp >> 2) * 32, n0 = (warp & 3) * 16;
    const int g = lane >> 2, t = lane & 3;
    __int128 *P = partials + it.p * nrhs + (long long)it.chunk * it.rank * nrhs;

    for (int kt = 0; kt < it.rank; kt += ST) {
        const int nk = min(ST, it.rank - kt);
        __int128 W[2][2][4];
#pragma unroll
        for (int fm = 0; fm < 2; ++fm)
#pragma unroll
            for (int fn = 0; fn < 2; ++fn)
#pragma unroll
                for (int i = 0; i < 4; ++i) W[fm][fn][i] = 0;
        for (int s0 = 0; s0 < it.len; s0 += SK) {
            __syncthreads();
            // 8-element chunks: (slice, row-of-tile, chunk of 8 along the stage)
            for (int e = tid; e < NSA * ST * (SK / 8); e += kSThreads) {
                const int c = e % (SK / 8), m = (e / (SK / 8)) % ST, p = e / ((SK / 8) * ST);
                const bool ok = m < nk;
                const bf16 *src = apool + p * astride + it.f + (long long)(it.r0 + s0 + c * 8) +
                                  (long long)(kt + (ok ? m : 0)) * it.n;
                cp16(As + (p * ST + m) * SLD + c * 8, src, ok);
            }
            for (int e = tid; e < NSB * ST * (SK / 8); e += kSThreads) {
                const int c = e % (SK / 8), n = (e / (SK / 8)) % ST, q = e / ((SK / 8) * ST);
                const bool ok = n < nj;
                const bf16 *src = xs + q * xstride + (long long)(it.in0 + it.r0 + s0 + c * 8) +
                                  (long long)(j0 + (ok ? n : 0)) * ldx;
                cp16(Bs + (q * ST + n) * SLD + c * 8, src, ok);
            }
            cp_wait_all();
            __syncthreads();
            stage_products<NSA, NSB, DMAX>(W, As, Bs, m0, n0, lane);
        }
#pragma unroll
        for (int fm = 0; fm < 2; ++fm)
#pragma unroll
            for (int fn = 0; fn < 2; ++fn)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int m = m0 + fm * 16 + g + (i >= 2 ? 8 : 0);
                    const int n = n0 + fn * 8 + 2 * t + (i & 1);
                    if (m < nk && n < nj) P[(kt + m) + (long long)(j0 + n) * it.rank] = W[fm][fn][i];
                }
    }
}

// Reduce: T = sig o 2^(E) sum_c W_c as double-double.
// T = sig o (sum over chunks of the 128-bit partials), as double-double.
// One thread per element of the schedule's concatenated element space:
// item i owns [rsum_i nrhs, (rsum_i + rank_i) nrhs), its element e = k + j
// rank; the item is found by binary search on rsum (no idle CTAs whatever
// the ranks), and the chunk sums run four loads deep (integer sums, so the
// order does not change the result).
template <int DMAX>
__global__ void sp_reduce_kernel(const SReduceItem *__restrict__ items, const int *__restrict__ rank_item,
                                 long long total,
                                 const __int128 *__restrict__ partials, const int *__restrict__ aexp,
                                 const int *__restrict__ xexp, const double *__restrict__ sigbase,
                                 int nrhs, double *__restrict__ T, long long lo_off)
{
    const long long E = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (E >= total) return;
    // the item from the rank-position table (element E sits at position
    // E / nrhs); the element within the item costs one 32-bit division
    // (rank * nrhs of one item stays below 2^31)
    const SReduceItem R = items[rank_item[E / nrhs]];
    const long long cnt = (long long)R.rank * nrhs;
    const int e = (int)(E - (long long)R.rsum * nrhs);
    const int j = e / R.rank, k = e - j * R.rank;
    const __int128 *P = partials + R.p * nrhs + e;
    __int128 W0 = 0, W1 = 0, W2 = 0, W3 = 0;
    int c = 0;
    for (; c + 3 < R.nch; c += 4) {
        W0 += P[(long long)c * cnt];
        W1 += P[(long long)(c + 1) * cnt];
        W2 += P[(long long)(c + 2) * cnt];
        W3 += P[(long long)(c + 3) * cnt];
    }
    for (; c < R.nch; ++c) W0 += P[(long long)c * cnt];
    const __int128 W = (W0 + W1) + (W2 + W3);
    double hi2, lo2;
    i128_to_dd_scaled(W, aexp[R.fexp + k] + xexp[j] - 7 * DMAX, hi2, lo2);
    if (R.sig >= 0) {
        // (hi2 + lo2) s as double-double: exact product of hi2, |l2| << |pr|
        const double s = sigbase[R.sig + k];
        const double pr = hi2 * s;
        const double l2 = fma(lo2, s, fma(hi2, s, -pr));
        hi2 = pr + l2;
        lo2 = l2 - (hi2 - pr);
    }
    T[R.t * nrhs + e] = hi2;
    T[lo_off + R.t * nrhs + e] = lo2;
}

template <int DMAX>
static void launch_reduce(const SSchedule &S, const __int128 *partials, const int *aexp, const int *xexp,
                          const double *sigbase, int nrhs, double *T, long long lo_off, cudaStream_t st)
{
    const long long total = (long long)S.rtotal * nrhs;
    if (S.reduces.empty() || total == 0) return;
    sp_reduce_kernel<DMAX><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(
        S.d_reduces, S.d_rank_item, total, partials, aexp, xexp, sigbase, nrhs, T, lo_off);
    note_launch();
}

// Slices of the double-double panel results, one exponent per (block,
// column) over the block's rank rows; one warp per (block, column).  Rows
// [rank, rp) of the slice panel are zero.
template <int NS>
__global__ void sp_tslice_kernel(const SReduceItem *__restrict__ items, int nitems,
                                 const double *__restrict__ T, long long lo_off, int nrhs,
                                 bf16 *__restrict__ ts, long long tstride, int *__restrict__ texp)
{
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (long long)nitems * nrhs) return;
    const int b = (int)(w / nrhs), j = (int)(w % nrhs);
    const SReduceItem R = items[b];
    const double *th = T + R.t * nrhs + (long long)j * R.rank;
    const double *tl = lo_off >= 0 ? th + lo_off : nullptr;
    double mx = 0.0;
    for (int k = lane; k < R.rank; k += 32) mx = fmax(mx, fabs(th[k]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const int e = scale_exp(mx);
    if (lane == 0) texp[(long long)b * nrhs + j] = e;
    bf16 *out = ts + R.tpad * nrhs + (long long)j * R.rp;
    const bf16 zero = __float2bfloat16(0.0f);
    for (int k = lane; k < R.rp; k += 32) {
        if (k < R.rank) {
            slice_dd<NS>(th[k], tl ? tl[k] : 0.0, e, out + k, tstride);
        } else {
#pragma unroll
            for (int p = 0; p < NS; ++p) out[k + p * tstride] = zero;
        }
    }
}

// Expand: Y = alpha * sum_terms A_t B_t + beta * Bin over one 64-row tile.
// A slices are row-major (row stride lda, zero padded to a multiple of 8),
// B is either the T-slice panel of a block (ld ldb = padded rank) or the X
// slices (leaf terms); everything is staged with 16-byte cp.async copies.
template <int NSA, int NSB, int DMAX>
__global__ void __launch_bounds__(kSThreads) sp_expand_kernel(
    const STerm *__restrict__ terms, const int *__restrict__ tile_row0,
    const int *__restrict__ tile_begin, const bf16 *__restrict__ apool, long long astride,
    const int *__restrict__ aexp, const bf16 *__restrict__ ts, long long tstride,
    const int *__restrict__ texp, const bf16 *__restrict__ xs, long long xstride, int ldx,
    const int *__restrict__ xexp, int nrhs, double alpha, const double *__restrict__ Bin,
    int ldbin, double beta, double *__restrict__ Y, int ldy)
{
    extern __shared__ __align__(16) unsigned char smem[];
    bf16 *As = reinterpret_cast<bf16 *>(smem);          // [NSA][ST][SLD]
    bf16 *Bs = As + NSA * ST * SLD;                      // [NSB][ST][SLD]
    __shared__ int rexp[ST], cexp[ST];
    const int tile = blockIdx.x;
    const int row0 = tile_row0[tile];
    const int j0 = blockIdx.y * ST;
    const int nj = min(ST, nrhs - j0);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m0 = (warp >> 2) * 32, n0 = (warp & 3) * 16;
    const int g = lane >> 2, t = lane & 3;

    double acch[2][2][4], accl[2][2][4];
#pragma unroll
    for (int fm = 0; fm < 2; ++fm)
#pragma unroll
        for (int fn = 0; fn < 2; ++fn)
#pragma unroll
            for (int i = 0; i < 4; ++i) acch[fm][fn][i] = accl[fm][fn][i] = 0.0;

    for (int q = tile_begin[tile]; q < tile_begin[tile + 1]; ++q) {
        const STerm tt = terms[q];
        __syncthreads();
        if (tid < ST) {
            rexp[tid] = aexp[tt.aexp + tid];
            cexp[tid] = tid < nj ? (tt.src == 0 ? texp[(long long)tt.blk * nrhs + j0 + tid]
                                               : xexp[j0 + tid])
                                 : 0;
        }
        __int128 W[2][2][4];
#pragma unroll
        for (int fm = 0; fm < 2; ++fm)
#pragma unroll
            for (int fn = 0; fn < 2; ++fn)
#pragma unroll
                for (int i = 0; i < 4; ++i) W[fm][fn][i] = 0;
        const int Kp = (tt.K + 7) & ~7;          // stored (zero padded) columns of A / rows of B
        for (int k0 = 0; k0 < tt.K; k0 += SK) {
            __syncthreads();
            for (int e = tid; e < NSA * ST * (SK / 8); e += kSThreads) {
                const int c = e % (SK / 8), m = (e / (SK / 8)) % ST, p = e / ((SK / 8) * ST);
                const bool ok = k0 + c * 8 < Kp;
                const bf16 *src = apool + p * astride + tt.a + (long long)m * tt.lda + (ok ? k0 + c * 8 : 0);
                cp16(As + (p * ST + m) * SLD + c * 8, src, ok);
            }
            for (int e = tid; e < NSB * ST * (SK / 8); e += kSThreads) {
                const int c = e % (SK / 8), n = (e / (SK / 8)) % ST, q2 = e / ((SK / 8) * ST);
                const bool ok = n < nj && k0 + c * 8 < Kp;
                const bf16 *src;
                if (tt.src == 0)
                    src = ts + q2 * tstride + tt.b * nrhs + (long long)(j0 + (ok ? n : 0)) * tt.ldb +
                          (ok ? k0 + c * 8 : 0);
                else
                    src = xs + q2 * xstride + (long long)(tt.x_row0 + (ok ? k0 + c * 8 : 0)) +
                          (long long)(j0 + (ok ? n : 0)) * ldx;
                cp16(Bs + (q2 * ST + n) * SLD + c * 8, src, ok);
            }
            cp_wait_all();
            __syncthreads();
            stage_products<NSA, NSB, DMAX>(W, As, Bs, m0, n0, lane);
        }
        // term -> double-double, accumulated with error-free sums
#pragma unroll
        for (int fm = 0; fm < 2; ++fm)
#pragma unroll
            for (int fn = 0; fn < 2; ++fn)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int m = m0 + fm * 16 + g + (i >= 2 ? 8 : 0);
                    const int n = n0 + fn * 8 + 2 * t + (i & 1);
                    double h, l;
                    i128_to_dd(W[fm][fn][i], h, l);
                    const int E = rexp[m] + cexp[n] - 7 * DMAX;
                    h = ldexp(h, E);
                    l = ldexp(l, E);
                    double s2, e2;
                    two_sum(acch[fm][fn][i], h, s2, e2);
                    acch[fm][fn][i] = s2;
                    accl[fm][fn][i] += e2 + l;
                }
    }
#pragma unroll
    for (int fm = 0; fm < 2; ++fm)
#pragma unroll
        for (int fn = 0; fn < 2; ++fn)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int m = m0 + fm * 16 + g + (i >= 2 ? 8 : 0);
                const int n = n0 + fn * 8 + 2 * t + (i & 1);
                if (n >= nj) continue;
                const double ah = alpha * acch[fm][fn][i], al = alpha * accl[fm][fn][i];
                double out;
                if (beta == 0.0) {
                    out = ah + al;
                } else {
                    const double b0 = beta * Bin[row0 + m + (long long)(j0 + n) * ldbin];
                    double s2, e2;
                    two_sum(b0, ah, s2, e2);
                    out = s2 + (e2 + al);
                }
                Y[row0 + m + (long long)(j0 + n) * ldy] = out;
            }
}

// ------------------------------------------------------------- host side

constexpr int kNS = 8;      // slices of the FP64-accurate products
constexpr int kD = 9;       // keep pairs p + q <= 9

static long long al32(long long x) { return (x + 31) & ~31LL; }
static int pad8(int x) { return (x + 7) & ~7; }

// Expand tile height: 128 rows on the tcgen05 kernels when every leaf is a
// multiple of 128 rows and no rank exceeds 256, else 64 rows on the
// mma.sync kernels.
// DPLR_GB300_SLICED_MMA=1 selects the mma.sync kernels everywhere.
static int sliced_tile_rows(const Plan *p)
{
    const char *env = std::getenv("DPLR_GB300_SLICED_MMA");
    if (env && env[0] == '1') return ST;
    for (const LeafDesc &L : p->leaves)
        if (L.b % tc::M != 0 || L.row0 % tc::M != 0) return ST;
    if (p->max_rank > 256) return ST;         // the tile-block layouts hold at most 4 rank tiles of 64
    return tc::M;
}

// The tcgen05 residual also takes leaves and blocks smaller than a tile
// when each lies inside one 128-row tile (n divides 128, rows aligned to n):
// they are stored as 128-row tile-blocks whose other rows are zero.
static bool fits_tile(int n, int row0)
{
    if (n % tc::M == 0) return row0 % tc::M == 0;
    return n % 16 == 0 && tc::M % n == 0 && row0 % n == 0;
}

static int resid_tile_rows(const Plan *p)
{
    const char *env = std::getenv("DPLR_GB300_SLICED_MMA");
    if (env && env[0] == '1') return ST;
    if (p->m % tc::M != 0 || p->max_rank > 256) return ST;
    for (const LeafDesc &L : p->leaves)
        if (!fits_tile(L.b, L.row0)) return ST;
    for (const LRDesc &L : p->lr)
        if (L.rank > 0 && !fits_tile(L.n, L.row0)) return ST;
    return tc::M;
}

int ensure_err_flag(Plan *p)
{
    if (p->tc_err_h) return 0;
    if (cudaHostAlloc((void **)&p->tc_err_h, sizeof(int), cudaHostAllocMapped) != cudaSuccess)
        return fail(DPLR_GPU_ENOMEM, "sliced products: cannot allocate the error flag");
    *p->tc_err_h = 0;
    if (cudaHostGetDevicePointer((void **)&p->tc_err_d, p->tc_err_h, 0) != cudaSuccess)
        return fail(DPLR_GPU_ECUDA, "sliced products: cannot map the error flag");
    return 0;
}

int set_wait_limit(int spins)
{
    const int v = spins > 0 ? spins : tc2::kSpin;
    DG_CUDA(cudaMemcpyToSymbol(tc2::g_wait_limit, &v, sizeof(int)));
    return 0;
}

int sliced_error(Plan *p)
{
    if (!p->tc_err_h) return 0;
    volatile int *f = p->tc_err_h;
    if (*f == 0) return 0;
    *f = 0;
    return fail(DPLR_GPU_ECUDA, "tensor-core slice product: a bounded wait expired");
}

// Panel launch of a schedule (mma.sync kernel; 16-row tiles).
template <int NS, int D>
static void launch_panel(const Plan *p, const SSchedule &S, const bf16 *apool, long long astride, const bf16 *xs,
                         long long xstride, int ldx, int nrhs, __int128 *partials, cudaStream_t st)
{
    const unsigned rt = (unsigned)((nrhs + ST - 1) / ST);
    sp_panel_kernel<NS, NS, D><<<dim3((unsigned)S.items.size(), rt), kSThreads,
                                 (size_t)(2 * NS) * ST * SLD * sizeof(bf16), st>>>(
        S.d_items, apool, astride, xs, xstride, ldx, nrhs, partials);
    note_launch();
}

// Expand launch of a schedule: Y = -/+ sum terms (+ Bin) (mma.sync kernel).
template <int NS, int D>
static void launch_expand(const Plan *p, const SSchedule &S, const bf16 *apool, long long astride, const int *aexp,
                          const bf16 *ts, long long tstride, const int *texp, const bf16 *xs, long long xstride,
                          int ldx, const int *xexp, int nrhs, bool neg, const double *Bin, int ldbin, bool addb,
                          double *Y, int ldy, cudaStream_t st)
{
    const unsigned ntiles = (unsigned)S.tile_row0.size();
    const unsigned rt = (unsigned)((nrhs + ST - 1) / ST);
    sp_expand_kernel<NS, NS, D><<<dim3(ntiles, rt), kSThreads, (size_t)(2 * NS) * ST * SLD * sizeof(bf16), st>>>(
        S.d_terms, S.d_tile_row0, S.d_tile_begin, apool, astride, aexp, ts, tstride, texp, xs, xstride, ldx,
        xexp, nrhs, neg ? -1.0 : 1.0, Bin, ldbin, addb ? 1.0 : 0.0, Y, ldy);
    note_launch();
}

template <class T>
static int dev_vec(const std::vector<T> &v, T **dst, long long *bytes)
{
    DG_ALLOC(dst, std::max<size_t>(v.size(), 1) * sizeof(T));
    *bytes += (long long)(std::max<size_t>(v.size(), 1) * sizeof(T));
    if (!v.empty()) DG_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

static void free_sschedule(SSchedule &A)
{
    cudaFree(A.d_pitems);
    cudaFree(A.d_xterms);
    cudaFree(A.d_rmax);
    A.d_pitems = nullptr;
    A.d_xterms = nullptr;
    A.d_rmax = nullptr;
    cudaFree(A.d_items);
    cudaFree(A.d_reduces);
    cudaFree(A.d_rank_item);
    A.d_rank_item = nullptr;
    cudaFree(A.d_tile_row0);
    cudaFree(A.d_tile_begin);
    cudaFree(A.d_terms);
    A.d_items = nullptr;
    A.d_reduces = nullptr;
    A.d_tile_row0 = A.d_tile_begin = nullptr;
    A.d_terms = nullptr;
}

void sliced_free(Plan *p)
{
    Sliced *S = (Sliced *)p->sliced;
    if (!S) return;
    cudaFree(S->pool);
    cudaFree(S->exps);
    free_sschedule(S->apply);
    cudaFree(S->xs);
    cudaFree(S->xexp);
    cudaFree(S->work);
    delete S;
    p->sliced = nullptr;
}

static size_t panel_smem(int nsa, int nsb) { return (size_t)(nsa + nsb) * ST * SLD * sizeof(bf16); }

// The reduce's element space: item i owns the rank positions [rsum_i,
// rsum_i + rank_i); the table maps each position to its item, so that a
// reduce thread finds its item with one load (element E is at position
// E / nrhs).
static int upload_rank_items(SSchedule &A, long long *bytes)
{
    A.rtotal = 0;
    std::vector<int> owner;
    for (size_t i = 0; i < A.reduces.size(); ++i) {
        SReduceItem &r = A.reduces[i];
        r.rsum = A.rtotal;
        A.rtotal += r.rank;
        owner.insert(owner.end(), r.rank, (int)i);
    }
    return dev_vec(owner, &A.d_rank_item, bytes);
}

static int upload_sschedule(SSchedule &A, long long *bytes)
{
    int rc;
    if ((rc = upload_rank_items(A, bytes))) return rc;
    if ((rc = dev_vec(A.items, &A.d_items, bytes)) || (rc = dev_vec(A.reduces, &A.d_reduces, bytes)) ||
        (rc = dev_vec(A.tile_row0, &A.d_tile_row0, bytes)) ||
        (rc = dev_vec(A.tile_begin, &A.d_tile_begin, bytes)) || (rc = dev_vec(A.terms, &A.d_terms, bytes)))
        return rc;
    return 0;
}

int sliced_build(Plan *p, int ns, cudaStream_t st)
{
    sliced_free(p);
    if (ns != kNS) return fail(DPLR_GPU_EINVAL, "sliced products: %d slices not built", ns);
    for (const LeafDesc &L : p->leaves)
        if (L.b % ST != 0 || L.row0 % ST != 0)
            return fail(DPLR_GPU_EINVAL, "sliced products need leaf sizes that are multiples of %d", ST);
    Sliced *S = new Sliced();
    p->sliced = S;
    S->ns = ns;
    if (resid_tile_rows(p) == tc::M) return sliced_build_tb(p, S, st);

    // layout: V column-major (ld n), U row-major (stride pad8(rank)), leaves row-major
    std::vector<long long> vs_off(p->lr.size()), us_off(p->lr.size()), ds_off(p->leaves.size());
    std::vector<int> ev_off(p->lr.size()), eu_off(p->lr.size()), ed_off(p->leaves.size());
    std::vector<SliceJob> vj;
    std::vector<RowSliceJob> uj;
    std::vector<int> vbase, ubase;
    long long el = 0;
    int nexp = 0, ncols = 0, nrows = 0;
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        const int rp = pad8(L.rank);
        vs_off[b] = el;
        el += al32((long long)L.n * L.rank);
        us_off[b] = el;
        el += al32((long long)L.n * rp);
        ev_off[b] = nexp;
        nexp += L.rank;
        eu_off[b] = nexp;
        nexp += L.n;
        if (L.rank == 0) continue;
        vbase.push_back(ncols);
        vj.push_back(SliceJob{L.v, vs_off[b], L.n, L.n, L.rank, ev_off[b]});
        ncols += L.rank;
        ubase.push_back(nrows);
        uj.push_back(RowSliceJob{L.u, us_off[b], L.n, L.n, L.rank, rp, eu_off[b]});
        nrows += L.n;
    }
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        const LeafDesc &L = p->leaves[i];
        ds_off[i] = el;
        el += al32((long long)L.b * L.b);
        ed_off[i] = nexp;
        nexp += L.b;
        ubase.push_back(nrows);
        uj.push_back(RowSliceJob{L.d, ds_off[i], L.b, L.b, L.b, L.b, ed_off[i]});
        nrows += L.b;
    }
    S->stride = al32(std::max<long long>(el, 1));
    cudaError_t e = dev_malloc((void **)&S->pool, (size_t)ns * S->stride * sizeof(bf16));
    if (e != cudaSuccess) return fail(DPLR_GPU_ENOMEM, "sliced products: cannot allocate slices");
    S->bytes += (long long)ns * S->stride * 2;
    S->nexp = nexp;
    int rc;
    if ((rc = dev_vec(std::vector<int>(std::max(nexp, 1), 0), &S->exps, &S->bytes))) return rc;
    {
        SliceJob *d_vj = nullptr;
        RowSliceJob *d_uj = nullptr;
        int *d_vb = nullptr, *d_ub = nullptr;
        long long tmp = 0;
        if ((rc = dev_vec(vj, &d_vj, &tmp)) || (rc = dev_vec(vbase, &d_vb, &tmp)) ||
            (rc = dev_vec(uj, &d_uj, &tmp)) || (rc = dev_vec(ubase, &d_ub, &tmp)))
            return rc;
        if (ncols > 0) {
            slice_cols_kernel<kNS><<<ncols, 256, 0, st>>>(d_vj, d_vb, (int)vj.size(), p->pool, S->pool,
                                                          S->stride, S->exps);
            note_launch();
        }
        if (nrows > 0) {
            slice_rows_kernel<kNS><<<(nrows + 127) / 128, 128, 0, st>>>(
                d_uj, d_ub, (int)uj.size(), nrows, p->pool, S->pool, S->stride, S->exps);
            note_launch();
        }
        cudaError_t e2 = cudaGetLastError();
        if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(st);
        cudaFree(d_vj);
        cudaFree(d_uj);
        cudaFree(d_vb);
        cudaFree(d_ub);
        if (e2 != cudaSuccess) return fail(DPLR_GPU_ECUDA, "slicing: %s", cudaGetErrorString(e2));
    }

    // op-N schedule
    SSchedule &A = S->apply;
    const int CH = 1024;
    long long poff = 0, tpad = 0;
    std::vector<int> ridx(p->lr.size(), -1);
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        if (L.rank == 0) continue;
        int nch = (L.n + CH - 1) / CH;
        for (int c = 0; c < nch; ++c) {
            SPanelItem it;
            it.f = vs_off[b];
            it.p = poff;
            it.n = L.n;
            it.rank = L.rank;
            it.in0 = L.col0;
            it.r0 = c * CH;
            it.len = std::min(CH, L.n - c * CH);
            it.chunk = c;
            A.items.push_back(it);
        }
        ridx[b] = (int)A.reduces.size();
        A.reduces.push_back(SReduceItem{poff, L.toff, L.sig, L.rank, nch, ev_off[b], pad8(L.rank), tpad});
        poff += (long long)nch * L.rank;
        tpad += pad8(L.rank);
        A.max_rank = std::max(A.max_rank, L.rank);
    }
    A.partial_per_rhs = poff;
    A.t_per_rhs = p->total_rank;
    A.tpad_per_rhs = tpad;
    const int TM = A.tile_m = sliced_tile_rows(p);
    const int ntiles = p->m / TM;
    std::vector<std::vector<STerm>> per(ntiles);
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        if (L.rank == 0) continue;
        const int rp = pad8(L.rank);
        for (int t0 = L.row0; t0 < L.row0 + L.n; t0 += TM) {
            STerm tt;
            tt.a = us_off[b] + (long long)(t0 - L.row0) * rp;
            tt.b = A.reduces[ridx[b]].tpad;
            tt.lda = rp;
            tt.K = L.rank;
            tt.aexp = eu_off[b] + (t0 - L.row0);
            tt.src = 0;
            tt.ldb = rp;
            tt.x_row0 = 0;
            tt.blk = ridx[b];
            per[t0 / TM].push_back(tt);
        }
    }
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        const LeafDesc &L = p->leaves[i];
        for (int t0 = L.row0; t0 < L.row0 + L.b; t0 += TM) {
            STerm tt;
            tt.a = ds_off[i] + (long long)(t0 - L.row0) * L.b;
            tt.b = 0;
            tt.lda = L.b;
            tt.K = L.b;
            tt.aexp = ed_off[i] + (t0 - L.row0);
            tt.src = 1;
            tt.ldb = 0;
            tt.x_row0 = L.row0;
            tt.blk = -1;
            per[t0 / TM].push_back(tt);
        }
    }
    for (int t = 0; t < ntiles; ++t) {
        A.tile_row0.push_back(t * TM);
        A.tile_begin.push_back((int)A.terms.size());
        A.terms.insert(A.terms.end(), per[t].begin(), per[t].end());
    }
    A.tile_begin.push_back((int)A.terms.size());
    if ((rc = upload_sschedule(A, &S->bytes))) return rc;
    if ((rc = ensure_err_flag(p))) return rc;
    DG_CUDA(cudaFuncSetAttribute(sp_panel_kernel<kNS, kNS, kD>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)panel_smem(kNS, kNS)));
    DG_CUDA(cudaFuncSetAttribute(sp_expand_kernel<kNS, kNS, kD>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)panel_smem(kNS, kNS)));
    return 0;
}

// Scratch of one sliced apply with nrhs columns: X slices, exponents,
// 128-bit partials, DD T, T slices and their exponents.
struct SWork {
    __int128 *partials;
    double *T;
    long long lo_off;
    bf16 *ts;
    long long tstride;
    int *texp;
};

static int sliced_scratch(Sliced *S, const SSchedule &A, int m, int nrhs, int ns, SWork &w)
{
    const size_t xs_need = (size_t)ns * m * nrhs;
    if (S->xs_elems < xs_need) {
        cudaFree(S->xs);
        S->xs = nullptr;
        S->xs_elems = 0;
        if (dev_malloc((void **)&S->xs, xs_need * sizeof(bf16)) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "sliced products: cannot allocate X slices");
        S->xs_elems = xs_need;
    }
    if (S->xexp_n < (size_t)nrhs) {
        cudaFree(S->xexp);
        S->xexp = nullptr;
        if (dev_malloc((void **)&S->xexp, nrhs * sizeof(int)) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "sliced products: cannot allocate exponents");
        S->xexp_n = nrhs;
    }
    auto r256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t part_bytes = r256((size_t)A.partial_per_rhs * nrhs * sizeof(__int128));
    const size_t t_bytes = r256((size_t)2 * A.t_per_rhs * nrhs * sizeof(double));
    const size_t ts_elems = (size_t)A.tpad_per_rhs * nrhs;
    const size_t ts_bytes = r256((size_t)ns * ts_elems * sizeof(bf16));
    const size_t te_bytes = (size_t)A.reduces.size() * nrhs * sizeof(int);
    const size_t need = part_bytes + t_bytes + ts_bytes + te_bytes + 1024;
    if (S->work_bytes < need) {
        cudaFree(S->work);
        S->work = nullptr;
        S->work_bytes = 0;
        if (cudaMalloc(&S->work, need) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "sliced products: cannot allocate scratch");
        S->work_bytes = need;
    }
    char *base = reinterpret_cast<char *>(S->work);
    w.partials = reinterpret_cast<__int128 *>(base);
    w.T = reinterpret_cast<double *>(base + part_bytes);
    w.lo_off = A.t_per_rhs * nrhs;
    w.ts = reinterpret_cast<bf16 *>(base + part_bytes + t_bytes);
    w.tstride = (long long)ts_elems;
    w.texp = reinterpret_cast<int *>(base + part_bytes + t_bytes + ts_bytes);
    return 0;
}

int sliced_residual(Plan *p, int nrhs, const double *X, int ldx, const double *B, int ldb,
                    double *R, int ldr, cudaStream_t st)
{
    Sliced *S = (Sliced *)p->sliced;
    if (!S) return fail(DPLR_GPU_ESTATE, "sliced residual: plan has no sliced factors");
    if (nrhs <= 0 || p->m == 0) return 0;
    if (S->apply.tile_m == tc::M) return sliced_residual_tb<kNS>(p, S, nrhs, X, ldx, B, ldb, R, ldr, st);
    const int m = p->m;
    const SSchedule &A = S->apply;
    SWork w;
    int rc = sliced_scratch(S, A, m, nrhs, kNS, w);
    if (rc) return rc;
    const long long xstride = (long long)m * nrhs;
    {
        ProfScope ps("slice_x", st, 0.0, 8.0 * m * nrhs + 2.0 * kNS * m * nrhs);
        xcol_exps(X, m, ldx, nrhs, S->xexp, st);
        xslice_kernel<kNS><<<xslice_grid(m, nrhs), 256, 0, st>>>(X, m, ldx, nrhs, S->xexp, S->xs, xstride);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }
    int npairs = 0;
    for (int d = 2; d <= kD; ++d)
        for (int pp = std::max(1, d - kNS); pp <= std::min(kNS, d - 1); ++pp) ++npairs;
    if (!A.items.empty()) {
        double fl = 0, by = 0;
        for (const SPanelItem &it : A.items) {
            fl += 2.0 * it.len * it.rank * nrhs;
            by += 2.0 * kNS * ((double)it.len * it.rank + (double)it.len * nrhs) + 16.0 * it.rank * nrhs;
        }
        {
            ProfScope ps("sliced_panel", st, fl * npairs, by);
            launch_panel<kNS, kD>(p, A, S->pool, S->stride, S->xs, xstride, m, nrhs, w.partials, st);
            DG_CUDA(cudaGetLastError());
        }
        ProfScope ps2("sliced_reduce", st, 0.0, 0.0);
        launch_reduce<kD>(A, w.partials, S->exps, S->xexp, p->pool, nrhs, w.T, w.lo_off, st);
        long long warps = (long long)A.reduces.size() * nrhs;
        sp_tslice_kernel<kNS><<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(
            A.d_reduces, (int)A.reduces.size(), w.T, w.lo_off, nrhs, w.ts, w.tstride, w.texp);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }
    if (!A.tile_row0.empty()) {
        double fl = 0, by = 0;
        for (const STerm &t : A.terms) {
            fl += 2.0 * A.tile_m * t.K * nrhs;
            by += 2.0 * kNS * ((double)A.tile_m * t.K) + 2.0 * kNS * t.K * nrhs;
        }
        ProfScope ps("sliced_expand", st, fl * npairs, by + 16.0 * m * nrhs);
        launch_expand<kNS, kD>(p, A, S->pool, S->stride, S->exps, w.ts, w.tstride, w.texp, S->xs, xstride, m,
                               S->xexp, nrhs, true, B, ldb, true, R, ldr, st);
        DG_CUDA(cudaGetLastError());
    }
    return 0;
}


// ====================================================== low-precision solve

// Slice counts of the inner solve: kMSMin..kMSMax slices, pairs p + q <= NS + 1.
constexpr int kMSMin = 3, kMSMax = 7;

static int pair_count(int ns, int dmax)
{
    int n = 0;
    for (int d = 2; d <= dmax; ++d)
        for (int p = std::max(1, d - ns); p <= std::min(ns, d - 1); ++p) ++n;
    return n;
}

void mixed_free(Plan *p)
{
    MixedSliced *M = (MixedSliced *)p->mixed;
    if (!M) return;
    cudaFree(M->pool);
    cudaFree(M->exps);
    for (SSchedule &L : M->level) free_sschedule(L);
    free_sschedule(M->leaf);
    cudaFree(M->xs);
    cudaFree(M->xexp);
    cudaFree(M->xexp2);
    cudaFree(M->work);
    cudaFree(M->kslices);
    cudaFree(M->kexps);
    for (SSchedule &C : M->capsched) free_sschedule(C);
    for (CapItem *d : M->d_capfb) cudaFree(d);
    delete M;
    p->mixed = nullptr;
}

template <int NS>
static int mixed_slice_t(const std::vector<SliceJob> &vj, const std::vector<int> &vbase, int ncols,
                         const std::vector<RowSliceJob> &zj, const std::vector<RowSliceJob> &lj,
                         const double *vpool, const double *zpool, const double *lpool, MixedSliced *M,
                         cudaStream_t st)
{
    SliceJob *d_vj = nullptr;
    RowSliceJob *d_zj = nullptr, *d_lj = nullptr;
    int *d_vb = nullptr, *d_zb = nullptr, *d_lb = nullptr;
    std::vector<int> zb, lb;
    int zr = 0, lr = 0;
    for (auto &j : zj) { zb.push_back(zr); zr += j.rows; }
    for (auto &j : lj) { lb.push_back(lr); lr += j.rows; }
    long long tmp = 0;
    int rc = 0;
    if ((rc = dev_vec(vj, &d_vj, &tmp)) || (rc = dev_vec(vbase, &d_vb, &tmp)) ||
        (rc = dev_vec(zj, &d_zj, &tmp)) || (rc = dev_vec(zb, &d_zb, &tmp)) ||
        (rc = dev_vec(lj, &d_lj, &tmp)) || (rc = dev_vec(lb, &d_lb, &tmp)))
        goto out;
    if (ncols > 0) {
        slice_cols_kernel<NS><<<ncols, 256, 0, st>>>(d_vj, d_vb, (int)vj.size(), vpool, M->pool, M->stride,
                                                     M->exps);
        note_launch();
    }
    // Z_l live in the factorisation's pool, leaf inverses in its leaf pool
    if (zr > 0) {
        slice_rows_kernel<NS><<<(zr + 127) / 128, 128, 0, st>>>(d_zj, d_zb, (int)zj.size(), zr, zpool, M->pool,
                                                               M->stride, M->exps);
        note_launch();
    }
    if (lr > 0) {
        slice_rows_kernel<NS><<<(lr + 127) / 128, 128, 0, st>>>(d_lj, d_lb, (int)lj.size(), lr, lpool, M->pool,
                                                               M->stride, M->exps);
        note_launch();
    }
    {
        cudaError_t e2 = cudaGetLastError();
        if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(st);
        if (e2 != cudaSuccess) rc = fail(DPLR_GPU_ECUDA, "mixed slicing: %s", cudaGetErrorString(e2));
    }
    if (!rc) {
        cudaError_t e3 = cudaFuncSetAttribute(sp_panel_kernel<NS, NS, NS + 1>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)panel_smem(NS, NS));
        if (e3 == cudaSuccess)
            e3 = cudaFuncSetAttribute(sp_expand_kernel<NS, NS, NS + 1>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)panel_smem(NS, NS));
        if (e3 != cudaSuccess) rc = fail(DPLR_GPU_ECUDA, "mixed solve: %s", cudaGetErrorString(e3));
    }
out:
    cudaFree(d_vj);
    cudaFree(d_vb);
    cudaFree(d_zj);
    cudaFree(d_zb);
    cudaFree(d_lj);
    cudaFree(d_lb);
    return rc;
}

int mixed_build(Plan *p, int ns, cudaStream_t st, bool fp64_caps)
{
    mixed_free(p);
    Fact *F = factor_of(p);
    if (!F) return fail(DPLR_GPU_ESTATE, "mixed solve: plan is not factored");
    if (ns < kMSMin || ns > kMSMax)
        return fail(DPLR_GPU_EINVAL, "mixed solve: %d slices (supported: %d to %d)", ns, kMSMin, kMSMax);
    for (const LeafDesc &L : p->leaves)
        if (L.b % ST != 0 || L.row0 % ST != 0)
            return fail(DPLR_GPU_EINVAL, "sliced products need leaf sizes that are multiples of %d", ST);
    MixedSliced *M = new MixedSliced();
    p->mixed = M;
    M->ns = ns;
    M->tc_caps = !fp64_caps;
    if (sliced_tile_rows(p) == tc::M) {
        switch (ns) {
        case 3: return mixed_build_tb_t<3>(p, M, F, st);
        case 4: return mixed_build_tb_t<4>(p, M, F, st);
        case 5: return mixed_build_tb_t<5>(p, M, F, st);
        case 6: return mixed_build_tb_t<6>(p, M, F, st);
        default: return mixed_build_tb_t<7>(p, M, F, st);
        }
    }
    const int m = p->m;
    const int nlev = (int)F->lv.size();

    // slice layout: V (column-major), Z_l (row-major, stride pad8(width)), leaf inverses (row-major)
    std::vector<long long> vs_off(p->lr.size()), zs_off(nlev), ls_off(p->leaves.size());
    std::vector<int> ev_off(p->lr.size()), ez_off(nlev), el_off(p->leaves.size());
    std::vector<SliceJob> vj;
    std::vector<RowSliceJob> zj, lj;
    std::vector<int> vbase;
    long long el = 0;
    int nexp = 0, ncols = 0;
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        vs_off[b] = el;
        el += al32((long long)L.n * L.rank);
        ev_off[b] = nexp;
        nexp += L.rank;
        if (L.rank == 0) continue;
        vbase.push_back(ncols);
        vj.push_back(SliceJob{L.v, vs_off[b], L.n, L.n, L.rank, ev_off[b]});
        ncols += L.rank;
    }
    for (int l = 0; l < nlev; ++l) {
        const int w = F->lv[l].width, wp = pad8(w);
        zs_off[l] = el;
        el += al32((long long)m * wp);
        ez_off[l] = nexp;
        nexp += m;
        if (w == 0) continue;
        zj.push_back(RowSliceJob{F->zoff[l], zs_off[l], m, m, w, wp, ez_off[l]});
    }
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        const LeafDesc &L = p->leaves[i];
        ls_off[i] = el;
        el += al32((long long)L.b * L.b);
        el_off[i] = nexp;
        nexp += L.b;
        lj.push_back(RowSliceJob{F->leafoff[i], ls_off[i], L.b, L.b, L.b, L.b, el_off[i]});
    }
    M->stride = al32(std::max<long long>(el, 1));
    if (dev_malloc((void **)&M->pool, (size_t)ns * M->stride * sizeof(bf16)) != cudaSuccess)
        return fail(DPLR_GPU_ENOMEM, "mixed solve: cannot allocate slices");
    M->bytes += (long long)ns * M->stride * 2;
    int rc;
    if ((rc = dev_vec(std::vector<int>(std::max(nexp, 1), 0), &M->exps, &M->bytes))) return rc;
    switch (ns) {
    case 3: rc = mixed_slice_t<3>(vj, vbase, ncols, zj, lj, p->pool, F->zpool, F->leafinv, M, st); break;
    case 4: rc = mixed_slice_t<4>(vj, vbase, ncols, zj, lj, p->pool, F->zpool, F->leafinv, M, st); break;
    case 5: rc = mixed_slice_t<5>(vj, vbase, ncols, zj, lj, p->pool, F->zpool, F->leafinv, M, st); break;
    case 6: rc = mixed_slice_t<6>(vj, vbase, ncols, zj, lj, p->pool, F->zpool, F->leafinv, M, st); break;
    default: rc = mixed_slice_t<7>(vj, vbase, ncols, zj, lj, p->pool, F->zpool, F->leafinv, M, st); break;
    }
    if (rc) return rc;

    // schedules: global reduce numbering over blocks (T / W slice panels)
    const int CH = 1024;
    std::vector<long long> tpad(p->lr.size(), 0);
    long long tp = 0;
    for (size_t b = 0; b < p->lr.size(); ++b) {
        tpad[b] = tp;
        tp += pad8(p->lr[b].rank);
    }
    M->tpad_per_rhs = tp;
    M->t_per_rhs = p->total_rank;
    M->nblocks = (int)p->lr.size();
    M->level.resize(nlev);
    const int TM = sliced_tile_rows(p);
    if ((rc = ensure_err_flag(p))) return rc;
    for (int l = 0; l < nlev; ++l) {
        SSchedule &S = M->level[l];
        S.tile_m = TM;
        long long poff = 0;
        const int wp = pad8(F->lv[l].width);
        for (int b : F->lv[l].blocks) {
            const LRDesc &L = p->lr[b];
            if (L.rank == 0) continue;
            const int nch = (L.n + CH - 1) / CH;
            for (int c = 0; c < nch; ++c) {
                SPanelItem it;
                it.f = vs_off[b];
                it.p = poff;
                it.n = L.n;
                it.rank = L.rank;
                it.in0 = L.col0;
                it.r0 = c * CH;
                it.len = std::min(CH, L.n - c * CH);
                it.chunk = c;
                S.items.push_back(it);
            }
            const int ridx = (int)S.reduces.size();
            S.reduces.push_back(SReduceItem{poff, L.toff, L.sig, L.rank, nch, ev_off[b], pad8(L.rank), tpad[b]});
            poff += (long long)nch * L.rank;
            S.max_rank = std::max(S.max_rank, L.rank);
            for (int t0 = L.row0; t0 < L.row0 + L.n; t0 += TM) {
                STerm tt;
                tt.a = zs_off[l] + (long long)t0 * wp;
                tt.b = tpad[b];
                tt.lda = wp;
                tt.K = L.rank;
                tt.aexp = ez_off[l] + t0;
                tt.src = 0;
                tt.ldb = pad8(L.rank);
                tt.x_row0 = 0;
                tt.blk = ridx;
                S.tile_row0.push_back(t0);
                S.tile_begin.push_back((int)S.terms.size());
                S.terms.push_back(tt);
            }
        }
        S.tile_begin.push_back((int)S.terms.size());
        S.partial_per_rhs = poff;
        S.t_per_rhs = p->total_rank;
        S.tpad_per_rhs = tp;
        if ((rc = upload_sschedule(S, &M->bytes))) return rc;
    }
    SSchedule &LS = M->leaf;
    LS.tile_m = TM;
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        const LeafDesc &L = p->leaves[i];
        for (int t0 = L.row0; t0 < L.row0 + L.b; t0 += TM) {
            STerm tt;
            tt.a = ls_off[i] + (long long)(t0 - L.row0) * L.b;
            tt.b = 0;
            tt.lda = L.b;
            tt.K = L.b;
            tt.aexp = el_off[i] + (t0 - L.row0);
            tt.src = 1;
            tt.ldb = 0;
            tt.x_row0 = L.row0;
            tt.blk = -1;
            LS.tile_row0.push_back(t0);
            LS.tile_begin.push_back((int)LS.terms.size());
            LS.terms.push_back(tt);
        }
    }
    LS.tile_begin.push_back((int)LS.terms.size());
    return upload_sschedule(LS, &M->bytes);
}

// Slice the columns of an m x n FP64 block (global exponent per column).
template <int NS>
static int slice_block(const double *X, int m, int ldx, int nrhs, bf16 *xs, int *xexp, cudaStream_t st)
{
    xcol_exps(X, m, ldx, nrhs, xexp, st);
    xslice_kernel<NS><<<xslice_grid(m, nrhs), 256, 0, st>>>(X, m, ldx, nrhs, xexp, xs, (long long)m * nrhs);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

// Scratch of the inner solve, carved from one allocation.
struct MWork {
    __int128 *partials;
    double *T, *W;
    long long lo_off;
    bf16 *ws;
    long long wstride;
    int *wexp;
};

static int mixed_scratch(MixedSliced *M, int m, int nrhs, MWork &w)
{
    const size_t xs_need = (size_t)M->ns * m * nrhs;
    if (M->xs_elems < xs_need) {
        cudaFree(M->xs);
        M->xs = nullptr;
        M->xs_elems = 0;
        if (dev_malloc((void **)&M->xs, xs_need * sizeof(bf16)) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "mixed solve: cannot allocate slices");
        M->xs_elems = xs_need;
    }
    if (M->xexp_n < (size_t)nrhs) {
        cudaFree(M->xexp);
        M->xexp = nullptr;
        if (dev_malloc((void **)&M->xexp, nrhs * sizeof(int)) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "mixed solve: cannot allocate exponents");
        M->xexp_n = nrhs;
    }
    long long part = 0;
    for (const SSchedule &L : M->level) part = std::max(part, L.partial_per_rhs);
    // every carve starts on a 256-byte boundary (16-byte copies need it)
    auto r256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t part_bytes = r256((size_t)part * nrhs * sizeof(__int128));
    const size_t t_bytes = r256((size_t)2 * M->t_per_rhs * nrhs * sizeof(double));
    const size_t w_bytes = r256((size_t)M->t_per_rhs * nrhs * sizeof(double));
    const size_t ws_bytes = r256((size_t)M->ns * M->tpad_per_rhs * nrhs * sizeof(bf16));
    size_t maxred = 0;
    for (const SSchedule &L : M->level) maxred = std::max(maxred, L.reduces.size());
    const size_t we_bytes = std::max<size_t>(maxred, 1) * nrhs * sizeof(int);
    const size_t need = part_bytes + t_bytes + w_bytes + ws_bytes + we_bytes + 1024;
    if (M->work_bytes < need) {
        cudaFree(M->work);
        M->work = nullptr;
        M->work_bytes = 0;
        if (cudaMalloc(&M->work, need) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "mixed solve: cannot allocate scratch");
        M->work_bytes = need;
    }
    char *base = reinterpret_cast<char *>(M->work);
    w.partials = reinterpret_cast<__int128 *>(base);
    w.T = reinterpret_cast<double *>(base + part_bytes);
    w.lo_off = M->t_per_rhs * nrhs;
    w.W = reinterpret_cast<double *>(base + part_bytes + t_bytes);
    w.ws = reinterpret_cast<bf16 *>(base + part_bytes + t_bytes + w_bytes);
    w.wstride = M->tpad_per_rhs * nrhs;
    w.wexp = reinterpret_cast<int *>(base + part_bytes + t_bytes + w_bytes + ws_bytes);
    return 0;
}

template <int NS>
static int mixed_solve_t(Plan *p, MixedSliced *M, Fact *F, int nrhs, const double *B, int ldb, double *X,
                         int ldx, cudaStream_t st)
{
    constexpr int D = NS + 1;
    const int m = p->m;
    MWork w;
    int rc = mixed_scratch(M, m, nrhs, w);
    if (rc) return rc;
    const long long xstride = (long long)m * nrhs;
    const double npairs = pair_count(NS, D);

    // leaf step: X = Leaf^-1 B
    if ((rc = slice_block<NS>(B, m, ldb, nrhs, M->xs, M->xexp, st))) return rc;
    {
        const SSchedule &LS = M->leaf;
        double fl = 0;
        for (const STerm &t : LS.terms) fl += 2.0 * LS.tile_m * t.K * nrhs;
        ProfScope ps("mixed_expand", st, fl * npairs, 0.0);
        launch_expand<NS, D>(p, LS, M->pool, M->stride, M->exps, w.ws, w.wstride, w.wexp, M->xs, xstride, m,
                             M->xexp, nrhs, false, nullptr, 0, false, X, ldx, st);
        DG_CUDA(cudaGetLastError());
    }
    for (int l = (int)M->level.size() - 1; l >= 0; --l) {
        const SSchedule &S = M->level[l];
        if (S.items.empty()) continue;
        if ((rc = slice_block<NS>(X, m, ldx, nrhs, M->xs, M->xexp, st))) return rc;
        double fl = 0;
        for (const SPanelItem &it : S.items) fl += 2.0 * it.len * it.rank * nrhs;
        {
            ProfScope ps("mixed_panel", st, fl * npairs, 0.0);
            launch_panel<NS, D>(p, S, M->pool, M->stride, M->xs, xstride, m, nrhs, w.partials, st);
        }
        launch_reduce<D>(S, w.partials, M->exps, M->xexp, p->pool, nrhs, w.T, w.lo_off, st);
        DG_CUDA(cudaGetLastError());
        // capacitance in FP64 on the high parts
        if ((rc = run_caps(F->lv[l].n, F->kpool, nullptr, 0, w.T, w.W, nrhs, st))) return rc;
        long long warps = (long long)S.reduces.size() * nrhs;
        sp_tslice_kernel<NS><<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(
            S.d_reduces, (int)S.reduces.size(), w.W, -1, nrhs, w.ws, w.wstride, w.wexp);
        note_launch();
        double fu = 0;
        for (const STerm &t : S.terms) fu += 2.0 * S.tile_m * t.K * nrhs;
        ProfScope ps2("mixed_expand", st, fu * npairs, 0.0);
        launch_expand<NS, D>(p, S, M->pool, M->stride, M->exps, w.ws, w.wstride, w.wexp, M->xs, xstride, m,
                             M->xexp, nrhs, true, X, ldx, true, X, ldx, st);
        DG_CUDA(cudaGetLastError());
    }
    return 0;
}

int mixed_solve(Plan *p, int nrhs, const double *B, int ldb, double *X, int ldx, cudaStream_t st)
{
    MixedSliced *M = (MixedSliced *)p->mixed;
    Fact *F = factor_of(p);
    if (!M || !F) return fail(DPLR_GPU_ESTATE, "mixed solve: not prepared");
    if (nrhs <= 0 || p->m == 0) return 0;
    if (M->leaf.tile_m == tc::M) {
        switch (M->ns) {
        case 3: return mixed_solve_tb<3>(p, M, F, nrhs, B, ldb, X, ldx, st);
        case 4: return mixed_solve_tb<4>(p, M, F, nrhs, B, ldb, X, ldx, st);
        case 5: return mixed_solve_tb<5>(p, M, F, nrhs, B, ldb, X, ldx, st);
        case 6: return mixed_solve_tb<6>(p, M, F, nrhs, B, ldb, X, ldx, st);
        default: return mixed_solve_tb<7>(p, M, F, nrhs, B, ldb, X, ldx, st);
        }
    }
    switch (M->ns) {
    case 3: return mixed_solve_t<3>(p, M, F, nrhs, B, ldb, X, ldx, st);
    case 4: return mixed_solve_t<4>(p, M, F, nrhs, B, ldb, X, ldx, st);
    case 5: return mixed_solve_t<5>(p, M, F, nrhs, B, ldb, X, ldx, st);
    case 6: return mixed_solve_t<6>(p, M, F, nrhs, B, ldb, X, ldx, st);
    default: return mixed_solve_t<7>(p, M, F, nrhs, B, ldb, X, ldx, st);
    }
}


// ====================================================== tcgen05 pipeline path
//
// With every leaf a multiple of 128 rows the products run on the
// warp-specialised tcgen05 kernels of tcpipe.cuh.  Their operands are cut
// into tile-blocks (R rows x 16 inner elements, contiguous, in the tensor
// core's K-major core-matrix order), so that one pipeline stage is a few
// contiguous bulk copies:
//   V (panel, B operand)   per block and rank tile of <= 64: row-blocks of 16
//                          block rows, pad16(tile ranks) rows each;
//   U, leaves, Z_l, leaf inverses (expand, A operand): 128-row tiles x
//                          16-element blocks of the inner dimension;
//   X slices (panel A operand in pairs, leaf-term B operand): 16-row blocks
//                          x 64-column tiles (column count padded to 128);
//   T / W slices (expand B operand): per block, 64-column tiles x 16-rank
//                          blocks.
// Padding rows and columns are zero.

namespace {

constexpr int kTbA = tc2::TB_A;     // 128 x 16
constexpr int kTbB = tc2::TB_B;     // 64 x 16

int pad16(int x) { return (x + 15) & ~15; }

// V into tile-blocks: one CTA per (job, rank column).
struct VSliceJob {
    long long src;          // column-major n x rank (ld n)
    long long sig;          // pool offset of sig (columns sliced as V sig_k), or -1
    long long dst[4];       // tile-block base of rank tiles 0..3
    int nr[4];              // padded rows of those tiles
    int n, rank, exp;
};

template <int NS>
__global__ void slice_v_tb_kernel(const VSliceJob *jobs, const int *col_base, int njobs, const double *src,
                                  bf16 *dst, long long stride, int *exps)
{
    __shared__ double red[256];
    const int gc = blockIdx.x;
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (col_base[mid] <= gc) lo = mid; else hi = mid - 1;
    }
    const VSliceJob &J = jobs[lo];
    const int k = gc - col_base[lo];
    const double *col = src + J.src + (long long)k * J.n;
    // with sig folded in, the column is the exact product V sig_k (TwoProd:
    // p + err); a rounded |p| below 2^e keeps the exact value below 2^e
    const double s = J.sig >= 0 ? src[J.sig + k] : 1.0;
    double mx = 0.0;
    for (int i = threadIdx.x; i < J.n; i += blockDim.x) mx = fmax(mx, fabs(col[i] * s));
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    const int e = scale_exp(red[0]);
    if (threadIdx.x == 0) exps[J.exp + k] = e;
    const int kt = k / 64, r = k % 64, nr = J.nr[kt];
    bf16 *base = dst + J.dst[kt];
    for (int i = threadIdx.x; i < J.n; i += blockDim.x) {
        bf16 *o = base + (long long)(i >> 4) * nr * 16 + tc2::tbo(r, i & 15);
        if (J.sig >= 0) {
            const double pr = col[i] * s;
            slice_dd<NS>(pr, fma(col[i], s, -pr), e, o, stride);
        } else {
            slice_d<NS>(col[i], e, o, stride);
        }
    }
}

// Row-sliced operands into 128-row tile-blocks.
struct RSliceJob {
    long long src;          // column-major rows x cols (ld)
    long long dst;          // tile-block base
    int ld, rows, cols, nkb, exp;
    int roff = 0;           // tile row of the first row (blocks smaller than a tile)
};

__device__ __forceinline__ int find_job(const int *base, int njobs, int g)
{
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (base[mid] <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Row slicing into 128-row tile-blocks: one thread per row, one exponent
// per row.
template <int NS>
__global__ void slice_r_tb_kernel(const RSliceJob *jobs, const int *row_base, int njobs, int total, const double *src,
                                  bf16 *dst, long long stride, int *exps)
{
    const int gr = blockIdx.x * blockDim.x + threadIdx.x;
    if (gr >= total) return;
    const int lo = find_job(row_base, njobs, gr);
    const RSliceJob &J = jobs[lo];
    const int r = gr - row_base[lo];
    double mx = 0.0;
    for (int k = 0; k < J.cols; ++k) mx = fmax(mx, fabs(src[J.src + r + (long long)k * J.ld]));
    const int e = scale_exp(mx);
    exps[J.exp + r] = e;
    const int rr = r + J.roff;
    bf16 *base = dst + J.dst + (long long)(rr >> 7) * J.nkb * kTbA;
    for (int k = 0; k < J.nkb * 16; ++k) {
        const double v = k < J.cols ? src[J.src + r + (long long)k * J.ld] : 0.0;
        slice_d<NS>(v, e, base + (long long)(k >> 4) * kTbA + tc2::tbo(rr & 127, k & 15), stride);
    }
}

// Pack the NS slices of 8 consecutive values into one 16-byte store per
// slice.  The balanced base-128 digits come out least significant first, so
// each slice is stored as soon as its 8 digits are known (only the 8 running
// values stay live).
template <int NS>
__device__ __forceinline__ void store8(long long (&v)[8], bf16 *out, long long stride)
{
#pragma unroll
    for (int p = NS - 1; p >= 0; --p) {
        uint32_t b[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            int a;
            if (p > 0) {
                const long long d = ((v[u] + 64) & 127) - 64;
                a = (int)d;
                v[u] = (v[u] - d) >> 7;
            } else {
                a = (int)v[u];
            }
            b[u] = digit_bits(a);
        }
        uint4 w;
        w.x = b[0] | (b[1] << 16);
        w.y = b[2] | (b[3] << 16);
        w.z = b[4] | (b[5] << 16);
        w.w = b[6] | (b[7] << 16);
        *reinterpret_cast<uint4 *>(out + p * stride) = w;
    }
}

// Four consecutive values of one column as NS bf16 digit slices: 8 bytes per
// slice at out + p * stride (the same balanced base-128 split as store8).
template <int NS>
__device__ __forceinline__ void store4(long long (&v)[4], bf16 *out, long long stride)
{
#pragma unroll
    for (int p = NS - 1; p >= 0; --p) {
        uint32_t b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int a;
            if (p > 0) {
                const long long d = ((v[u] + 64) & 127) - 64;
                a = (int)d;
                v[u] = (v[u] - d) >> 7;
            } else {
                a = (int)v[u];
            }
            b[u] = digit_bits(a);
        }
        uint2 w;
        w.x = b[0] | (b[1] << 16);
        w.y = b[2] | (b[3] << 16);
        *reinterpret_cast<uint2 *>(out + p * stride) = w;
    }
}

// X (m x nrhs) into 16-row x 64-column tile-blocks, coalesced: one warp per
// (row-block rb, group of 8 columns); lane l holds column 8 g + l / 4 and
// rows 4 (l % 4) .. 4 (l % 4) + 3 of the row-block, so four lanes read one
// column's 128 contiguous bytes and the warp writes, per slice, the 256
// contiguous bytes of two core matrices.  Columns >= nrhs are zero.
template <int NS>
__global__ void xslice_tb4_kernel(const double *__restrict__ X, int m, int ldx, int nrhs, int xnjt,
                                  const int *__restrict__ xexp, bf16 *__restrict__ xs, long long stride)
{
    const int nrb = m >> 4, ncg = xnjt * 8;
    const long long nw = (long long)nrb * ncg;
    const int lane = threadIdx.x & 31;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long wstep = ((long long)gridDim.x * blockDim.x) >> 5;
    const int q = lane & 3;
    const bool vec = (ldx & 1) == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0;
    for (long long w = w0; w < nw; w += wstep) {
        const int g = (int)(w % ncg), rb = (int)(w / ncg);
        const int j = g * 8 + (lane >> 2);
        const bool live = j < nrhs;
        const int sh = live ? 7 * NS - xexp[j] : 0;
        const double *col = X + (long long)(live ? j : 0) * ldx + rb * 16 + q * 4;
        double x[4];
        if (live && vec) {
            const double2 a = __ldg(reinterpret_cast<const double2 *>(col));
            const double2 b = __ldg(reinterpret_cast<const double2 *>(col + 2));
            x[0] = a.x, x[1] = a.y, x[2] = b.x, x[3] = b.y;
        } else {
#pragma unroll
            for (int u = 0; u < 4; ++u) x[u] = live ? __ldg(col + u) : 0.0;
        }
        long long y[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) y[u] = scaled_int(x[u], sh);
        bf16 *out = xs + ((long long)rb * xnjt + (j >> 6)) * kTbB + tc2::tbo(j & 63, q * 4);
        store4<NS>(y, out, stride);
    }
}

// T / W (rank x nrhs per block, FP64 or double-double) into tile-blocks of
// 64 columns x 16 ranks, one exponent per (block, column); one warp per
// (block, column j < njt * 64).
template <int NS>
__global__ void __launch_bounds__(256) tslice_tb_kernel(const SReduceItem *__restrict__ items, int nitems,
                                                        const double *__restrict__ T, long long lo_off, int nrhs,
                                                        int njt, bf16 *__restrict__ ts, long long tstride,
                                                        int *__restrict__ texp)
{
    // one CTA per (block, 64-column tile); thread = (column jl, 8 ranks kg)
    __shared__ int cexp[64];
    const int b = blockIdx.x, jt = blockIdx.y;
    if (b >= nitems) return;
    const SReduceItem R = items[b];
    const int ngrp = R.rp >> 3;                   // 8-rank groups of the padded rank
    if (threadIdx.x < 64) cexp[threadIdx.x] = INT_MIN;
    __syncthreads();
    // column exponents: scale_exp is monotone, so the max of the per-thread
    // exponents is the exponent of the column's largest entry
    for (int w = threadIdx.x; w < 64 * ngrp; w += blockDim.x) {
        const int jl = w & 63, kg = w >> 6, j = jt * 64 + jl;
        if (j >= nrhs) continue;
        const double *th = T + R.t * nrhs + (long long)j * R.rank;
        double mx = 0.0;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int k = kg * 8 + u;
            if (k < R.rank) mx = fmax(mx, fabs(th[k]));
        }
        if (mx > 0.0) atomicMax(&cexp[jl], scale_exp(mx));
    }
    __syncthreads();
    if (threadIdx.x < 64) {
        if (cexp[threadIdx.x] == INT_MIN) cexp[threadIdx.x] = 0;     // all-zero column
        if (jt * 64 + threadIdx.x < nrhs) texp[(long long)b * nrhs + jt * 64 + threadIdx.x] = cexp[threadIdx.x];
    }
    __syncthreads();
    bf16 *base = ts + R.tpad * njt + (long long)jt * (R.rp >> 4) * kTbB;
    for (int w = threadIdx.x; w < 64 * ngrp; w += blockDim.x) {
        const int jl = w & 63, kg = w >> 6, j = jt * 64 + jl;
        const int k0 = kg * 8;
        bf16 *o = base + (long long)(k0 >> 4) * kTbB + tc2::tbo(jl, k0 & 15);
        long long y[8];
        if (j < nrhs) {
            const double *th = T + R.t * nrhs + (long long)j * R.rank;
            const double *tl = lo_off >= 0 ? th + lo_off : nullptr;
            const int sh = 7 * NS - cexp[jl];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int k = k0 + u;
                y[u] = k < R.rank ? scaled_int(th[k], sh) + (tl ? scaled_int(tl[k], sh) : 0) : 0;
            }
        } else {
#pragma unroll
            for (int u = 0; u < 8; ++u) y[u] = 0;
        }
        store8<NS>(y, o, tstride);
    }
}

// Alignment exponents of the multi-term expand: per tile row the largest
// row exponent of the tile's terms (fixed once the factors are sliced), and
// per tile and right-hand side the largest column exponent (T or X slices,
// per call).  Empty tiles and columns get 0, as the kernel expects.
__global__ void tile_rmax_kernel(const XTerm *__restrict__ terms, const int *__restrict__ tile_begin, int ntiles,
                                 const int *__restrict__ aexp, int *__restrict__ rmax)
{
    const int tile = blockIdx.x, row = threadIdx.x;
    if (tile >= ntiles) return;
    int r = -100000;
    for (int q = tile_begin[tile]; q < tile_begin[tile + 1]; ++q) r = max(r, aexp[terms[q].aexp + row]);
    rmax[(long long)tile * tc2::M + row] = r < -99999 ? 0 : r;
}

__global__ void tile_cmax_kernel(const XTerm *__restrict__ terms, const int *__restrict__ tile_begin, int ntiles,
                                 const int *__restrict__ texp, const int *__restrict__ xexp, int nrhs,
                                 int *__restrict__ cmax)
{
    const int tile = blockIdx.x, j = blockIdx.y * blockDim.x + threadIdx.x;
    if (tile >= ntiles || j >= nrhs) return;
    int c = -100000;
    for (int q = tile_begin[tile]; q < tile_begin[tile + 1]; ++q) {
        const XTerm tt = terms[q];
        c = max(c, tt.src == 0 ? texp[(long long)tt.blk * nrhs + j] : xexp[j]);
    }
    cmax[(long long)tile * nrhs + j] = c < -99999 ? 0 : c;
}

int upload_tb(SSchedule &S, long long *bytes)
{
    int rc;
    if ((rc = upload_rank_items(S, bytes))) return rc;
    if ((rc = dev_vec(S.pitems, &S.d_pitems, bytes)) || (rc = dev_vec(S.reduces, &S.d_reduces, bytes)) ||
        (rc = dev_vec(S.tile_row0, &S.d_tile_row0, bytes)) || (rc = dev_vec(S.tile_begin, &S.d_tile_begin, bytes)) ||
        (rc = dev_vec(S.xterms, &S.d_xterms, bytes)))
        return rc;
    return 0;
}

// V tile-block layout of every low-rank block (shared by both builders).
struct VLayout {
    std::vector<VSliceJob> jobs;
    std::vector<int> col_base;
    int ncols = 0;
};

// fold_sig: slice V diag(sig) (the panel then yields T = S V^T x directly and
// the reduce does no FP64 scaling).
long long layout_v(const Plan *p, std::vector<std::array<long long, 4>> &vdst, std::vector<std::array<int, 4>> &vnr,
                   long long el, const std::vector<int> &ev_off, VLayout &VL, bool fold_sig)
{
    vdst.assign(p->lr.size(), {0, 0, 0, 0});
    vnr.assign(p->lr.size(), {0, 0, 0, 0});
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        if (L.rank == 0) continue;
        VSliceJob J{};
        J.src = L.v;
        J.sig = fold_sig ? L.sig : -1;
        J.n = L.n;
        J.rank = L.rank;
        J.exp = ev_off[b];
        for (int kt = 0; kt * 64 < L.rank; ++kt) {
            const int nr = pad16(std::min(64, L.rank - kt * 64));
            vdst[b][kt] = el;
            vnr[b][kt] = nr;
            J.dst[kt] = el;
            J.nr[kt] = nr;
            el += (long long)(L.n / 16) * nr * 16;
        }
        VL.col_base.push_back(VL.ncols);
        VL.jobs.push_back(J);
        VL.ncols += L.rank;
    }
    return el;
}

// Panel items of one block (row chunks of CH rows x rank tiles of 64).
// Each (chunk, rank, right-hand side) leaves one 128-bit partial that the
// reduce reads back.  Measured on the N = 2^18 solve, 4096-row chunks for
// the residual's all-level panel cut the reduce (1.55 -> 1.40 ms per step)
// but slowed the panel more (8.40 -> 9.17 ms): both panels keep 1024 rows.
constexpr int kInnerChunk = 1024, kResidChunk = 1024;

void panel_items(const LRDesc &L, const std::array<long long, 4> &vdst, const std::array<int, 4> &vnr, long long poff,
                 std::vector<PItem> &out, int CH = kInnerChunk)
{
    const int nch = (L.n + CH - 1) / CH;
    for (int c = 0; c < nch; ++c) {
        const int r0 = c * CH, len = std::min(CH, L.n - r0);
        for (int kt = 0; kt * 64 < L.rank; ++kt) {
            PItem it;
            it.v = vdst[kt];
            it.p = poff;
            it.rank = L.rank;
            it.kt = kt * 64;
            it.nr = vnr[kt];
            it.xrb0 = (L.col0 + r0) / 16;
            it.vrb0 = r0 / 16;
            it.nkb = len / 16;
            it.chunk = c;
            out.push_back(it);
        }
    }
}

int xnjt_of(int nrhs) { return 2 * ((nrhs + 127) / 128); }

// X slices (tile-blocks) and their exponents for nrhs columns.
template <int NS>
// known_exps: xexp already holds the column exponents (gathered by the
// expand that wrote X, kNoExp for all-zero columns); only the fix-up runs.
int slice_x_tb(const double *X, int m, int ldx, int nrhs, bf16 *&xs, size_t &xs_elems, int *&xexp, size_t &xexp_n,
               cudaStream_t st, bool known_exps = false)
{
    const int xnjt = xnjt_of(nrhs);
    const size_t need = (size_t)NS * (m / 16) * xnjt * kTbB;
    if (xs_elems < need) {
        cudaFree(xs);
        xs = nullptr;
        xs_elems = 0;
        if (dev_malloc((void **)&xs, need * sizeof(bf16)) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "sliced products: cannot allocate X slices");
        xs_elems = need;
    }
    if (xexp_n < (size_t)nrhs) {
        cudaFree(xexp);
        xexp = nullptr;
        if (dev_malloc((void **)&xexp, nrhs * sizeof(int)) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "sliced products: cannot allocate exponents");
        xexp_n = nrhs;
    }
    if (known_exps) {
        xcol_fix_kernel<<<(nrhs + 255) / 256, 256, 0, st>>>(xexp, nrhs);
        note_launch();
    } else {
        xcol_exps(X, m, ldx, nrhs, xexp, st);
    }
    const long long warps = (long long)(m / 16) * xnjt * 8;
    const int grid = (int)std::min<long long>((warps * 32 + 255) / 256, 152LL * 32);
    xslice_tb4_kernel<NS><<<grid, 256, 0, st>>>(X, m, ldx, nrhs, xnjt, xexp, xs, (long long)(m / 16) * xnjt * kTbB);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

template <int NS, int D>
int tb_attrs()
{
    DG_CUDA(cudaFuncSetAttribute(tc2::panel_kernel<NS, D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc2::Cfg<NS>::SMEM));
    DG_CUDA(cudaFuncSetAttribute(tc2::expand_kernel<NS, D, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc2::Cfg<NS>::SMEM));
    if constexpr (D <= 8)
        DG_CUDA(cudaFuncSetAttribute(tc2::expand_kernel<NS, D, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     tc2::Cfg<NS>::SMEM));
    return 0;
}

int grid_of(long long units)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (int)std::max<long long>(1, std::min<long long>(units, sms));
}

template <int NS, int D>
void launch_panel_tb(const Plan *p, const SSchedule &S, const bf16 *vpool, long long vstride, const bf16 *xs,
                     int m, int nrhs, __int128 *partials, cudaStream_t st)
{
    const int njp = (nrhs + 127) / 128;
    const int n = (int)S.pitems.size();
    if (n == 0) return;
    tc2::panel_kernel<NS, D><<<grid_of((long long)n * njp), tc2::THREADS, tc2::Cfg<NS>::SMEM, st>>>(
        S.d_pitems, n, njp, vpool, vstride, xs, (long long)(m / 16) * xnjt_of(nrhs) * kTbB, xnjt_of(nrhs), nrhs,
        partials, p->tc_err_d);
    note_launch();
}

template <int NS, int D>
void launch_expand_tb(const Plan *p, const SSchedule &S, const bf16 *apool, long long astride, const int *aexp,
                      const bf16 *ts, long long tstride, const int *texp, const bf16 *xs, int m, const int *xexp,
                      int nrhs, bool neg, const double *Bin, int ldbin, bool addb, double *Y, int ldy,
                      cudaStream_t st, const int *rmaxt = nullptr, const int *cmaxt = nullptr, int *yexp = nullptr,
                      int rscale = 1)
{
    const int njt = (nrhs + 63) / 64;
    const int nt = (int)S.tile_row0.size();
    if (nt == 0) return;
    const long long xstride = (long long)(m / 16) * xnjt_of(nrhs) * kTbB;
    bool single = true;                         // every tile one term: the 64-bit epilogue applies
    for (size_t t = 0; t + 1 < S.tile_begin.size(); ++t) single = single && S.tile_begin[t + 1] - S.tile_begin[t] == 1;
    if constexpr (D <= 8) {
        if (single) {
            tc2::expand_kernel<NS, D, true><<<grid_of((long long)nt * njt), tc2::THREADS, tc2::Cfg<NS>::SMEM, st>>>(
                S.d_xterms, S.d_tile_row0, S.d_tile_begin, nt, njt, apool, astride, aexp, ts, tstride, texp, xs,
                xstride, xnjt_of(nrhs), xexp, nrhs, neg ? 1 : 0, Bin, ldbin, addb ? 1 : 0, Y, ldy, nullptr, nullptr,
                nrhs <= tc2::kColCap ? yexp : nullptr, rscale, p->tc_err_d);
            note_launch();
            return;
        }
    }
    tc2::expand_kernel<NS, D, false><<<grid_of((long long)nt * njt), tc2::THREADS, tc2::Cfg<NS>::SMEM, st>>>(
        S.d_xterms, S.d_tile_row0, S.d_tile_begin, nt, njt, apool, astride, aexp, ts, tstride, texp, xs, xstride,
        xnjt_of(nrhs), xexp, nrhs, neg ? 1 : 0, Bin, ldbin, addb ? 1 : 0, Y, ldy, rmaxt, cmaxt, nullptr, rscale,
        p->tc_err_d);
    note_launch();
}

}  // namespace

// -------------------------------------------------- exact-slice residual
// Row exponent of a padding row of a tile-block (a block smaller than the
// tile): below every real one, so that it never sets a tile's alignment;
// its rows are zero and add nothing whatever the shift.
constexpr int kPadExp = -(1 << 20);

static int sliced_build_tb(Plan *p, Sliced *S, cudaStream_t st)
{
    // Exponent slots: V per rank, U and leaves per row.  A block or leaf of
    // n < 128 rows gets a whole tile of slots (eu_off / ed_off: the tile's
    // row 0), its rows at roff = row0 % 128, the others padding.
    std::vector<int> ev_off(p->lr.size()), eu_off(p->lr.size()), ed_off(p->leaves.size());
    std::vector<std::pair<int, int>> pads;           // [begin, end) of padding slots
    int nexp = 0;
    auto rows_slots = [&](int n, int row0) {
        const int base = nexp;
        if (n % tc2::M == 0) {
            nexp += n;
        } else {
            const int roff = row0 % tc2::M;
            if (roff > 0) pads.push_back({base, base + roff});
            if (roff + n < tc2::M) pads.push_back({base + roff + n, base + tc2::M});
            nexp += tc2::M;
        }
        return base;
    };
    for (size_t b = 0; b < p->lr.size(); ++b) {
        ev_off[b] = nexp;
        nexp += p->lr[b].rank;
        eu_off[b] = rows_slots(p->lr[b].n, p->lr[b].row0);
    }
    for (size_t i = 0; i < p->leaves.size(); ++i) ed_off[i] = rows_slots(p->leaves[i].b, p->leaves[i].row0);
    auto small = [](int n) { return n % tc2::M != 0; };
    auto roff_of = [&](int n, int row0) { return small(n) ? row0 % tc2::M : 0; };
    VLayout VL;
    std::vector<std::array<long long, 4>> vdst;
    std::vector<std::array<int, 4>> vnr;
    long long el = layout_v(p, vdst, vnr, 0, ev_off, VL, true);
    // every U row and leaf row has its own exponent
    std::vector<long long> ua(p->lr.size(), 0), la(p->leaves.size(), 0);
    std::vector<RSliceJob> uj, lj;
    std::vector<int> ubase, lbase;
    int nurows = 0, nlrows = 0;
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        if (L.rank == 0) continue;
        const int nkb = (L.rank + 15) / 16;
        const int ro = roff_of(L.n, L.row0);
        ua[b] = el;
        el += (long long)std::max(1, L.n / tc2::M) * nkb * kTbA;
        ubase.push_back(nurows);
        uj.push_back(RSliceJob{L.u, ua[b], L.n, L.n, L.rank, nkb, eu_off[b] + ro, ro});
        nurows += L.n;
    }
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        const LeafDesc &L = p->leaves[i];
        const int ro = roff_of(L.b, L.row0);
        la[i] = el;
        el += (long long)std::max(1, L.b / tc2::M) * (L.b / 16) * kTbA;
        lbase.push_back(nlrows);
        lj.push_back(RSliceJob{L.d, la[i], L.b, L.b, L.b, L.b / 16, ed_off[i] + ro, ro});
        nlrows += L.b;
    }
    S->stride = al32(std::max<long long>(el, 1));
    if (dev_malloc((void **)&S->pool, (size_t)kNS * S->stride * sizeof(bf16)) != cudaSuccess)
        return fail(DPLR_GPU_ENOMEM, "sliced products: cannot allocate slices");
    S->bytes += (long long)kNS * S->stride * 2;
    DG_CUDA(cudaMemsetAsync(S->pool, 0, (size_t)kNS * S->stride * sizeof(bf16), st));
    S->nexp = nexp;
    int rc;
    {
        std::vector<int> e0(std::max(nexp, 1), 0);
        for (const auto &pr : pads) std::fill(e0.begin() + pr.first, e0.begin() + pr.second, kPadExp);
        if ((rc = dev_vec(e0, &S->exps, &S->bytes))) return rc;
    }
    {
        VSliceJob *d_vj = nullptr;
        RSliceJob *d_uj = nullptr, *d_lj = nullptr;
        int *d_vb = nullptr, *d_ub = nullptr, *d_lb = nullptr;
        long long tmp = 0;
        if ((rc = dev_vec(VL.jobs, &d_vj, &tmp)) || (rc = dev_vec(VL.col_base, &d_vb, &tmp)) ||
            (rc = dev_vec(uj, &d_uj, &tmp)) || (rc = dev_vec(ubase, &d_ub, &tmp)) || (rc = dev_vec(lj, &d_lj, &tmp)) ||
            (rc = dev_vec(lbase, &d_lb, &tmp)))
            return rc;
        if (VL.ncols > 0) {
            slice_v_tb_kernel<kNS><<<VL.ncols, 256, 0, st>>>(d_vj, d_vb, (int)VL.jobs.size(), p->pool, S->pool,
                                                            S->stride, S->exps);
            note_launch();
        }
        if (nurows > 0) {
            slice_r_tb_kernel<kNS><<<(nurows + 127) / 128, 128, 0, st>>>(d_uj, d_ub, (int)uj.size(), nurows,
                                                                        p->pool, S->pool, S->stride, S->exps);
            note_launch();
        }
        if (nlrows > 0) {
            slice_r_tb_kernel<kNS><<<(nlrows + 127) / 128, 128, 0, st>>>(d_lj, d_lb, (int)lj.size(), nlrows,
                                                                        p->pool, S->pool, S->stride, S->exps);
            note_launch();
        }
        cudaError_t e2 = cudaGetLastError();
        if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(st);
        cudaFree(d_vj);
        cudaFree(d_vb);
        cudaFree(d_uj);
        cudaFree(d_ub);
        cudaFree(d_lj);
        cudaFree(d_lb);
        if (e2 != cudaSuccess) return fail(DPLR_GPU_ECUDA, "slicing: %s", cudaGetErrorString(e2));
    }
    // schedule: panel items, reduces, 128-row tiles
    SSchedule &A = S->apply;
    A.tile_m = tc2::M;
    long long poff = 0, tpre = 0;
    std::vector<int> ridx(p->lr.size(), -1);
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        if (L.rank == 0) continue;
        panel_items(L, vdst[b], vnr[b], poff, A.pitems, kResidChunk);
        const int nch = (L.n + kResidChunk - 1) / kResidChunk;
        const int nkb = (L.rank + 15) / 16;
        ridx[b] = (int)A.reduces.size();
        A.reduces.push_back(SReduceItem{poff, L.toff, -1, L.rank, nch, ev_off[b], nkb * 16, tpre});   // sig in V
        poff += (long long)nch * L.rank;
        tpre += (long long)nkb * kTbB;
        A.max_rank = std::max(A.max_rank, L.rank);
    }
    A.partial_per_rhs = poff;
    A.t_per_rhs = p->total_rank;
    A.tpre = tpre;
    const int ntiles = p->m / tc2::M;
    std::vector<std::vector<XTerm>> per(ntiles);
    for (size_t b = 0; b < p->lr.size(); ++b) {
        const LRDesc &L = p->lr[b];
        if (L.rank == 0) continue;
        const int nkb = (L.rank + 15) / 16;
        // each term keeps its own row and column exponents (one read-out per
        // term): sharing them across levels costs the residual about 3x in
        // accuracy on the N = 2^18 kernel matrix
        if (small(L.n)) {                     // one tile, the block's rows inside it
            per[L.row0 / tc2::M].push_back(XTerm{ua[b], A.reduces[ridx[b]].tpad, L.rank, eu_off[b], 0, ridx[b]});
            continue;
        }
        for (int t0 = L.row0; t0 < L.row0 + L.n; t0 += tc2::M)
            per[t0 / tc2::M].push_back(XTerm{ua[b] + (long long)((t0 - L.row0) / tc2::M) * nkb * kTbA,
                                             A.reduces[ridx[b]].tpad, L.rank, eu_off[b] + (t0 - L.row0), 0, ridx[b]});
    }
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        const LeafDesc &L = p->leaves[i];
        if (small(L.b)) {
            per[L.row0 / tc2::M].push_back(XTerm{la[i], L.row0 / 16, L.b, ed_off[i], 1, -1});
            continue;
        }
        for (int t0 = L.row0; t0 < L.row0 + L.b; t0 += tc2::M)
            per[t0 / tc2::M].push_back(XTerm{la[i] + (long long)((t0 - L.row0) / tc2::M) * (L.b / 16) * kTbA,
                                             L.row0 / 16, L.b, ed_off[i] + (t0 - L.row0), 1, -1});
    }
    for (int t = 0; t < ntiles; ++t) {
        A.tile_row0.push_back(t * tc2::M);
        A.tile_begin.push_back((int)A.xterms.size());
        A.xterms.insert(A.xterms.end(), per[t].begin(), per[t].end());
    }
    A.tile_begin.push_back((int)A.xterms.size());
    if ((rc = upload_tb(A, &S->bytes))) return rc;
    if (ntiles > 0) {
        DG_ALLOC(&A.d_rmax, (size_t)ntiles * tc2::M * sizeof(int));
        S->bytes += (long long)ntiles * tc2::M * sizeof(int);
        tile_rmax_kernel<<<ntiles, tc2::M, 0, st>>>(A.d_xterms, A.d_tile_begin, ntiles, S->exps, A.d_rmax);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }
    if ((rc = ensure_err_flag(p))) return rc;
    return tb_attrs<kNS, kD>();
}

// NSR slices of the stored ones (the residual uses all 8).
template <int NSR>
static int sliced_residual_tb(Plan *p, Sliced *S, int nrhs, const double *X, int ldx, const double *B, int ldb,
                              double *R, int ldr, cudaStream_t st)
{
    constexpr int DR = NSR + 1;
    const int m = p->m;
    const SSchedule &A = S->apply;
    const int njt = (nrhs + 63) / 64;
    int rc;
    {
        ProfScope ps("slice_x", st, 0.0, 8.0 * m * nrhs + 2.0 * NSR * m * nrhs);
        if ((rc = slice_x_tb<NSR>(X, m, ldx, nrhs, S->xs, S->xs_elems, S->xexp, S->xexp_n, st))) return rc;
    }
    // scratch: partials, DD T, T slices, T exponents (256-byte carves)
    auto r256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t part_bytes = r256((size_t)A.partial_per_rhs * nrhs * sizeof(__int128));
    const size_t t_bytes = r256((size_t)2 * A.t_per_rhs * nrhs * sizeof(double));
    const long long tstride = A.tpre * njt;
    const size_t ts_bytes = r256((size_t)NSR * tstride * sizeof(bf16));
    const size_t te_bytes = r256((size_t)std::max<size_t>(A.reduces.size(), 1) * nrhs * sizeof(int));
    const int ntiles = (int)A.tile_row0.size();
    const size_t cm_bytes = r256((size_t)std::max(ntiles, 1) * nrhs * sizeof(int));
    const size_t need = part_bytes + t_bytes + ts_bytes + te_bytes + cm_bytes;
    if (S->work_bytes < need) {
        cudaFree(S->work);
        S->work = nullptr;
        S->work_bytes = 0;
        if (cudaMalloc(&S->work, need) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "sliced products: cannot allocate scratch");
        S->work_bytes = need;
    }
    char *base = reinterpret_cast<char *>(S->work);
    __int128 *partials = reinterpret_cast<__int128 *>(base);
    double *T = reinterpret_cast<double *>(base + part_bytes);
    const long long lo_off = A.t_per_rhs * nrhs;
    bf16 *ts = reinterpret_cast<bf16 *>(base + part_bytes + t_bytes);
    int *texp = reinterpret_cast<int *>(base + part_bytes + t_bytes + ts_bytes);
    int *cmax = reinterpret_cast<int *>(base + part_bytes + t_bytes + ts_bytes + te_bytes);
    int npairs = 0;
    for (int d = 2; d <= DR; ++d)
        for (int pp = std::max(1, d - NSR); pp <= std::min(NSR, d - 1); ++pp) ++npairs;
    if (!A.pitems.empty()) {
        double fl = 0, by = 0;
        for (const PItem &it : A.pitems) {
            fl += 2.0 * it.nkb * 16 * std::min(64, it.rank - it.kt) * nrhs;
            by += 2.0 * NSR * ((double)it.nkb * 16 * it.nr + (double)it.nkb * 16 * nrhs);
        }
        {
            ProfScope ps("sliced_panel", st, fl * npairs, by);
            launch_panel_tb<NSR, DR>(p, A, S->pool, S->stride, S->xs, m, nrhs, partials, st);
            DG_CUDA(cudaGetLastError());
        }
        {
            ProfScope ps2("sliced_reduce", st, 0.0, 16.0 * A.partial_per_rhs * nrhs);
            launch_reduce<DR>(A, partials, S->exps, S->xexp, p->pool, nrhs, T, lo_off, st);
        }
        ProfScope ps3("sliced_tslice", st, 0.0, 0.0);
        tslice_tb_kernel<NSR><<<dim3((unsigned)A.reduces.size(), (unsigned)njt), 256, 0, st>>>(
            A.d_reduces, (int)A.reduces.size(), T, lo_off, nrhs, njt, ts, tstride, texp);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }
    if (!A.tile_row0.empty()) {
        double fl = 0, by = 0;
        for (const XTerm &t : A.xterms) {
            fl += 2.0 * tc2::M * t.K * nrhs;
            by += 2.0 * NSR * ((double)tc2::M * pad16(t.K)) + 2.0 * NSR * pad16(t.K) * nrhs;
        }
        ProfScope ps("sliced_expand", st, fl * npairs, by + 16.0 * m * nrhs);
        tile_cmax_kernel<<<dim3((unsigned)ntiles, (unsigned)((nrhs + 127) / 128)), 128, 0, st>>>(
            A.d_xterms, A.d_tile_begin, ntiles, texp, S->xexp, nrhs, cmax);
        note_launch();
        launch_expand_tb<NSR, DR>(p, A, S->pool, S->stride, S->exps, ts, tstride, texp, S->xs, m, S->xexp, nrhs,
                                  true, B, ldb, true, R, ldr, st, A.d_rmax, cmax);
        DG_CUDA(cudaGetLastError());
    }
    return 0;
}

// -------------------------------------------------- mixed inner solve
// Tensor-core capacitance: per level, the nodes whose two blocks both have
// rank 128 get K^-1 (256 x 256, FP64) cut into 8 exact slices with row
// exponents; K^-1 [T1; T2] is then two output tiles of 128 rows (the W of
// the ne and of the sw block, ld 128, at T offset * nrhs), each the sum of
// two terms K^-1[tile, 0:128] T1 + K^-1[tile, 128:256] T2 with the T slices'
// own column exponents -- the multi-term expand, products exact, one
// rounding per output (at least FP64 accuracy).  Other nodes stay on the
// FP64 kernel.
static int build_tc_caps(Plan *p, MixedSliced *M, Fact *F, cudaStream_t st)
{
    const int nlev = (int)F->lv.size();
    M->capsched.assign(nlev, SSchedule());
    M->capfb.assign(nlev, std::vector<CapItem>());
    M->d_capfb.assign(nlev, nullptr);
    std::vector<RSliceJob> kj;
    std::vector<int> kb;
    long long kel = 0;
    int krows = 0, kexp = 0, rc;
    for (int l = 0; l < nlev; ++l) {
        const SSchedule &S = M->level[l];
        std::unordered_map<long long, int> ridx;          // T offset -> reduce index of the level
        for (size_t i = 0; i < S.reduces.size(); ++i) ridx[S.reduces[i].t] = (int)i;
        SSchedule &CS = M->capsched[l];
        CS.tile_m = tc2::M;
        for (const CapItem &c : F->lv[l].n.caps) {
            const auto i1 = ridx.find(c.t1), i2 = ridx.find(c.t2);
            if (c.r1 != tc2::M || c.r2 != tc2::M || i1 == ridx.end() || i2 == ridx.end()) {
                M->capfb[l].push_back(c);
                continue;
            }
            kj.push_back(RSliceJob{c.k, kel, 2 * tc2::M, 2 * tc2::M, 2 * tc2::M, 2 * tc2::M / 16, kexp});
            kb.push_back(krows);
            krows += 2 * tc2::M;
            for (int t = 0; t < 2; ++t) {
                CS.tile_row0.push_back((int)(t == 0 ? c.t1 : c.t2));
                CS.tile_begin.push_back((int)CS.xterms.size());
                const long long a = kel + (long long)t * 16 * kTbA;
                CS.xterms.push_back(XTerm{a, S.reduces[i1->second].tpad, tc2::M, kexp + t * tc2::M, 0, i1->second});
                CS.xterms.push_back(XTerm{a + 8 * kTbA, S.reduces[i2->second].tpad, tc2::M, kexp + t * tc2::M, 0,
                                          i2->second});
            }
            kel += 2LL * 16 * kTbA;
            kexp += 2 * tc2::M;
        }
        CS.tile_begin.push_back((int)CS.xterms.size());
        if ((rc = upload_tb(CS, &M->bytes))) return rc;
        if ((rc = dev_vec(M->capfb[l], &M->d_capfb[l], &M->bytes))) return rc;
    }
    if (kj.empty()) return 0;
    M->kstride = al32(kel);
    if (dev_malloc((void **)&M->kslices, (size_t)kNS * M->kstride * sizeof(bf16)) != cudaSuccess)
        return fail(DPLR_GPU_ENOMEM, "mixed solve: cannot allocate capacitance slices");
    M->bytes += (long long)kNS * M->kstride * 2;
    if ((rc = dev_vec(std::vector<int>(kexp, 0), &M->kexps, &M->bytes))) return rc;
    RSliceJob *d_kj = nullptr;
    int *d_kb = nullptr;
    long long tmp = 0;
    if ((rc = dev_vec(kj, &d_kj, &tmp)) || (rc = dev_vec(kb, &d_kb, &tmp))) return rc;
    slice_r_tb_kernel<kNS><<<(krows + 127) / 128, 128, 0, st>>>(d_kj, d_kb, (int)kj.size(), krows, F->kpool,
                                                               M->kslices, M->kstride, M->kexps);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_kj);
    cudaFree(d_kb);
    if (e != cudaSuccess) return fail(DPLR_GPU_ECUDA, "capacitance slicing: %s", cudaGetErrorString(e));
    return tb_attrs<kNS, kD>();
}

template <int NS>
static int mixed_build_tb_t(Plan *p, MixedSliced *M, Fact *F, cudaStream_t st)
{
    const int m = p->m;
    const int nlev = (int)F->lv.size();
    std::vector<int> ev_off(p->lr.size()), ez_off(nlev), el_off(p->leaves.size());
    int nexp = 0;
    for (size_t b = 0; b < p->lr.size(); ++b) {
        ev_off[b] = nexp;
        nexp += p->lr[b].rank;
    }
    for (int l = 0; l < nlev; ++l) {
        ez_off[l] = nexp;
        nexp += m;
    }
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        el_off[i] = nexp;
        nexp += p->leaves[i].b;
    }
    VLayout VL;
    std::vector<std::array<long long, 4>> vdst;
    std::vector<std::array<int, 4>> vnr;
    long long el = layout_v(p, vdst, vnr, 0, ev_off, VL, true);
    std::vector<long long> za(nlev, 0), la(p->leaves.size(), 0);
    std::vector<int> nkbw(nlev, 0);
    std::vector<RSliceJob> zj, lj;
    std::vector<int> zb, lb;
    int zr = 0, lr = 0;
    for (int l = 0; l < nlev; ++l) {
        const int w = F->lv[l].width;
        nkbw[l] = (w + 15) / 16;
        za[l] = el;
        el += (long long)(m / tc2::M) * nkbw[l] * kTbA;
        if (w == 0) continue;
        zb.push_back(zr);
        zj.push_back(RSliceJob{F->zoff[l], za[l], m, m, w, nkbw[l], ez_off[l]});
        zr += m;
    }
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        const LeafDesc &L = p->leaves[i];
        la[i] = el;
        el += (long long)(L.b / tc2::M) * (L.b / 16) * kTbA;
        lb.push_back(lr);
        lj.push_back(RSliceJob{F->leafoff[i], la[i], L.b, L.b, L.b, L.b / 16, el_off[i]});
        lr += L.b;
    }
    M->stride = al32(std::max<long long>(el, 1));
    if (dev_malloc((void **)&M->pool, (size_t)NS * M->stride * sizeof(bf16)) != cudaSuccess)
        return fail(DPLR_GPU_ENOMEM, "mixed solve: cannot allocate slices");
    M->bytes += (long long)NS * M->stride * 2;
    DG_CUDA(cudaMemsetAsync(M->pool, 0, (size_t)NS * M->stride * sizeof(bf16), st));
    int rc;
    if ((rc = dev_vec(std::vector<int>(std::max(nexp, 1), 0), &M->exps, &M->bytes))) return rc;
    {
        VSliceJob *d_vj = nullptr;
        RSliceJob *d_zj = nullptr, *d_lj = nullptr;
        int *d_vb = nullptr, *d_zb = nullptr, *d_lb = nullptr;
        long long tmp = 0;
        if ((rc = dev_vec(VL.jobs, &d_vj, &tmp)) || (rc = dev_vec(VL.col_base, &d_vb, &tmp)) ||
            (rc = dev_vec(zj, &d_zj, &tmp)) || (rc = dev_vec(zb, &d_zb, &tmp)) || (rc = dev_vec(lj, &d_lj, &tmp)) ||
            (rc = dev_vec(lb, &d_lb, &tmp)))
            return rc;
        if (VL.ncols > 0) {
            slice_v_tb_kernel<NS><<<VL.ncols, 256, 0, st>>>(d_vj, d_vb, (int)VL.jobs.size(), p->pool, M->pool,
                                                           M->stride, M->exps);
            note_launch();
        }
        if (zr > 0) {
            slice_r_tb_kernel<NS><<<(zr + 127) / 128, 128, 0, st>>>(d_zj, d_zb, (int)zj.size(), zr, F->zpool,
                                                                   M->pool, M->stride, M->exps);
            note_launch();
        }
        if (lr > 0) {
            slice_r_tb_kernel<NS><<<(lr + 127) / 128, 128, 0, st>>>(d_lj, d_lb, (int)lj.size(), lr, F->leafinv,
                                                                   M->pool, M->stride, M->exps);
            note_launch();
        }
        cudaError_t e2 = cudaGetLastError();
        if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(st);
        cudaFree(d_vj);
        cudaFree(d_vb);
        cudaFree(d_zj);
        cudaFree(d_zb);
        cudaFree(d_lj);
        cudaFree(d_lb);
        if (e2 != cudaSuccess) return fail(DPLR_GPU_ECUDA, "mixed slicing: %s", cudaGetErrorString(e2));
    }
    // W tile-block offsets over all blocks (per 64-column rhs tile)
    std::vector<long long> tpre(p->lr.size(), 0);
    long long tp = 0;
    for (size_t b = 0; b < p->lr.size(); ++b) {
        tpre[b] = tp;
        tp += (long long)((p->lr[b].rank + 15) / 16) * kTbB;
    }
    M->t_per_rhs = p->total_rank;
    M->tpad_per_rhs = tp;             // per 64-column tile
    M->nblocks = (int)p->lr.size();
    M->level.resize(nlev);
    for (int l = 0; l < nlev; ++l) {
        SSchedule &S = M->level[l];
        S.tile_m = tc2::M;
        S.tpre = tp;
        long long poff = 0;
        for (int b : F->lv[l].blocks) {
            const LRDesc &L = p->lr[b];
            if (L.rank == 0) continue;
            panel_items(L, vdst[b], vnr[b], poff, S.pitems, kInnerChunk);
            const int nch = (L.n + kInnerChunk - 1) / kInnerChunk;
            const int ridx = (int)S.reduces.size();
            S.reduces.push_back(SReduceItem{poff, L.toff, -1, L.rank, nch, ev_off[b], pad16(L.rank), tpre[b]});   // sig in V
            poff += (long long)nch * L.rank;
            S.max_rank = std::max(S.max_rank, L.rank);
            for (int t0 = L.row0; t0 < L.row0 + L.n; t0 += tc2::M) {
                S.tile_row0.push_back(t0);
                S.tile_begin.push_back((int)S.xterms.size());
                S.xterms.push_back(XTerm{za[l] + (long long)(t0 / tc2::M) * nkbw[l] * kTbA, tpre[b], L.rank,
                                         ez_off[l] + t0, 0, ridx});
            }
        }
        S.tile_begin.push_back((int)S.xterms.size());
        S.partial_per_rhs = poff;
        S.t_per_rhs = p->total_rank;
        if ((rc = upload_tb(S, &M->bytes))) return rc;
    }
    if (M->tc_caps && (rc = build_tc_caps(p, M, F, st))) return rc;
    SSchedule &LS = M->leaf;
    LS.tile_m = tc2::M;
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        const LeafDesc &L = p->leaves[i];
        for (int t0 = L.row0; t0 < L.row0 + L.b; t0 += tc2::M) {
            LS.tile_row0.push_back(t0);
            LS.tile_begin.push_back((int)LS.xterms.size());
            LS.xterms.push_back(XTerm{la[i] + (long long)((t0 - L.row0) / tc2::M) * (L.b / 16) * kTbA, L.row0 / 16,
                                      L.b, el_off[i] + (t0 - L.row0), 1, -1});
        }
    }
    LS.tile_begin.push_back((int)LS.xterms.size());
    if ((rc = upload_tb(LS, &M->bytes))) return rc;
    if ((rc = ensure_err_flag(p))) return rc;
    return tb_attrs<NS, NS + 1>();
}

template <int NS>
static int mixed_solve_tb(Plan *p, MixedSliced *M, Fact *F, int nrhs, const double *B, int ldb, double *X, int ldx,
                          cudaStream_t st)
{
    constexpr int D = NS + 1;
    const int m = p->m;
    const int njt = (nrhs + 63) / 64;
    // scratch: partials, DD T, W, W slices, W exponents
    auto r256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
    long long part = 0;
    for (const SSchedule &L : M->level) part = std::max(part, L.partial_per_rhs);
    size_t maxred = 1;
    for (const SSchedule &L : M->level) maxred = std::max(maxred, L.reduces.size());
    const size_t part_bytes = r256((size_t)part * nrhs * sizeof(__int128));
    const size_t t_bytes = r256((size_t)2 * M->t_per_rhs * nrhs * sizeof(double));
    const size_t w_bytes = r256((size_t)M->t_per_rhs * nrhs * sizeof(double));
    const long long wstride = M->tpad_per_rhs * njt;
    const size_t ws_bytes = r256((size_t)NS * wstride * sizeof(bf16));
    const size_t we_bytes = r256(maxred * nrhs * sizeof(int));
    // tensor-core capacitance: T in 8 slices and their exponents
    const bool tcc = M->tc_caps && M->kslices;
    const long long tstride8 = M->tpad_per_rhs * njt;
    const size_t t8_bytes = tcc ? r256((size_t)kNS * tstride8 * sizeof(bf16)) : 0;
    const size_t te8_bytes = tcc ? r256(maxred * nrhs * sizeof(int)) : 0;
    const size_t need = part_bytes + t_bytes + w_bytes + ws_bytes + we_bytes + t8_bytes + te8_bytes;
    if (M->work_bytes < need) {
        cudaFree(M->work);
        M->work = nullptr;
        M->work_bytes = 0;
        if (cudaMalloc(&M->work, need) != cudaSuccess) return fail(DPLR_GPU_ENOMEM, "mixed solve: cannot allocate scratch");
        M->work_bytes = need;
    }
    char *base = reinterpret_cast<char *>(M->work);
    __int128 *partials = reinterpret_cast<__int128 *>(base);
    double *T = reinterpret_cast<double *>(base + part_bytes);
    const long long lo_off = M->t_per_rhs * nrhs;
    double *W = reinterpret_cast<double *>(base + part_bytes + t_bytes);
    bf16 *ws = reinterpret_cast<bf16 *>(base + part_bytes + t_bytes + w_bytes);
    int *wexp = reinterpret_cast<int *>(base + part_bytes + t_bytes + w_bytes + ws_bytes);
    bf16 *ts8 = reinterpret_cast<bf16 *>(base + part_bytes + t_bytes + w_bytes + ws_bytes + we_bytes);
    int *texp8 = reinterpret_cast<int *>(base + part_bytes + t_bytes + w_bytes + ws_bytes + we_bytes + t8_bytes);
    const double npairs = pair_count(NS, D);
    int rc;

    // The expand that writes X gathers X's column exponents (into xexp2,
    // while xexp still describes the slices being read), so slicing X for the
    // next level needs no exponent pass over it.
    const bool gather = nrhs <= tc2::kColCap;
    if (gather && M->xexp2_n < (size_t)nrhs) {
        cudaFree(M->xexp2);
        M->xexp2 = nullptr;
        M->xexp2_n = 0;
        if (dev_malloc((void **)&M->xexp2, nrhs * sizeof(int)) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "mixed solve: cannot allocate exponents");
        M->xexp2_n = nrhs;
    }
    auto start_gather = [&]() {
        if (!gather) return;
        xcol_init_kernel<<<(nrhs + 255) / 256, 256, 0, st>>>(M->xexp2, nrhs);
        note_launch();
    };
    auto end_gather = [&]() {
        if (!gather) return;
        std::swap(M->xexp, M->xexp2);
        std::swap(M->xexp_n, M->xexp2_n);
    };

    // leaf step: X = Leaf^-1 B
    {
        ProfScope ps("mixed_slice_x", st, 0.0, (8.0 + 2.0 * NS) * m * nrhs);
        if ((rc = slice_x_tb<NS>(B, m, ldb, nrhs, M->xs, M->xs_elems, M->xexp, M->xexp_n, st))) return rc;
        start_gather();
    }
    {
        const SSchedule &LS = M->leaf;
        double fl = 0;
        for (const XTerm &t : LS.xterms) fl += 2.0 * tc2::M * t.K * nrhs;
        ProfScope ps("mixed_expand", st, fl * npairs, 0.0);
        launch_expand_tb<NS, D>(p, LS, M->pool, M->stride, M->exps, ws, wstride, wexp, M->xs, m, M->xexp, nrhs, false,
                                nullptr, 0, false, X, ldx, st, nullptr, nullptr, gather ? M->xexp2 : nullptr);
        DG_CUDA(cudaGetLastError());
        end_gather();
    }
    for (int l = (int)M->level.size() - 1; l >= 0; --l) {
        const SSchedule &S = M->level[l];
        if (S.pitems.empty()) continue;
        {
            ProfScope ps("mixed_slice_x", st, 0.0, (8.0 + 2.0 * NS) * m * nrhs);
            if ((rc = slice_x_tb<NS>(X, m, ldx, nrhs, M->xs, M->xs_elems, M->xexp, M->xexp_n, st, gather)))
                return rc;
        }
        double fl = 0;
        for (const PItem &it : S.pitems) fl += 2.0 * it.nkb * 16 * std::min(64, it.rank - it.kt) * nrhs;
        {
            ProfScope ps("mixed_panel", st, fl * npairs, 0.0);
            launch_panel_tb<NS, D>(p, S, M->pool, M->stride, M->xs, m, nrhs, partials, st);
        }
        {
            ProfScope ps("mixed_reduce", st, 0.0, 0.0);
            launch_reduce<D>(S, partials, M->exps, M->xexp, p->pool, nrhs, T, lo_off, st);
            DG_CUDA(cudaGetLastError());
        }
        if (tcc && !M->capsched[l].xterms.empty()) {
            // W = K^-1 [T1; T2] on the tensor cores for the rank-128 nodes
            {
                ProfScope ps("mixed_tslice", st, 0.0, 0.0);
                tslice_tb_kernel<kNS><<<dim3((unsigned)S.reduces.size(), (unsigned)njt), 256, 0, st>>>(
                    S.d_reduces, (int)S.reduces.size(), T, lo_off, nrhs, njt, ts8, tstride8, texp8);
                note_launch();
            }
            {
                const SSchedule &CS = M->capsched[l];
                const double fc = 2.0 * tc2::M * tc2::M * nrhs * (double)CS.xterms.size() * pair_count(kNS, kD);
                ProfScope ps("capacitance_tc", st, fc, 0.0);
                launch_expand_tb<kNS, kD>(p, CS, M->kslices, M->kstride, M->kexps, ts8, tstride8, texp8, M->xs, m,
                                          M->xexp, nrhs, false, nullptr, 0, false, W, tc2::M, st, nullptr, nullptr,
                                          nullptr, nrhs);
                DG_CUDA(cudaGetLastError());
            }
            if ((rc = run_cap_list(M->capfb[l], M->d_capfb[l], F->kpool, nullptr, 0, T, W, nrhs, st))) return rc;
        } else if ((rc = run_caps(F->lv[l].n, F->kpool, nullptr, 0, T, W, nrhs, st))) {
            return rc;
        }
        {
            ProfScope ps("mixed_tslice", st, 0.0, 0.0);
            tslice_tb_kernel<NS><<<dim3((unsigned)S.reduces.size(), (unsigned)njt), 256, 0, st>>>(
                S.d_reduces, (int)S.reduces.size(), W, -1, nrhs, njt, ws, wstride, wexp);
            note_launch();
            start_gather();
        }
        double fu = 0;
        for (const XTerm &t : S.xterms) fu += 2.0 * tc2::M * t.K * nrhs;
        ProfScope ps2("mixed_expand", st, fu * npairs, 0.0);
        launch_expand_tb<NS, D>(p, S, M->pool, M->stride, M->exps, ws, wstride, wexp, M->xs, m, M->xexp, nrhs, true, X,
                                ldx, true, X, ldx, st, nullptr, nullptr, gather ? M->xexp2 : nullptr);
        DG_CUDA(cudaGetLastError());
        end_gather();
    }
    return 0;
}


}  // namespace dg
