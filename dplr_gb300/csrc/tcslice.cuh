// tcslice.cuh -- tcgen05 building blocks shared by the exact-slice product
// kernels of tcpipe.cuh: tile shape, tensor-memory sizing, mbarrier and
// tcgen05 fences, commit and load waits, and the exact integer arithmetic of
// the read-out (FP32 accumulator -> int64, 128-bit shifts, 128-bit integer
// -> FP64 rounded to nearest).
//
// The slice arithmetic: products of 7-bit slices summed over at most 256
// inner elements stay below 2^24, so each slice diagonal's FP32 accumulator
// holds an exact integer when it is read out of tensor memory.
#pragma once

#include <cstdint>

namespace dg {
namespace tc {

constexpr int M = 128;          // tile rows (TMEM lanes)
constexpr int N = 64;           // tile columns (right-hand sides)

// Tensor-memory columns allocated for D - 1 diagonals of N columns (a power
// of two >= 32, as tcgen05.alloc requires).
__host__ __device__ constexpr int tmem_cols(int D)
{
    return (D - 1) * N <= 32 ? 32 : (D - 1) * N <= 64 ? 64 : (D - 1) * N <= 128 ? 128
         : (D - 1) * N <= 256 ? 256 : 512;
}

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *b, int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count));
}

__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}

__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

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

__device__ __forceinline__ void record_error(int *err, int code)
{
    if (err) atomicCAS(err, 0, code);
}

}  // namespace tc
}  // namespace dg
