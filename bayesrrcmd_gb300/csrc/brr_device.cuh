// Device-side helpers shared by the packer and sweep kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace brr {

constexpr int kThreads = 256;          // threads per CTA of every kernel
constexpr int kMaxSpec = 64;           // largest number of markers resolved per grid round
constexpr int kMaxGroups = 64;
constexpr int kMaxK = 16;
constexpr int kChunk = 64;             // individuals per 16-byte code chunk

__host__ __device__ __forceinline__ int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ __forceinline__ int64_t imax64(int64_t a, int64_t b) { return a > b ? a : b; }

// Status codes written by kernels into the context's error word.
constexpr int kDevOk = 0;
constexpr int kDevTimeout = 1;
constexpr int kDevRange = 2;

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_add_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void red_add_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void red_add_u32(unsigned *p, unsigned v)
{
    asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t global_timer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// cp.async (Ampere-style LDGSTS) 16-byte copy global -> shared, L2-only caching.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
// cp.async 4-byte copy global -> shared (L1-allocating form, the only one for 4 bytes).
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
// cp.async 8-byte copy global -> shared.
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Exact fixed-point exchange.  A partial sum is converted with integer
// operations only into a 128-bit integer X = value * 2^60 (truncated below
// 2^-60), split as X = hi * 2^56 + lo with 0 <= lo < 2^56, and the two words
// are added with 64-bit integer atomics: the sum over CTAs is exact and does
// not depend on the order of arrival.  Values must satisfy |value| < 2^41.
struct Fx {
    long long hi;
    unsigned long long lo;
};

__device__ __forceinline__ bool fx_from_double(double p, __int128 &x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(p);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e == 0) {            // zero or subnormal: below the grid
        x = 0;
        return true;
    }
    if (e >= 1023 + 41)      // out of range (also inf / nan)
        return false;
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = e - 1015; // value * 2^60 = m * 2^(e - 1075 + 60)
    __int128 v;
    if (sh >= 0)
        v = (__int128)m << sh;
    else if (sh > -64)
        v = (__int128)(m >> (-sh));
    else
        v = 0;
    x = (b >> 63) ? -v : v;
    return true;
}

__device__ __forceinline__ bool fx_from_float(float f, __int128 &x)
{
    const unsigned b = __float_as_uint(f);
    const int e = (int)((b >> 23) & 0xFF);
    if (e == 0) {
        x = 0;
        return true;
    }
    if (e >= 127 + 41)
        return false;
    const unsigned long long m = (b & 0x7FFFFFu) | 0x800000u;
    const int sh = e - 90;   // value * 2^60 = m * 2^(e - 150 + 60)
    __int128 v;
    if (sh >= 0)
        v = (__int128)m << sh;
    else if (sh > -64)
        v = (__int128)(m >> (-sh));
    else
        v = 0;
    x = (b >> 31) ? -v : v;
    return true;
}

__device__ __forceinline__ Fx fx_split(__int128 x)
{
    Fx f;
    f.lo = (unsigned long long)(x & (((__int128)1 << 56) - 1));
    f.hi = (long long)(x >> 56);
    return f;
}

// sum = hi * 2^-4 + lo * 2^-60 with lo < 2^64, evaluated with exact partial
// conversions and two roundings.
__host__ __device__ __forceinline__ double fx_join(long long hi, unsigned long long lo)
{
    const double a = (double)hi * 0.0625;
    const double b = (double)(lo >> 32) * 3.7252902984619140625e-09;      // 2^-28
    const double c = (double)(lo & 0xFFFFFFFFull) * 8.673617379884035e-19; // 2^-60
    return a + (b + c);
}

// Error-free transformation a + b = s + e (Knuth TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Double-float addition (hi, lo) += (bh, bl), renormalised.
__device__ __forceinline__ void df_add(float &hi, float &lo, float bh, float bl)
{
    float s, e;
    two_sum(hi, bh, s, e);
    e = __fadd_rn(e, __fadd_rn(lo, bl));
    hi = __fadd_rn(s, e);
    lo = __fsub_rn(e, __fsub_rn(hi, s));
}

// Split an FP64 value into a normalised double-float pair.
__device__ __forceinline__ void df_from_double(double v, float &hi, float &lo)
{
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
}

// Double-float product (ah, al) * (bh, bl): exact product of the high words by
// FMA, cross terms added once, renormalised (relative error below 2^-44).
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float &h, float &l)
{
    const float p = __fmul_rn(ah, bh);
    const float e = __fmaf_rn(ah, bh, -p);
    const float t = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, e));
    h = __fadd_rn(p, t);
    l = __fsub_rn(t, __fsub_rn(h, p));
}

// Fixed-point sum (hi, lo) (value hi * 2^-4 + lo * 2^-60; lo is an unsigned
// 64-bit sum of 56-bit parts) to a double-float pair with integer operations
// only: the 128-bit value is assembled with its carry, the magnitude is
// normalised by a leading-zero count and its top 48 bits become two exact
// floats (truncation, relative error below 2^-47).
__device__ __forceinline__ void fx_to_df(long long hi, unsigned long long lo, float &h, float &l)
{
    // X = hi * 2^56 + lo as (xh, xl) = (X >> 64, X mod 2^64)
    unsigned long long xl = ((unsigned long long)hi << 56) + lo;
    unsigned long long xh = (unsigned long long)(hi >> 8) + (xl < lo ? 1ull : 0ull);
    const bool neg = (long long)xh < 0;
    if (neg) {
        xl = ~xl + 1ull;
        xh = ~xh + (xl == 0ull ? 1ull : 0ull);
    }
    if ((xh | xl) == 0ull) {
        h = l = 0.f;
        return;
    }
    const int lz = xh ? __clzll((long long)xh) : 64 + __clzll((long long)xl);
    unsigned long long th;
    if (lz >= 64)
        th = xl << (lz - 64);
    else if (lz == 0)
        th = xh;
    else
        th = (xh << lz) | (xl >> (64 - lz));
    const unsigned m1 = (unsigned)(th >> 40);              // top 24 bits (bit 23 set)
    const unsigned m2 = (unsigned)(th >> 16) & 0xFFFFFFu;  // next 24 bits
    // bit 127 of the normalised magnitude weighs 2^(67 - lz); m1's lowest bit 2^(44 - lz)
    const int e1 = 44 - lz;
    const float s1 = __int_as_float((e1 + 127) << 23);
    const float s2 = __int_as_float((e1 - 24 + 127) << 23);
    h = __fmul_rn(__uint2float_rn(m1), s1);
    l = __fmul_rn(__uint2float_rn(m2), s2);
    if (neg) {
        h = -h;
        l = -l;
    }
}

}  // namespace brr
