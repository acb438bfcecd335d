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
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Exact split of an FP64 value into two integers on fixed grids 2^-20 and
// 2^-60, so that a sum over CTAs is an exact, order-independent integer sum.
// Valid for |p| < 2^41; returns false otherwise.
__device__ __forceinline__ bool fixed_split(double p, long long *hi, long long *lo)
{
    if (!(fabs(p) < 2199023255552.0))
        return false;
    const double ph = rint(p * 1048576.0);
    const double rem = p - ph * (1.0 / 1048576.0);
    const double pl = rint(rem * 1152921504606846976.0);
    *hi = (long long)ph;
    *lo = (long long)pl;
    return true;
}

__device__ __forceinline__ double fixed_join(long long hi, long long lo)
{
    return (double)hi * (1.0 / 1048576.0) + (double)lo * (1.0 / 1152921504606846976.0);
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

}  // namespace brr
