// Batched Gibbs sweeps of C chains on shared genotypes, with the dot products
// and the residual updates on the tensor cores (tcgen05, kind::f16).
//
// Reference semantics per chain: BayesRBase::processColumn over the dense
// kernel (src/BayesRBase.cpp:287-392, src/densebayesrkernel.cpp:10-20), every
// chain visiting the markers in one shared order (any scan order is a valid
// Gibbs sweep; the per-marker draws u, z stay per chain).
//
// Layout.  Individuals are cut into G slices (one CTA each, a multiple of 16
// individuals per slice).  For a block of 32 markers every CTA holds:
//   g   : the block's genotypes over its slice, FP16, [marker t][individual i]
//         in the no-swizzle K-major core-matrix layout (8 rows x 16 bytes);
//   E   : all chains' residuals over the slice as exact fixed point
//         E = eps * 2^40, four balanced 11-bit limbs per value, FP16, rows
//         r = 4*chain + limb, stored MN-major (8 consecutive rows in 16 bytes);
//   W   : the block's update coefficients, FP16 limbs, [row r][marker t].
// Tensor-core products (all partial sums are integers below 2^24, exact in FP32):
//   dots   D1[r][t] = sum_i E[r][i] * g[t][i]      (M = 128 rows per tile, N = 32)
//   Gram   P[t'][t] = sum_i g[t'][i] * g[t][i]     (integer block Gram)
//   update D2[i][r] = sum_t g[t][i] * W[r][t]      (M = 128 individuals, N = 4C)
// Per block:
//   1. every CTA computes D1 and P over its slice and adds them, as exact
//      integers, into global accumulators; grid barrier 1;
//   2. one warp per chain resolves the 32 markers in order: lane t samples
//      marker t from num_t = sigma_t (dot_t - colmean_t * sum(E)) 2^-40 +
//      beta_old (N-1) (FP64; the component is decided in FP32 with a
//      rigorous error bound and in FP64 whenever the bound cannot certify it,
//      so the decisions are the FP64 ones; acum is kept to FP32 precision);
//      when marker p changes, the later markers' dots
//      move by W_p P[p][t] - C_p S_t exactly (W_p = round(dBeta sigma_p 2^40),
//      C_p = round(dBeta sigma_p colmean_p 2^40)); grid barrier 2;
//   3. every CTA applies E_i += sum_p W_p g_p[i] - sum_p C_p through D2 and
//      renormalises the limbs.
// Every wait is bounded (timeout -> error word, the CTAs leave, TMEM freed).
#include <cuda_fp16.h>

#include "brr_internal.h"
#include "brr_device.cuh"
#include "brr_pick.cuh"
#include "brr_stream.h"

namespace brr {
namespace {

constexpr int kBT = 256;               // threads per CTA
constexpr int kBW = kBT / 32;
static_assert(kBW == 8, "the update pass deals tiles to two groups of four warps");
constexpr int kTmemCols = 512;
constexpr int kCounterGap = 32;        // words between the two barrier counters
constexpr long long kLimbHalf = 1024;  // balanced limbs in [-1024, 1023]
constexpr unsigned kMinSmemPerCta = 116u * 1024u;

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle: start address, leading-dimension
// byte offset (the stride between core matrices along K) and stride-dimension
// byte offset (the stride between core matrices along M or N).
__device__ __forceinline__ uint64_t smem_desc(unsigned addr, unsigned lbo, unsigned sbo)
{
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16 with FP16 operands and FP32 accumulation.
__device__ __forceinline__ uint32_t idesc_f16(int M, int N, bool a_mn)
{
    return (1u << 4) | ((a_mn ? 1u : 0u) << 15) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(unsigned d_tmem, uint64_t a, uint64_t b, uint32_t idesc, unsigned accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                 "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
                 : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 consecutive TMEM columns of this warp's 32 lanes.
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                   "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                   "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k)
        v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void mbar_init1(uint64_t *m)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(m)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_done(uint64_t *m, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_addr(m)), "r"(parity)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *m, unsigned parity, uint64_t timeout_ns)
{
    if (mbar_done(m, parity))
        return true;
    const uint64_t t0 = global_timer_ns();
    unsigned spins = 0;
    while (!mbar_done(m, parity)) {
        if ((++spins & 63u) == 0 && global_timer_ns() - t0 > timeout_ns)
            return false;
    }
    return true;
}

__device__ __forceinline__ bool counter_wait(const unsigned long long *c, unsigned long long target, const int *err,
                                             uint64_t timeout_ns)
{
    if (ld_acquire_u64(c) >= target)
        return true;
    const uint64_t t0 = global_timer_ns();
    unsigned spins = 0;
    while (ld_acquire_u64(c) < target) {
        if ((++spins & 255u) == 0) {
            if (*(volatile const int *)err != kDevOk || global_timer_ns() - t0 > timeout_ns)
                return false;
        }
    }
    return true;
}

// Balanced radix-2^11 digits of x: x = sum_l d_l 2^(11 l), d_l in [-1024, 1023].
// Returns false when x needs more than four digits.
__device__ __forceinline__ bool split4(long long x, int (&d)[kBatchLimbs])
{
#pragma unroll
    for (int l = 0; l < kBatchLimbs - 1; ++l) {
        const long long r = ((x + kLimbHalf) & 2047) - kLimbHalf;
        d[l] = (int)r;
        x = (x - r) >> 11;
    }
    d[kBatchLimbs - 1] = (int)x;
    return x >= -kLimbHalf && x < kLimbHalf;
}

__device__ __forceinline__ long long join4(const int (&d)[kBatchLimbs])
{
    long long x = d[kBatchLimbs - 1];
#pragma unroll
    for (int l = kBatchLimbs - 2; l >= 0; --l)
        x = x * 2048 + d[l];
    return x;
}

// floor(v / 2048 + 1/2) of an integer-valued float |v| < 2^21 (the carry that
// brings a limb into [-1024, 1023]): y = v / 2048 + 1/2 has a fraction that is
// a multiple of 2^-11, so floor(y) is the nearest integer to y - 1/2 + 2^-12 =
// v / 2048 + 2^-12, formed exactly by one FMA and rounded by adding and
// removing 1.5 * 2^23.
__device__ __forceinline__ float limb_carry(float v)
{
    const float q = __fmaf_rn(v, 1.f / 2048.f, 1.f / 4096.f);
    return __fsub_rn(__fadd_rn(q, 12582912.f), 12582912.f);
}

__device__ __forceinline__ unsigned short h_bits(int v) { return __half_as_ushort(__int2half_rn(v)); }
__device__ __forceinline__ int h_int(unsigned short b) { return __half2int_rn(__ushort_as_half(b)); }

// Genotype of a 2-bit BED code {0: 2, 1: missing, 2: 1, 3: 0}.
__device__ __forceinline__ unsigned short g_half(unsigned code)
{
    // FP16 bit patterns of 2.0, 0.0 (missing genotypes are rejected before), 1.0, 0.0
    return code == 0u ? (unsigned short)0x4000 : (code == 2u ? (unsigned short)0x3C00 : (unsigned short)0);
}

struct BatchPlan {
    unsigned off_g, off_e, off_w, off_codes, off_p, total;
    int nres;            // resolver warps per CTA (chains per CTA, at most 8)
    unsigned sbo_g;      // stride between 8-marker groups of g (= kext/8 * 128)
    unsigned lbo_e;      // stride between 8-individual groups of E (= R/8 * 128)
};

__host__ __device__ inline BatchPlan batch_plan(int C, int kext, int G)
{
    BatchPlan p;
    p.nres = (C + G - 1) / G;
    if (p.nres > kBW)
        p.nres = kBW;
    const unsigned R = 4u * (unsigned)C;
    p.sbo_g = (unsigned)(kext / 8) * 128u;
    p.lbo_e = (R / 8u) * 128u;
    p.off_g = 0;
    p.off_e = p.off_g + 32u * (unsigned)kext * 2u;
    p.off_w = p.off_e + R * (unsigned)kext * 2u;
    p.off_codes = p.off_w + R * 32u * 2u;
    p.off_p = p.off_codes + 32u * (unsigned)(kext / 4);
    p.total = p.off_p + (unsigned)p.nres * kBatchBlock * 33u * 4u;
    p.total = (p.total + 1023u) & ~1023u;
    // every CTA allocates all 512 TMEM columns and waits at grid barriers, so
    // no two CTAs may share an SM: at least half the SM's shared memory each
    if (p.total < kMinSmemPerCta)
        p.total = kMinSmemPerCta;
    return p;
}

// PROF: the variant that counts phase cycles on CTA 0 (the plain variant reads
// no clock, whose reads would constrain the scheduling of every CTA's code).
template <int KM, bool PROF>
__global__ void __launch_bounds__(kBT, 1) k_sweep_batch(BatchArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t s_mbar;
    __shared__ unsigned s_tmem;
    __shared__ int s_abort;
    __shared__ uint32_t s_j[kBatchBlock];
    __shared__ float s_cl[kBatchMaxChains][kBatchLimbs];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int s = blockIdx.x;
    const int C = a.C, R = 4 * C, MT = R / 128;
    const int kext = a.kext;
    const int lo = a.slice_lo[s];
    const int ns = a.slice_lo[s + 1] - lo;
    const BatchPlan pl = batch_plan(C, kext, a.G);
    uint8_t *g_t = smem + pl.off_g;
    uint8_t *e_t = smem + pl.off_e;
    uint8_t *w_t = smem + pl.off_w;
    uint8_t *s_codes = smem + pl.off_codes;
    int *s_pbuf = reinterpret_cast<int *>(smem + pl.off_p);
    const int nblocks = (int)((a.M + kBatchBlock - 1) / kBatchBlock);
    const int KS = kext / 16;                       // K steps of the dot GEMM
    const int NT = (kext + 127) / 128;              // individual tiles of the update GEMM
    const int TPP = kTmemCols / R;                  // update tiles per TMEM pass
    const double inv2f = 1.0 / (double)(1ll << kBatchFrac);
    unsigned long long *cnt1 = a.counter, *cnt2 = a.counter + kCounterGap;
    long long *prof = (PROF && s == 0) ? a.prof : nullptr;
    long long ph[8] = {0, 0, 0, 0, 0, 0, 0, 0};

    if (tid == 0) {
        s_abort = 0;
        mbar_init1(&s_mbar);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s_tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }

    // ---- residuals of all chains over the slice, with the updateMu shift, as limbs
    for (int idx = tid; idx < (C / 2) * kext; idx += kBT) {
        const int i = idx % kext, cp = idx / kext;
        uint32_t w[4];
        bool ok = true;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int c = 2 * cp + h;
            long long x = 0;
            if (i < ns)
                x = a.E[(size_t)c * a.N + lo + i] + a.dmu[c];
            int d[kBatchLimbs];
            ok = split4(x, d) && ok;
            w[2 * h] = (uint32_t)h_bits(d[0]) | ((uint32_t)h_bits(d[1]) << 16);
            w[2 * h + 1] = (uint32_t)h_bits(d[2]) | ((uint32_t)h_bits(d[3]) << 16);
        }
        if (!ok)
            atomicCAS(a.err, kDevOk, kDevRange);
        *reinterpret_cast<uint4 *>(e_t + (i >> 3) * pl.lbo_e + cp * 128 + (i & 7) * 16) = make_uint4(w[0], w[1], w[2], w[3]);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = s_tmem;
    unsigned mphase = 0;
    const unsigned ug = smem_addr(g_t), ue = smem_addr(e_t), uw = smem_addr(w_t);

    for (int b = 0; b < nblocks; ++b) {
        long long t0 = prof ? clock64() : 0;
        // ---- block records and genotype codes of the slice
        if (tid < kBatchBlock) {
            const int64_t q = (int64_t)b * kBatchBlock + tid;
            s_j[tid] = q < a.M ? a.rec[q].j : 0xFFFFFFFFu;
        }
        __syncthreads();
        const int wpm = kext / 16;                       // 32-bit code words per marker
        const int nw_ok = (ns + 15) / 16;                // words holding individuals of the slice
        for (int idx = tid; idx < kBatchBlock * wpm; idx += kBT) {
            const int t = idx / wpm, w = idx % wpm;
            uint32_t v = 0;
            const uint32_t j = s_j[t];
            if (j != 0xFFFFFFFFu && w < nw_ok)
                v = __ldg(reinterpret_cast<const uint32_t *>(a.codes + (size_t)j * a.col_stride + lo / 4) + w);
            reinterpret_cast<uint32_t *>(s_codes)[t * wpm + w] = v;
        }
        __syncthreads();
        for (int idx = tid; idx < kBatchBlock * (kext / 8); idx += kBT) {
            const int t = idx & 31, ic = idx >> 5;
            const unsigned v = reinterpret_cast<const unsigned short *>(s_codes)[t * (kext / 8) + ic];
            uint32_t w[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const int i0 = ic * 8 + 2 * h;
                const unsigned short g0 = i0 < ns ? g_half((v >> (4 * h)) & 3u) : (unsigned short)0;
                const unsigned short g1 = i0 + 1 < ns ? g_half((v >> (4 * h + 2)) & 3u) : (unsigned short)0;
                w[h] = (uint32_t)g0 | ((uint32_t)g1 << 16);
            }
            *reinterpret_cast<uint4 *>(g_t + (t >> 3) * pl.sbo_g + ic * 128 + (t & 7) * 16) =
                make_uint4(w[0], w[1], w[2], w[3]);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();

        // ---- dots and block Gram on the tensor cores
        if (tid == 0) {
            const uint32_t id_dot = idesc_f16(128, 32, true), id_gram = idesc_f16(128, 32, false);
            for (int mt = 0; mt < MT; ++mt)
                for (int ks = 0; ks < KS; ++ks)
                    umma_f16(tmem + (unsigned)(mt * 32), smem_desc(ue + mt * 2048 + ks * 2 * pl.lbo_e, pl.lbo_e, 128),
                             smem_desc(ug + ks * 256, 128, pl.sbo_g), id_dot, ks > 0);
            // rows 32..127 of the A tile read past the block's genotypes into
            // shared memory that is not part of it; those rows are not used
            for (int ks = 0; ks < KS; ++ks)
                umma_f16(tmem + 64u, smem_desc(ug + ks * 256, 128, pl.sbo_g), smem_desc(ug + ks * 256, 128, pl.sbo_g),
                         id_gram, ks > 0);
            umma_commit(&s_mbar);
        }
        if (!mbar_wait_bounded(&s_mbar, mphase & 1u, a.timeout_ns)) {
            atomicCAS(a.err, kDevOk, kDevTimeout);
            s_abort = 1;
        }
        ++mphase;
        tc_fence_after();
        if (prof)
            ph[0] += clock64() - t0, t0 = clock64();
        // publish: row r = 4c + l of tile mt; lanes 4k..4k+3 hold the limbs of one chain
        if (warp < MT * 4) {
            const int mt = warp >> 2, q4 = warp & 3;
            float f[32];
            tmem_ld32(tmem + ((unsigned)(q4 * 32) << 16) + (unsigned)(mt * 32), f);
            const int l = lane & 3;
            const int c = (mt * 128 + q4 * 32 + lane) >> 2;
            long long v[32];
#pragma unroll
            for (int t = 0; t < 32; ++t)
                v[t] = (long long)(int)f[t] * (1ll << (11 * l));
            const bool up2 = (l & 2) != 0, up1 = (l & 1) != 0;
            long long k16[16], k8[8];
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                const long long send = up2 ? v[k] : v[k + 16];
                const long long keep = up2 ? v[k + 16] : v[k];
                k16[k] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const long long send = up1 ? k16[k] : k16[k + 8];
                const long long keep = up1 ? k16[k + 8] : k16[k];
                k8[k] = keep + __shfl_xor_sync(0xffffffffu, send, 1);
            }
            unsigned long long *acc = a.acc + ((size_t)(s % kBatchCopies) * C + c) * kBatchBlock + 8 * l;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                atomicAdd(acc + k, (unsigned long long)k8[k]);
        }
        if (warp == 0) {
            float f[32];
            tmem_ld32(tmem + 64u, f);
            unsigned *pacc = a.pacc + ((size_t)(b & 1) * kBatchPCopies + (s % kBatchPCopies)) * (kBatchBlock * kBatchBlock) +
                             lane * kBatchBlock;
            for (int t = 0; t < lane; ++t)
                atomicAdd(pacc + t, (unsigned)(int)f[t]);
        }
        tc_fence_before();
        __syncthreads();
        if (tid == 0)
            red_release_add_u64(cnt1, 1ull);
        if (prof)
            ph[1] += clock64() - t0, t0 = clock64();

        // ---- the block's integer Gram (lower triangle), summed over its copies
        // once per CTA into shared memory for all the CTA's chains (the
        // genotypes are shared): row t holds P[t][p] for p < t, 33 words apart.
        // A CTA that resolves chains first waits for every CTA's dot products.
        const int *sP = s_pbuf;
        if (s < C) {
            const long long tw = prof ? clock64() : 0;
            if (tid == 0 && !counter_wait(cnt1, (unsigned long long)(a.G + a.phantom) * (unsigned long long)(b + 1),
                                          a.err, a.timeout_ns)) {
                atomicCAS(a.err, kDevOk, kDevTimeout);
                s_abort = 1;
            }
            __syncthreads();   // orders tid 0's acquire before the loads below
            if (prof)
                ph[4] += clock64() - tw;
            if (!s_abort) {
                const unsigned *pk_base = a.pacc + (size_t)(b & 1) * kBatchPCopies * (kBatchBlock * kBatchBlock);
                for (int e = tid; e < kBatchBlock * kBatchBlock; e += kBT) {
                    const int t = e >> 5, pp = e & 31;
                    if (pp < t) {
                        unsigned v = 0;
#pragma unroll
                        for (int cp = 0; cp < kBatchPCopies; ++cp)
                            v += __ldcg(pk_base + (size_t)cp * (kBatchBlock * kBatchBlock) + e);
                        s_pbuf[t * 33 + pp] = (int)v;
                    }
                }
            }
            __syncthreads();
        }

        // ---- resolve: one warp per chain
        for (int k = warp;; k += kBW) {
            const int c = s + a.G * k;
            if (c >= C || s_abort)
                break;
            const int64_t q = (int64_t)b * kBatchBlock + lane;
            bool done = q >= a.M;
            BatchRec rc{};
            ChainRec cr{0.0, 1.0, 0.0, 0.0};
            if (!done) {
                rc = a.rec[q];
                cr = a.crec[(size_t)c * a.M + q];
            }
            const double bold = cr.beta_old, u = cr.u, z = cr.z;
            const float uf = __double2float_rn(u);
            const int grp = done ? 0 : rc.group;
            const double *gc = a.gconst + ((size_t)c * a.n_groups + grp) * kMaxK * 4;
            const float *gcf = a.gcf + ((size_t)c * a.n_groups + grp) * kMaxK * 2;
            const int K = a.gK[grp];
            const long long tl = prof ? clock64() : 0;
            int steps = 0;
            long long dot = 0;
#pragma unroll
            for (int cp = 0; cp < kBatchCopies; ++cp) {
                unsigned long long *p = a.acc + ((size_t)cp * C + c) * kBatchBlock + lane;
                dot += (long long)ld_relaxed_u64(p);
                *p = 0ull;
            }
            long long sumE = a.sumE[c];
            // num_t from the exact integer dot and residual total, once per
            // block in FP64; then carried as a double-float pair through the
            // block's changes: after marker p changes, num_t moves by
            // dBeta_p x_p.x_t = dBeta_p sigma_p sigma_t (P[p][t] - colmean_t S_p)
            const double num0 = fma(rc.sigma * inv2f, (double)dot,
                                    fma(-rc.sigma * rc.colmean * inv2f, (double)sumE, bold * ((double)a.N - 1.0)));
            float nh, nl, sh, sl, mh, ml, zh, zl, boh, bol;
            df_from_double(num0, nh, nl);
            df_from_double(rc.sigma, sh, sl);
            df_from_double(rc.colmean, mh, ml);
            df_from_double(z, zh, zl);
            df_from_double(bold, boh, bol);
            const float Sf = (float)rc.S;
            const float4 *gdf = a.gdf + ((size_t)c * a.n_groups + grp) * kMaxK;
            float bnh = boh, bnl = bol, acum_f = 0.f;
            double acum_d = 0.0;
            bool acum_is_d = false;
            int fcomp = -1;
            long long Wl = 0, Csum = 0;
            const float two40 = (float)(1ll << kBatchFrac);
            // certified stability margin of the current decision: while num^2
            // moves by Delta with H * Delta <= wmar (H: the spread of the
            // group's h_k, h_0 = 0 included) no cumulative probability crosses
            // u, so a marker is evaluated again only when a correction moves it
            // beyond its margin (the decisions are those of an evaluation at the
            // current num)
            float H = 0.f;
            {
                float hmax = 0.f, hmin = 0.f;
                for (int k = 1; k < K; ++k) {
                    hmax = fmaxf(hmax, gcf[2 * k + 1]);
                    hmin = fminf(hmin, gcf[2 * k + 1]);
                }
                H = (hmax - hmin) * 1.000001f;
            }
            float sref = 0.f, wmar = -1.f;
            int comp = -1;
            bool fbd = false;   // the decision came from the FP64 sampler
            double fb_beta = bold, fb_acum = 0.0;
            for (;; ++steps) {
                const float sx = __fmaf_rn(nh, nh, 2.f * nh * nl);
                const float delta = fabsf(sx - sref) * 1.000001f + 4e-7f * (sx + sref);
                const bool need = !done && !(H * delta <= wmar);
                if (__any_sync(0xffffffffu, need)) {
                    int cm;
                    float w;
                    const bool okm = pick_margin<KM>(sx, uf, gcf, K, cm, w);
                    if (need) {
                        comp = cm;
                        fbd = false;
                        sref = sx;
                        wmar = okm ? w : -1.f;
                    }
                    const bool slow = need && !okm;
                    if (__any_sync(0xffffffffu, slow) && slow) {
                        // 700 guards possibly active or u near a boundary: the
                        // guarded FP32 sampler, then FP64
                        int c2;
                        float a0;
                        if (pick_f32<KM>(nh, nl, uf, gcf, K, c2, a0)) {
                            comp = c2;
                        } else {
                            const Pick pk = pick_marker<false, KM>((double)nh + (double)nl, u, z, bold, gc, K);
                            comp = pk.comp;
                            fb_acum = pk.acum0;
                            fb_beta = pk.beta;
                            fbd = true;
                        }
                    }
                }
                const bool cert = !fbd;
                const bool chg = !done && (bold != 0.0 || comp > 0);
                const unsigned mask = __ballot_sync(0xffffffffu, chg);
                const int p = mask ? __ffs(mask) - 1 : 32;
                if (!done && lane <= p) {
                    // the decision of marker t is final (src/BayesRBase.cpp:346-366)
                    fcomp = comp;
                    if (comp == 0) {
                        bnh = bnl = 0.f;
                    } else if (comp > 0) {
                        if (cert) {
                            const float4 k4 = gdf[comp];   // {sdk hi, lo, invden hi, lo}
                            float ah, al, bh, bl;
                            df_mul(zh, zl, k4.x, k4.y, ah, al);
                            df_mul(nh, nl, k4.z, k4.w, bh, bl);
                            df_add(ah, al, bh, bl);
                            bnh = ah;
                            bnl = al;
                        } else {
                            df_from_double(fb_beta, bnh, bnl);
                        }
                    }
                    acum_is_d = !cert;
                    acum_d = fb_acum;
                    done = true;
                }
                if (!mask)
                    break;
                // marker p's update: dBeta sigma_p (double-float) and the exact
                // fixed-point coefficients W_p = round(dBeta sigma_p 2^40),
                // C_p = round(dBeta sigma_p colmean_p 2^40)
                float uh = 0.f, ul = 0.f;
                long long Wp = 0, Cp = 0;
                if (lane == p) {
                    float dh = boh, dl = bol;
                    df_add(dh, dl, -bnh, -bnl);
                    df_mul(dh, dl, sh, sl, uh, ul);
                    float ch, cl;
                    df_mul(uh, ul, mh, ml, ch, cl);
                    Wp = __float2ll_rn(__fmul_rn(uh, two40)) + __float2ll_rn(__fmul_rn(ul, two40));
                    Cp = __float2ll_rn(__fmul_rn(ch, two40)) + __float2ll_rn(__fmul_rn(cl, two40));
                    Wl = Wp;
                }
                uh = __shfl_sync(0xffffffffu, uh, p);
                ul = __shfl_sync(0xffffffffu, ul, p);
                const float Sp = __shfl_sync(0xffffffffu, Sf, p);
                Wp = __shfl_sync(0xffffffffu, Wp, p);
                Cp = __shfl_sync(0xffffffffu, Cp, p);
                Csum += Cp;
                if (lane > p) {
                    const float P = (float)sP[lane * 33 + p];
                    // r = P - colmean_t S_p, G = sigma_t r, num += (dBeta sigma_p) G
                    const float qh = __fmul_rn(mh, Sp);
                    const float ql = __fmaf_rn(ml, Sp, __fmaf_rn(mh, Sp, -qh));
                    float rh = P, rl = 0.f;
                    df_add(rh, rl, -qh, -ql);
                    float gh, gl, xh, xl;
                    df_mul(sh, sl, rh, rl, gh, gl);
                    df_mul(uh, ul, gh, gl, xh, xl);
                    df_add(nh, nl, xh, xl);
                }
                sumE += Wp * (long long)Sp - (long long)a.N * Cp;
            }
            // acum of an FP32 decision: P(component 0) of the FP32 sampler at
            // the marker's final num
            {
                int c2;
                float a0;
                pick_f32<KM>(nh, nl, uf, gcf, K, c2, a0);
                acum_f = a0;
            }
            if (q < a.M) {
                const size_t cj = (size_t)c * a.M + rc.j;
                a.beta[cj] = fcomp == 0 ? 0.0 : (fcomp > 0 ? (double)bnh + (double)bnl : bold);
                a.acum[cj] = acum_is_d ? acum_d : (double)acum_f;
                a.chosen[cj] = fcomp >= 0 ? 1 : 0;
                if (fcomp >= 0)
                    a.comp[cj] = fcomp;
            }
            a.wx[(size_t)c * (kBatchBlock + 1) + lane] = Wl;
            if (lane == 0) {
                a.wx[(size_t)c * (kBatchBlock + 1) + kBatchBlock] = Csum;
                a.sumE[c] = sumE;
            }
            __syncwarp();
            if (lane == 0)
                red_release_add_u64(cnt2, 1ull);
            if (prof && k == 0) {
                ph[5] += clock64() - tl;
                ph[6] += steps + 1;
            }
        }
        const long long t2 = prof ? clock64() : 0;
        if (tid == 0 && !s_abort &&
            !counter_wait(cnt2, (unsigned long long)C * (unsigned long long)(b + 1), a.err, a.timeout_ns)) {
            atomicCAS(a.err, kDevOk, kDevTimeout);
            s_abort = 1;
        }
        __syncthreads();
        if (prof) {
            ph[7] += clock64() - t2;
            ph[2] += clock64() - t0, t0 = clock64();
        }
        if (s_abort)
            break;

        // ---- update coefficients as limbs: W tile [row 4c+l][marker t], constants per chain
        for (int idx = tid; idx < C * kBatchBlock; idx += kBT) {
            const int c = idx >> 5, t = idx & 31;
            int d[kBatchLimbs];
            if (!split4((long long)__ldcg((const unsigned long long *)a.wx + (size_t)c * (kBatchBlock + 1) + t), d))
                atomicCAS(a.err, kDevOk, kDevRange);
#pragma unroll
            for (int l = 0; l < kBatchLimbs; ++l) {
                const int n = 4 * c + l;
                *reinterpret_cast<unsigned short *>(w_t + (n >> 3) * 512 + (t >> 3) * 128 + (n & 7) * 16 + (t & 7) * 2) =
                    h_bits(d[l]);
            }
        }
        for (int c = tid; c < C; c += kBT) {
            int d[kBatchLimbs];
            if (!split4((long long)__ldcg((const unsigned long long *)a.wx + (size_t)c * (kBatchBlock + 1) + kBatchBlock), d))
                atomicCAS(a.err, kDevOk, kDevRange);
#pragma unroll
            for (int l = 0; l < kBatchLimbs; ++l)
                s_cl[c][l] = (float)d[l];
        }
        // the block Gram accumulators of this block are read by now: clear them for block b+2
        if (s == 0)
            for (int e = tid; e < kBatchPCopies * kBatchBlock * kBatchBlock; e += kBT)
                a.pacc[(size_t)(b & 1) * kBatchPCopies * (kBatchBlock * kBatchBlock) + e] = 0u;
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();

        // ---- residual update D2[i][4c+l] = sum_t g[t][i] W[4c+l][t], TPP tiles of 128 individuals per pass
        const uint32_t id_upd = idesc_f16(128, R, true);
        for (int t0p = 0; t0p < NT; t0p += TPP) {
            const int nt = NT - t0p < TPP ? NT - t0p : TPP;
            if (tid == 0) {
                for (int it = 0; it < nt; ++it)
                    for (int ks = 0; ks < 2; ++ks)
                        umma_f16(tmem + (unsigned)(it * R),
                                 smem_desc(ug + (t0p + it) * 2048 + ks * 2 * pl.sbo_g, pl.sbo_g, 128),
                                 smem_desc(uw + ks * 256, 128, 512), id_upd, ks > 0);
                umma_commit(&s_mbar);
            }
            if (!mbar_wait_bounded(&s_mbar, mphase & 1u, a.timeout_ns)) {
                atomicCAS(a.err, kDevOk, kDevTimeout);
                s_abort = 1;
            }
            ++mphase;
            tc_fence_after();
            // the pass's tiles dealt to the two groups of four warps in pairs;
            // an odd last tile split between them by chains (both groups read
            // the same TMEM lanes, the warp's quarter, at other columns)
            const int q4 = warp & 3, wg = warp >> 2;
            auto update_tile = [&](int it, int ck0, int ck1) {
                const int i = (t0p + it) * 128 + q4 * 32 + lane;
                bool ok = true;
                for (int ck = ck0; ck < ck1; ++ck) {
                    float f[32];
                    tmem_ld32(tmem + ((unsigned)(q4 * 32) << 16) + (unsigned)(it * R + ck * 32), f);
                    if (i < ns) {
                        // limbs + update - constant, renormalised with carries, all in
                        // FP32 on exact integers (|values| < 2^17)
#pragma unroll
                        for (int cc = 0; cc < 8; cc += 2) {
                            const int c = ck * 8 + cc;     // chains c, c+1: rows 4c .. 4c+7
                            uint4 *ep = reinterpret_cast<uint4 *>(e_t + (i >> 3) * pl.lbo_e + (c >> 1) * 128 + (i & 7) * 16);
                            uint4 w4 = *ep;
                            uint32_t *w = reinterpret_cast<uint32_t *>(&w4);
#pragma unroll
                            for (int h = 0; h < 2; ++h) {
                                const float2 e01 = __half22float2(*reinterpret_cast<const __half2 *>(&w[2 * h]));
                                const float2 e23 = __half22float2(*reinterpret_cast<const __half2 *>(&w[2 * h + 1]));
                                const float *cl = s_cl[c + h];
                                const float *d = &f[(cc + h) * 4];
                                float v0 = __fsub_rn(__fadd_rn(e01.x, d[0]), cl[0]);
                                const float k0 = limb_carry(v0);
                                v0 = __fmaf_rn(-2048.f, k0, v0);
                                float v1 = __fadd_rn(__fsub_rn(__fadd_rn(e01.y, d[1]), cl[1]), k0);
                                const float k1 = limb_carry(v1);
                                v1 = __fmaf_rn(-2048.f, k1, v1);
                                float v2 = __fadd_rn(__fsub_rn(__fadd_rn(e23.x, d[2]), cl[2]), k1);
                                const float k2 = limb_carry(v2);
                                v2 = __fmaf_rn(-2048.f, k2, v2);
                                const float v3 = __fadd_rn(__fsub_rn(__fadd_rn(e23.y, d[3]), cl[3]), k2);
                                ok = ok && v3 >= -1024.f && v3 < 1024.f;
                                const __half2 n01 = __floats2half2_rn(v0, v1), n23 = __floats2half2_rn(v2, v3);
                                w[2 * h] = *reinterpret_cast<const uint32_t *>(&n01);
                                w[2 * h + 1] = *reinterpret_cast<const uint32_t *>(&n23);
                            }
                            *ep = w4;
                        }
                    }
                }
                if (!ok)
                    atomicCAS(a.err, kDevOk, kDevRange);
            };
            for (int it = wg; it < (nt & ~1); it += 2)
                update_tile(it, 0, R / 32);
            if (nt & 1)
                update_tile(nt - 1, wg * (R / 64), (wg + 1) * (R / 64));
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
        }
        if (prof)
            ph[3] += clock64() - t0;
        if (s_abort)
            break;
    }

    // ---- residuals back to HBM; per-slice sum(E) and sum(eps^2) per chain
    for (int cp = 0; cp < C / 2; ++cp) {
        long long se[2] = {0, 0};
        double sq[2] = {0.0, 0.0};
        for (int i = tid; i < ns; i += kBT) {
            const uint4 w4 = *reinterpret_cast<const uint4 *>(e_t + (i >> 3) * pl.lbo_e + cp * 128 + (i & 7) * 16);
            const uint32_t w[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                int d[kBatchLimbs];
#pragma unroll
                for (int l = 0; l < kBatchLimbs; ++l) {
                    const uint32_t word = w[2 * h + (l >> 1)];
                    d[l] = h_int((unsigned short)((l & 1) ? (word >> 16) : (word & 0xFFFFu)));
                }
                const long long x = join4(d);
                a.E[(size_t)(2 * cp + h) * a.N + lo + i] = x;
                se[h] += x;
                const double e = (double)x * inv2f;
                sq[h] = fma(e, e, sq[h]);
            }
        }
        // fixed-order reduction: lanes, then warps
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                se[h] += __shfl_xor_sync(0xffffffffu, se[h], o);
                sq[h] += __shfl_xor_sync(0xffffffffu, sq[h], o);
            }
        }
        __shared__ long long r_se[kBW][2];
        __shared__ double r_sq[kBW][2];
        if (lane == 0) {
            r_se[warp][0] = se[0];
            r_se[warp][1] = se[1];
            r_sq[warp][0] = sq[0];
            r_sq[warp][1] = sq[1];
        }
        __syncthreads();
        if (tid < 2) {
            long long t = 0;
            double u = 0.0;
            for (int w = 0; w < kBW; ++w) {
                t += r_se[w][tid];
                u += r_sq[w][tid];
            }
            double *pp = a.part + ((size_t)s * C + 2 * cp + tid) * 2;
            pp[0] = __longlong_as_double(t);
            pp[1] = u;
        }
        __syncthreads();
    }
    if (prof && tid == 0)
        for (int k = 0; k < 8; ++k)
            prof[k] = ph[k];

    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

__global__ void k_batch_draws(uint32_t seed, uint32_t chain0, uint32_t it, int64_t M,
                              const uint32_t *__restrict__ order, const double *__restrict__ beta,
                              ChainRec *__restrict__ crec)
{
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (q >= M)
        return;
    const uint32_t j = order[q];
    double u, z;
    marker_draws(StreamKey{seed, chain0 + (uint32_t)c}, it, j, &u, &z);
    crec[(size_t)c * M + q] = ChainRec{beta[(size_t)c * M + j], u, z, 0.0};
}

__global__ void k_batch_gather(const uint32_t *__restrict__ order, int64_t M, const double *__restrict__ scale,
                               const int64_t *__restrict__ counts, const int32_t *__restrict__ group,
                               BatchRec *__restrict__ rec)
{
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= M)
        return;
    const uint32_t j = order[q];
    BatchRec r;
    r.sigma = scale[2 * j];
    r.colmean = scale[2 * j + 1];
    r.S = (double)(counts[4 * (size_t)j + 1] + 2 * counts[4 * (size_t)j + 2]);
    r.j = j;
    r.group = group[j];
    rec[q] = r;
}

// Per chain: component counts per group and the exact fixed-point sum of the
// squared non-zero betas per group over the markers whose component was drawn
// (src/BayesRBase.cpp:200-202, :348-366).
__global__ void __launch_bounds__(256) k_batch_stats(int64_t M, const int32_t *__restrict__ group,
                                                     const int32_t *__restrict__ comp,
                                                     const uint8_t *__restrict__ chosen,
                                                     const double *__restrict__ beta, int n_groups,
                                                     unsigned long long *__restrict__ out)
{
    __shared__ unsigned long long sv[kMaxGroups * kMaxK];
    __shared__ unsigned long long sb[kMaxGroups][2];
    const int c = blockIdx.y;
    const int32_t *cc = comp + (size_t)c * M;
    const double *bc = beta + (size_t)c * M;
    unsigned long long *o = out + (size_t)c * (n_groups * kMaxK + 2 * n_groups);
    for (int i = threadIdx.x; i < n_groups * kMaxK; i += blockDim.x)
        sv[i] = 0ull;
    for (int i = threadIdx.x; i < n_groups; i += blockDim.x)
        sb[i][0] = sb[i][1] = 0ull;
    __syncthreads();
    const uint8_t *ch = chosen + (size_t)c * M;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < M; j += (int64_t)gridDim.x * blockDim.x) {
        if (!ch[j])
            continue;
        const int g = group[j], k = cc[j];
        atomicAdd(&sv[g * kMaxK + k], 1ull);
        if (k >= 1) {
            __int128 x;
            fx_from_double(bc[j] * bc[j], x);
            const Fx f = fx_split(x);
            atomicAdd(&sb[g][0], (unsigned long long)f.hi);
            atomicAdd(&sb[g][1], f.lo);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_groups * kMaxK; i += blockDim.x)
        if (sv[i])
            atomicAdd(&o[i], sv[i]);
    for (int i = threadIdx.x; i < n_groups; i += blockDim.x) {
        atomicAdd(&o[n_groups * kMaxK + 2 * i], sb[i][0]);
        atomicAdd(&o[n_groups * kMaxK + 2 * i + 1], sb[i][1]);
    }
}

template <int KM>
cudaError_t launch_batch_km(const BatchArgs &a, cudaStream_t st)
{
    const size_t smem = batch_smem_bytes(a.C, a.kext, a.G);
    const void *f = a.prof ? (const void *)k_sweep_batch<KM, true> : (const void *)k_sweep_batch<KM, false>;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    BatchArgs args = a;
    void *params[] = {&args};
    return cudaLaunchCooperativeKernel(f, dim3((unsigned)a.G), dim3(kBT), params, smem, st);
}

}  // namespace

size_t batch_smem_bytes(int C, int kext, int G) { return batch_plan(C, kext, G).total; }

int batch_max_ctas_per_sm(int C, int kext, size_t smem)
{
    int n = 1 << 30;
    const void *fs[4] = {(const void *)k_sweep_batch<4, false>, (const void *)k_sweep_batch<16, false>,
                         (const void *)k_sweep_batch<4, true>, (const void *)k_sweep_batch<16, true>};
    for (const void *f : fs) {
        int m = 0;
        if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, f, kBT, smem) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        n = m < n ? m : n;
    }
    (void)C;
    (void)kext;
    return n;
}

cudaError_t launch_batch_gather(const uint32_t *order, int64_t M, const double *scale, const int64_t *counts,
                                const int32_t *group, BatchRec *rec, cudaStream_t st)
{
    k_batch_gather<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(order, M, scale, counts, group, rec);
    return cudaGetLastError();
}

cudaError_t launch_batch_draws(uint32_t seed, uint32_t chain0, uint32_t it, int64_t M, int C, const uint32_t *order,
                               const double *beta, ChainRec *crec, cudaStream_t st)
{
    k_batch_draws<<<dim3((unsigned)((M + 255) / 256), (unsigned)C), 256, 0, st>>>(seed, chain0, it, M, order, beta,
                                                                                  crec);
    return cudaGetLastError();
}

cudaError_t launch_batch_stats(int64_t M, int C, const int32_t *group, const int32_t *comp, const uint8_t *chosen,
                               const double *beta, int n_groups, unsigned long long *out, cudaStream_t st)
{
    const int bx = (int)((M + 255) / 256 < 64 ? (M + 255) / 256 : 64);
    k_batch_stats<<<dim3((unsigned)bx, (unsigned)C), 256, 0, st>>>(M, group, comp, chosen, beta, n_groups, out);
    return cudaGetLastError();
}

cudaError_t launch_sweep_batch(const BatchArgs &a, int kmax, cudaStream_t st)
{
    if (kmax <= 4)
        return launch_batch_km<4>(a, st);
    if (kmax <= 8)
        return launch_batch_km<8>(a, st);
    return launch_batch_km<16>(a, st);
}

}  // namespace brr
