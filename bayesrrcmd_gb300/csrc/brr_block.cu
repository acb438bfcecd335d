// Gram-blocked sweep of the FP32C form over dense markers, software-pipelined
// (sm_103a).
//
// Replaces BayesRBase::processColumn (src/BayesRBase.cpp:287-392) over the
// dense kernel (src/densebayesrkernel.cpp:10-20) for whole sweeps, like the
// restart sweep of brr_sweep.cu, with the precomputed marker Gram matrix
// (packed lower triangle, FP64, brr_gram.cu).
//
// The sweep order is cut into blocks of B consecutive markers.  One CTA per SM
// owns a slice of individuals and keeps its residual slice in shared memory in
// fixed point, E = eps * 2^50 as a signed 64-bit integer stored as four
// balanced 16-bit limbs.  Block q's dot products sum_i g_i E_i (g in {0,1,2}
// the genotype) are exact integer sums: dp2a (two int16 x int8 products per
// instruction) over the limbs, one warp per 8 markers; they are summed across
// CTAs by exact 128-bit fixed-point integer atomics, and a grid-wide counter
// barrier publishes the sums.  The residual update adds dBeta * x rounded to
// the 2^-50 grid.  Every CTA then
// resolves block q identically: the markers are sampled in order of the
// block, and after every marker p that changes the residual the later markers'
// dot products move by dBeta_p * G[p, t] (exact sequential chain up to
// rounding).  The block's rank-U residual update follows.
//
// Pipelining, two blocks deep: block q+2's dot products are computed against
// the residual that holds the updates of blocks q-1 and earlier, while block q
// is being resolved.  When block t is resolved, the updates of blocks t-2 and
// t-1 enter through the cross Gram entries G[p, t'] (p in block t-2: "far",
// p in block t-1: "near", t' in block t).  Per CTA and iteration r:
//   8 dot warps:            rank-U update of block r-1; cp.async of block
//                           r+3's code slices into the slot block r-1 held;
//                           dots of block r+2, publish, arrive at barrier r+2;
//   the resolve warp:       near corrections of block r-1 (Gram entries in
//                           shared memory, bulk-copied one iteration ahead),
//                           resolve block r;
//   the chore warp:         bulk copy (TMA) of block r+1's triangle and near
//                           entries into shared memory; staged Gram entries of
//                           block r+3; zeroed accumulators of block r+4 (first
//                           CTA); a non-blocking arrival on the dot warps'
//                           named barrier; the Gram loads of block r+4;
//                           outputs of block r-1;
//   the input warp:         the far corrections of block r-1 for block r+1
//                           (entries read from the staging slot in L2), then
//                           wait for barrier r+1 (arrived one iteration
//                           earlier) and assemble block r+1's inputs from its
//                           published sums.
// So neither the grid barrier's latency nor the input assembly is on the path
// of the dot warps or of the resolve warp.  The ten warps other than the
// resolve warp iterate in step (named barrier 3 at the top of each iteration);
// the resolve warp runs on its own, tied to them by two signals in shared
// memory (mbarriers, two per signal by block parity):
//   GO(q)        320 arrivals in the others' iteration q-1: the dot threads
//                after block q-2's update, the input warp after block q's
//                inputs, the chore warp after block q-2's outputs; so block q
//                can be resolved while the others finish iteration q-1;
//   RESOLVED(q)  the resolve warp's 32 lanes after block q's decisions; the
//                others wait for it at the top of iteration q+1.
// Block q's decisions (parity q % 2) are read by the others in iteration q+1
// and overwritten by block q+2, which waits for GO(q+2), i.e. for those reads;
// a signal's next phase on the same mbarrier needs the other side's progress
// past the previous one, so no phase is ever skipped.
//
// Buffers and why their counts suffice (iteration r: the dot warps publish
// block r+2 and arrive at barrier r+2; the input warp passes barrier r+1 and
// reads block r+1's sums and staged far entries; a CTA in iteration r has
// passed barrier r, and every CTA arrives at barrier q+2 only after it passed
// barrier q):
//  * two sets of barrier counters, barrier q on set q % 2, each set 8 counters
//    (CTA s on counter s % 8, target its CTA count * (q / 2 + 1)): arrivals on
//    a set beyond barrier q come only from CTAs that passed barrier q;
//  * 8 fixed-point accumulator buffers (block q in buffer q % 8), each with 8
//    copies (CTA s adds into copy s % 8, the reader sums them): the first CTA
//    zeroes block q+4's buffer in iteration q before arriving at barrier q+2;
//    every CTA publishes block q+4 in iteration q+2, after it passed barrier
//    q+2; the buffer last held block q-4, whose sums every CTA read in
//    iteration q-5, before arriving at barrier q-2 (passed by the first CTA);
//  * 8 Gram staging slots in global memory (block q in slot q % 8: triangle,
//    near, far entries), written in iteration q-3 before the arrival at
//    barrier q-1, read (bulk copy of triangle and near, far loads) in
//    iteration q-1 after barrier q-1 or, for blocks 0-2, after barrier 0;
//    slot q % 8 last held block q-8, read in iteration q-9 (its bulk copy
//    waited for in iteration q-8), before every CTA's arrival at barrier q-5,
//    which the writers have passed; 2
//    shared-memory Gram slots (block q copied in iteration q-1, read in
//    iteration q; the slot's previous block q-2 was read in iteration q-2);
//  * rings of 4B records and 4B code slots (B markers per block): records of
//    blocks r..r+3 (block r+3 issued at the top of iteration r, into the slot
//    of block r-1, read by nobody after iteration r-1); codes of blocks
//    r-1..r+2, block r+3 issued by the dot warps after the update of block
//    r-1, into its slot.
#include <cuda_runtime.h>

#include <string>

#include "brr_device.cuh"
#include "brr_internal.h"
#include "brr_pick.cuh"



namespace brr {

namespace {

// Roles by warp.  Warp w issues from sub-partition w % 4: the eight dot warps
// 0-7 put two on every sub-partition (their dot products and updates are the
// longest role), and the resolve, input and chore warps 8-10 take the third
// slot of sub-partitions 0-2.  Measured against the resolve warp alone with
// the input warp on sub-partition 3 (three dot warps on sub-partitions 0 and
// 1): 3 % more marker-updates/s at N = M = 100,000 although the resolve warp
// now shares its sub-partition with two dot warps.
constexpr int kDotWarps = 8;
constexpr int kResolveWarp = 8;    // samples the blocks
constexpr int kInputWarp = 9;      // grid barrier, inputs of the next block
constexpr int kChoreWarp = 10;     // Gram copies and gathers, outputs
constexpr int kBlockThreads = (kDotWarps + 3) * 32;
// index 0..7 of a dot warp, -1 for the other roles
__host__ __device__ constexpr int dot_index(int w) { return w < kDotWarps ? w : -1; }
static_assert(kResolveWarp >= kDotWarps && kInputWarp >= kDotWarps && kChoreWarp >= kDotWarps,
              "the dot warps are warps 0..7");
constexpr int kAccBufs = 8;
constexpr int kAccCopies = 8;   // CTA s adds into copy s % 8: 19 atomics per address and block, not 152
constexpr int kAccBufWords = kAccCopies * kMaxSpec * 4;
// Barrier counters: per barrier parity 8 counters 128 bytes apart; CTA s arrives
// on counter s % 8, so 19 arrivals (not 152) serialise on one address.
constexpr int kCounters = 8;
constexpr int kCounterStride = 16;
constexpr int kStageSlots = 8;
constexpr int kIdSlots = 8;

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

// Gram entries of one block in shared memory: the triangle G[p, t], p < t
// within the block, then the near entries G[p, t] of the previous block's p and
// this block's t.
__host__ __device__ inline size_t block_gram_entries(int B) { return (size_t)B * (B - 1) / 2 + (size_t)B * B; }
// A staging slot adds the far entries G[p, t], p in the block before the
// previous one.
__host__ __device__ inline size_t block_stage_entries(int B) { return block_gram_entries(B) + (size_t)B * B; }

struct PipePlan {
    size_t planes;          // residual limb planes: 8 words per 4 individuals
    size_t fix;             // residual in fixed point: one int64 per individual
    size_t codes;           // R x slot_bytes genotype codes
    size_t recs;            // R x BlockRec
    size_t gram;            // 2 x block_gram_entries double-float Gram entries
    size_t pairs;           // B(B-1)/2 x 2 bytes: pair positions (a < b)
    size_t gcf;             // n_groups x kMaxK x {dc, h}
    size_t gbf;             // n_groups x kMaxK x {sdk hi, lo, invden hi, lo}
    size_t mbar;            // 2 mbarriers of the Gram copies
    size_t total;
};

__host__ __device__ inline PipePlan make_pipe_plan(int slice_max, int slot_bytes, int B, int n_groups)
{
    PipePlan p;
    const size_t R = 4 * (size_t)B;
    size_t o = 0;
    p.planes = o;
    o += al16((size_t)slice_max / 4 * 32);
    p.fix = o;
    o += al16((size_t)slice_max * 8);
    p.codes = o;
    o += al16(R * slot_bytes);
    p.recs = o;
    o += R * sizeof(BlockRec);
    p.gram = o;
    o += al16(2 * block_gram_entries(B) * sizeof(float2));
    p.pairs = o;
    o += al16((size_t)B * (B - 1) / 2 * 2);
    p.gcf = o;
    o += al16((size_t)n_groups * kMaxK * 2 * sizeof(float));
    p.gbf = o;
    o += al16((size_t)n_groups * kMaxK * 4 * sizeof(float));
    p.mbar = o;
    o += 16;
    p.total = al16(o);
    return p;
}

// ---- mbarrier and bulk-copy (TMA) primitives
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *m, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *m, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *m)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(m)) : "memory");
}

// Waits (suspending in hardware for a while) for the phase with the given
// parity; false when the hardware's time window passed first.
__device__ __forceinline__ bool mbar_try(uint64_t *m, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(m)), "r"(parity)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_test(uint64_t *m, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(m)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16)
// completing on mbarrier m.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, uint64_t *m)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(m))
                 : "memory");
}

// Orders this thread's generic-proxy view of memory (global writes of other
// CTAs it has acquired, shared-memory reads of the slot being refilled) before
// its later async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async;" ::: "memory"); }

// SM clock read ordered with the surrounding memory operations and barriers.
__device__ __forceinline__ long long clk()
{
    long long t;
    asm volatile("mov.u64 %0, %%clock64;" : "=l"(t)::"memory");
    return t;
}

__device__ __forceinline__ void dot_warps_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// Before the arrival at a grid barrier the dot warps wait on named barrier 2
// for their own work and for the chore warp's staging stores; the chore warp
// only signals it and goes on.
__device__ __forceinline__ void arrive_sync() { asm volatile("bar.sync 2, 288;" ::: "memory"); }
__device__ __forceinline__ void chore_signal() { asm volatile("bar.arrive 2, 288;" ::: "memory"); }

// The ten warps other than the resolve warp: iteration barrier (named barrier
// 3) with the OR of a flag over its 320 threads.
constexpr int kOtherThreads = 320;
__device__ __forceinline__ bool others_any(bool v)
{
    unsigned r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, 3, 320, q;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(r)
                 : "r"((unsigned)v)
                 : "memory");
    return r != 0;
}

// A double-float written by another CTA before a grid barrier this thread has
// passed (read at L2, not from a stale L1 line).
__device__ __forceinline__ float2 ld_relaxed_f2(const float2 *p)
{
    float2 v;
    asm volatile("ld.relaxed.gpu.global.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p) : "memory");
    return v;
}

// ---- fixed-point residual: E = eps * 2^kFrac, |E| < 2^62, as four balanced
// 16-bit limbs E = l0 + l1 2^16 + l2 2^32 + l3 2^48 (l_k in [-2^15, 2^15)).
// The limb planes of 4 individuals i0..i3 (byte position b of the codes) are 8
// words: limb k's pair (i0, i1) at word 2(k ^ (b & 3)) and (i2, i3) at the next
// word, each pair as two int16 (low half first).  The XOR with b & 3 makes the
// lane that reads position b see the limbs in the order its reduction wants.
constexpr int kFrac = 50;
constexpr long long kFixMax = 1ll << 62;

// A code byte (4 individuals, 2 bits each) as the byte selector of __byte_perm:
// code k of the byte in bits 4k..4k+1 of the result.  Selecting from
// kGenoBytes gives the 4 genotype bytes (code 0: 2, 2: 1, 1 and 3: 0), from
// kMissBytes the 4 missing-indicator bytes (code 1), with no table lookup.
constexpr unsigned kGenoBytes = 0x00010002u;
constexpr unsigned kMissBytes = 0x00000100u;
__device__ __forceinline__ unsigned code_nibbles(unsigned v)
{
    const unsigned x = (v | (v << 4)) & 0x0F0Fu;
    return (x | (x << 2)) & 0x3333u;
}

__device__ __forceinline__ void split_limbs(long long E, int (&l)[4])
{
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        l[k] = (int)((E << 48) >> 48);
        E = (E - l[k]) >> 16;
    }
    l[3] = (int)E;
}

__device__ __forceinline__ void store_fix4(uint32_t *planes, int b, const long long (&E)[4])
{
    uint2 *w = reinterpret_cast<uint2 *>(planes + 8 * b);
    const int p = b & 3;
    int l0[4], l1[4], l2[4], l3[4];
    split_limbs(E[0], l0);
    split_limbs(E[1], l1);
    split_limbs(E[2], l2);
    split_limbs(E[3], l3);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        w[k ^ p] = make_uint2(__byte_perm((unsigned)l0[k], (unsigned)l1[k], 0x5410),
                              __byte_perm((unsigned)l2[k], (unsigned)l3[k], 0x5410));
}

// Double-float value to the fixed-point grid (truncation below 2^-60, then
// rounding to the nearest multiple of 2^-kFrac); false when out of range.
__device__ __forceinline__ bool df_to_fix(float h, float l, long long &E)
{
    __int128 x1, x2;
    if (!fx_from_float(h, x1) || !fx_from_float(l, x2))
        return false;
    const __int128 x = (x1 + x2 + ((__int128)1 << (59 - kFrac))) >> (60 - kFrac);   // nearest
    if (x >= (__int128)kFixMax || x <= -(__int128)kFixMax)
        return false;
    E = (long long)x;
    return true;
}

// Double-float value times 2^kFrac to the nearest integer by the hardware
// conversions, for the residual changes of the update: the scaled high part is
// an integer whenever it reaches 2^23, and then the sum is the nearest integer
// to the scaled value; below that it is within one unit of it.  False when out
// of range or not a number.  The exact df_to_fix (two 128-bit shifts) stays for
// the residual itself.
static_assert(kFrac == 50, "df_to_fix_near scales by 2^50");
__device__ __forceinline__ bool df_to_fix_near(float h, float l, long long &E)
{
    const float sh = h * 0x1p50f, sl = l * 0x1p50f;
    if (!(fabsf(sh) < 0x1p61f) || !(fabsf(sl) < 0x1p61f))
        return false;
    E = __float2ll_rn(sh) + __float2ll_rn(sl);
    return E < kFixMax && E > -kFixMax;
}

__device__ __forceinline__ void fix_to_df(long long E, float &h, float &l)
{
    const Fx f = fx_split((__int128)E << (60 - kFrac));
    fx_to_df(f.hi, f.lo, h, l);
}

// Waits for phase `parity` of m, at most timeout_ns; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *m, unsigned parity, uint64_t timeout_ns)
{
    if (mbar_test(m, parity))
        return true;
    const uint64_t t0 = global_timer_ns();
    unsigned spins = 0;
    while (!mbar_test(m, parity)) {
        if ((++spins & 63u) == 0 && global_timer_ns() - t0 > timeout_ns)
            return false;
    }
    return true;
}

}  // namespace

// Records of the Gram-blocked FP32C dense sweep (all markers in parallel, the
// FP64 work of the sweep's per-marker constants done once here).
__global__ void k_gather_block(const uint32_t *__restrict__ order, int64_t M, int64_t N,
                               const double *__restrict__ table, const double *__restrict__ scale,
                               const double *__restrict__ beta, const double *__restrict__ u,
                               const double *__restrict__ z, const int32_t *__restrict__ group, double S,
                               BlockRec *__restrict__ rec)
{
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= M)
        return;
    const uint32_t j = order[q];
    BlockRec r;
#pragma unroll
    for (int c = 0; c < 4; ++c)
        df_from_double(table[4 * j + c], r.x[2 * c], r.x[2 * c + 1]);
    const double sigma = scale[2 * j], cm = scale[2 * j + 1], xm = table[4 * j + 1];
    const double bo = beta[j];
    df_from_double(sigma, r.sig[0], r.sig[1]);
    df_from_double(__dsub_rn(__dmul_rn(bo, (double)(N - 1)), __dmul_rn(__dmul_rn(sigma, cm), S)), r.cst[0],
                   r.cst[1]);
    df_from_double(__dadd_rn(__dmul_rn(sigma, cm), xm), r.dm[0], r.dm[1]);
    df_from_double(bo, r.bo[0], r.bo[1]);
    df_from_double(z[j], r.zf[0], r.zf[1]);
    r.uf = __double2float_rn(u[j]);
    r.bnz = bo != 0.0 ? 1u : 0u;
    r.beta_old = bo;
    r.u = u[j];
    r.z = z[j];
    r.j = j;
    r.group = group[j];
    r.pad[0] = r.pad[1] = r.pad[2] = r.pad[3] = 0u;
    rec[q] = r;
}

// After a blocked sweep: FP64 beta (markers that chose a component) and acum.
__global__ void k_block_finish(int64_t M, const uint8_t *__restrict__ chosen, const float2 *__restrict__ beta_df,
                               const float2 *__restrict__ acum_df, double *__restrict__ beta,
                               double *__restrict__ acum)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= M)
        return;
    const float2 a = acum_df[j];
    acum[j] = __dadd_rn((double)a.x, (double)a.y);
    if (chosen[j]) {
        const float2 b = beta_df[j];
        beta[j] = __dadd_rn((double)b.x, (double)b.y);
    }
}

// One halving exchange of a warp's reduce-scatter over double-float sums:
// lanes of the lower half (upper false) keep entries [0, H), the others
// [H, 2H), each adding the partner's copy; the kept sums move to [0, H).
template <int H>
__device__ __forceinline__ void df_rs_step(float (&h)[kMaxSpec / 8], float (&l)[kMaxSpec / 8], bool upper, int off)
{
#pragma unroll
    for (int i = 0; i < H; ++i) {
        const float kh = upper ? h[i + H] : h[i], kl = upper ? l[i + H] : l[i];
        const float sh = upper ? h[i] : h[i + H], sl = upper ? l[i] : l[i + H];
        const float rh = __shfl_xor_sync(0xffffffffu, sh, off);
        const float rl = __shfl_xor_sync(0xffffffffu, sl, off);
        h[i] = kh;
        l[i] = kl;
        df_add(h[i], l[i], rh, rl);
    }
}

// Butterfly step of a double-float all-reduce (both partners get the same sum).
__device__ __forceinline__ void df_xor_add(float &h, float &l, int off)
{
    const float rh = __shfl_xor_sync(0xffffffffu, h, off);
    const float rl = __shfl_xor_sync(0xffffffffu, l, off);
    df_add(h, l, rh, rl);
}

// Outputs of one resolved block, written by one warp of the CTA whose turn it
// is (block q by CTA q mod G, one iteration later, off the critical path): new
// beta as double-float (z * sdk + num * invden for a component k > 0, 0 for
// component 0), acum (P(component 0) of the FP32 sampler at the final num, or
// of the FP64 evaluation), chosen flag and component, by marker id.
struct BlockOut {
    float2 x[kMaxSpec];   // final num (double-float)
    float2 fb[kMaxSpec];  // beta of an FP64 decision
    float2 fa[kMaxSpec];  // acum of an FP64 decision
    float2 zf[kMaxSpec];  // z
    float uf[kMaxSpec];
    uint32_t j[kMaxSpec];
    int group[kMaxSpec];
    int code[kMaxSpec];   // comp & 0xFF | FP64 decision << 8; -2: no marker
};

template <int KM>
__device__ __forceinline__ void write_block_outputs(const SweepArgs &a, const BlockOut &o, const float *gcf,
                                                    const int32_t *gk, const float *gbf, int lane)
{
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int m = lane + 32 * h;
        const int oc = o.code[m];
        if (oc == -2)
            continue;
        const int c = (oc & 0x80) ? -1 : (oc & 0xFF);
        const bool fp64 = (oc & 0x100) != 0;
        const int g = o.group[m];
        const float2 x = o.x[m];
        float bh = 0.f, bl = 0.f;
        float2 acum;
        if (fp64) {
            if (c > 0) {
                bh = o.fb[m].x;
                bl = o.fb[m].y;
            }
            acum = o.fa[m];
        } else {
            if (c > 0) {
                const float4 gc = reinterpret_cast<const float4 *>(gbf + (size_t)g * kMaxK * 4)[c];
                float ph, pl;
                df_mul(o.zf[m].x, o.zf[m].y, gc.x, gc.y, bh, bl);
                df_mul(x.x, x.y, gc.z, gc.w, ph, pl);
                df_add(bh, bl, ph, pl);
            }
            int c2;
            float a0;
            pick_f32<KM>(x.x, x.y, o.uf[m], gcf + (size_t)g * kMaxK * 2, gk[g], c2, a0);
            acum = make_float2(a0, 0.f);
        }
        const uint32_t j = o.j[m];
        a.beta_df[j] = make_float2(bh, bl);
        a.acum_df[j] = acum;
        a.chosen[j] = c >= 0 ? 1 : 0;
        if (c >= 0)
            a.comp[j] = c;
    }
}

// One CTA of 11 warps per SM (8 dot warps, the resolve, chore and input
// warps).  The register file is split between the SM's four sub-partitions
// (16K registers each) and warps are placed round-robin, so the sub-partitions
// holding three warps bound every thread to 168 registers: the launch bound is
// stated for 12 warps to give the compiler that limit.  PROF: the variant that
// counts phase cycles on the first CTA (the clock reads constrain the code's
// scheduling, so the plain variant has none).
template <int KM, bool MISS, bool PROF>
__global__ void __launch_bounds__(12 * 32, 1) k_sweep_block(SweepArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    // per block parity: residual-changing markers of the block (positions,
    // dBeta, standardised code values), and the block's prepared inputs
    __shared__ int s_upd[2][kMaxSpec];
    __shared__ float2 s_dB[2][kMaxSpec];
    __shared__ float4 s_x[2][kMaxSpec][2];
    __shared__ int s_nupd[2];
    __shared__ float2 s_inum[2][kMaxSpec];   // num from the block's dot products (double-float)
    __shared__ float s_iuf[2][kMaxSpec];
    __shared__ unsigned s_imeta[2][kMaxSpec]; // group | K << 8 | (beta_old != 0) << 16
    __shared__ float s_H[kMaxGroups];
    __shared__ int32_t s_gk[kMaxGroups];
    __shared__ BlockOut s_out[2];
    __shared__ long long s_D[kMaxSpec][4];   // residual change per update and code, fixed point
    __shared__ unsigned s_uoff[kMaxSpec];    // offset of each update's codes in the ring
    // marker ids of blocks q (slot q % kIdSlots), copied from the sweep order
    // one iteration before they are read: blocks r+1 .. r+4 are resident in
    // iteration r while block r+5's ids are in flight
    __shared__ __align__(16) uint32_t s_ids[kIdSlots][kMaxSpec];
    __shared__ int s_abort;
    __shared__ int s_cp_issued;
    // resolve warp <-> other warps: GO(q) on s_mb[q & 1] (320 arrivals: the dot
    // threads after block q-2's update, the input warp after block q's inputs,
    // the chore warp after block q-2's outputs), RESOLVED(q) on s_mb[2 + (q & 1)]
    // (the resolve warp's 32 lanes after block q's decisions)
    __shared__ __align__(8) uint64_t s_mb[4];

    const int B = a.B;
    const unsigned Bu = (unsigned)B;
    const unsigned R = 4u * Bu;
    const unsigned Rm = R - 1u;
    const int sidx = blockIdx.x;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int dw = dot_index(warp);                       // dot warps: 0..7
    const int dtid = dw >= 0 ? dw * 32 + lane : kBlockThreads;   // dot warps: 0..255
    const int otid = tid - (warp > kResolveWarp ? 32 : 0);       // the other warps: 0..319
    const int lo = a.slice_lo[sidx];
    const int ns = a.slice_lo[sidx + 1] - lo;
    const int nbytes = ((ns + kChunk - 1) / kChunk) * 16;
    const int64_t byte_lo = lo / 4;
    const PipePlan plan = make_pipe_plan(a.slice_max, a.slot_bytes, B, a.n_groups);
    const int npairs = B * (B - 1) / 2;
    const unsigned gent = (unsigned)block_gram_entries(B);    // per shared-memory Gram slot
    const unsigned gst = (unsigned)block_stage_entries(B);    // per staging slot
    const unsigned M32 = (unsigned)a.M;
    const int nblk = (int)((M32 + Bu - 1) / Bu);
    auto nb_of = [&](int q) { return (int)min(Bu, M32 - (unsigned)q * Bu); };

    uint32_t *planes = reinterpret_cast<uint32_t *>(smem + plan.planes);
    long long *fix = reinterpret_cast<long long *>(smem + plan.fix);
    uint8_t *ring_codes = smem + plan.codes;
    BlockRec *ring_rec = reinterpret_cast<BlockRec *>(smem + plan.recs);
    float2 *gbuf = reinterpret_cast<float2 *>(smem + plan.gram);
    uint8_t *pair_ab = smem + plan.pairs;
    float *gcf = reinterpret_cast<float *>(smem + plan.gcf);
    float *gbf = reinterpret_cast<float *>(smem + plan.gbf);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + plan.mbar);
    float2 *gstage = reinterpret_cast<float2 *>(a.gstage);

    // ---- prologue: residual slice (with eps -= mu_new) to fixed point, tables
    {
        float muh, mul;
        df_from_double(-a.mu_new, muh, mul);
        for (int b = tid; b < a.slice_max / 4; b += kBlockThreads) {
            long long E[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                E[i] = 0;
                const int ii = 4 * b + i;
                if (ii < ns) {
                    float h = a.eps_hi[lo + ii], l = a.eps_lo[lo + ii];
                    df_add(h, l, muh, mul);
                    if (!df_to_fix(h, l, E[i])) {
                        atomicCAS(a.err, kDevOk, kDevRange);
                        E[i] = 0;
                    }
                }
            }
            store_fix4(planes, b, E);
            reinterpret_cast<longlong2 *>(fix)[2 * b] = make_longlong2(E[0], E[1]);
            reinterpret_cast<longlong2 *>(fix)[2 * b + 1] = make_longlong2(E[2], E[3]);
        }
    }
    for (int i = tid; i < a.n_groups; i += kBlockThreads) {
        s_gk[i] = a.gK[i];
        const double *row = a.gconst + (size_t)i * kMaxK * 4;
        double hmax = 0.0, hmin = 0.0;
        for (int k = 1; k < a.gK[i]; ++k) {
            hmax = fmax(hmax, row[4 * k + 2]);
            hmin = fmin(hmin, row[4 * k + 2]);
        }
        s_H[i] = (float)((hmax - hmin) * (1.0 + 1e-6));
    }
    for (int i = tid; i < a.n_groups * kMaxK; i += kBlockThreads) {
        const int g = i / kMaxK, k = i - g * kMaxK;
        const double *row = a.gconst + (size_t)g * kMaxK * 4;
        gcf[2 * i] = k == 0 ? 0.f : (float)(row[4 * k] - row[0]);
        gcf[2 * i + 1] = k == 0 ? 0.f : (float)row[4 * k + 2];
        df_from_double(row[4 * k + 3], gbf[4 * i], gbf[4 * i + 1]);
        df_from_double(row[4 * k + 1], gbf[4 * i + 2], gbf[4 * i + 3]);
    }
    for (int pb = 1 + tid; pb < B; pb += kBlockThreads)
        for (int pa = 0; pa < pb; ++pa) {
            const int p = pb * (pb - 1) / 2 + pa;
            pair_ab[2 * p] = (uint8_t)pa;
            pair_ab[2 * p + 1] = (uint8_t)pb;
        }
    if (tid == 0) {
        s_abort = 0;
        s_nupd[0] = 0;
        s_nupd[1] = 0;
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        mbar_init(&s_mb[0], kOtherThreads);
        mbar_init(&s_mb[1], kOtherThreads);
        mbar_init(&s_mb[2], 32);
        mbar_init(&s_mb[3], 32);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();

    // ---- ring of records and genotype code slices (cp.async)
    unsigned rec_issued = 0;
    auto issue_recs = [&](unsigned upto, int idx, int stride) {
        upto = min(upto, M32);
        if (upto <= rec_issued)
            return;
        constexpr unsigned kParts = sizeof(BlockRec) / 16;
        const unsigned n = (upto - rec_issued) * kParts;
        for (unsigned e = (unsigned)idx; e < n; e += (unsigned)stride) {
            const unsigned q = rec_issued + e / kParts;
            const unsigned c = e % kParts;
            cp_async16(reinterpret_cast<unsigned char *>(&ring_rec[q & Rm]) + 16 * c,
                       reinterpret_cast<const unsigned char *>(&a.brec[q]) + 16 * c);
        }
        rec_issued = upto;
    };
    // Code slices of a block, copied by the dot warps: thread t copies chunk
    // my_c of the block's markers my_q, my_q + per_pass, ...; the marker ids come
    // from the id ring in shared memory.
    const unsigned chunks = (unsigned)nbytes / 16u;
    const unsigned per_pass = chunks ? (unsigned)(kDotWarps * 32) / chunks : 0u;
    const unsigned my_q = chunks ? (unsigned)dtid / chunks : 0u;
    const unsigned my_c = chunks ? (unsigned)dtid - my_q * chunks : 0u;
    // ids of block q into its ring slot (threads idx, idx + stride, ...): 16-byte
    // copies of four ids, 4-byte copies for a partial last group
    auto issue_ids = [&](int q, int idx, int stride) {
        if (q >= nblk)
            return;
        const unsigned qb = (unsigned)q * Bu, nbq = (unsigned)nb_of(q);
        uint32_t *dst = s_ids[q % kIdSlots];
        for (unsigned g = (unsigned)idx; 4u * g < nbq; g += (unsigned)stride) {
            if (4u * g + 4u <= nbq) {
                cp_async16(dst + 4u * g, a.order + qb + 4u * g);
            } else {
                for (unsigned m = 4u * g; m < nbq; ++m)
                    cp_async4(dst + m, a.order + qb + m);
            }
        }
    };
    auto issue_block_codes = [&](int q) {
        if (q >= nblk || dw < 0 || my_q >= per_pass)
            return;
        const unsigned qb = (unsigned)q * Bu, nbq = (unsigned)nb_of(q);
        const uint32_t *ids = s_ids[q % kIdSlots];
        for (unsigned m = my_q; m < nbq; m += per_pass)
            cp_async16(ring_codes + ((qb + m) & Rm) * a.slot_bytes + 16 * my_c,
                       a.codes + (int64_t)ids[m] * a.col_stride + byte_lo + 16 * my_c);
    };

    // ---- Gram entries of block q (chore warp): CTA s gathers entries
    // e = s + G*(l + 32*i) from the packed Gram into staging slot q % 8.  The
    // first kGather entries of each thread are loaded one iteration before they
    // are stored, so that the random reads of the Gram never delay the
    // signal before the barrier arrival (more than kGather entries per lane, on
    // grids below 80 CTAs, are loaded when stored).
    constexpr int kGather = 4;
    float2 gval[kGather];
    int gent_mine[kGather] = {-1, -1, -1, -1};
    auto gram_entry = [&](int q, unsigned e, float2 *out) -> bool {
        const unsigned q0 = (unsigned)q * Bu;
        const int nbq = nb_of(q);
        unsigned pa, pb, qa;
        if (e < (unsigned)npairs) {
            pa = pair_ab[2 * e];
            pb = pair_ab[2 * e + 1];
            if ((int)pb >= nbq)
                return false;
            qa = q0 + pa;
        } else {
            // near (block q-1) or far (block q-2) entries; those blocks are full
            const unsigned c = e - (unsigned)npairs;
            const unsigned back = c < Bu * Bu ? 1u : 2u;
            if ((unsigned)q < back)
                return false;
            const unsigned cc = c - (back - 1u) * Bu * Bu;
            pa = cc / Bu;
            pb = cc - pa * Bu;
            if ((int)pb >= nbq)
                return false;
            qa = q0 - back * Bu + pa;
        }
        const int64_t ja = s_ids[(qa / Bu) % kIdSlots][qa % Bu], jb = s_ids[q % kIdSlots][pb];
        const int64_t hi = ja > jb ? ja : jb, lw = ja > jb ? jb : ja;
        *out = __ldg(&a.gram[hi * (hi - 1) / 2 + lw]);
        return true;
    };
    auto gather_load = [&](int q) {
#pragma unroll
        for (int k = 0; k < kGather; ++k) {
            gent_mine[k] = -1;
            const unsigned e = (unsigned)sidx + (unsigned)(lane + 32 * k) * (unsigned)a.G;
            if (e < gst && gram_entry(q, e, &gval[k]))
                gent_mine[k] = (int)e;
        }
    };
    auto gather_store = [&](int q) {
        float2 *slot = gstage + (size_t)(q % kStageSlots) * gst;
#pragma unroll
        for (int k = 0; k < kGather; ++k)
            if (gent_mine[k] >= 0)
                slot[gent_mine[k]] = gval[k];
        for (unsigned e = (unsigned)sidx + (unsigned)(lane + 32 * kGather) * (unsigned)a.G; e < gst;
             e += 32u * (unsigned)a.G) {
            float2 v;
            if (gram_entry(q, e, &v))
                slot[e] = v;
        }
    };

    auto publish = [&](unsigned long long *acc, __int128 x) {
        const Fx f = fx_split(x);
        red_add_u64(acc, (unsigned long long)f.hi);
        red_add_u64(acc + 1, f.lo);
    };

    // ---- partial dot products of block q against the current residual (dot
    // warps), exact in integers.  Warp w owns markers w, w+8, ..., w+56 of the
    // block; its lanes stride over the slice's code bytes (lane l reads byte
    // positions b = l mod 32).  Accumulator slot s = 4 m' + k' of lane l holds
    // marker w + 8 (m' ^ (l >> 2)) and limb k' ^ (l & 3) (the plane order of its
    // byte positions), so value s of lane l is value s ^ l of the warp and the
    // reduction is a butterfly without selects: after it lane l holds limb
    // l & 3 of marker w + 8 (l >> 2), and four lanes combine a marker's limbs.
    auto dot_block = [&](int q) {
        const unsigned q0 = (unsigned)q * Bu;
        const int nbq = nb_of(q);
        constexpr int MPW = kMaxSpec / 8;
        int A[MPW * 4], Mx[MPW * 4];
        unsigned cofs[MPW];
#pragma unroll
        for (int k = 0; k < MPW; ++k) {
            // markers past the end of a short block read a stale slot; their
            // sums are never published
            const unsigned m = (unsigned)dw + 8u * ((unsigned)k ^ (unsigned)(lane >> 2));
            cofs[k] = ((q0 + m) & Rm) * (unsigned)a.slot_bytes;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                A[4 * k + t] = 0;
                Mx[4 * k + t] = 0;
            }
        }
        // all 8 slots are summed; with B < 64 the slots past the block read ring
        // slots of other blocks and are never published
        for (int b = lane; b < nbytes; b += 32) {
            const uint4 w0 = reinterpret_cast<const uint4 *>(planes)[2 * b];
            const uint4 w1 = reinterpret_cast<const uint4 *>(planes)[2 * b + 1];
            const int wv[8] = {(int)w0.x, (int)w0.y, (int)w0.z, (int)w0.w,
                               (int)w1.x, (int)w1.y, (int)w1.z, (int)w1.w};
#pragma unroll
            for (int k = 0; k < MPW; ++k) {
                const unsigned v = ring_codes[cofs[k] + b];
                const unsigned sel = code_nibbles(v);
                const int g = (int)__byte_perm(kGenoBytes, 0u, sel);
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    A[4 * k + t] = __dp2a_lo(wv[2 * t], g, A[4 * k + t]);
                    A[4 * k + t] = __dp2a_hi(wv[2 * t + 1], g, A[4 * k + t]);
                }
                if (MISS) {
                    const int mm = (int)__byte_perm(kMissBytes, 0u, sel);
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        Mx[4 * k + t] = __dp2a_lo(wv[2 * t], mm, Mx[4 * k + t]);
                        Mx[4 * k + t] = __dp2a_hi(wv[2 * t + 1], mm, Mx[4 * k + t]);
                    }
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int i = 0; i < o; ++i) {
                A[i] += __shfl_xor_sync(0xffffffffu, A[i + o], o);
                if (MISS)
                    Mx[i] += __shfl_xor_sync(0xffffffffu, Mx[i + o], o);
            }
        }
        // limb l & 3 of marker w + 8 (l >> 2): combine the four limbs (int128)
        const int limb = lane & 3;
        auto combine = [&](int v) {
            __int128 x = (__int128)(long long)v << (16 * limb);
            unsigned long long xl = (unsigned long long)x, xh = (unsigned long long)(x >> 64);
#pragma unroll
            for (int o = 1; o <= 2; o <<= 1) {
                const unsigned long long yl = __shfl_xor_sync(0xffffffffu, xl, o);
                const unsigned long long yh = __shfl_xor_sync(0xffffffffu, xh, o);
                const unsigned long long sl = xl + yl;
                xh = xh + yh + (sl < xl ? 1ull : 0ull);
                xl = sl;
            }
            return (__int128)(((unsigned __int128)xh << 64) | xl);
        };
        const __int128 T = combine(A[0]);
        const __int128 Tm = MISS ? combine(Mx[0]) : (__int128)0;
        const int m = dw + 8 * (lane >> 2);
        if (limb == 0 && m < nbq) {
            unsigned long long *acc =
                a.acc + (size_t)(q % kAccBufs) * kAccBufWords + ((size_t)(sidx % kAccCopies) * kMaxSpec + m) * 4;
            publish(acc, T << (60 - kFrac));
            if (MISS && Tm != 0)
                publish(acc + 2, Tm << (60 - kFrac));
        }
    };
    auto arrive = [&](int q) {
        red_release_add_u64(a.counter + ((size_t)(q & 1) * kCounters + (size_t)(sidx % kCounters)) * kCounterStride,
                            1ull);
    };

    // profiling (first CTA): dot side on thread 0, resolve side on the resolve
    // warp's lane 0
    const bool prof_d = PROF && sidx == 0 && tid == 0;
    const bool prof_r = PROF && sidx == 0 && tid == kResolveWarp * 32;
    long long ph[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    long long tp = (prof_d || prof_r) ? clk() : 0;
    auto mark = [&](bool on, int k) {
        if (on) {
            const long long t = clk();
            ph[k] += t - tp;
            tp = t;
        }
    };
    unsigned long long *fb_counter = PROF ? reinterpret_cast<unsigned long long *>(a.prof + 8) : nullptr;
    long long steps = 0;
    const bool prof_h = PROF && sidx == 0 && tid == kInputWarp * 32;
    // event timeline (counting variant): kTimelineIters iterations around the
    // middle of the sweep, every CTA
    const int tl_r0 = nblk / 2 > kTimelineIters / 2 ? nblk / 2 - kTimelineIters / 2 : 0;
    auto stamp = [&](int r, int e) {
        if (PROF && a.tline && r >= tl_r0 && r < tl_r0 + kTimelineIters)
            a.tline[((size_t)(r - tl_r0) * (size_t)a.G + (size_t)sidx) * kTimelineEvents + e] = global_timer_ns();
    };
    int cp_issued = -1, cp_waited = -1;   // resolve warp: Gram copies issued / waited for

    // ---- rank-U residual update of block q (dot warps, run at the start of the
    // next iteration while the resolve warp works on block q+1):
    // E += round(dBeta_u * x_u(code) * 2^kFrac) (df_to_fix_near)
    auto apply_update = [&](int q) {
        const int par = q & 1;
        const int U = s_nupd[par];
        if (U == 0)
            return;
        const unsigned qb = (unsigned)q * Bu;
        if (dtid < 4 * U) {
            const int u = dtid >> 2, code = dtid & 3;
            const float2 dB = s_dB[par][u];
            const float4 xv = s_x[par][u][code >> 1];
            const float xh = (code & 1) ? xv.z : xv.x, xl = (code & 1) ? xv.w : xv.y;
            float dh, dl;
            df_mul(dB.x, dB.y, xh, xl, dh, dl);
            long long D = 0;
            if (!df_to_fix_near(dh, dl, D))
                atomicCAS(a.err, kDevOk, kDevRange);
            s_D[u][code] = D;
            if (code == 0)
                s_uoff[u] = ((qb + (unsigned)s_upd[par][u]) & Rm) * (unsigned)a.slot_bytes;
        }
        if (tid == 0)
            stamp(q + 1, 12);
        dot_warps_sync();
        if (tid == 0)
            stamp(q + 1, 13);
        // The sum of the residual is left as it was at the sweep start: the
        // standardised columns sum to zero, so a dense update moves it only
        // by rounding (dBeta times a column sum of order 1e-11).
        for (int b = dtid; b < nbytes; b += kDotWarps * 32) {
            const longlong2 e01 = reinterpret_cast<const longlong2 *>(fix)[2 * b];
            const longlong2 e23 = reinterpret_cast<const longlong2 *>(fix)[2 * b + 1];
            long long E[4] = {e01.x, e01.y, e23.x, e23.y};
            // four updates' code bytes loaded at a time
            int u = 0;
            for (; u + 4 <= U; u += 4) {
                unsigned v[4];
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    v[k] = ring_codes[s_uoff[u + k] + b];
#pragma unroll
                for (int k = 0; k < 4; ++k)
#pragma unroll
                    for (int i = 0; i < 4; ++i)
                        E[i] += s_D[u + k][(v[k] >> (2 * i)) & 3u];
            }
            for (; u < U; ++u) {
                const unsigned v = ring_codes[s_uoff[u] + b];
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    E[i] += s_D[u][(v >> (2 * i)) & 3u];
            }
            // padding individuals past the slice end keep a zero residual
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                if (4 * b + i >= ns)
                    E[i] = 0;
                if (E[i] >= kFixMax || E[i] <= -kFixMax) {
                    atomicCAS(a.err, kDevOk, kDevRange);
                    E[i] = 0;
                }
            }
            reinterpret_cast<longlong2 *>(fix)[2 * b] = make_longlong2(E[0], E[1]);
            reinterpret_cast<longlong2 *>(fix)[2 * b + 1] = make_longlong2(E[2], E[3]);
            store_fix4(planes, b, E);
        }
        if (tid == 0)
            stamp(q + 1, 14);
        dot_warps_sync();
        if (tid == 0)
            stamp(q + 1, 15);
    };

    constexpr int kCopyThread = kChoreWarp * 32; // issues the Gram bulk copies

    // ---- inputs of block q (the input warp, one iteration before block q is
    // resolved): first the far corrections dBeta_p * G[p, t] of block q-2's
    // residual-changing markers p (their updates are not in the residual the
    // dot products saw; block q-2's decisions and block q's staged entries are
    // known before barrier q, so they are read while the last CTAs arrive);
    // then wait for barrier q (lane c < 8 polls counter c) and form per marker
    // num = sigma * sum(g*eps) + cst + dm * sum_missing(eps) + far as
    // double-float, with the FP32 sampler's per-marker values.
    long long th_poll = 0, th_in = 0;
    auto prepare_inputs = [&](int q, bool prof) {
        const int par = q & 1, nbq = nb_of(q);
        const unsigned qb = (unsigned)q * Bu;
        // far corrections (block q-2 has the parity of q), eight rows of
        // entries in flight at a time
        float fh[2] = {0.f, 0.f}, fl[2] = {0.f, 0.f};
        if (q >= 2) {
            const int Uf = s_nupd[par];
            const float2 *gfar = gstage + (size_t)(q % kStageSlots) * gst + gent;
            for (int u0 = 0; u0 < Uf; u0 += 8) {
                float2 g[8][2];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int p = u0 + k < Uf ? s_upd[par][u0 + k] : 0;
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        g[k][h] = u0 + k < Uf ? ld_relaxed_f2(gfar + (size_t)p * B + lane + 32 * h)
                                              : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    if (u0 + k >= Uf)
                        break;
                    const float2 dB = s_dB[par][u0 + k];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        float ph2, pl2;
                        df_mul(dB.x, dB.y, g[k][h].x, g[k][h].y, ph2, pl2);
                        df_add(fh[h], fl[h], ph2, pl2);
                    }
                }
            }
        }
        if (lane == 0)
            stamp(q - 1, 10);
        const long long t0 = prof ? clk() : 0;
        bool ok = true;
        if (lane < kCounters) {
            // lane c waits for the CTAs s = c (mod 8), and the phantom arrivals on counter 0
            const unsigned long long per = (unsigned long long)((q >> 1) + 1);
            const int nc = lane < a.G ? (a.G - lane + kCounters - 1) / kCounters : 0;
            const unsigned long long target = (unsigned long long)(nc + (lane == 0 ? a.phantom : 0)) * per;
            const unsigned long long *ctr =
                a.counter + ((size_t)(q & 1) * kCounters + (size_t)lane) * kCounterStride;
            if (ld_acquire_u64(ctr) < target) {
                const uint64_t tw = global_timer_ns();
                unsigned spins = 0;
                while (ld_acquire_u64(ctr) < target) {
                    if ((++spins & 255u) == 0 &&
                        (*(volatile int *)a.err != kDevOk || global_timer_ns() - tw > a.timeout_ns)) {
                        atomicCAS(a.err, kDevOk, kDevTimeout);
                        ok = false;
                        break;
                    }
                }
            }
        }
        ok = __all_sync(0xffffffffu, ok);
        if (!ok && lane == 0)
            s_abort = 1;
        __syncwarp();
        if (lane == 0)
            stamp(q - 1, 2);
        const long long t1 = prof ? clk() : 0;
        if (!ok)
            return;
        // the published sums of the lane's two markers, every load issued
        // before the first use; the copies' 56-bit low words sum to less than
        // 2^64 (152 parts at most)
        const unsigned long long *accb = a.acc + (size_t)(q % kAccBufs) * kAccBufWords;
        long long th64[2] = {0, 0}, sh64[2] = {0, 0};
        unsigned long long tl64[2] = {0ull, 0ull}, sl64[2] = {0ull, 0ull};
#pragma unroll
        for (int c = 0; c < kAccCopies; ++c) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const unsigned long long *ac = accb + ((size_t)c * kMaxSpec + lane + 32 * h) * 4;
                th64[h] += (long long)ld_relaxed_u64(ac);
                tl64[h] += ld_relaxed_u64(ac + 1);
                if (MISS) {
                    sh64[h] += (long long)ld_relaxed_u64(ac + 2);
                    sl64[h] += ld_relaxed_u64(ac + 3);
                }
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int m = lane + 32 * h;
            float nh = 0.f, nl = 0.f, uf = 2.f;
            unsigned meta = 2u << 8;
            if (m < nbq) {
                const BlockRec &rc = ring_rec[(qb + m) & Rm];
                float th, tl;
                fx_to_df(th64[h], tl64[h], th, tl);
                df_mul(rc.sig[0], rc.sig[1], th, tl, nh, nl);
                df_add(nh, nl, rc.cst[0], rc.cst[1]);
                if (MISS) {
                    float sh, sl, qh, ql;
                    fx_to_df(sh64[h], sl64[h], sh, sl);
                    df_mul(rc.dm[0], rc.dm[1], sh, sl, qh, ql);
                    df_add(nh, nl, qh, ql);
                }
                df_add(nh, nl, fh[h], fl[h]);
                uf = rc.uf;
                meta = (unsigned)rc.group | ((unsigned)s_gk[rc.group] << 8) | (rc.bnz ? 1u << 16 : 0u);
            }
            s_inum[par][m] = make_float2(nh, nl);
            s_iuf[par][m] = uf;
            s_imeta[par][m] = meta;
        }
        if (prof) {
            const long long t2 = clk();
            th_poll += t1 - t0;
            th_in += t2 - t1;
        }
    };

    // ---- first blocks: records 0..3 and codes 0..2 resident; the Gram entries
    // of blocks 0..2 staged and blocks 0 and 1's dot products published before
    // the arrivals at barriers 0 and 1; block 0's inputs assembled
    issue_recs(4u * Bu, tid, kBlockThreads);
    for (int q = 0; q < 5; ++q)
        issue_ids(q, tid, kBlockThreads);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    for (int q = 0; q < 3; ++q)
        issue_block_codes(q);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    if (dw >= 0) {
        dot_block(0);
        if (nblk > 1)
            dot_block(1);
        arrive_sync();
        if (tid == 0) {
            arrive(0);
            if (nblk > 1)
                arrive(1);
        }
    } else if (warp == kChoreWarp) {
        for (int q = 0; q < 3 && q < nblk; ++q) {
            gather_load(q);
            gather_store(q);
        }
        if (nblk > 3)
            gather_load(3);
        __syncwarp();
        chore_signal();
    } else if (warp == kInputWarp) {
        prepare_inputs(0, false);
    }

    int r = 0;
    if (prof_d || prof_r)
        tp = clk();
    // profiling: per role, the clock from the iteration's start to the end of
    // its work (dot side on thread 0, chore warp, resolve warp, input warp)
    long long t_it = 0, t_end = 0;
    const bool prof_e = PROF && sidx == 0 && (tid & 31) == 0 &&
                        (tid == 0 || warp == kChoreWarp || warp == kResolveWarp || warp == kInputWarp);
    // Waits for a role signal, at most the wait limit; false on timeout or
    // when another warp aborted.
    auto role_wait = [&](uint64_t *m, unsigned parity) -> bool {
        if (mbar_test(m, parity))
            return true;
        const uint64_t t0 = global_timer_ns();
        unsigned spins = 0;
        while (!mbar_try(m, parity)) {
            if ((++spins & 15u) == 0) {
                if (*(volatile int *)&s_abort)
                    return false;
                if (global_timer_ns() - t0 > a.timeout_ns) {
                    atomicCAS(a.err, kDevOk, kDevTimeout);
                    s_abort = 1;
                    return false;
                }
            }
        }
        return true;
    };
    // GO(0): block 0's inputs and records are in place
    cp_async_wait_all();
    __syncthreads();
    if (warp != kResolveWarp)
        mbar_arrive(&s_mb[0]);

    if (warp == kResolveWarp) {
        // ---- resolve warp: block r once GO(r) (inputs of block r, the
        // residual-changing markers of block r-2 applied and read, its outputs
        // read), then RESOLVED(r)
        for (; r < nblk; ++r) {
            const bool ok = role_wait(&s_mb[r & 1], (unsigned)((r >> 1) & 1));
            if (__any_sync(0xffffffffu, !ok || *(volatile int *)&s_abort != 0))
                break;
            if (lane == 0)
                stamp(r, 6);
            if (prof_e)
                t_it = clk();
            const unsigned q0 = (unsigned)r * Bu;
            const int nb = nb_of(r);
            // ---- resolve side
            mark(prof_r, 8);
            {
                const int par = r & 1;
                float nh[2], nl[2], ufr[2];
                int grp[2], kk[2];
                bool own[2], bnz[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int m = lane + 32 * h;
                    own[h] = m < nb;
                    const float2 n = s_inum[par][m];
                    nh[h] = n.x;
                    nl[h] = n.y;
                    ufr[h] = s_iuf[par][m];
                    const unsigned meta = s_imeta[par][m];
                    grp[h] = (int)(meta & 0xFFu);
                    kk[h] = (int)((meta >> 8) & 0xFFu);
                    bnz[h] = (meta >> 16) != 0u;
                }
                // Gram entries of block r (copied one iteration ahead)
                bool gok = mbar_wait(&mbar[r & 1], (unsigned)((r >> 1) & 1), a.timeout_ns);
                gok = __all_sync(0xffffffffu, gok);
                if (gok)
                    cp_waited = r;
                if (!gok) {
                    if (lane == 0) {
                        atomicCAS(a.err, kDevOk, kDevTimeout);
                        s_abort = 1;
                    }
                } else {
                    const float2 *gtri = gbuf + (size_t)(r & 1) * gent;
                    const float2 *gcross = gtri + npairs;
                    // updates of block r-1, not yet in the residual the dot products saw
                    const int pp = (r - 1) & 1;
                    const int Up = r > 0 ? s_nupd[pp] : 0;
                    for (int u = 0; u < Up; ++u) {
                        const int p = s_upd[pp][u];
                        const float2 dB = s_dB[pp][u];
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            if (!own[h])
                                continue;
                            const float2 g2 = gcross[p * B + lane + 32 * h];
                            float ph2, pl2;
                            df_mul(dB.x, dB.y, g2.x, g2.y, ph2, pl2);
                            df_add(nh[h], nl[h], ph2, pl2);
                        }
                    }
                    __syncwarp();
                    mark(prof_r, 7);


                    // ---- resolve block r: lane l owns markers l and l+32; a
                    // decision is kept while its certified margin covers the move of
                    // num^2; ballots find the first residual-changing marker p, the
                    // later markers move by dBeta_p * G[p, t]
                    float ch[2] = {0.f, 0.f}, cl[2] = {0.f, 0.f};
                    float fbh[2] = {0.f, 0.f}, fbl[2] = {0.f, 0.f}, fah[2] = {0.f, 0.f}, fal[2] = {0.f, 0.f};
                    float sref[2] = {0.f, 0.f}, wmar[2] = {-1.f, -1.f}, hg[2];
                    int comp[2] = {-1, -1};
                    bool fb[2] = {false, false};
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        hg[h] = s_H[grp[h]];
                    int next = 0, nupd = 0;
                    while (true) {
                        const long long tl0 = prof_r ? clk() : 0;
                        bool need[2], upd[2];
                        float sx[2];
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            float xh = nh[h], xl = nl[h];
                            df_add(xh, xl, ch[h], cl[h]);
                            sx[h] = __fmaf_rn(xh, xh, 2.f * xh * xl);
                            const float delta = fabsf(sx[h] - sref[h]) * 1.000001f + 4e-7f * (sx[h] + sref[h]);
                            need[h] = own[h] && lane + 32 * h >= next && !(hg[h] * delta <= wmar[h]);
                        }
                        const unsigned need_halves = (__ballot_sync(0xffffffffu, need[0]) ? 1u : 0u) |
                                                     (__ballot_sync(0xffffffffu, need[1]) ? 2u : 0u);
                        if (need_halves) {
                            bool slow[2];
#pragma unroll
                            for (int h = 0; h < 2; ++h) {
                                slow[h] = false;
                                // a half none of whose markers needs a new decision is skipped
                                if (!(need_halves & (1u << h)))
                                    continue;
                                int c;
                                float w;
                                const bool okm =
                                    pick_margin<KM>(sx[h], ufr[h], gcf + (size_t)grp[h] * kMaxK * 2, kk[h], c, w);
                                if (need[h]) {
                                    comp[h] = c;
                                    fb[h] = false;
                                    sref[h] = sx[h];
                                    wmar[h] = okm ? w : -1.f;
                                }
                                slow[h] = need[h] && !okm;
                            }
                            if (__any_sync(0xffffffffu, slow[0] || slow[1])) {
#pragma unroll
                                for (int h = 0; h < 2; ++h) {
                                    if (!slow[h])
                                        continue;
                                    // 700 guards possibly active, or u near a boundary:
                                    // the guarded FP32 sampler, then FP64
                                    float xh = nh[h], xl = nl[h];
                                    df_add(xh, xl, ch[h], cl[h]);
                                    int c;
                                    float a0;
                                    if (pick_f32<KM>(xh, xl, ufr[h], gcf + (size_t)grp[h] * kMaxK * 2, kk[h], c,
                                                     a0)) {
                                        comp[h] = c;
                                    } else {
                                        const BlockRec &rc = ring_rec[(q0 + lane + 32 * h) & Rm];
                                        const Pick r64 = pick_marker<false, KM>(
                                            (double)xh + (double)xl, rc.u, rc.z, rc.beta_old,
                                            a.gconst + (size_t)grp[h] * kMaxK * 4, kk[h]);
                                        comp[h] = r64.comp;
                                        df_from_double(r64.acum0, fah[h], fal[h]);
                                        df_from_double(r64.beta, fbh[h], fbl[h]);
                                        fb[h] = true;
                                        if (sidx == 0 && fb_counter)
                                            atomicAdd(fb_counter, 1ull);
                                    }
                                }
                            }
                        }
#pragma unroll
                        for (int h = 0; h < 2; ++h)
                            upd[h] = own[h] && lane + 32 * h >= next && (bnz[h] || comp[h] > 0);
                        const long long tl1 = prof_r ? clk() : 0;
                        if (prof_r)
                            ph[9] += tl1 - tl0;
                        ++steps;
                        const unsigned b0 = __ballot_sync(0xffffffffu, upd[0]);
                        const unsigned b1 = __ballot_sync(0xffffffffu, upd[1]);
                        const int p = b0 ? __ffs(b0) - 1 : (b1 ? 32 + __ffs(b1) - 1 : kMaxSpec);
                        if (p >= nb)
                            break;
                        // dBeta_p = beta_old - beta_new as double-float, by the owner
                        const int owner = p & 31;
                        const bool half = p >= 32;
                        float dh = 0.f, dl = 0.f;
                        if (lane == owner) {
                            const BlockRec &rc = ring_rec[(q0 + p) & Rm];
                            const int c = half ? comp[1] : comp[0];
                            if (c >= 0) {
                                float bh = 0.f, bl = 0.f;
                                if (c > 0) {
                                    if (half ? fb[1] : fb[0]) {
                                        bh = half ? fbh[1] : fbh[0];
                                        bl = half ? fbl[1] : fbl[0];
                                    } else {
                                        float xh = half ? nh[1] : nh[0], xl = half ? nl[1] : nl[0];
                                        df_add(xh, xl, half ? ch[1] : ch[0], half ? cl[1] : cl[0]);
                                        const float4 gc =
                                            reinterpret_cast<const float4 *>(gbf + (size_t)rc.group * kMaxK * 4)[c];
                                        float ph2, pl2;
                                        df_mul(rc.zf[0], rc.zf[1], gc.x, gc.y, bh, bl);
                                        df_mul(xh, xl, gc.z, gc.w, ph2, pl2);
                                        df_add(bh, bl, ph2, pl2);
                                    }
                                }
                                dh = rc.bo[0];
                                dl = rc.bo[1];
                                df_add(dh, dl, -bh, -bl);
                            }
                        }
                        dh = __shfl_sync(0xffffffffu, dh, owner);
                        dl = __shfl_sync(0xffffffffu, dl, owner);
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int m = lane + 32 * h;
                            if (own[h] && m > p) {
                                const float2 g2 = gtri[m * (m - 1) / 2 + p];
                                float ph2, pl2;
                                df_mul(dh, dl, g2.x, g2.y, ph2, pl2);
                                df_add(ch[h], cl[h], ph2, pl2);
                            }
                        }
                        if (lane == 0) {
                            s_upd[par][nupd] = p;
                            s_dB[par][nupd] = make_float2(dh, dl);
                        }
                        if (lane == owner) {
                            const float4 *xs = reinterpret_cast<const float4 *>(ring_rec[(q0 + p) & Rm].x);
                            s_x[par][nupd][0] = xs[0];
                            s_x[par][nupd][1] = xs[1];
                        }
                        ++nupd;
                        next = p + 1;
                        if (prof_r)
                            ph[10] += clk() - tl1;
                    }
                    if (lane == 0)
                        s_nupd[par] = nupd;
                    // the decisions of the markers whose outputs this CTA writes
                    // (sweep position p by CTA p mod G)
                    {
                        BlockOut &o = s_out[r & 1];
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int m = lane + 32 * h;
                            if ((q0 + (unsigned)m) % (unsigned)a.G != (unsigned)sidx) {
                                o.code[m] = -2;
                                continue;
                            }
                            float xh = nh[h], xl = nl[h];
                            df_add(xh, xl, ch[h], cl[h]);
                            o.x[m] = make_float2(xh, xl);
                            o.fb[m] = make_float2(fbh[h], fbl[h]);
                            o.fa[m] = make_float2(fah[h], fal[h]);
                            o.uf[m] = ufr[h];
                            o.group[m] = grp[h];
                            o.code[m] = own[h] ? ((comp[h] & 0xFF) | (fb[h] ? 0x100 : 0)) : -2;
                            if (own[h]) {
                                const BlockRec &rc = ring_rec[(q0 + m) & Rm];
                                o.zf[m] = make_float2(rc.zf[0], rc.zf[1]);
                                o.j[m] = rc.j;
                            }
                        }
                    }
                    mark(prof_r, 3);
                }
            }
            if (prof_e)
                t_end += clk() - t_it;
            __syncwarp();
            if (lane == 0)
                stamp(r, 7);
            mbar_arrive(&s_mb[2 + (r & 1)]);   // RESOLVED(r)
        }
    } else {
        // ---- the other warps, iteration r once block r-1 is resolved (its
        // decisions, and the ring and shared Gram slots it read, are free);
        // the iteration ends with the others' barrier (cp.async data of every
        // thread visible)
        for (; r < nblk; ++r) {
            const bool ok = r == 0 || role_wait(&s_mb[2 + ((r - 1) & 1)], (unsigned)(((r - 1) >> 1) & 1));
            if (others_any(!ok || *(volatile int *)&s_abort != 0))
                break;
            if (tid == 0)
                stamp(r, 0);
            if (prof_e)
                t_it = clk();
            mark(prof_d, 0);
            issue_recs((unsigned)(r + 4) * Bu, otid, kOtherThreads);
            issue_ids(r + 5, otid, kOtherThreads);
            cp_async_commit();

            if (warp == kChoreWarp) {
                // ---- chore warp: Gram copy of block r+1 (its staging was published
                // by barrier r, which this warp passed in the previous iteration;
                // blocks 0..2 by barrier 0), issued early so that the L2 burst of
                // 152 CTAs copying the same slot overlaps the dot products; staged
                // Gram entries of block r+3 (loaded in the previous iteration) and
                // the zeroed accumulators of block r+4, signalled to the dot warps
                // before their arrival at barrier r+2; then the Gram loads of
                // block r+4 and the outputs of block r-1
                auto issue_bulk_next = [&]() {
                    if (lane == 0 && r + 1 < nblk) {
                        const int q = r + 1;
                        fence_proxy_async();
                        mbar_expect_tx(&mbar[q & 1], (unsigned)(gent * sizeof(float2)));
                        bulk_copy_g2s(gbuf + (size_t)(q & 1) * gent, gstage + (size_t)(q % kStageSlots) * gst,
                                      (unsigned)(gent * sizeof(float2)), &mbar[q & 1]);
                        cp_issued = q;
                    }
                };
                if (lane == 0 && r == 0) {
                    fence_proxy_async();
                    mbar_expect_tx(&mbar[0], (unsigned)(gent * sizeof(float2)));
                    bulk_copy_g2s(gbuf, gstage, (unsigned)(gent * sizeof(float2)), &mbar[0]);
                    cp_issued = 0;
                }
                issue_bulk_next();
                if (r + 3 < nblk)
                    gather_store(r + 3);
                // block r+4's accumulators, zeroed in shares of 32 words by the
                // first CTAs
                if (r + 4 < nblk)
                    for (int i = sidx * 32 + lane; i < kAccBufWords; i += 32 * a.G)
                        a.acc[(size_t)((r + 4) % kAccBufs) * kAccBufWords + i] = 0ull;
                __syncwarp();
                chore_signal();
                if (lane == 0)
                    stamp(r, 4);
                if (r + 4 < nblk)
                    gather_load(r + 4);
                if (lane == 0)
                    stamp(r, 11);
                if (r >= 1)
                    write_block_outputs<KM>(a, s_out[(r - 1) & 1], gcf, s_gk, gbf, lane);
                if (lane == 0)
                    stamp(r, 5);
                mbar_arrive(&s_mb[(r + 1) & 1]);   // GO(r+1): block r-1's outputs read
            } else if (warp == kInputWarp) {
                // ---- input warp: block r+1's inputs
                if (r + 1 < nblk)
                    prepare_inputs(r + 1, prof_h);
                if (lane == 0)
                    stamp(r, 3);
                mbar_arrive(&s_mb[(r + 1) & 1]);   // GO(r+1): block r+1's inputs
            } else if (dw >= 0) {
                // ---- dot side: update of block r-1, the code slices of block r+3
                // into the slot block r-1 held, dots of block r+2 and their
                // publication
                if (r >= 1)
                    apply_update(r - 1);
                mbar_arrive(&s_mb[(r + 1) & 1]);   // GO(r+1): block r-1's decisions applied
                if (tid == 0)
                    stamp(r, 8);
                mark(prof_d, 4);
                issue_block_codes(r + 3);
                cp_async_commit();
                if (r + 2 < nblk)
                    dot_block(r + 2);
                if (tid == 0)
                    stamp(r, 9);
                arrive_sync();
                if (tid == 0 && r + 2 < nblk)
                    arrive(r + 2);
                if (tid == 0)
                    stamp(r, 1);
                mark(prof_d, 1);
            }
            if (prof_e)
                t_end += clk() - t_it;
            cp_async_wait_all();
            mark(prof_d, 11);
        }
    }
    __syncthreads();
    // the last block: residual update and outputs
    if (!s_abort && r == nblk) {
        if (dw >= 0)
            apply_update(nblk - 1);
        else if (warp == kChoreWarp)
            write_block_outputs<KM>(a, s_out[(nblk - 1) & 1], gcf, s_gk, gbf, lane);
    }
    if (prof_d) {
        a.prof[0] = ph[0];
        a.prof[1] = ph[1];
        a.prof[4] = ph[4];
        a.prof[5] = r;

    }
    if (prof_h) {
        a.prof[2] = th_poll;
        a.prof[11] = th_in;
    }
    if (prof_e)
        a.prof[tid == 0 ? 12 : (warp == kChoreWarp ? 13 : (warp == kResolveWarp ? 14 : 15))] = t_end;
    if (prof_r) {
        a.prof[3] = ph[3];
        a.prof[6] = steps;
        a.prof[7] = ph[7];
        a.prof[9] = ph[9];
        a.prof[10] = ph[10];

    }   // a.prof[8]: FP64 fallbacks of the certified sampler (first CTA)
    cp_async_wait_all();

    // bulk copies still in flight after an abort: wait for them (bounded)
    if (tid == kCopyThread)
        s_cp_issued = cp_issued;
    __syncthreads();
    if (tid == kResolveWarp * 32) {
        for (int q = cp_waited + 1; q <= s_cp_issued; ++q)
            mbar_wait(&mbar[q & 1], (unsigned)((q >> 1) & 1), a.timeout_ns);
    }
    __syncthreads();

    // ---- epilogue: residual back to HBM, per-slice sums
    double s1 = 0.0, s2 = 0.0;
    for (int b = tid; b < nbytes; b += kBlockThreads) {
        const longlong2 e01 = reinterpret_cast<const longlong2 *>(fix)[2 * b];
        const longlong2 e23 = reinterpret_cast<const longlong2 *>(fix)[2 * b + 1];
        const long long E[4] = {e01.x, e01.y, e23.x, e23.y};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (4 * b + i < ns) {
                float h, l;
                fix_to_df(E[i], h, l);
                a.eps_hi[lo + 4 * b + i] = h;
                a.eps_lo[lo + 4 * b + i] = l;
                const double e = (double)h + (double)l;
                s1 += e;
                s2 = fma(e, e, s2);
            }
        }
    }
    __shared__ double s_red[kBlockThreads / 32][2];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane == 0) {
        s_red[warp][0] = s1;
        s_red[warp][1] = s2;
    }
    __syncthreads();
    if (tid == 0) {
        double t1 = 0.0, t2 = 0.0;
        for (int q = 0; q < kBlockThreads / 32; ++q) {
            t1 += s_red[q][0];
            t2 += s_red[q][1];
        }
        a.part[2 * sidx] = t1;
        a.part[2 * sidx + 1] = t2;
        if (sidx == 0) {
            a.stats_out[0] = 0.0;
            *a.rounds_out = r;
        }
    }
}

// --------------------------------------------------------------------------
// Launchers

cudaError_t launch_gather_block(const uint32_t *order, int64_t M, int64_t N, const double *table,
                                const double *scale, const double *beta, const double *u, const double *z,
                                const int32_t *group, double eps_total, BlockRec *rec, cudaStream_t st)
{
    k_gather_block<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(order, M, N, table, scale, beta, u, z, group,
                                                                eps_total, rec);
    return cudaGetLastError();
}

cudaError_t launch_block_finish(int64_t M, const uint8_t *chosen, const float2 *beta_df, const float2 *acum_df,
                                double *beta, double *acum, cudaStream_t st)
{
    k_block_finish<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(M, chosen, beta_df, acum_df, beta, acum);
    return cudaGetLastError();
}

size_t sweep_block_smem_bytes(const SweepArgs &a)
{
    return make_pipe_plan(a.slice_max, a.slot_bytes, a.B, a.n_groups).total;
}

size_t sweep_block_stage_bytes(int B) { return (size_t)kStageSlots * block_stage_entries(B) * sizeof(float2); }

int sweep_block_threads() { return kBlockThreads; }

template <int KM, bool MISS>
static cudaError_t launch_block_km(const SweepArgs &a, size_t smem, cudaStream_t st)
{
    const void *f = a.prof ? (const void *)k_sweep_block<KM, MISS, true> : (const void *)k_sweep_block<KM, MISS, false>;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    SweepArgs args = a;
    void *params[] = {&args};
    return cudaLaunchCooperativeKernel(f, dim3(a.G), dim3(kBlockThreads), params, smem, st);
}

cudaError_t launch_sweep_block(const SweepArgs &a, size_t smem, cudaStream_t st)
{
    if (a.kmax <= 4)
        return a.has_missing ? launch_block_km<4, true>(a, smem, st) : launch_block_km<4, false>(a, smem, st);
    return a.has_missing ? launch_block_km<kMaxK, true>(a, smem, st) : launch_block_km<kMaxK, false>(a, smem, st);
}

int sweep_block_max_ctas_per_sm(size_t smem, std::string *why)
{
    int n = 1 << 30;
    const void *fs[8] = {(const void *)k_sweep_block<4, false, false>,     (const void *)k_sweep_block<4, true, false>,
                         (const void *)k_sweep_block<kMaxK, false, false>, (const void *)k_sweep_block<kMaxK, true, false>,
                         (const void *)k_sweep_block<4, false, true>,      (const void *)k_sweep_block<4, true, true>,
                         (const void *)k_sweep_block<kMaxK, false, true>,  (const void *)k_sweep_block<kMaxK, true, true>};
    for (const void *f : fs) {
        int m = 0;
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, f, kBlockThreads, smem);
        if (e != cudaSuccess) {
            if (why) {
                cudaFuncAttributes fa{};
                cudaFuncGetAttributes(&fa, f);
                *why = std::string(cudaGetErrorString(e)) + " (dynamic shared memory " + std::to_string(smem) +
                       " B, static " + std::to_string(fa.sharedSizeBytes) + " B, " + std::to_string(fa.numRegs) +
                       " registers)";
            }
            cudaGetLastError();
            return 0;
        }
        if (m < 1 && why) {
            cudaFuncAttributes fa{};
            cudaFuncGetAttributes(&fa, f);
            *why = "0 per SM (dynamic shared memory " + std::to_string(smem) + " B, static " +
                   std::to_string(fa.sharedSizeBytes) + " B, " + std::to_string(fa.numRegs) + " registers, at most " +
                   std::to_string(fa.maxThreadsPerBlock) + " threads)";
        }
        n = m < n ? m : n;
    }
    return n;
}

}  // namespace brr
