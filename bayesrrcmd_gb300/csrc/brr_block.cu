// Gram-blocked sweep of the FP32C form over dense markers, software-pipelined
// (sm_103a).
//
// Replaces BayesRBase::processColumn (src/BayesRBase.cpp:287-392) over the
// dense kernel (src/densebayesrkernel.cpp:10-20) for whole sweeps, like the
// restart sweep of brr_sweep.cu, with the precomputed marker Gram matrix
// (packed lower triangle, FP64, brr_gram.cu).
//
// The sweep order is cut into blocks of B consecutive markers.  One CTA per SM
// owns a slice of individuals and keeps its residual slice in shared memory as
// double-float.  Block q's dot products x_t . eps are computed by every CTA
// over its slice and summed across CTAs by exact 128-bit fixed-point integer
// atomics; a grid-wide counter barrier publishes the sums.  Every CTA then
// resolves block q identically: the markers are sampled in order of the
// block, and after every marker p that changes the residual the later markers'
// dot products move by dBeta_p * G[p, t] (exact sequential chain up to
// rounding).  The block's rank-U residual update follows.
//
// Pipelining: block q+1's dot products are computed against the residual
// before block q's update, while block q is being resolved; when block q+1 is
// resolved, the updates of block q enter through the cross Gram entries
// G[p, t], p in block q, t in block q+1.  So per CTA
//   warps 0-7 (dot warps):  dots of block r+1, publish, stage Gram entries of
//                           block r+2, arrive at barrier r+1;
//   warp 8 (resolve warp):  wait for barrier r (arrived one iteration
//                           earlier), bulk-copy block r+1's Gram entries
//                           into shared memory (TMA, mbarrier), assemble block
//                           r's dot products with the corrections of block
//                           r-1, resolve block r;
//   all warps:              rank-U update of block r.
// The grid barrier is polled about one iteration after its last arrival, so
// its latency leaves the critical path.
//
// Buffers and why their counts suffice (iteration r: dot side publishes block
// r+1, stages block r+2, arrives at barrier r+1; resolve side waits for barrier
// r, reads block r's sums, copies block r+1's Gram entries):
//  * two barrier counters, barrier q on counter q % 2 with target
//    (G + phantom) * (q / 2 + 1): a CTA arrives at barrier q+2 only after its
//    resolve warp passed barrier q, so two barriers at most are open;
//  * 8 fixed-point accumulator buffers (block q in buffer q % 8): the first
//    CTA zeroes block q+3's buffer in iteration q before arriving at barrier
//    q+1, after it passed barrier q-1, which every CTA arrived at after it had
//    read the sums of block q-3 and earlier (the buffer last held block q-5);
//    publishes of block q+3 come after barrier q+1;
//  * 8 Gram staging slots in global memory (block q in slot q % 8), written in
//    iteration q-2 after barrier q-3, when every CTA has finished copying the
//    entries of block q-5 and earlier; 2 shared-memory Gram slots;
//  * ring of 4B records and 4B code slots: iteration r holds blocks r..r+2
//    (codes) and r..r+3 (records).
#include <cuda_runtime.h>

#include "brr_device.cuh"
#include "brr_internal.h"
#include "brr_pick.cuh"

namespace brr {

namespace {

constexpr int kDotWarps = 8;
constexpr int kBlockThreads = (kDotWarps + 1) * 32;
constexpr int kAccBufs = 8;
constexpr int kStageSlots = 8;

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

// Gram entries of one block: the triangle G[p, t], p < t within the block,
// then the cross entries G[p, t] of the previous block's p and this block's t.
__host__ __device__ inline size_t block_gram_entries(int B) { return (size_t)B * (B - 1) / 2 + (size_t)B * B; }

struct PipePlan {
    size_t eps_hi, eps_lo;  // double-float residual slice
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
    p.eps_hi = o;
    o += al16((size_t)slice_max * 4);
    p.eps_lo = o;
    o += al16((size_t)slice_max * 4);
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

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async;" ::: "memory"); }

// SM clock read ordered with the surrounding memory operations and barriers.
__device__ __forceinline__ long long clk()
{
    long long t;
    asm volatile("mov.u64 %0, %%clock64;" : "=l"(t)::"memory");
    return t;
}

__device__ __forceinline__ void dot_warps_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

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

// FP32 component selection with a rigorous error bound, falling back to the
// FP64 evaluation of pick_marker when the bound cannot certify the decision.
// With D_k = logL_k - logL_0 = dc_k + h_k*num^2 (dc_0 = h_0 = 0) evaluated by one
// FMA from rounded inputs, |error(D_k)| <= 3u(|dc_k| + |h_k num^2|) with
// u = 2^-24.  The 700 guards compare differences of D (the logL_0 offset
// cancels); a guard whose difference lies within the error band of 700
// falls back.  Probabilities then carry at most 2*max_err + 2^-21 relative
// error, so a u within tol = 4e-5 + 4*max_err of a cumulative bound falls back.
template <int KM>
__device__ __forceinline__ bool pick_f32(float xh, float xl, float uf, const float *__restrict__ gcf, int K,
                                         int &comp, float &a0out)
{
    // num = xh + xl (double-float); num^2 to FP32 within 3u
    const float n2 = __fmaf_rn(xh, xh, 2.f * xh * xl);
    float D[KM];
    float maxerr = 0.f;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        if (k == 0 || k >= K) {
            D[k] = k == 0 ? 0.f : -INFINITY;
        } else {
            const float dc = gcf[2 * k], h = gcf[2 * k + 1];
            D[k] = __fmaf_rn(h, n2, dc);
            maxerr = fmaxf(maxerr, 3.0e-7f * (fabsf(dc) + fabsf(h * n2)));
        }
    }
    float dmax = 0.f, dmax1 = D[1], dmin1 = D[1];
#pragma unroll
    for (int k = 1; k < KM; ++k) {
        if (k < K) {
            dmax = fmaxf(dmax, D[k]);
            dmax1 = fmaxf(dmax1, D[k]);
            dmin1 = fminf(dmin1, D[k]);
        }
    }
    const float band = 2.f * maxerr + 1e-3f;
    const float spread = dmax1 - dmin1;
    bool unsure = fabsf(spread - 700.f) < band || fabsf(dmax1 - 700.f) < band || fabsf(-dmin1 - 700.f) < band;
    const bool wide = spread > 700.f;
    const bool guard0 = (dmax1 > 700.f) || (-dmin1 > 700.f);
    float e[KM];
    float es = 0.f;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        e[k] = k < K ? __expf(D[k] - dmax) : 0.f;
        es += e[k];
    }
    const float ies = __frcp_rn(es);
    int chosen = -1;
    float acum = 0.f, prev = 0.f, a0 = 0.f;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        if (k < K && chosen < 0) {
            bool guard;
            if (k == 0) {
                guard = guard0;
            } else {
                const float d1 = dmax1 - D[k], d2 = D[k] - dmin1;
                if (wide && (fabsf(d1 - 700.f) < band || fabsf(d2 - 700.f) < band))
                    unsure = true;
                guard = wide && (d1 > 700.f || d2 > 700.f);
            }
            const float pk = guard ? 0.f : e[k] * ies;
            if (k == 0)
                a0 = pk;
            prev = acum;
            acum += pk;
            if (uf <= acum)
                chosen = k;
        }
    }
    const float tol = 4e-5f + 4.f * maxerr;
    const bool close = chosen >= 0 ? ((uf > acum - tol) || (chosen > 0 && uf < prev + tol)) : (uf < acum + tol);
    comp = chosen;
    a0out = a0;
    return !(unsure || close);
}

// Branch-free certified FP32 decision with a stability margin.  With
// D_k = dc_k + h_k * s (s = num^2, D_0 = 0) the component is the first k with
// u * sum(e) <= c_k (e_k = exp(D_k - max D), c_k the running sums).  Returns
// false when the 700 guards of the log-likelihood differences could matter
// (any difference beyond 600) or when u lies within the certified error tol of
// a boundary; the caller then takes the guarded or the FP64 path.
// On success *w is a margin in log-probability: while the true s moves by Delta
// with H * Delta <= w (H: largest h_k - smallest, h_0 = 0 included), every
// cumulative probability changes by a factor within exp(+-H * Delta), which
// cannot carry a boundary across u, so the decision stays the same.
template <int KM>
__device__ __forceinline__ bool pick_margin(float s, float uf, const float *__restrict__ gcf, int K, int &comp,
                                            float &w)
{
    float D[KM];
    float maxerr = 0.f;
    D[0] = 0.f;
#pragma unroll
    for (int k = 1; k < KM; ++k) {
        const float dc = gcf[2 * k], h = gcf[2 * k + 1];
        D[k] = k < K ? __fmaf_rn(h, s, dc) : -INFINITY;
        maxerr = k < K ? fmaxf(maxerr, 3.0e-7f * (fabsf(dc) + fabsf(h * s))) : maxerr;
    }
    float dmax = 0.f, dmax1 = D[1], dmin1 = D[1];
#pragma unroll
    for (int k = 1; k < KM; ++k) {
        dmax = fmaxf(dmax, D[k]);
        dmax1 = fmaxf(dmax1, D[k]);
        dmin1 = k < K ? fminf(dmin1, D[k]) : dmin1;
    }
    const bool far = (dmax1 - dmin1) < 600.f && dmax1 < 600.f && dmin1 > -600.f;
    float c[KM];
    float run = 0.f;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        run = __fadd_rn(run, __expf(D[k] - dmax));   // exp(-inf) = 0 beyond K
        c[k] = run;
    }
    const float es = run;
    const float target = uf * es;
    const float tol = (4e-5f + 4.f * maxerr) * es;
    int chosen = 0;
    bool close = false;
    float up = es, lo = 0.f;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        if (k < K) {
            const bool below = c[k] < target;
            chosen += below ? 1 : 0;
            close = close || fabsf(c[k] - target) < tol;
            lo = below ? c[k] : lo;
        }
    }
#pragma unroll
    for (int k = KM - 1; k >= 0; --k)
        up = (k < K && c[k] >= target) ? c[k] : up;
    comp = chosen < K ? chosen : -1;
    const float w1 = __logf(up - tol) - __logf(target);
    const float w2 = chosen > 0 ? __logf(target) - __logf(lo + tol) : 50.f;
    w = fminf(fminf(w1, w2) - 1e-5f, 50.f);
    return far && !close && chosen < K && w > 0.f;
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

template <int KM, bool MISS>
__global__ void __launch_bounds__(kBlockThreads, 1) k_sweep_block(SweepArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_upd[kMaxSpec];
    __shared__ float2 s_dB[kMaxSpec];
    __shared__ float s_dfl[kMaxSpec][8];
    __shared__ float s_H[kMaxGroups];
    __shared__ int32_t s_gk[kMaxGroups];
    __shared__ BlockOut s_out[2];
    __shared__ int s_abort, s_nupd;

    const int B = a.B;
    const unsigned Bu = (unsigned)B;
    const unsigned R = 4u * Bu;
    const unsigned Rm = R - 1u;
    const int sidx = blockIdx.x;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int lo = a.slice_lo[sidx];
    const int ns = a.slice_lo[sidx + 1] - lo;
    const int nbytes = ((ns + kChunk - 1) / kChunk) * 16;
    const int64_t byte_lo = lo / 4;
    const PipePlan plan = make_pipe_plan(a.slice_max, a.slot_bytes, B, a.n_groups);
    const int npairs = B * (B - 1) / 2;
    const unsigned gent = (unsigned)block_gram_entries(B);
    const unsigned M32 = (unsigned)a.M;
    const int nblk = (int)((M32 + Bu - 1) / Bu);
    auto nb_of = [&](int q) { return (int)min(Bu, M32 - (unsigned)q * Bu); };

    float *eh = reinterpret_cast<float *>(smem + plan.eps_hi);
    float *el = reinterpret_cast<float *>(smem + plan.eps_lo);
    uint8_t *ring_codes = smem + plan.codes;
    BlockRec *ring_rec = reinterpret_cast<BlockRec *>(smem + plan.recs);
    float2 *gbuf = reinterpret_cast<float2 *>(smem + plan.gram);
    uint8_t *pair_ab = smem + plan.pairs;
    float *gcf = reinterpret_cast<float *>(smem + plan.gcf);
    float *gbf = reinterpret_cast<float *>(smem + plan.gbf);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + plan.mbar);
    float2 *gstage = reinterpret_cast<float2 *>(a.gstage);

    // ---- prologue: residual slice (with eps -= mu_new), group constants
    {
        float muh, mul;
        df_from_double(-a.mu_new, muh, mul);
        for (int i = tid; i < a.slice_max; i += kBlockThreads) {
            float h = 0.f, l = 0.f;
            if (i < ns) {
                h = a.eps_hi[lo + i];
                l = a.eps_lo[lo + i];
                df_add(h, l, muh, mul);
            }
            eh[i] = h;
            el[i] = l;
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
        s_nupd = 0;
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();

    // ---- ring of records and genotype code slices (cp.async)
    unsigned rec_issued = 0, code_issued = 0;
    auto issue_recs = [&](unsigned upto) {
        upto = min(upto, M32);
        if (upto <= rec_issued)
            return;
        constexpr unsigned kParts = sizeof(BlockRec) / 16;
        const unsigned n = (upto - rec_issued) * kParts;
        for (unsigned e = tid; e < n; e += kBlockThreads) {
            const unsigned q = rec_issued + e / kParts;
            const unsigned c = e % kParts;
            cp_async16(reinterpret_cast<unsigned char *>(&ring_rec[q & Rm]) + 16 * c,
                       reinterpret_cast<const unsigned char *>(&a.brec[q]) + 16 * c);
        }
        rec_issued = upto;
    };
    const unsigned chunks = (unsigned)nbytes / 16u;
    const unsigned per_pass = chunks ? (unsigned)kBlockThreads / chunks : 0u;
    const unsigned my_q = chunks ? (unsigned)tid / chunks : 0u;
    const unsigned my_c = chunks ? (unsigned)tid - my_q * chunks : 0u;
    auto issue_codes = [&](unsigned upto) {
        upto = min(upto, M32);
        if (upto <= code_issued)
            return;
        if (my_q < per_pass) {
            for (unsigned q = code_issued + my_q; q < upto; q += per_pass) {
                const uint32_t j = ring_rec[q & Rm].j;
                cp_async16(ring_codes + (q & Rm) * a.slot_bytes + 16 * my_c,
                           a.codes + (int64_t)j * a.col_stride + byte_lo + 16 * my_c);
            }
        }
        code_issued = upto;
    };

    // ---- Gram entries of block q (dot warps): CTA s gathers entries
    // e = s + G*(t + 256*i) from the packed Gram into staging slot q % 8.
    double gval = 0.0;
    int gent_mine = -1;
    auto gram_entry = [&](int q, unsigned e, double *out) -> bool {
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
            if (q == 0)
                return false;
            const unsigned c = e - (unsigned)npairs;
            pa = c / Bu;   // position in block q-1 (full: q-1 < nblk-1)
            pb = c - pa * Bu;
            if ((int)pb >= nbq)
                return false;
            qa = q0 - Bu + pa;
        }
        const int64_t ja = ring_rec[qa & Rm].j, jb = ring_rec[(q0 + pb) & Rm].j;
        const int64_t hi = ja > jb ? ja : jb, lw = ja > jb ? jb : ja;
        *out = __ldg(&a.gram[hi * (hi - 1) / 2 + lw]);
        return true;
    };
    auto gather_load = [&](int q) {
        gent_mine = -1;
        const unsigned e = (unsigned)sidx + (unsigned)tid * (unsigned)a.G;
        if (e < gent && gram_entry(q, e, &gval))
            gent_mine = (int)e;
    };
    auto split2 = [](double v) {
        float h, l;
        df_from_double(v, h, l);
        return make_float2(h, l);
    };
    auto gather_store = [&](int q) {
        float2 *slot = gstage + (size_t)(q % kStageSlots) * gent;
        if (gent_mine >= 0)
            slot[gent_mine] = split2(gval);
        for (unsigned e = (unsigned)sidx + (unsigned)(tid + kDotWarps * 32) * (unsigned)a.G; e < gent;
             e += (unsigned)(kDotWarps * 32) * (unsigned)a.G) {
            double v;
            if (gram_entry(q, e, &v))
                slot[e] = split2(v);
        }
    };

    auto publish = [&](unsigned long long *acc, __int128 x) {
        const Fx f = fx_split(x);
        red_add_u64(acc, (unsigned long long)f.hi);
        red_add_u64(acc + 1, f.lo);
    };

    // ---- partial dot products of block q against the current residual (dot
    // warps).  Warp w owns markers w, w+8, ... of the block; its lanes stride
    // over the slice's code bytes.  Per byte the four products g*hi (exact)
    // are combined by error-free TwoSums; rounding errors and g*lo go to the
    // low word.  Missing genotypes are summed apart.  The warp's 8 sums are
    // reduce-scattered so that 8 lanes convert and publish in parallel.
    auto dot_block = [&](int q) {
        const unsigned q0 = (unsigned)q * Bu;
        const int nbq = nb_of(q);
        constexpr int MPW = kMaxSpec / 8;
        float Ah[MPW], Al[MPW], Mh[MPW], Ml[MPW];
        unsigned cofs[MPW];
#pragma unroll
        for (int k = 0; k < MPW; ++k) {
            Ah[k] = Al[k] = Mh[k] = Ml[k] = 0.f;
            // markers past the end of a short block read a stale slot; their
            // sums are never published
            cofs[k] = ((q0 + (unsigned)(warp + 8 * k)) & Rm) * (unsigned)a.slot_bytes;
        }
        const int mpw = (B + 7) / 8;
        for (int b = lane; b < nbytes; b += 32) {
            const float4 h = reinterpret_cast<const float4 *>(eh)[b];
            const float4 l = reinterpret_cast<const float4 *>(el)[b];
#pragma unroll
            for (int k = 0; k < MPW; ++k) {
                if (k < mpw) {
                    const unsigned v = ring_codes[cofs[k] + b];
                    const unsigned x = ~v, lo1 = x & 0x55u, hi1 = (x >> 1) & 0x55u;
                    const unsigned two = lo1 & hi1, one = lo1 & ~hi1;
                    const float g0 = (two & 1u) ? 2.f : ((one & 1u) ? 1.f : 0.f);
                    const float g1 = (two & 4u) ? 2.f : ((one & 4u) ? 1.f : 0.f);
                    const float g2 = (two & 16u) ? 2.f : ((one & 16u) ? 1.f : 0.f);
                    const float g3 = (two & 64u) ? 2.f : ((one & 64u) ? 1.f : 0.f);
                    float s01, e01, s23, e23, s4, e4, sa, ea;
                    two_sum(__fmul_rn(g0, h.x), __fmul_rn(g1, h.y), s01, e01);
                    two_sum(__fmul_rn(g2, h.z), __fmul_rn(g3, h.w), s23, e23);
                    two_sum(s01, s23, s4, e4);
                    two_sum(Ah[k], s4, sa, ea);
                    Ah[k] = sa;
                    const float lo4 =
                        __fmaf_rn(g0, l.x, __fmaf_rn(g1, l.y, __fmaf_rn(g2, l.z, __fmul_rn(g3, l.w))));
                    Al[k] = __fadd_rn(Al[k], __fadd_rn(__fadd_rn(__fadd_rn(e01, e23), e4), __fadd_rn(ea, lo4)));
                    if (MISS) {
                        const unsigned mm = v & ~(v >> 1) & 0x55u;   // code 01: missing
                        if (mm) {
                            if (mm & 1u) df_add(Mh[k], Ml[k], h.x, l.x);
                            if (mm & 4u) df_add(Mh[k], Ml[k], h.y, l.y);
                            if (mm & 16u) df_add(Mh[k], Ml[k], h.z, l.z);
                            if (mm & 64u) df_add(Mh[k], Ml[k], h.w, l.w);
                        }
                    }
                }
            }
        }
        df_rs_step<4>(Ah, Al, lane & 16, 16);
        df_rs_step<2>(Ah, Al, lane & 8, 8);
        df_rs_step<1>(Ah, Al, lane & 4, 4);
        df_xor_add(Ah[0], Al[0], 2);
        df_xor_add(Ah[0], Al[0], 1);
        if (MISS) {
            df_rs_step<4>(Mh, Ml, lane & 16, 16);
            df_rs_step<2>(Mh, Ml, lane & 8, 8);
            df_rs_step<1>(Mh, Ml, lane & 4, 4);
            df_xor_add(Mh[0], Ml[0], 2);
            df_xor_add(Mh[0], Ml[0], 1);
        }
        const int kk = ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
        const int m = warp + 8 * kk;
        if ((lane & 3) == 0 && m < nbq) {
            unsigned long long *acc = a.acc + ((size_t)(q % kAccBufs) * kMaxSpec + m) * 4;
            __int128 x1, x2, m1 = 0, m2 = 0;
            const bool ok = fx_from_float(Ah[0], x1) && fx_from_float(Al[0], x2) &&
                            (!MISS || (fx_from_float(Mh[0], m1) && fx_from_float(Ml[0], m2)));
            if (ok) {
                publish(acc, x1 + x2);
                if (MISS && (Mh[0] != 0.f || Ml[0] != 0.f))
                    publish(acc + 2, m1 + m2);
            } else {
                atomicCAS(a.err, kDevOk, kDevRange);
            }
        }
    };
    auto arrive = [&](int q) { red_release_add_u64(a.counter + (q & 1), 1ull); };

    // profiling (first CTA): dot side on thread 0, resolve side on warp 8 lane 0
    const bool prof_d = a.prof != nullptr && sidx == 0 && tid == 0;
    const bool prof_r = a.prof != nullptr && sidx == 0 && tid == kDotWarps * 32;
    long long ph[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    long long tp = (prof_d || prof_r) ? clk() : 0;
    auto mark = [&](bool on, int k) {
        if (on) {
            const long long t = clk();
            ph[k] += t - tp;
            tp = t;
        }
    };
    unsigned long long *fb_counter = a.prof ? reinterpret_cast<unsigned long long *>(a.prof + 8) : nullptr;
    long long steps = 0;
    int cp_issued = -1, cp_waited = -1;   // resolve warp: Gram copies issued / waited for

    // ---- first blocks: records 0..2 and codes 0..1 resident, block 0's dot
    // products and the Gram entries of blocks 0 and 1 staged, barrier 0
    issue_recs(3u * Bu);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    issue_codes(2u * Bu);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    if (warp < kDotWarps) {
        gather_load(0);
        dot_block(0);
        gather_store(0);
        if (nblk > 1) {
            gather_load(1);
            gather_store(1);
        }
        dot_warps_sync();
        if (tid == 0)
            arrive(0);
    }

    int r = 0;
    for (; r < nblk; ++r) {
        cp_async_wait_all();
        __syncthreads();
        if (s_abort)
            break;
        mark(prof_d, 0);
        issue_codes((unsigned)(r + 3) * Bu);
        issue_recs((unsigned)(r + 4) * Bu);
        cp_async_commit();
        const unsigned q0 = (unsigned)r * Bu;
        const int nb = nb_of(r);

        if (warp < kDotWarps) {
            // ---- dot side
            if (r >= 1 && sidx == (r - 1) % a.G && warp == kDotWarps - 1)
                write_block_outputs<KM>(a, s_out[(r - 1) & 1], gcf, s_gk, gbf, lane);
            if (r + 2 < nblk)
                gather_load(r + 2);
            if (r + 1 < nblk)
                dot_block(r + 1);
            if (r + 2 < nblk)
                gather_store(r + 2);
            if (sidx == 0 && r + 3 < nblk && tid < 4 * kMaxSpec)
                a.acc[(size_t)((r + 3) % kAccBufs) * kMaxSpec * 4 + tid] = 0ull;
            dot_warps_sync();
            if (tid == 0 && r + 1 < nblk)
                arrive(r + 1);
            mark(prof_d, 1);
        } else {
            // ---- resolve side: barrier r
            mark(prof_r, 8);
            bool ok = true;
            if (lane == 0) {
                const unsigned long long target =
                    (unsigned long long)(a.G + a.phantom) * (unsigned long long)((r >> 1) + 1);
                const unsigned long long *ctr = a.counter + (r & 1);
                if (ld_acquire_u64(ctr) < target) {
                    const uint64_t t0 = global_timer_ns();
                    unsigned spins = 0;
                    while (ld_acquire_u64(ctr) < target) {
                        if ((++spins & 255u) == 0 &&
                            (*(volatile int *)a.err != kDevOk || global_timer_ns() - t0 > a.timeout_ns)) {
                            atomicCAS(a.err, kDevOk, kDevTimeout);
                            ok = false;
                            break;
                        }
                    }
                }
                if (ok) {
                    // the staged entries were written by generic stores of other
                    // CTAs; the bulk copies read them through the async proxy
                    fence_proxy_async();
                    if (r == 0) {
                        mbar_expect_tx(&mbar[0], (unsigned)(gent * sizeof(float2)));
                        bulk_copy_g2s(gbuf, gstage, (unsigned)(gent * sizeof(float2)), &mbar[0]);
                        cp_issued = 0;
                    }
                    if (r + 1 < nblk) {
                        const int q = r + 1;
                        mbar_expect_tx(&mbar[q & 1], (unsigned)(gent * sizeof(float2)));
                        bulk_copy_g2s(gbuf + (size_t)(q & 1) * gent, gstage + (size_t)(q % kStageSlots) * gent,
                                      (unsigned)(gent * sizeof(float2)), &mbar[q & 1]);
                        cp_issued = q;
                    }
                } else {
                    s_abort = 1;
                }
            }
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            mark(prof_r, 2);
            if (ok) {
                // ---- block inputs: num = sigma * sum(g*eps) + cst + dm * sum_missing(eps)
                float nh[2], nl[2], ufr[2];
                int grp[2], kk[2];
                bool own[2], bnz[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int m = lane + 32 * h;
                    own[h] = m < nb;
                    nh[h] = nl[h] = 0.f;
                    ufr[h] = 2.f;
                    grp[h] = 0;
                    kk[h] = 2;
                    bnz[h] = false;
                    if (own[h]) {
                        const BlockRec &rc = ring_rec[(q0 + m) & Rm];
                        const unsigned long long *acc = a.acc + ((size_t)(r % kAccBufs) * kMaxSpec + m) * 4;
                        float th, tl;
                        fx_to_df((long long)ld_relaxed_u64(acc), ld_relaxed_u64(acc + 1), th, tl);
                        df_mul(rc.sig[0], rc.sig[1], th, tl, nh[h], nl[h]);
                        df_add(nh[h], nl[h], rc.cst[0], rc.cst[1]);
                        if (MISS) {
                            float sh, sl, qh, ql;
                            fx_to_df((long long)ld_relaxed_u64(acc + 2), ld_relaxed_u64(acc + 3), sh, sl);
                            df_mul(rc.dm[0], rc.dm[1], sh, sl, qh, ql);
                            df_add(nh[h], nl[h], qh, ql);
                        }
                        ufr[h] = rc.uf;
                        grp[h] = rc.group;
                        kk[h] = s_gk[rc.group];
                        bnz[h] = rc.bnz != 0u;
                    }
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
                    const int Up = s_nupd;
                    for (int u = 0; u < Up; ++u) {
                        const int p = s_upd[u];
                        const float2 dB = s_dB[u];
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
                        if (__any_sync(0xffffffffu, need[0] || need[1])) {
                            bool slow[2];
#pragma unroll
                            for (int h = 0; h < 2; ++h) {
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
                            s_upd[nupd] = p;
                            s_dB[nupd] = make_float2(dh, dl);
                        }
                        ++nupd;
                        next = p + 1;
                        if (prof_r)
                            ph[10] += clk() - tl1;
                    }
                    if (lane == 0)
                        s_nupd = nupd;
                    // the block's decisions for the CTA that writes them out
                    if (sidx == r % a.G) {
                        BlockOut &o = s_out[r & 1];
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int m = lane + 32 * h;
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
        }
        __syncthreads();
        mark(prof_d, 11);
        if (s_abort)
            break;

        // ---- rank-U residual update of block r: eps += dBeta_u * x_u
        const int U = s_nupd;
        if (U > 0) {
            if (tid < 4 * U) {
                const int u = tid >> 2, code = tid & 3;
                const BlockRec &rc = ring_rec[(q0 + s_upd[u]) & Rm];
                const float2 dB = s_dB[u];
                df_mul(dB.x, dB.y, rc.x[2 * code], rc.x[2 * code + 1], s_dfl[u][2 * code], s_dfl[u][2 * code + 1]);
            }
            __syncthreads();
            // The sum of the residual is left as it was at the sweep start: the
            // standardised columns sum to zero, so a dense update moves it only
            // by rounding (dBeta times a column sum of order 1e-11).
            for (int b = tid; b < nbytes; b += kBlockThreads) {
                float4 h = reinterpret_cast<float4 *>(eh)[b];
                float4 l = reinterpret_cast<float4 *>(el)[b];
                for (int u = 0; u < U; ++u) {
                    const unsigned v = ring_codes[((q0 + s_upd[u]) & Rm) * a.slot_bytes + b];
                    const float *d = s_dfl[u];
                    df_add(h.x, l.x, d[2 * (v & 3u)], d[2 * (v & 3u) + 1]);
                    df_add(h.y, l.y, d[2 * ((v >> 2) & 3u)], d[2 * ((v >> 2) & 3u) + 1]);
                    df_add(h.z, l.z, d[2 * ((v >> 4) & 3u)], d[2 * ((v >> 4) & 3u) + 1]);
                    df_add(h.w, l.w, d[2 * (v >> 6)], d[2 * (v >> 6) + 1]);
                }
                // padding individuals past the slice end keep a zero residual
                const int i0 = 4 * b;
                if (i0 + 3 >= ns) {
                    if (i0 + 0 >= ns) { h.x = 0.f; l.x = 0.f; }
                    if (i0 + 1 >= ns) { h.y = 0.f; l.y = 0.f; }
                    if (i0 + 2 >= ns) { h.z = 0.f; l.z = 0.f; }
                    if (i0 + 3 >= ns) { h.w = 0.f; l.w = 0.f; }
                }
                reinterpret_cast<float4 *>(eh)[b] = h;
                reinterpret_cast<float4 *>(el)[b] = l;
            }
        }
        mark(prof_d, 4);
    }
    // outputs of the last block
    if (!s_abort && r == nblk && sidx == (nblk - 1) % a.G && warp == kDotWarps - 1)
        write_block_outputs<KM>(a, s_out[(nblk - 1) & 1], gcf, s_gk, gbf, lane);
    if (prof_d) {
        a.prof[0] = ph[0];
        a.prof[1] = ph[1];
        a.prof[4] = ph[4];
        a.prof[5] = r;
        a.prof[11] = ph[11];
    }
    if (prof_r) {
        a.prof[2] = ph[2];
        a.prof[3] = ph[3];
        a.prof[6] = steps;
        a.prof[7] = ph[7];
        a.prof[9] = ph[9];
        a.prof[10] = ph[10];
    }   // a.prof[8]: FP64 fallbacks of the certified sampler (first CTA)
    cp_async_wait_all();
    // bulk copies still in flight after an abort: wait for them (bounded)
    if (tid == kDotWarps * 32) {
        for (int q = cp_waited + 1; q <= cp_issued; ++q)
            mbar_wait(&mbar[q & 1], (unsigned)((q >> 1) & 1), a.timeout_ns);
    }
    __syncthreads();

    // ---- epilogue: residual back to HBM, per-slice sums
    double s1 = 0.0, s2 = 0.0;
    for (int i = tid; i < ns; i += kBlockThreads) {
        a.eps_hi[lo + i] = eh[i];
        a.eps_lo[lo + i] = el[i];
        const double e = (double)eh[i] + (double)el[i];
        s1 += e;
        s2 = fma(e, e, s2);
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

size_t sweep_block_stage_bytes(int B) { return (size_t)kStageSlots * block_gram_entries(B) * sizeof(float2); }

int sweep_block_threads() { return kBlockThreads; }

template <int KM, bool MISS>
static cudaError_t launch_block_km(const SweepArgs &a, size_t smem, cudaStream_t st)
{
    cudaError_t e =
        cudaFuncSetAttribute(k_sweep_block<KM, MISS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    SweepArgs args = a;
    void *params[] = {&args};
    return cudaLaunchCooperativeKernel((const void *)k_sweep_block<KM, MISS>, dim3(a.G), dim3(kBlockThreads), params,
                                       smem, st);
}

cudaError_t launch_sweep_block(const SweepArgs &a, size_t smem, cudaStream_t st)
{
    if (a.kmax <= 4)
        return a.has_missing ? launch_block_km<4, true>(a, smem, st) : launch_block_km<4, false>(a, smem, st);
    return a.has_missing ? launch_block_km<kMaxK, true>(a, smem, st) : launch_block_km<kMaxK, false>(a, smem, st);
}

int sweep_block_max_ctas_per_sm(size_t smem)
{
    int n = 1 << 30;
    const void *fs[4] = {(const void *)k_sweep_block<4, false>, (const void *)k_sweep_block<4, true>,
                         (const void *)k_sweep_block<kMaxK, false>, (const void *)k_sweep_block<kMaxK, true>};
    for (const void *f : fs) {
        int m = 0;
        if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, f, kBlockThreads, smem) != cudaSuccess)
            return 0;
        n = m < n ? m : n;
    }
    return n;
}

}  // namespace brr
