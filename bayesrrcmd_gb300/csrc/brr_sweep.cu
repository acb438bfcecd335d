// Persistent Gibbs-sweep kernel and its per-iteration helpers (sm_103a).
//
// Replaces BayesRBase::processColumn (src/BayesRBase.cpp:287-392) driven once
// per marker by AnalysisGraph::exec (src/sequential.cpp:23-26,
// src/limitsequencegraph.cpp:46-55), with the dense kernel
// (src/densebayesrkernel.cpp:10-20) or the ragged kernel
// (src/sparsebayesrkernel.cpp:10-34, src/raggedbayesrkernel.cpp:10-35,
// src/SparseBayesRRG.cpp:76-92).
//
// Layout: one CTA per SM, each owning a contiguous slice of individuals; the
// residual slice lives in shared memory for the whole sweep.  Markers are
// walked in the sweep order in "rounds": a round computes the dot products of
// the next B markers against the current residual (each CTA over its slice),
// sums them across CTAs through exact fixed-point atomics and one grid-wide
// counter barrier, then every CTA samples the B markers redundantly and
// identically.  The first marker whose sample changes the residual
// (beta_old != 0 or beta_new != 0) ends the round: its update is applied and
// the next round starts right after it.  Every sampled marker therefore sees
// exactly the residual of the sequential chain.
#include "brr_device.cuh"
#include "brr_internal.h"
#include "brr_stream.h"

namespace brr {

enum { kFormFP64 = 0, kFormFP32C = 1 };
enum { kKindDense = 0, kKindRagged = 1 };

// --------------------------------------------------------------------------
// Per-iteration helpers.

__global__ void k_draws(uint32_t seed, uint32_t chain, uint32_t it, int64_t M, double *u, double *z)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= M)
        return;
    marker_draws(StreamKey{seed, chain}, it, (uint32_t)j, &u[j], &z[j]);
}

__global__ void k_gather(int form, int kind, const uint32_t *__restrict__ order, int64_t M,
                         const double *__restrict__ table, const double *__restrict__ scale,
                         const double *__restrict__ beta, const double *__restrict__ u,
                         const double *__restrict__ z, const int32_t *__restrict__ group,
                         const double *__restrict__ colsum, SweepRec *rec)
{
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= M)
        return;
    const uint32_t j = order[q];
    SweepRec r;
    if (kind == kKindDense) {
        if (form == kFormFP64) {
            r.t[0] = table[4 * j];
            r.t[1] = table[4 * j + 1];
            r.t[2] = table[4 * j + 2];
            r.t[3] = table[4 * j + 3];
        } else {
            r.t[0] = scale[2 * j];       // sigma
            r.t[1] = scale[2 * j + 1];   // column mean
            r.t[2] = table[4 * j + 1];   // value of a missing genotype
            r.t[3] = colsum[j];          // sum of the column
        }
    } else {
        r.t[0] = table[4 * j];           // mean
        r.t[1] = table[4 * j + 1];       // sd
        r.t[2] = 1.0 / table[4 * j + 1]; // 1/sd
        r.t[3] = table[4 * j + 3];       // Zsum
    }
    r.beta_old = beta[j];
    r.u = u[j];
    r.z = z[j];
    r.j = j;
    r.group = group[j];
    rec[q] = r;
}

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

// updateMu, first half: eps += mu_old, and per-block sum(eps) (src/DenseBayesRRmz.cpp:38-39).
__global__ void __launch_bounds__(kThreads) k_mu_prep(int form, int64_t N, double mu_old, double *eps,
                                                      float *eps_hi, float *eps_lo, double *part)
{
    __shared__ double red[kThreads / 32];
    double s = 0.0;
    float mh, ml;
    df_from_double(mu_old, mh, ml);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        if (form == kFormFP64) {
            const double e = __dadd_rn(eps[i], mu_old);
            eps[i] = e;
            s += e;
        } else {
            float h = eps_hi[i], l = eps_lo[i];
            df_add(h, l, mh, ml);
            eps_hi[i] = h;
            eps_lo[i] = l;
            s += (double)h + (double)l;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q)
            t += red[q];
        part[blockIdx.x] = t;
    }
}

// FP64 residual refresh eps = y - mu - X beta over the non-zero betas.  Each
// thread owns one byte of codes (four individuals) and walks the non-zero
// markers in a fixed order, so the result is deterministic.
__global__ void __launch_bounds__(kThreads) k_refresh(int form, int kind, int64_t N, const double *__restrict__ ystd,
                                                      double mu, const uint8_t *__restrict__ codes,
                                                      int64_t col_stride, const double *__restrict__ table,
                                                      const uint32_t *__restrict__ nz_j,
                                                      const double *__restrict__ nz_beta, int64_t n_nz, double *eps,
                                                      float *eps_hi, float *eps_lo)
{
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t i0 = 4 * b;
    if (i0 >= N)
        return;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t q = 0; q < n_nz; ++q) {
        const uint32_t j = nz_j[q];
        const double bj = nz_beta[q];
        const unsigned v = codes[(int64_t)j * col_stride + b];
        double x[4];
        if (kind == kKindDense) {
            const double l0 = table[4 * j], l1 = table[4 * j + 1], l2 = table[4 * j + 2], l3 = table[4 * j + 3];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned c = (v >> (2 * k)) & 3u;
                x[k] = (c & 2u) ? ((c & 1u) ? l3 : l2) : ((c & 1u) ? l1 : l0);
            }
        } else {
            // the ragged epsilon update leaves missing genotypes unchanged
            // (src/raggedbayesrkernel.cpp:26-27): x = (g - mean)/sd, 0 if missing
            const double mean = table[4 * j], sd = table[4 * j + 1];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned c = (v >> (2 * k)) & 3u;
                const double g = c == 0u ? 2.0 : (c == 2u ? 1.0 : 0.0);
                x[k] = c == 1u ? 0.0 : (g - mean) / sd;
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            acc[k] = fma(bj, x[k], acc[k]);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int64_t i = i0 + k;
        if (i < N) {
            const double e = (ystd[i] - mu) - acc[k];
            if (form == kFormFP64) {
                eps[i] = e;
            } else {
                float h, l;
                df_from_double(e, h, l);
                eps_hi[i] = h;
                eps_lo[i] = l;
            }
        }
    }
}

// --------------------------------------------------------------------------
// Shared-memory plan of the sweep kernel (byte offsets, all 16-aligned).
struct SmemPlan {
    size_t eps0, eps1;      // FP64 residual | double-float hi, lo
    size_t ring_codes;      // dense: R x slot_bytes
    size_t ring_rec;        // R x SweepRec
    size_t ring_roff;       // ragged: R x 8 int32
    size_t gconst;          // n_groups x kMaxK x 4 doubles
    size_t gk;              // n_groups ints
    size_t gtab;            // FP32C dense: 256 float4 + 256 bytes
    size_t total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline SmemPlan make_plan(int form, int kind, int slice_max, int slot_bytes, int B, int n_groups,
                                              size_t rec_bytes = sizeof(SweepRec))
{
    SmemPlan p;
    const int R = 4 * B;
    size_t o = 0;
    p.eps0 = o;
    o += align16((size_t)slice_max * (form == kFormFP64 ? 8 : 4));
    p.eps1 = o;
    if (form != kFormFP64)
        o += align16((size_t)slice_max * 4);
    p.ring_codes = o;
    if (kind == kKindDense)
        o += align16((size_t)R * slot_bytes);
    p.ring_rec = o;
    o += (size_t)R * rec_bytes;
    p.ring_roff = o;
    if (kind == kKindRagged)
        o += (size_t)R * 8 * sizeof(int32_t);
    p.gconst = o;
    o += align16((size_t)n_groups * kMaxK * 4 * sizeof(double));
    p.gk = o;
    o += align16((size_t)n_groups * sizeof(int32_t));
    p.gtab = o;
    if (form != kFormFP64 && kind == kKindDense)
        o += 256 * 16 + 256;
    p.total = align16(o);
    return p;
}

// Team of LPM lanes inside a warp that computes one marker's partial dot product.
struct Team {
    unsigned mask;
    int lane;      // lane within the team
    int base;      // warp lane of the team's first lane
};

__device__ __forceinline__ Team make_team(int lpm)
{
    Team t;
    const int wl = threadIdx.x & 31;
    t.lane = wl & (lpm - 1);
    t.base = wl - t.lane;
    t.mask = lpm == 32 ? 0xffffffffu : (((1u << lpm) - 1u) << t.base);
    return t;
}

__device__ __forceinline__ double team_sum_d(double v, const Team &t, int lpm)
{
    for (int o = lpm >> 1; o > 0; o >>= 1)
        v += __shfl_xor_sync(t.mask, v, o);
    return v;
}
__device__ __forceinline__ void team_df_sum(float &h, float &l, const Team &t, int lpm)
{
    for (int o = lpm >> 1; o > 0; o >>= 1) {
        const float bh = __shfl_xor_sync(t.mask, h, o);
        const float bl = __shfl_xor_sync(t.mask, l, o);
        df_add(h, l, bh, bl);
    }
}

__device__ __forceinline__ double lut_select(unsigned c, double l0, double l1, double l2, double l3)
{
    return (c & 2u) ? ((c & 1u) ? l3 : l2) : ((c & 1u) ? l1 : l0);
}

// Component selection for one marker by one thread (src/BayesRBase.cpp:309-366).
// logL_k = c_k + h_k*num^2 with c_k = log(pi_k) - log(sigmaG/sigmaE*(N-1)*cVa_k + 1)/2
// and h_k = 1/(2*denom_k*sigmaE).  P(k) = exp(logL_k - max)/sum, zeroed where the
// reference's 700 guards fire (any |logL_q - logL_k| > 700 over q >= 1); the
// walk picks the first k whose cumulative probability reaches u.
// FP32 = true evaluates the exponentials in single precision from the FP64
// log-likelihood differences and keeps the decision only when u is further
// than 2e-5 from every cumulative bound it was compared with (the FP32 error
// is below 5e-6); otherwise the FP64 evaluation decides.
struct Pick {
    int comp;       // chosen component, -1 if none
    double beta;    // new beta (beta_old when none)
    double acum0;   // P(component 0) as stored in acum
};

template <bool FP32, int KM>
__device__ __forceinline__ Pick pick_marker(double num, double u, double z, double beta_old,
                                            const double *__restrict__ gc, int K)
{
    double L[KM];
    const double n2 = num * num;
#pragma unroll
    for (int k = 0; k < KM; ++k)
        L[k] = k < K ? (k == 0 ? gc[0] : fma(gc[4 * k + 2], n2, gc[4 * k])) : -INFINITY;
    double lmax = L[0], lmax1 = L[1], lmin1 = L[1];
#pragma unroll
    for (int k = 1; k < KM; ++k) {
        if (k < K) {
            lmax = fmax(lmax, L[k]);
            lmax1 = fmax(lmax1, L[k]);
            lmin1 = fmin(lmin1, L[k]);
        }
    }
    // the guards of components q >= 1 can only fire when the log-likelihoods of
    // components 1..K-1 span more than 700
    const bool wide = lmax1 - lmin1 > 700.0;
    const bool guard0 = (lmax1 - L[0] > 700.0) || (L[0] - lmin1 > 700.0);
    auto guarded = [&](int k) -> bool {
        return k == 0 ? guard0 : (wide && ((lmax1 - L[k] > 700.0) || (L[k] - lmin1 > 700.0)));
    };
    Pick res;
    res.comp = -1;
    res.beta = beta_old;
    res.acum0 = 0.0;
    bool decided = false;
    if (FP32) {
        float e[KM];
        float es = 0.f;
#pragma unroll
        for (int k = 0; k < KM; ++k) {
            e[k] = k < K ? __expf((float)(L[k] - lmax)) : 0.f;
            es += e[k];
        }
        const float ies = __frcp_rn(es);
        int chosen = -1;
        float acum = 0.f, prev = 0.f, a0 = 0.f;
        const float uf = (float)u;
#pragma unroll
        for (int k = 0; k < KM; ++k) {
            if (k < K && chosen < 0) {
                const float pk = guarded(k) ? 0.f : e[k] * ies;
                if (k == 0)
                    a0 = pk;
                prev = acum;
                acum += pk;
                if (uf <= acum)
                    chosen = k;
            }
        }
        const float tol = 2e-5f;
        const bool close = chosen >= 0 ? ((uf > acum - tol) || (chosen > 0 && uf < prev + tol)) : (uf < acum + tol);
        if (!close) {
            res.comp = chosen;
            res.acum0 = (double)a0;
            decided = true;
        }
    }
    if (!decided) {
        double e[KM];
        double es = 0.0;
#pragma unroll
        for (int k = 0; k < KM; ++k) {
            e[k] = k < K ? exp(L[k] - lmax) : 0.0;
            es += e[k];
        }
        const double ies = 1.0 / es;
        int chosen = -1;
        double acum = 0.0, a0 = 0.0;
#pragma unroll
        for (int k = 0; k < KM; ++k) {
            if (k < K && chosen < 0) {
                const double pk = guarded(k) ? 0.0 : e[k] * ies;
                if (k == 0)
                    a0 = pk;
                acum += pk;
                if (u <= acum)
                    chosen = k;
            }
        }
        res.comp = chosen;
        res.acum0 = a0;
    }
    if (res.comp == 0) {
        res.beta = 0.0;
    } else if (res.comp > 0) {
        const double sdk = gc[4 * res.comp + 3], invden = gc[4 * res.comp + 1];
        res.beta = __dadd_rn(__dmul_rn(z, sdk), __dmul_rn(num, invden));
    }
    return res;
}

// --------------------------------------------------------------------------
template <int FORM, int KIND, int KM>
__global__ void __launch_bounds__(kThreads, 1) k_sweep(SweepArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_beta[kMaxSpec];
    __shared__ double s_acum[kMaxSpec];
    __shared__ int s_comp[kMaxSpec];
    __shared__ int s_first;
    __shared__ int s_abort;
    __shared__ double s_scal[4];          // ragged: shift, epsSum; dense FP32C: residual total
    __shared__ double s_delta[4];         // update coefficients of the current round
    __shared__ float s_dfl[8];            // double-float split of the update coefficients
    __shared__ double s_red[kThreads / 32][2];

    const int B = a.B;
    const int lpm = kThreads / B;
    const int R = 4 * B;
    const int sidx = blockIdx.x;
    const int tid = threadIdx.x;
    const int lo = a.slice_lo[sidx];
    const int ns = a.slice_lo[sidx + 1] - lo;
    const int nbytes = ((ns + kChunk - 1) / kChunk) * 16;
    const int64_t byte_lo = lo / 4;
    const SmemPlan plan = make_plan(FORM, KIND, a.slice_max, a.slot_bytes, B, a.n_groups);

    double *eps64 = reinterpret_cast<double *>(smem + plan.eps0);
    float *eh = reinterpret_cast<float *>(smem + plan.eps0);
    float *el = reinterpret_cast<float *>(smem + plan.eps1);
    uint8_t *ring_codes = smem + plan.ring_codes;
    SweepRec *ring_rec = reinterpret_cast<SweepRec *>(smem + plan.ring_rec);
    int32_t *ring_roff = reinterpret_cast<int32_t *>(smem + plan.ring_roff);
    double *gconst = reinterpret_cast<double *>(smem + plan.gconst);
    int32_t *gk = reinterpret_cast<int32_t *>(smem + plan.gk);
    float4 *gtab = reinterpret_cast<float4 *>(smem + plan.gtab);
    uint8_t *mtab = smem + plan.gtab + 256 * 16;

    // ---- prologue: residual slice, constants, tables
    float muh, mul;
    df_from_double(-a.mu_new, muh, mul);
    for (int i = tid; i < a.slice_max; i += kThreads) {
        if (FORM == kFormFP64) {
            eps64[i] = i < ns ? __dsub_rn(a.eps[lo + i], a.mu_new) : 0.0;
        } else {
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
    for (int i = tid; i < a.n_groups * kMaxK * 4; i += kThreads)
        gconst[i] = a.gconst[i];
    for (int i = tid; i < a.n_groups; i += kThreads)
        gk[i] = a.gK[i];
    if (FORM != kFormFP64 && KIND == kKindDense) {
        for (int v = tid; v < 256; v += kThreads) {
            float g[4];
            unsigned m = 0;
            for (int k = 0; k < 4; ++k) {
                const unsigned c = (v >> (2 * k)) & 3u;
                g[k] = c == 0u ? 2.f : (c == 2u ? 1.f : 0.f);
                if (c == 1u)
                    m |= 1u << k;
            }
            gtab[v] = make_float4(g[0], g[1], g[2], g[3]);
            mtab[v] = (uint8_t)m;
        }
    }
    if (tid == 0) {
        s_abort = 0;
        s_scal[0] = 0.0;          // ragged shift
        s_scal[1] = a.epsSum;     // ragged running sum
        s_scal[2] = a.eps_total;  // dense FP32C: sum of the residual
    }
    __syncthreads();

    // ---- prefetch machinery (ring slots are positions modulo R, a power of two)
    const unsigned M32 = (unsigned)a.M;
    const unsigned Rm = (unsigned)R - 1u;
    unsigned rec_issued = 0, code_issued = 0;
    auto issue_recs = [&](unsigned upto) {
        upto = min(upto, M32);
        if (upto <= rec_issued)
            return;
        const unsigned n = (upto - rec_issued) * 4u;
        for (unsigned e = tid; e < n; e += kThreads) {
            const unsigned q = rec_issued + (e >> 2);
            const unsigned c = e & 3u;
            cp_async16(reinterpret_cast<unsigned char *>(&ring_rec[q & Rm]) + 16 * c,
                       reinterpret_cast<const unsigned char *>(&a.rec[q]) + 16 * c);
        }
        rec_issued = upto;
    };
    // each thread owns one 16-byte chunk of codes of one marker per pass
    const unsigned chunks = (unsigned)nbytes / 16u;
    const unsigned per_pass = chunks ? (unsigned)kThreads / chunks : 0u;
    const unsigned my_q = chunks ? (unsigned)tid / chunks : 0u;
    const unsigned my_c = chunks ? (unsigned)tid - my_q * chunks : 0u;
    auto issue_codes = [&](unsigned upto) {
        upto = min(upto, M32);
        if (upto <= code_issued)
            return;
        if (KIND == kKindDense) {
            if (my_q < per_pass) {
                for (unsigned q = code_issued + my_q; q < upto; q += per_pass) {
                    const uint32_t j = ring_rec[q & Rm].j;
                    cp_async16(ring_codes + (q & Rm) * a.slot_bytes + 16 * my_c,
                               a.codes + (int64_t)j * a.col_stride + byte_lo + 16 * my_c);
                }
            }
        } else {
            // offsets of the slice's sub-lists, copied asynchronously into the ring
            const unsigned n = (upto - code_issued) * 8u;
            for (unsigned e = tid; e < n; e += kThreads) {
                const unsigned q = code_issued + (e >> 3);
                const unsigned k = e & 7u;
                if (k < 6u) {
                    const uint32_t j = ring_rec[q & Rm].j;
                    const int64_t base = (int64_t)j * a.G + sidx;
                    cp_async4(&ring_roff[(q & Rm) * 8 + k], &a.roff[k >> 1][base + (k & 1)]);
                }
            }
        }
        code_issued = upto;
    };

    issue_recs(3u * B);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    issue_codes(2u * B);
    cp_async_commit();

    int lpm_log2 = 0;
    while ((1 << lpm_log2) < lpm)
        ++lpm_log2;
    const Team tm = make_team(lpm);
    const int team = tid >> lpm_log2;
    const double Nm1 = (double)(a.N - 1);
    const bool prof = a.prof != nullptr && blockIdx.x == 0 && tid == 0;
    long long ph[6] = {0, 0, 0, 0, 0, 0};
    long long tp = prof ? clock64() : 0;
    auto mark = [&](int k) {
        if (prof) {
            const long long t = clock64();
            ph[k] += t - tp;
            tp = t;
        }
    };
    auto publish = [&](unsigned long long *acc, __int128 x) {
        const Fx f = fx_split(x);
        red_add_u64(acc, (unsigned long long)f.hi);
        red_add_u64(acc + 1, f.lo);
    };

    unsigned start = 0;
    long long r = 0;
    int rb = 0;   // r % 3
    while (start < M32) {
        cp_async_wait_all();
        __syncthreads();
        issue_codes(start + 2u * B);
        issue_recs(start + 3u * B);
        cp_async_commit();
        const int nb = (int)min((unsigned)B, M32 - start);
        if (tid == 0)
            s_first = kMaxSpec;
        mark(0);

        // ---- partial dot products of this slice, published as exact fixed point
        if (team < nb) {
            const unsigned slot = (start + team) & Rm;
            const SweepRec &rc = ring_rec[slot];
            unsigned long long *acc = a.acc + (rb * kMaxSpec + team) * 4;
            bool ok = true;
            if (KIND == kKindDense) {
                const uint8_t *cb = ring_codes + slot * a.slot_bytes;
                if (FORM == kFormFP64) {
                    const double l0 = rc.t[0], l1 = rc.t[1], l2 = rc.t[2], l3 = rc.t[3];
                    double p = 0.0;
                    for (int b = tm.lane; b < nbytes; b += lpm) {
                        const unsigned v = cb[b];
                        const double2 e01 = reinterpret_cast<const double2 *>(eps64)[2 * b];
                        const double2 e23 = reinterpret_cast<const double2 *>(eps64)[2 * b + 1];
                        p = fma(lut_select(v & 3u, l0, l1, l2, l3), e01.x, p);
                        p = fma(lut_select((v >> 2) & 3u, l0, l1, l2, l3), e01.y, p);
                        p = fma(lut_select((v >> 4) & 3u, l0, l1, l2, l3), e23.x, p);
                        p = fma(lut_select((v >> 6) & 3u, l0, l1, l2, l3), e23.y, p);
                    }
                    p = team_sum_d(p, tm, lpm);
                    if (tm.lane == 0) {
                        __int128 x;
                        ok = fx_from_double(p, x);
                        if (ok)
                            publish(acc, x);
                    }
                } else {
                    // A = sum over non-missing of g*eps in double-float: the
                    // products g*hi are exact, each is added with an
                    // error-free TwoSum into one of two interleaved chains and
                    // the rounding errors plus the g*lo terms are accumulated
                    // in the low words.  Sm = sum of eps over missing genotypes.
                    float A0 = 0.f, L0 = 0.f, A1 = 0.f, L1 = 0.f, mh = 0.f, ml = 0.f;
                    for (int b = tm.lane; b < nbytes; b += lpm) {
                        const unsigned v = cb[b];
                        const float4 g = gtab[v];
                        const float4 h = reinterpret_cast<const float4 *>(eh)[b];
                        const float4 l = reinterpret_cast<const float4 *>(el)[b];
                        float s, e;
                        two_sum(A0, __fmul_rn(g.x, h.x), s, e); A0 = s; L0 = __fmaf_rn(g.x, l.x, __fadd_rn(L0, e));
                        two_sum(A1, __fmul_rn(g.y, h.y), s, e); A1 = s; L1 = __fmaf_rn(g.y, l.y, __fadd_rn(L1, e));
                        two_sum(A0, __fmul_rn(g.z, h.z), s, e); A0 = s; L0 = __fmaf_rn(g.z, l.z, __fadd_rn(L0, e));
                        two_sum(A1, __fmul_rn(g.w, h.w), s, e); A1 = s; L1 = __fmaf_rn(g.w, l.w, __fadd_rn(L1, e));
                        const unsigned mm = mtab[v];
                        if (mm) {
                            if (mm & 1u) df_add(mh, ml, h.x, l.x);
                            if (mm & 2u) df_add(mh, ml, h.y, l.y);
                            if (mm & 4u) df_add(mh, ml, h.z, l.z);
                            if (mm & 8u) df_add(mh, ml, h.w, l.w);
                        }
                    }
                    float Ah = A0, Al = L0;
                    df_add(Ah, Al, A1, L1);
                    team_df_sum(Ah, Al, tm, lpm);
                    team_df_sum(mh, ml, tm, lpm);
                    if (tm.lane == 0) {
                        __int128 x1, x2, m1, m2;
                        ok = fx_from_float(Ah, x1) && fx_from_float(Al, x2) && fx_from_float(mh, m1) &&
                             fx_from_float(ml, m2);
                        if (ok) {
                            publish(acc, x1 + x2);
                            if (mh != 0.f || ml != 0.f)
                                publish(acc + 2, m1 + m2);
                        }
                    }
                }
            } else {
                const int32_t *ro = ring_roff + slot * 8;
                if (FORM == kFormFP64) {
                    double p = 0.0;
                    for (int e = ro[0] + tm.lane; e < ro[1]; e += lpm)
                        p += eps64[a.ridx[0][e]];
                    double p2 = 0.0;
                    for (int e = ro[2] + tm.lane; e < ro[3]; e += lpm)
                        p2 += eps64[a.ridx[1][e]];
                    p = team_sum_d(p + 2.0 * p2, tm, lpm);
                    if (tm.lane == 0) {
                        __int128 x;
                        ok = fx_from_double(p, x);
                        if (ok)
                            publish(acc, x);
                    }
                } else {
                    float h = 0.f, l = 0.f;
                    for (int e = ro[0] + tm.lane; e < ro[1]; e += lpm) {
                        const int i = a.ridx[0][e];
                        df_add(h, l, eh[i], el[i]);
                    }
                    for (int e = ro[2] + tm.lane; e < ro[3]; e += lpm) {
                        const int i = a.ridx[1][e];
                        df_add(h, l, 2.f * eh[i], 2.f * el[i]);
                    }
                    team_df_sum(h, l, tm, lpm);
                    if (tm.lane == 0) {
                        __int128 x1, x2;
                        ok = fx_from_float(h, x1) && fx_from_float(l, x2);
                        if (ok)
                            publish(acc, x1 + x2);
                    }
                }
            }
            if (!ok)
                atomicCAS(a.err, kDevOk, kDevRange);
        }
        __syncthreads();
        mark(1);

        // ---- grid barrier: one counter; release orders this CTA's
        // accumulator updates (ordered before it by bar.sync), acquire orders
        // the reads below.  The wait is bounded.
        if (tid == 0) {
            red_release_add_u64(a.counter, 1ull);
            const unsigned long long target = (unsigned long long)(a.G + a.phantom) * (unsigned long long)(r + 1);
            const uint64_t t0 = global_timer_ns();
            unsigned spins = 0;
            while (ld_acquire_u64(a.counter) < target) {
                if ((++spins & 255u) == 0) {
                    if (*(volatile int *)a.err != kDevOk || global_timer_ns() - t0 > a.timeout_ns) {
                        atomicCAS(a.err, kDevOk, kDevTimeout);
                        s_abort = 1;
                        break;
                    }
                }
            }
        }
        __syncthreads();
        mark(2);
        if (s_abort)
            break;

        // ---- redundant sampling of the round's markers in every CTA, one thread per marker
        if (tid < nb) {
            const SweepRec &rc = ring_rec[(start + tid) & Rm];
            const unsigned long long *acc = a.acc + (rb * kMaxSpec + tid) * 4;
            const double tot = fx_join((long long)ld_relaxed_u64(acc), ld_relaxed_u64(acc + 1));
            double num;
            if (KIND == kKindDense) {
                if (FORM == kFormFP64) {
                    num = tot + rc.beta_old * Nm1;
                } else {
                    const double sm = fx_join((long long)ld_relaxed_u64(acc + 2), ld_relaxed_u64(acc + 3));
                    const double sigma = rc.t[0], cm = rc.t[1], xm = rc.t[2];
                    num = (sigma * (tot - cm * (s_scal[2] - sm)) + xm * sm) + rc.beta_old * Nm1;
                }
            } else {
                const double mean = rc.t[0], isd = rc.t[2], Zsum = rc.t[3];
                num = (rc.beta_old * ((double)a.N - 1.0) - mean * s_scal[1] * isd) + (tot + s_scal[0] * Zsum) * isd;
            }
            const int g = rc.group;
            const Pick pk = pick_marker<FORM != kFormFP64, KM>(num, rc.u, rc.z, rc.beta_old,
                                                           gconst + (size_t)g * kMaxK * 4, gk[g]);
            s_beta[tid] = pk.beta;
            s_acum[tid] = pk.acum0;
            s_comp[tid] = pk.comp;
            if (rc.beta_old != 0.0 || pk.beta != 0.0)
                atomicMin(&s_first, tid);
        }
        __syncthreads();
        mark(3);

        const int first = s_first;
        const int last = first < nb ? first : nb - 1;
        if (blockIdx.x == 0) {
            // outputs of the resolved markers, only from CTA 0
            if (tid <= last) {
                const SweepRec &rc = ring_rec[(start + tid) & Rm];
                const int c = s_comp[tid];
                a.beta[rc.j] = s_beta[tid];
                a.acum[rc.j] = s_acum[tid];
                a.chosen[rc.j] = c >= 0 ? 1 : 0;
                if (c >= 0)
                    a.comp[rc.j] = c;
            }
            // all CTAs have read the accumulators of round r-1: recycle them
            if (tid < 4 * kMaxSpec)
                a.acc[((rb + 2) % 3) * kMaxSpec * 4 + tid] = 0ull;
        }

        // ---- apply the residual update of the first changing marker
        if (first < nb) {
            const unsigned slot = (start + first) & Rm;
            const SweepRec &rc = ring_rec[slot];
            const double dBeta = rc.beta_old - s_beta[first];
            if (KIND == kKindDense) {
                const uint8_t *cb = ring_codes + slot * a.slot_bytes;
                if (FORM == kFormFP64) {
                    const double l0 = rc.t[0], l1 = rc.t[1], l2 = rc.t[2], l3 = rc.t[3];
                    for (int i = tid; i < ns; i += kThreads) {
                        const unsigned c = (cb[i >> 2] >> (2 * (i & 3))) & 3u;
                        eps64[i] = __dadd_rn(eps64[i], __dmul_rn(dBeta, lut_select(c, l0, l1, l2, l3)));
                    }
                } else {
                    if (tid < 4) {
                        // delta per code: dBeta * (v - colmean) * sigma, missing: dBeta * xm
                        const double sigma = rc.t[0], cm = rc.t[1], xm = rc.t[2];
                        const double gv = tid == 0 ? 2.0 : (tid == 2 ? 1.0 : 0.0);
                        const double d = tid == 1 ? dBeta * xm : dBeta * ((gv - cm) * sigma);
                        float h, l;
                        df_from_double(d, h, l);
                        s_dfl[2 * tid] = h;
                        s_dfl[2 * tid + 1] = l;
                    } else if (tid == 32) {
                        // the residual total moves by dBeta times the column sum
                        s_scal[2] = s_scal[2] + dBeta * rc.t[3];
                    }
                    __syncthreads();
                    for (int i = tid; i < ns; i += kThreads) {
                        const unsigned c = (cb[i >> 2] >> (2 * (i & 3))) & 3u;
                        float h = eh[i], l = el[i];
                        df_add(h, l, s_dfl[2 * c], s_dfl[2 * c + 1]);
                        eh[i] = h;
                        el[i] = l;
                    }
                }
            } else {
                const int32_t *ro = ring_roff + slot * 8;
                if (tid == 0) {
                    const double mean = rc.t[0], isd = rc.t[2], Zsum = rc.t[3];
                    const double meanAdj = dBeta * mean * isd;
                    const double oneAdj = dBeta * isd;
                    s_delta[0] = oneAdj;
                    s_delta[1] = 2.0 * oneAdj;
                    s_delta[2] = meanAdj;
                    s_scal[0] = s_scal[0] - meanAdj;
                    s_scal[1] = s_scal[1] + ((dBeta * Zsum) * isd - ((dBeta * mean) * (double)a.N) * isd);
                    float h, l;
                    for (int k = 0; k < 3; ++k) {
                        df_from_double(s_delta[k], h, l);
                        s_dfl[2 * k] = h;
                        s_dfl[2 * k + 1] = l;
                    }
                }
                __syncthreads();
                for (int k = 0; k < 3; ++k) {
                    const uint16_t *ix = a.ridx[k];
                    for (int e = ro[2 * k] + tid; e < ro[2 * k + 1]; e += kThreads) {
                        const int i = ix[e];
                        if (FORM == kFormFP64) {
                            eps64[i] = __dadd_rn(eps64[i], s_delta[k]);
                        } else {
                            float h = eh[i], l = el[i];
                            df_add(h, l, s_dfl[2 * k], s_dfl[2 * k + 1]);
                            eh[i] = h;
                            el[i] = l;
                        }
                    }
                }
            }
        }
        __syncthreads();
        mark(4);
        start += (unsigned)(last + 1);
        ++r;
        rb = rb == 2 ? 0 : rb + 1;
    }
    if (prof) {
        for (int k = 0; k < 5; ++k)
            a.prof[k] = ph[k];
        a.prof[5] = r;
    }
    cp_async_wait_all();
    __syncthreads();

    // ---- epilogue: residual back to HBM, per-slice sums
    double s1 = 0.0, s2 = 0.0;
    const double shift = (KIND == kKindRagged) ? s_scal[0] : 0.0;
    float shh, shl;
    df_from_double(shift, shh, shl);
    for (int i = tid; i < ns; i += kThreads) {
        double e;
        if (FORM == kFormFP64) {
            e = KIND == kKindRagged ? __dadd_rn(eps64[i], shift) : eps64[i];
            a.eps[lo + i] = e;
        } else {
            float h = eh[i], l = el[i];
            if (KIND == kKindRagged)
                df_add(h, l, shh, shl);
            a.eps_hi[lo + i] = h;
            a.eps_lo[lo + i] = l;
            e = (double)h + (double)l;
        }
        s1 += e;
        s2 = fma(e, e, s2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((tid & 31) == 0) {
        s_red[tid >> 5][0] = s1;
        s_red[tid >> 5][1] = s2;
    }
    __syncthreads();
    if (tid == 0) {
        double t1 = 0.0, t2 = 0.0;
        for (int q = 0; q < kThreads / 32; ++q) {
            t1 += s_red[q][0];
            t2 += s_red[q][1];
        }
        a.part[2 * sidx] = t1;
        a.part[2 * sidx + 1] = t2;
        if (blockIdx.x == 0) {
            a.stats_out[0] = s_scal[1];
            *a.rounds_out = r;
        }
    }
}

// --------------------------------------------------------------------------
// Blocked sweep of the FP32C form over dense markers, with the precomputed
// marker Gram matrix (packed lower triangle, FP64).  Every grid round
// resolves exactly B consecutive markers of the sweep order: the B dot
// products against the residual at the start of the block are exchanged as in
// k_sweep; then, in every CTA, all markers of the block are sampled in
// parallel, the first one that changes the residual (p) is kept, the dot
// products of the later markers are moved by dBeta_p * G[p, t], and the later
// markers are sampled again, until no later marker changes the residual.  This
// is the sequential chain exactly (up to rounding): marker t sees
// x_t . (eps + sum_{p<t} dBeta_p x_p).  The rank-U residual update of the block
// follows.  Genotype slices, records and the block's Gram entries are
// prefetched with cp.async one round ahead.
struct BlockPlan {
    SmemPlan base;  // residual, code ring, group constants, decode tables
    size_t brec;    // R x BlockRec
    size_t gram;    // 2 x npairs double-float entries
    size_t pairs;   // npairs x 2 bytes (positions a < b)
    size_t gcf;     // n_groups x kMaxK x {dc, h} floats: FP32 log-likelihood constants
    size_t gbf;     // n_groups x kMaxK x {sdk hi, lo, invden hi, lo}: double-float beta constants
    size_t total;
};

__host__ __device__ inline BlockPlan make_block_plan(int slice_max, int slot_bytes, int B, int n_groups)
{
    BlockPlan p;
    p.base = make_plan(kFormFP32C, kKindDense, slice_max, slot_bytes, B, n_groups, 0);
    const size_t npairs = (size_t)B * (B - 1) / 2;
    size_t o = p.base.total;
    p.brec = o;
    o += (size_t)4 * B * sizeof(BlockRec);
    p.gram = o;
    o += align16(2 * npairs * sizeof(float2));
    p.pairs = o;
    o += align16(npairs * 2);
    p.gcf = o;
    o += align16((size_t)n_groups * kMaxK * 2 * sizeof(float));
    p.gbf = o;
    o += align16((size_t)n_groups * kMaxK * 4 * sizeof(float));
    p.total = align16(o);
    return p;
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

// New beta of a marker that chose component k > 0, as double-float:
// beta = z * sdk_k + num * invden_k (the FP64 expression of pick_marker).
__device__ __forceinline__ void beta_df(const BlockRec &rc, const float *__restrict__ gbf, int k, float nh, float nl,
                                        float &bh, float &bl)
{
    const float4 c = reinterpret_cast<const float4 *>(gbf)[k];
    float ph, pl;
    df_mul(rc.zf[0], rc.zf[1], c.x, c.y, bh, bl);
    df_mul(nh, nl, c.z, c.w, ph, pl);
    df_add(bh, bl, ph, pl);
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

// Outputs of one resolved block (first CTA, one warp): new beta as double-float
// (z * sdk + num * invden for a component k > 0, 0 for component 0), acum
// (P(component 0) of the FP32 sampler at the final num, or of the FP64
// evaluation), chosen flag and component, by marker id.  Runs while the CTA
// waits at the next grid barrier; the block's records stay in the ring until then.
template <int KM>
__device__ __forceinline__ void write_block_outputs(const SweepArgs &a, const BlockRec *ring_rec, unsigned q0,
                                                    unsigned Rm, const float *gcf, const int32_t *gk,
                                                    const float *gbf, const float2 *s_ox, const float2 *s_oa,
                                                    const float2 *s_ob, const int *s_oc, int lane)
{
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int m = lane + 32 * h;
        const int oc = s_oc[m];
        if (oc == -2)
            continue;
        const BlockRec &rc = ring_rec[(q0 + m) & Rm];
        const int c = (oc & 0x80) ? -1 : (oc & 0xFF);
        const bool fp64 = (oc & 0x100) != 0;
        const float2 x = s_ox[m];
        float bh = 0.f, bl = 0.f;
        float2 acum;
        if (fp64) {
            const float2 fbv = s_oa[m];
            if (c > 0) {
                bh = fbv.x;
                bl = fbv.y;
            }
            acum = s_ob[m];
        } else {
            if (c > 0)
                beta_df(rc, gbf + (size_t)rc.group * kMaxK * 4, c, x.x, x.y, bh, bl);
            int c2;
            float a0;
            pick_f32<KM>(x.x, x.y, rc.uf, gcf + (size_t)rc.group * kMaxK * 2, gk[rc.group], c2, a0);
            acum = make_float2(a0, 0.f);
        }
        a.beta_df[rc.j] = make_float2(bh, bl);
        a.acum_df[rc.j] = acum;
        a.chosen[rc.j] = c >= 0 ? 1 : 0;
        if (c >= 0)
            a.comp[rc.j] = c;
    }
}

template <int KM, bool MISS>
__global__ void __launch_bounds__(kThreads, 1) k_sweep_block(SweepArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_upd[kMaxSpec];
    __shared__ float2 s_dB[kMaxSpec];
    __shared__ float2 s_num[kMaxSpec];     // num at the block start (double-float)
    __shared__ float s_uf[kMaxSpec];
    __shared__ unsigned s_meta[kMaxSpec];  // group | K << 8 | (beta_old != 0) << 16
    __shared__ float2 s_ox[kMaxSpec];      // first CTA: final num
    __shared__ float2 s_oa[kMaxSpec];      // first CTA: beta of an FP64 decision
    __shared__ float2 s_ob[kMaxSpec];      // first CTA: acum of an FP64 decision
    __shared__ int s_oc[kMaxSpec];         // first CTA: comp | FP64 decision << 8; -2: no marker
    __shared__ float s_H[kMaxGroups];      // largest minus smallest h_k of each group (h_0 = 0)
    __shared__ float s_dfl[kMaxSpec][8];
    __shared__ int s_abort, s_nupd;

    const int B = a.B;
    const int lpm = kThreads / B;
    const int R = 4 * B;
    const int sidx = blockIdx.x;
    const int tid = threadIdx.x;
    const int lo = a.slice_lo[sidx];
    const int ns = a.slice_lo[sidx + 1] - lo;
    const int nbytes = ((ns + kChunk - 1) / kChunk) * 16;
    const int64_t byte_lo = lo / 4;
    const BlockPlan bp = make_block_plan(a.slice_max, a.slot_bytes, B, a.n_groups);
    const SmemPlan &plan = bp.base;
    const int npairs = B * (B - 1) / 2;

    float *eh = reinterpret_cast<float *>(smem + plan.eps0);
    float *el = reinterpret_cast<float *>(smem + plan.eps1);
    uint8_t *ring_codes = smem + plan.ring_codes;
    BlockRec *ring_rec = reinterpret_cast<BlockRec *>(smem + bp.brec);
    double *gconst = reinterpret_cast<double *>(smem + plan.gconst);
    int32_t *gk = reinterpret_cast<int32_t *>(smem + plan.gk);
    float4 *gtab = reinterpret_cast<float4 *>(smem + plan.gtab);
    uint8_t *mtab = smem + plan.gtab + 256 * 16;
    float2 *gbuf = reinterpret_cast<float2 *>(smem + bp.gram);
    uint8_t *pair_ab = smem + bp.pairs;
    float *gcf = reinterpret_cast<float *>(smem + bp.gcf);
    float *gbf = reinterpret_cast<float *>(smem + bp.gbf);

    // ---- prologue
    float muh, mul;
    df_from_double(-a.mu_new, muh, mul);
    for (int i = tid; i < a.slice_max; i += kThreads) {
        float h = 0.f, l = 0.f;
        if (i < ns) {
            h = a.eps_hi[lo + i];
            l = a.eps_lo[lo + i];
            df_add(h, l, muh, mul);
        }
        eh[i] = h;
        el[i] = l;
    }
    for (int i = tid; i < a.n_groups * kMaxK * 4; i += kThreads)
        gconst[i] = a.gconst[i];
    for (int i = tid; i < a.n_groups; i += kThreads) {
        gk[i] = a.gK[i];
        const double *row = a.gconst + (size_t)i * kMaxK * 4;
        double hmax = 0.0, hmin = 0.0;
        for (int k = 1; k < a.gK[i]; ++k) {
            hmax = fmax(hmax, row[4 * k + 2]);
            hmin = fmin(hmin, row[4 * k + 2]);
        }
        s_H[i] = (float)((hmax - hmin) * (1.0 + 1e-6));
    }
    for (int i = tid; i < a.n_groups * kMaxK; i += kThreads) {
        const int g = i / kMaxK, k = i - g * kMaxK;
        const double *row = a.gconst + (size_t)g * kMaxK * 4;
        gcf[2 * i] = k == 0 ? 0.f : (float)(row[4 * k] - row[0]);
        gcf[2 * i + 1] = k == 0 ? 0.f : (float)row[4 * k + 2];
        df_from_double(row[4 * k + 3], gbf[4 * i], gbf[4 * i + 1]);
        df_from_double(row[4 * k + 1], gbf[4 * i + 2], gbf[4 * i + 3]);
    }
    for (int v = tid; v < 256; v += kThreads) {
        float g[4];
        unsigned m = 0;
        for (int k = 0; k < 4; ++k) {
            const unsigned c = (v >> (2 * k)) & 3u;
            g[k] = c == 0u ? 2.f : (c == 2u ? 1.f : 0.f);
            if (c == 1u)
                m |= 1u << k;
        }
        gtab[v] = make_float4(g[0], g[1], g[2], g[3]);
        mtab[v] = (uint8_t)m;
    }
    for (int pb = 1 + tid; pb < B; pb += kThreads)
        for (int pa = 0; pa < pb; ++pa) {
            const int p = pb * (pb - 1) / 2 + pa;
            pair_ab[2 * p] = (uint8_t)pa;
            pair_ab[2 * p + 1] = (uint8_t)pb;
        }
    if (tid == 0)
        s_abort = 0;
    __syncthreads();

    const unsigned M32 = (unsigned)a.M;
    const unsigned Rm = (unsigned)R - 1u;
    unsigned rec_issued = 0, code_issued = 0;
    auto issue_recs = [&](unsigned upto) {
        upto = min(upto, M32);
        if (upto <= rec_issued)
            return;
        constexpr unsigned kParts = sizeof(BlockRec) / 16;
        const unsigned n = (upto - rec_issued) * kParts;
        for (unsigned e = tid; e < n; e += kThreads) {
            const unsigned q = rec_issued + e / kParts;
            const unsigned c = e % kParts;
            cp_async16(reinterpret_cast<unsigned char *>(&ring_rec[q & Rm]) + 16 * c,
                       reinterpret_cast<const unsigned char *>(&a.brec[q]) + 16 * c);
        }
        rec_issued = upto;
    };
    const unsigned chunks = (unsigned)nbytes / 16u;
    const unsigned per_pass = chunks ? (unsigned)kThreads / chunks : 0u;
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
    // Cooperative Gram gather: CTA s loads pairs p = s, s+G, ... of the block
    // starting at q0 (issued early into registers, stored to the global staging
    // buffer before the CTA arrives at the round barrier, which publishes them).
    // Thread t of CTA s owns pairs p = s + (t + k*kThreads)*G; the first one is
    // loaded ahead into a register, any further ones (small grids only) at store time.
    double gval = 0.0;
    int gpair = -1;
    unsigned gq0 = 0;
    auto gram_entry = [&](unsigned q0, int p, unsigned nb, double *out) -> bool {
        const unsigned pa = pair_ab[2 * p], pb = pair_ab[2 * p + 1];
        if (pb >= nb)
            return false;
        const int64_t ja = ring_rec[(q0 + pa) & Rm].j, jb = ring_rec[(q0 + pb) & Rm].j;
        const int64_t hi = ja > jb ? ja : jb, lw = ja > jb ? jb : ja;
        *out = __ldg(&a.gram[hi * (hi - 1) / 2 + lw]);
        return true;
    };
    auto gather_load = [&](unsigned q0) {
        gpair = -1;
        gq0 = q0;
        if (q0 >= M32)
            return;
        const int p = sidx + tid * a.G;
        if (p < npairs && gram_entry(q0, p, min((unsigned)B, M32 - q0), &gval))
            gpair = p;
    };
    // entries are staged as double-float pairs (hi, lo) for the FP32 resolve
    float2 *gstage2 = reinterpret_cast<float2 *>(a.gstage);
    auto split2 = [](double v) {
        float h, l;
        df_from_double(v, h, l);
        return make_float2(h, l);
    };
    auto gather_store = [&](int buf) {
        if (gpair >= 0)
            gstage2[(size_t)buf * npairs + gpair] = split2(gval);
        if (gq0 >= M32)
            return;
        const unsigned nb = min((unsigned)B, M32 - gq0);
        for (int p = sidx + (tid + kThreads) * a.G; p < npairs; p += kThreads * a.G) {
            double v;
            if (gram_entry(gq0, p, nb, &v))
                gstage2[(size_t)buf * npairs + p] = split2(v);
        }
    };
    auto copy_stage = [&](int buf) {
        const unsigned n16 = (unsigned)(npairs * 8 + 15) / 16u;
        for (unsigned e = tid; e < n16; e += kThreads)
            cp_async16(reinterpret_cast<unsigned char *>(gbuf + (size_t)buf * npairs) + 16 * e,
                       reinterpret_cast<const unsigned char *>(a.gstage + (size_t)buf * npairs) + 16 * e);
    };

    issue_recs(3u * B);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    issue_codes(2u * B);
    cp_async_commit();
    gather_load(0u);
    gather_store(0);   // block 0's entries, published by the first round barrier

    int lpm_log2 = 0;
    while ((1 << lpm_log2) < lpm)
        ++lpm_log2;
    const Team tm = make_team(lpm);
    const int team = tid >> lpm_log2;
    const bool prof = a.prof != nullptr && blockIdx.x == 0 && tid == 0;
    long long ph[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    long long tp = prof ? clock64() : 0;
    auto mark = [&](int k) {
        if (prof) {
            const long long t = clock64();
            ph[k] += t - tp;
            tp = t;
        }
    };
    auto publish = [&](unsigned long long *acc, __int128 x) {
        const Fx f = fx_split(x);
        red_add_u64(acc, (unsigned long long)f.hi);
        red_add_u64(acc + 1, f.lo);
    };

    unsigned start = 0;
    long long r = 0, steps = 0;
    int rb = 0;
    unsigned long long *fb_counter = a.prof ? reinterpret_cast<unsigned long long *>(a.prof + 8) : nullptr;
    while (start < M32) {
        cp_async_wait_all();
        __syncthreads();
        issue_codes(start + 2u * B);
        issue_recs(start + 3u * B);
        cp_async_commit();
        gather_load(start + (unsigned)B);   // next block's Gram entries, in flight during the dots
        const int nb = (int)min((unsigned)B, M32 - start);
        const float2 *gcur = gbuf + (size_t)(r & 1) * npairs;
        mark(0);

        // ---- partial dot products (double-float, exact integer genotypes).
        // Warp w owns markers w, w+8, ... of the block; its lanes stride over
        // the slice's code bytes, so each residual value is read once per warp
        // and kept in registers for all of the warp's markers.  Per byte the
        // four products g*hi (exact) are combined by error-free TwoSums and one
        // TwoSum enters the running sum; rounding errors and g*lo go to the
        // low word.  Missing genotypes are summed apart (double-float).
        {
            const int warp = tid >> 5, lane = tid & 31;
            constexpr int MPW = kMaxSpec / 8;   // markers per warp
            float Ah[MPW], Al[MPW], Mh[MPW], Ml[MPW];
            unsigned cofs[MPW];
#pragma unroll
            for (int k = 0; k < MPW; ++k) {
                Ah[k] = Al[k] = Mh[k] = Ml[k] = 0.f;
                // markers past the end of a short last block read a stale ring
                // slot; their sums are never published
                cofs[k] = ((start + (unsigned)(warp + 8 * k)) & Rm) * (unsigned)a.slot_bytes;
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
                        const float lo4 = __fmaf_rn(g0, l.x, __fmaf_rn(g1, l.y, __fmaf_rn(g2, l.z, __fmul_rn(g3, l.w))));
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
            const long long te0 = prof ? clock64() : 0;
            // reduce-scatter: after three halving exchanges lane l holds the
            // partial sum of marker kk(l) over 8 lanes; two more exchanges
            // complete it over the warp, and lanes 0, 4, ..., 28 publish
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
            if ((lane & 3) == 0 && m < nb) {
                unsigned long long *acc = a.acc + (rb * kMaxSpec + m) * 4;
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
            if (prof)
                ph[8] += clock64() - te0;
        }
        gather_store((int)((r + 1) & 1));
        __syncthreads();
        mark(1);
        if (blockIdx.x == 0 && r > 0 && (tid >> 5) == 1)
            write_block_outputs<KM>(a, ring_rec, start - (unsigned)B, Rm, gcf, gk, gbf, s_ox, s_oa, s_ob, s_oc,
                                    tid - 32);

        // ---- grid barrier
        if (tid == 0) {
            red_release_add_u64(a.counter, 1ull);
            const unsigned long long target = (unsigned long long)(a.G + a.phantom) * (unsigned long long)(r + 1);
            const uint64_t t0 = global_timer_ns();
            unsigned spins = 0;
            while (ld_acquire_u64(a.counter) < target) {
                if ((++spins & 255u) == 0) {
                    if (*(volatile int *)a.err != kDevOk || global_timer_ns() - t0 > a.timeout_ns) {
                        atomicCAS(a.err, kDevOk, kDevTimeout);
                        s_abort = 1;
                        break;
                    }
                }
            }
        }
        __syncthreads();
        mark(2);
        if (s_abort)
            break;
        if (r == 0) {
            // block 0's entries were staged before the first barrier
            copy_stage(0);
            cp_async_commit();
            cp_async_wait_all();
        }
        copy_stage((int)((r + 1) & 1));   // next block's entries: complete before the next round
        cp_async_commit();

        // ---- per-marker inputs of the resolve, one thread per marker:
        // num = sigma * sum(g*eps) + cst + dm * sum_missing(eps) (double-float)
        if (tid < kMaxSpec) {
            const int m = tid;
            float nh = 0.f, nl = 0.f, uf = 2.f;
            unsigned meta = 2u << 8;
            if (m < nb) {
                const BlockRec &rc = ring_rec[(start + m) & Rm];
                const unsigned long long *acc = a.acc + (rb * kMaxSpec + m) * 4;
                float th, tl;
                fx_to_df((long long)ld_relaxed_u64(acc), ld_relaxed_u64(acc + 1), th, tl);
                df_mul(rc.sig[0], rc.sig[1], th, tl, nh, nl);
                df_add(nh, nl, rc.cst[0], rc.cst[1]);
                if (MISS) {
                    float sh, sl, qh, ql;
                    fx_to_df((long long)ld_relaxed_u64(acc + 2), ld_relaxed_u64(acc + 3), sh, sl);
                    df_mul(rc.dm[0], rc.dm[1], sh, sl, qh, ql);
                    df_add(nh, nl, qh, ql);
                }
                uf = rc.uf;
                meta = (unsigned)rc.group | ((unsigned)gk[rc.group] << 8) | (rc.bnz ? 1u << 16 : 0u);
            }
            s_num[m] = make_float2(nh, nl);
            s_uf[m] = uf;
            s_meta[m] = meta;
        }
        __syncthreads();
        if (prof)
            mark(5);

        // ---- resolve the block in warp 0 (lane l owns markers l and l+32),
        // in FP32 / double-float only: after every residual-changing marker p
        // the later markers move by dBeta_p * G[p, t] and are sampled again.
        // Ballots find p, shuffles broadcast dBeta_p; no CTA barrier inside the
        // loop.  Both markers of a lane are evaluated without branches; the
        // FP64 evaluation of an uncertified decision is a separate, rare branch.
        if (tid < 32) {
            const int lane = tid;
            float nh[2], nl[2], ufr[2], ch[2] = {0.f, 0.f}, cl[2] = {0.f, 0.f};
            float a0h[2] = {0.f, 0.f}, a0l[2] = {0.f, 0.f}, fbh[2] = {0.f, 0.f}, fbl[2] = {0.f, 0.f};
            int comp[2] = {-1, -1}, grp[2], kk[2];
            bool own[2], bnz[2], fb[2] = {false, false};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int m = lane + 32 * h;
                own[h] = m < nb;
                const float2 n = s_num[m];
                nh[h] = n.x;
                nl[h] = n.y;
                ufr[h] = s_uf[m];
                const unsigned meta = s_meta[m];
                grp[h] = (int)(meta & 0xFFu);
                kk[h] = (int)((meta >> 8) & 0xFFu);
                bnz[h] = (meta >> 16) != 0u;
            }
            float sref[2] = {0.f, 0.f}, wmar[2] = {-1.f, -1.f}, hg[2];
#pragma unroll
            for (int h = 0; h < 2; ++h)
                hg[h] = s_H[grp[h]];
            int next = 0, nupd = 0;
            while (true) {
                const long long tl0 = prof ? clock64() : 0;
                bool need[2], upd[2];
                float sx[2];
                // a decision is kept while its certified margin covers the move of num^2
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
                        const bool ok = pick_margin<KM>(sx[h], ufr[h], gcf + (size_t)grp[h] * kMaxK * 2, kk[h], c, w);
                        if (need[h]) {
                            comp[h] = c;
                            fb[h] = false;
                            sref[h] = sx[h];
                            wmar[h] = ok ? w : -1.f;
                        }
                        slow[h] = need[h] && !ok;
                    }
                    if (__any_sync(0xffffffffu, slow[0] || slow[1])) {
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            if (!slow[h])
                                continue;
                            // 700 guards possibly active, or u near a boundary: the
                            // guarded FP32 sampler, then FP64
                            float xh = nh[h], xl = nl[h];
                            df_add(xh, xl, ch[h], cl[h]);
                            int c;
                            float a0;
                            if (pick_f32<KM>(xh, xl, ufr[h], gcf + (size_t)grp[h] * kMaxK * 2, kk[h], c, a0)) {
                                comp[h] = c;
                            } else {
                                const BlockRec &rc = ring_rec[(start + lane + 32 * h) & Rm];
                                const Pick r64 = pick_marker<false, KM>((double)xh + (double)xl, rc.u, rc.z,
                                                                        rc.beta_old, gconst + (size_t)grp[h] * kMaxK * 4,
                                                                        kk[h]);
                                comp[h] = r64.comp;
                                df_from_double(r64.acum0, a0h[h], a0l[h]);
                                df_from_double(r64.beta, fbh[h], fbl[h]);
                                fb[h] = true;
                                if (blockIdx.x == 0 && fb_counter)
                                    atomicAdd(fb_counter, 1ull);
                            }
                        }
                    }
                }
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    upd[h] = own[h] && lane + 32 * h >= next && (bnz[h] || comp[h] > 0);
                const long long tl1 = prof ? clock64() : 0;
                if (prof)
                    ph[6] += tl1 - tl0;
                ++steps;
                const unsigned b0 = __ballot_sync(0xffffffffu, upd[0]);
                const unsigned b1 = __ballot_sync(0xffffffffu, upd[1]);
                const int p = b0 ? __ffs(b0) - 1 : (b1 ? 32 + __ffs(b1) - 1 : kMaxSpec);
                if (p >= nb)
                    break;
                // dBeta_p = beta_old - beta_new as double-float, computed by the owner
                const int owner = p & 31;
                const bool half = p >= 32;
                float dh = 0.f, dl = 0.f;
                if (lane == owner) {
                    const BlockRec &rc = ring_rec[(start + p) & Rm];
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
                                beta_df(rc, gbf + (size_t)rc.group * kMaxK * 4, c, xh, xl, bh, bl);
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
                        // corr += dBeta * G[p, m] in double-float
                        const float2 g2 = gcur[m * (m - 1) / 2 + p];
                        float ph, pl;
                        df_mul(dh, dl, g2.x, g2.y, ph, pl);
                        df_add(ch[h], cl[h], ph, pl);
                    }
                }
                if (lane == 0) {
                    s_upd[nupd] = p;
                    s_dB[nupd] = make_float2(dh, dl);
                }
                ++nupd;
                next = p + 1;
                if (prof)
                    ph[7] += clock64() - tl1;
            }
            if (lane == 0)
                s_nupd = nupd;
            // first CTA: the block's decisions, written out during the next barrier wait
            if (blockIdx.x == 0) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int m = lane + 32 * h;
                    float xh = nh[h], xl = nl[h];
                    df_add(xh, xl, ch[h], cl[h]);
                    s_ox[m] = make_float2(xh, xl);
                    s_oa[m] = fb[h] ? make_float2(fbh[h], fbl[h]) : make_float2(a0h[h], a0l[h]);
                    s_ob[m] = make_float2(a0h[h], a0l[h]);
                    s_oc[m] = own[h] ? ((comp[h] & 0xFF) | (fb[h] ? 0x100 : 0)) : -2;
                }
            }
        }
        __syncthreads();
        mark(3);

        if (blockIdx.x == 0 && tid < 4 * kMaxSpec)
            a.acc[((rb + 2) % 3) * kMaxSpec * 4 + tid] = 0ull;

        // ---- rank-U residual update of the block: eps += dBeta_u * x_u
        const int U = s_nupd;
        if (U > 0) {
            if (tid < 4 * U) {
                const int u = tid >> 2, code = tid & 3;
                const BlockRec &rc = ring_rec[(start + s_upd[u]) & Rm];
                const float2 dB = s_dB[u];
                df_mul(dB.x, dB.y, rc.x[2 * code], rc.x[2 * code + 1], s_dfl[u][2 * code], s_dfl[u][2 * code + 1]);
            }
            __syncthreads();
            // The sum of the residual is left as it was at the sweep start: the
            // standardised columns sum to zero, so a dense update moves it only
            // by rounding (dBeta times a column sum of order 1e-11).
            for (int b = tid; b < nbytes; b += kThreads) {
                float4 h = reinterpret_cast<float4 *>(eh)[b];
                float4 l = reinterpret_cast<float4 *>(el)[b];
                for (int u = 0; u < U; ++u) {
                    const unsigned v = ring_codes[((start + s_upd[u]) & Rm) * a.slot_bytes + b];
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
        __syncthreads();
        mark(4);
        start += (unsigned)nb;
        ++r;
        rb = rb == 2 ? 0 : rb + 1;
    }
    if (blockIdx.x == 0 && r > 0 && !s_abort && (tid >> 5) == 1)
        write_block_outputs<KM>(a, ring_rec, start - (unsigned)((M32 - 1) % (unsigned)B + 1), Rm, gcf, gk, gbf, s_ox,
                                s_oa, s_ob, s_oc, tid - 32);
    if (prof) {
        for (int k = 0; k < 5; ++k)
            a.prof[k] = ph[k];
        a.prof[5] = r;
        a.prof[6] = steps;
        a.prof[7] = ph[5];
        a.prof[9] = ph[6];
        a.prof[10] = ph[7];
        a.prof[11] = ph[8];
    }   // a.prof[8]: FP64 fallbacks of the certified sampler (first CTA)
    cp_async_wait_all();
    __syncthreads();

    // ---- epilogue
    double s1 = 0.0, s2 = 0.0;
    for (int i = tid; i < ns; i += kThreads) {
        a.eps_hi[lo + i] = eh[i];
        a.eps_lo[lo + i] = el[i];
        const double e = (double)eh[i] + (double)el[i];
        s1 += e;
        s2 = fma(e, e, s2);
    }
    __shared__ double s_red[kThreads / 32][2];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((tid & 31) == 0) {
        s_red[tid >> 5][0] = s1;
        s_red[tid >> 5][1] = s2;
    }
    __syncthreads();
    if (tid == 0) {
        double t1 = 0.0, t2 = 0.0;
        for (int q = 0; q < kThreads / 32; ++q) {
            t1 += s_red[q][0];
            t2 += s_red[q][1];
        }
        a.part[2 * sidx] = t1;
        a.part[2 * sidx + 1] = t2;
        if (blockIdx.x == 0) {
            a.stats_out[0] = 0.0;
            *a.rounds_out = r;
        }
    }
}

// Sweep statistics from the resolved markers (src/BayesRBase.cpp:353-355):
// v[g][k] counts the markers that chose component k, betasqnG[g] sums the
// squares of the non-zero betas.  Counts and the fixed-point square sums are
// integer atomics, so the result does not depend on the order of summation.
__global__ void __launch_bounds__(kThreads) k_sweep_stats(int64_t M, const int32_t *__restrict__ group,
                                                          const int32_t *__restrict__ comp,
                                                          const uint8_t *__restrict__ chosen,
                                                          const double *__restrict__ beta, int n_groups,
                                                          unsigned long long *__restrict__ out)
{
    // out: [n_groups*kMaxK] counts, then [n_groups][2] fixed-point sums
    __shared__ unsigned long long sv[kMaxGroups * kMaxK];
    __shared__ unsigned long long sb[kMaxGroups][2];
    for (int i = threadIdx.x; i < n_groups * kMaxK; i += blockDim.x)
        sv[i] = 0ull;
    for (int i = threadIdx.x; i < n_groups; i += blockDim.x) {
        sb[i][0] = 0ull;
        sb[i][1] = 0ull;
    }
    __syncthreads();
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < M; j += (int64_t)gridDim.x * blockDim.x) {
        if (!chosen[j])
            continue;
        const int g = group[j], c = comp[j];
        atomicAdd(&sv[g * kMaxK + c], 1ull);
        if (c >= 1) {
            __int128 x;
            fx_from_double(beta[j] * beta[j], x);
            const Fx f = fx_split(x);
            atomicAdd(&sb[g][0], (unsigned long long)f.hi);
            atomicAdd(&sb[g][1], f.lo);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_groups * kMaxK; i += blockDim.x)
        if (sv[i])
            atomicAdd(&out[i], sv[i]);
    for (int i = threadIdx.x; i < n_groups; i += blockDim.x) {
        atomicAdd(&out[n_groups * kMaxK + 2 * i], sb[i][0]);
        atomicAdd(&out[n_groups * kMaxK + 2 * i + 1], sb[i][1]);
    }
}

// --------------------------------------------------------------------------
// Launchers.

cudaError_t launch_draws(uint32_t seed, uint32_t chain, uint32_t it, int64_t M, double *u, double *z, cudaStream_t st)
{
    k_draws<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(seed, chain, it, M, u, z);
    return cudaGetLastError();
}

cudaError_t launch_gather(int form, int kind, const uint32_t *order, int64_t M, const double *table,
                          const double *scale, const double *beta, const double *u, const double *z,
                          const int32_t *group, const double *colsum, SweepRec *rec, cudaStream_t st)
{
    k_gather<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(form, kind, order, M, table, scale, beta, u, z, group,
                                                          colsum, rec);
    return cudaGetLastError();
}

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

cudaError_t launch_mu_prep(int form, int64_t N, double mu_old, double *eps, float *eps_hi, float *eps_lo,
                           double *part, int nblocks, cudaStream_t st)
{
    k_mu_prep<<<nblocks, kThreads, 0, st>>>(form, N, mu_old, eps, eps_hi, eps_lo, part);
    return cudaGetLastError();
}

cudaError_t launch_refresh(int form, int kind, int64_t N, const double *ystd, double mu, const uint8_t *codes,
                           int64_t col_stride, const double *table, const uint32_t *nz_j, const double *nz_beta,
                           int64_t n_nz, double *eps, float *eps_hi, float *eps_lo, cudaStream_t st)
{
    const int64_t nb = (N + 3) / 4;
    k_refresh<<<(unsigned)((nb + kThreads - 1) / kThreads), kThreads, 0, st>>>(
        form, kind, N, ystd, mu, codes, col_stride, table, nz_j, nz_beta, n_nz, eps, eps_hi, eps_lo);
    return cudaGetLastError();
}

cudaError_t launch_sweep_stats(int64_t M, const int32_t *group, const int32_t *comp, const uint8_t *chosen,
                               const double *beta, int n_groups, unsigned long long *out, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long) * (n_groups * kMaxK + 2 * n_groups), st);
    if (e != cudaSuccess)
        return e;
    const int blocks = (int)imin64((M + kThreads - 1) / kThreads, 152);
    k_sweep_stats<<<blocks, kThreads, 0, st>>>(M, group, comp, chosen, beta, n_groups, out);
    return cudaGetLastError();
}

size_t sweep_smem_bytes(int form, int kind, const SweepArgs &a)
{
    return make_plan(form, kind, a.slice_max, a.slot_bytes, a.B, a.n_groups).total;
}

template <int FORM, int KIND, int KM>
static cudaError_t launch_one(const SweepArgs &a, size_t smem, cudaStream_t st)
{
    cudaError_t e = cudaFuncSetAttribute(k_sweep<FORM, KIND, KM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    SweepArgs args = a;
    void *params[] = {&args};
    return cudaLaunchCooperativeKernel((const void *)k_sweep<FORM, KIND, KM>, dim3(a.G), dim3(kThreads), params, smem,
                                       st);
}

template <int KM>
static const void *sweep_fn(int form, int kind)
{
    if (form == kFormFP64)
        return kind == kKindDense ? (const void *)k_sweep<kFormFP64, kKindDense, KM>
                                  : (const void *)k_sweep<kFormFP64, kKindRagged, KM>;
    return kind == kKindDense ? (const void *)k_sweep<kFormFP32C, kKindDense, KM>
                              : (const void *)k_sweep<kFormFP32C, kKindRagged, KM>;
}

template <int KM>
static cudaError_t launch_km(int form, int kind, const SweepArgs &a, size_t smem, cudaStream_t st)
{
    if (form == kFormFP64 && kind == kKindDense)
        return launch_one<kFormFP64, kKindDense, KM>(a, smem, st);
    if (form == kFormFP32C && kind == kKindDense)
        return launch_one<kFormFP32C, kKindDense, KM>(a, smem, st);
    if (form == kFormFP64 && kind == kKindRagged)
        return launch_one<kFormFP64, kKindRagged, KM>(a, smem, st);
    return launch_one<kFormFP32C, kKindRagged, KM>(a, smem, st);
}

// Components per group up to 4 (the reference default S has three variance
// ratios) use the 4-wide sampler; larger mixtures the 16-wide one.
cudaError_t launch_sweep(int form, int kind, const SweepArgs &a, size_t smem, cudaStream_t st)
{
    return a.kmax <= 4 ? launch_km<4>(form, kind, a, smem, st) : launch_km<kMaxK>(form, kind, a, smem, st);
}

size_t sweep_block_smem_bytes(const SweepArgs &a)
{
    return make_block_plan(a.slice_max, a.slot_bytes, a.B, a.n_groups).total;
}

template <int KM, bool MISS>
static cudaError_t launch_block_km(const SweepArgs &a, size_t smem, cudaStream_t st)
{
    cudaError_t e =
        cudaFuncSetAttribute(k_sweep_block<KM, MISS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    SweepArgs args = a;
    void *params[] = {&args};
    return cudaLaunchCooperativeKernel((const void *)k_sweep_block<KM, MISS>, dim3(a.G), dim3(kThreads), params, smem,
                                       st);
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
        cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, f, kThreads, smem) != cudaSuccess)
            return 0;
        n = m < n ? m : n;
    }
    return n;
}

int sweep_max_ctas_per_sm(int form, int kind, size_t smem)
{
    int n = 0, m = 0;
    const void *f4 = sweep_fn<4>(form, kind), *f16 = sweep_fn<kMaxK>(form, kind);
    cudaFuncSetAttribute(f4, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(f16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f4, kThreads, smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, f16, kThreads, smem) != cudaSuccess)
        return 0;
    return n < m ? n : m;
}

}  // namespace brr
