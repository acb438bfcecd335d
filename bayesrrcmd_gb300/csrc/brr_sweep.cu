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
                         const double *__restrict__ z, const int32_t *__restrict__ group, SweepRec *rec)
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
            r.t[3] = 0.0;
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

__host__ __device__ inline SmemPlan make_plan(int form, int kind, int slice_max, int slot_bytes, int B, int n_groups)
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
    o += (size_t)R * sizeof(SweepRec);
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

// Team of LPM lanes inside a warp.
struct Team {
    unsigned mask;
    int lane;      // lane within the team
    int base;      // warp lane of the team's first lane
};

__device__ __forceinline__ Team make_team(int lpm)
{
    Team t;
    const int wl = threadIdx.x & 31;
    t.lane = wl % lpm;
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
__device__ __forceinline__ double team_max_d(double v, const Team &t, int lpm)
{
    for (int o = lpm >> 1; o > 0; o >>= 1)
        v = fmax(v, __shfl_xor_sync(t.mask, v, o));
    return v;
}
__device__ __forceinline__ double team_min_d(double v, const Team &t, int lpm)
{
    for (int o = lpm >> 1; o > 0; o >>= 1)
        v = fmin(v, __shfl_xor_sync(t.mask, v, o));
    return v;
}
__device__ __forceinline__ float team_sum_f(float v, const Team &t, int lpm)
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

// Component selection for one marker by a team (src/BayesRBase.cpp:309-366).
// Lane l evaluates components k = l, l+lpm, ...; lane 0 returns the result.
// logL_k = c_k + h_k*num^2 with c_k = log(pi_k) - log(sigmaG/sigmaE*(N-1)*cVa_k + 1)/2
// and h_k = 1/(2*denom_k*sigmaE); P_k = exp(logL_k - max)/sum, zeroed where the
// reference's 700 guards fire (any |logL_q - logL_k| > 700 over q >= 1).
struct Pick {
    int comp;       // chosen component, -1 if none
    double beta;    // new beta (beta_old when none)
    double acum0;   // P(component 0) as stored in acum
};

template <bool FP32>
__device__ Pick pick_component(const Team &tm, int lpm, double num, double u, double z, double beta_old,
                               const double *__restrict__ gc, int K)
{
    constexpr int kPer = kMaxK / 4;   // components per lane when lpm >= 4
    double L[kPer];
    double lmax = -INFINITY, lmax1 = -INFINITY, lmin1 = INFINITY;
    const double n2 = num * num;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int k = tm.lane + i * lpm;
        L[i] = -INFINITY;
        if (k < K) {
            const double c = gc[4 * k + 0], h = gc[4 * k + 2];
            L[i] = k == 0 ? c : fma(h, n2, c);
            lmax = fmax(lmax, L[i]);
            if (k >= 1) {
                lmax1 = fmax(lmax1, L[i]);
                lmin1 = fmin(lmin1, L[i]);
            }
        }
    }
    lmax = team_max_d(lmax, tm, lpm);
    lmax1 = team_max_d(lmax1, tm, lpm);
    lmin1 = team_min_d(lmin1, tm, lpm);

    // probabilities
    float pf[kPer];
    double pd[kPer];
    bool fallback = false;
    Pick res;
    res.comp = -1;
    res.beta = beta_old;
    res.acum0 = 0.0;
    if (FP32) {
        float e[kPer];
        float es = 0.f;
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
            const int k = tm.lane + i * lpm;
            e[i] = k < K ? expf((float)(L[i] - lmax)) : 0.f;
            es += e[i];
        }
        es = team_sum_f(es, tm, lpm);
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
            const int k = tm.lane + i * lpm;
            const bool guard = (lmax1 - L[i] > 700.0) || (L[i] - lmin1 > 700.0);
            pf[i] = (k < K && !guard) ? e[i] / es : 0.f;
        }
        // walk in FP32 on lane 0; certify the decision against the FP32 error
        int chosen = -1;
        float acum = 0.f, prev = 0.f;
        float a0 = 0.f;
        for (int k = 0; k < K; ++k) {
            const float pk = __shfl_sync(tm.mask, pf[k / lpm], tm.base + (k % lpm));
            if (k == 0)
                a0 = pk;
            prev = acum;
            acum = k == 0 ? pk : acum + pk;
            if (chosen < 0 && (double)u <= (double)acum)
                chosen = k;
            if (chosen >= 0 && k == chosen)
                break;
        }
        const float tol = 2e-5f;
        bool close;
        if (chosen >= 0)
            close = ((float)u > acum - tol) || (chosen > 0 && (float)u < prev + tol);
        else
            close = (float)u < acum + tol;
        fallback = __shfl_sync(tm.mask, close ? 1 : 0, tm.base) != 0;
        if (!fallback) {
            res.comp = chosen;
            res.acum0 = (double)a0;
        }
    }
    if (!FP32 || fallback) {
        double e[kPer];
        double es = 0.0;
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
            const int k = tm.lane + i * lpm;
            e[i] = k < K ? exp(L[i] - lmax) : 0.0;
            es += e[i];
        }
        es = team_sum_d(es, tm, lpm);
        const double ies = 1.0 / es;
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
            const int k = tm.lane + i * lpm;
            const bool guard = (lmax1 - L[i] > 700.0) || (L[i] - lmin1 > 700.0);
            pd[i] = (k < K && !guard) ? e[i] * ies : 0.0;
        }
        int chosen = -1;
        double acum = 0.0, a0 = 0.0;
        for (int k = 0; k < K; ++k) {
            const double pk = __shfl_sync(tm.mask, pd[k / lpm], tm.base + (k % lpm));
            if (k == 0)
                a0 = pk;
            acum = k == 0 ? pk : acum + pk;
            if (chosen < 0 && u <= acum)
                chosen = k;
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
template <int FORM, int KIND>
__global__ void __launch_bounds__(kThreads, 1) k_sweep(SweepArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_num[kMaxSpec];
    __shared__ double s_beta[kMaxSpec];
    __shared__ double s_acum[kMaxSpec];
    __shared__ int s_comp[kMaxSpec];
    __shared__ int s_first;
    __shared__ int s_abort;
    __shared__ double s_scal[8];          // ragged: shift, epsSum; dense FP32C: slice sum
    __shared__ double s_delta[8];         // update coefficients of the current round
    __shared__ float s_dfl[8];            // double-float split of the update coefficients
    __shared__ unsigned long long s_bsq[kMaxGroups][2];
    __shared__ int s_v[kMaxGroups * kMaxK];
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
    for (int i = tid; i < kMaxGroups * kMaxK; i += kThreads)
        s_v[i] = 0;
    if (tid < kMaxGroups) {
        s_bsq[tid][0] = 0ull;
        s_bsq[tid][1] = 0ull;
    }
    if (tid == 0) {
        s_abort = 0;
        s_scal[0] = 0.0;        // ragged shift
        s_scal[1] = a.epsSum;   // ragged running sum
        s_scal[2] = 0.0;        // dense FP32C slice sum
    }
    __syncthreads();

    // dense FP32C: slice sum of the residual (kept current across updates)
    auto slice_sum = [&]() {
        double s = 0.0;
        if (FORM != kFormFP64 && KIND == kKindDense) {
            for (int i = tid; i < ns; i += kThreads)
                s += (double)eh[i] + (double)el[i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                s += __shfl_xor_sync(0xffffffffu, s, o);
            if ((tid & 31) == 0)
                s_red[tid >> 5][0] = s;
            __syncthreads();
            if (tid == 0) {
                double t = 0.0;
                for (int q = 0; q < kThreads / 32; ++q)
                    t += s_red[q][0];
                s_scal[2] = t;
            }
            __syncthreads();
        }
    };
    slice_sum();

    // ---- prefetch machinery
    int64_t rec_issued = 0, code_issued = 0;
    auto issue_recs = [&](int64_t upto) {
        upto = imin64(upto, a.M);
        const int64_t n = upto - rec_issued;
        for (int64_t e = tid; e < n * 4; e += kThreads) {
            const int64_t q = rec_issued + e / 4;
            const int c = (int)(e % 4);
            cp_async16(reinterpret_cast<unsigned char *>(&ring_rec[q % R]) + 16 * c,
                       reinterpret_cast<const unsigned char *>(&a.rec[q]) + 16 * c);
        }
        rec_issued = imax64(rec_issued, upto);
    };
    auto issue_codes = [&](int64_t upto) {
        upto = imin64(upto, a.M);
        const int64_t n = upto - code_issued;
        if (KIND == kKindDense) {
            const int chunks = nbytes / 16;
            for (int64_t e = tid; e < n * chunks; e += kThreads) {
                const int64_t q = code_issued + e / chunks;
                const int c = (int)(e % chunks);
                const uint32_t j = ring_rec[q % R].j;
                cp_async16(ring_codes + (q % R) * a.slot_bytes + 16 * c,
                           a.codes + (int64_t)j * a.col_stride + byte_lo + 16 * c);
            }
        } else {
            // offsets of the slice's sub-lists, copied asynchronously into the ring
            for (int64_t e = tid; e < n * 6; e += kThreads) {
                const int64_t q = code_issued + e / 6;
                const int k = (int)(e % 6);
                const uint32_t j = ring_rec[q % R].j;
                const int64_t base = (int64_t)j * a.G + sidx;
                cp_async4(&ring_roff[(q % R) * 8 + k], &a.roff[k >> 1][base + (k & 1)]);
            }
        }
        code_issued = imax64(code_issued, upto);
    };

    issue_recs(3 * (int64_t)B);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    issue_codes(2 * (int64_t)B);
    cp_async_commit();

    const Team tm = make_team(lpm);
    const int team = tid / lpm;
    const double Nm1 = (double)(a.N - 1);

    int64_t start = 0;
    long long r = 0;
    while (start < a.M) {
        cp_async_wait_all();
        __syncthreads();
        issue_codes(start + 2 * (int64_t)B);
        issue_recs(start + 3 * (int64_t)B);
        cp_async_commit();
        const int nb = (int)imin64(B, a.M - start);
        if (tid == 0)
            s_first = kMaxSpec;

        // ---- partial dot products of this slice
        if (team < nb) {
            const int64_t q = start + team;
            const int slot = (int)(q % R);
            const SweepRec &rc = ring_rec[slot];
            double part = 0.0;
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
                    part = team_sum_d(p, tm, lpm);
                } else {
                    // sum g*eps exactly per product, pairwise over the four
                    // genotypes of a byte, Kahan across bytes; lo parts plain.
                    float A = 0.f, cA = 0.f, sl = 0.f, mh = 0.f, ml = 0.f;
                    for (int b = tm.lane; b < nbytes; b += lpm) {
                        const unsigned v = cb[b];
                        const float4 g = gtab[v];
                        const float4 h = reinterpret_cast<const float4 *>(eh)[b];
                        const float4 l = reinterpret_cast<const float4 *>(el)[b];
                        const float s4 = __fadd_rn(__fadd_rn(__fmul_rn(g.x, h.x), __fmul_rn(g.y, h.y)),
                                                   __fadd_rn(__fmul_rn(g.z, h.z), __fmul_rn(g.w, h.w)));
                        const float y = __fsub_rn(s4, cA);
                        const float t2 = __fadd_rn(A, y);
                        cA = __fsub_rn(__fsub_rn(t2, A), y);
                        A = t2;
                        sl = fmaf(g.x, l.x, sl);
                        sl = fmaf(g.y, l.y, sl);
                        sl = fmaf(g.z, l.z, sl);
                        sl = fmaf(g.w, l.w, sl);
                        const unsigned mm = mtab[v];
                        if (mm) {
                            if (mm & 1u) df_add(mh, ml, h.x, l.x);
                            if (mm & 2u) df_add(mh, ml, h.y, l.y);
                            if (mm & 4u) df_add(mh, ml, h.z, l.z);
                            if (mm & 8u) df_add(mh, ml, h.w, l.w);
                        }
                    }
                    float Al = __fsub_rn(sl, cA);
                    team_df_sum(A, Al, tm, lpm);
                    team_df_sum(mh, ml, tm, lpm);
                    const double Ad = (double)A + (double)Al;
                    const double Sm = (double)mh + (double)ml;
                    const double sigma = rc.t[0], cm = rc.t[1], xm = rc.t[2];
                    part = sigma * (Ad - cm * (s_scal[2] - Sm)) + xm * Sm;
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
                    part = team_sum_d(p + 2.0 * p2, tm, lpm);
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
                    part = (double)h + (double)l;
                }
            }
            if (tm.lane == 0) {
                long long ph, pl;
                if (!fixed_split(part, &ph, &pl)) {
                    atomicCAS(a.err, kDevOk, kDevRange);
                    ph = 0;
                    pl = 0;
                }
                unsigned long long *acc = a.acc + ((r % 3) * kMaxSpec + team) * 2;
                red_add_u64(acc, (unsigned long long)ph);
                red_add_u64(acc + 1, (unsigned long long)pl);
            }
        }
        __syncthreads();

        // ---- grid barrier: one counter, bounded wait
        if (tid == 0) {
            __threadfence();
            red_release_add_u64(a.counter, 1ull);
            const unsigned long long target = (unsigned long long)a.G * (unsigned long long)(r + 1);
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
            __threadfence();
        }
        __syncthreads();
        if (s_abort)
            break;

        // ---- redundant sampling of the round's markers in every CTA
        if (team < nb) {
            const int64_t q = start + team;
            const SweepRec &rc = ring_rec[q % R];
            double tot = 0.0;
            if (tm.lane == 0) {
                const unsigned long long *acc = a.acc + ((r % 3) * kMaxSpec + team) * 2;
                tot = fixed_join((long long)ld_relaxed_u64(acc), (long long)ld_relaxed_u64(acc + 1));
            }
            tot = __shfl_sync(tm.mask, tot, tm.base);
            double num;
            if (KIND == kKindDense) {
                num = tot + rc.beta_old * Nm1;
            } else {
                const double mean = rc.t[0], isd = rc.t[2], Zsum = rc.t[3];
                num = (rc.beta_old * ((double)a.N - 1.0) - mean * s_scal[1] * isd) + (tot + s_scal[0] * Zsum) * isd;
            }
            const int g = rc.group;
            const Pick pk = pick_component<FORM != kFormFP64>(tm, lpm, num, rc.u, rc.z, rc.beta_old,
                                                              gconst + (size_t)g * kMaxK * 4, gk[g]);
            if (tm.lane == 0) {
                s_num[team] = num;
                s_beta[team] = pk.beta;
                s_acum[team] = pk.acum0;
                s_comp[team] = pk.comp;
                if (rc.beta_old != 0.0 || pk.beta != 0.0)
                    atomicMin(&s_first, team);
            }
        }
        __syncthreads();

        const int first = s_first;
        const int last = first < nb ? first : nb - 1;
        if (blockIdx.x == 0) {
            // outputs and sweep statistics, only from CTA 0
            if (team <= last && tm.lane == 0) {
                const SweepRec &rc = ring_rec[(start + team) % R];
                const int c = s_comp[team];
                a.beta[rc.j] = s_beta[team];
                a.acum[rc.j] = s_acum[team];
                if (c >= 0) {
                    a.comp[rc.j] = c;
                    atomicAdd(&s_v[rc.group * kMaxK + c], 1);
                    if (c >= 1) {
                        long long ph, pl;
                        const double b = s_beta[team];
                        fixed_split(b * b, &ph, &pl);
                        atomicAdd(&s_bsq[rc.group][0], (unsigned long long)ph);
                        atomicAdd(&s_bsq[rc.group][1], (unsigned long long)pl);
                    }
                }
            }
            if (tid < 2 * kMaxSpec)
                a.acc[((r + 2) % 3) * kMaxSpec * 2 + tid] = 0ull;
        }

        // ---- apply the residual update of the first changing marker
        if (first < nb) {
            const int slot = (int)((start + first) % R);
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
                    }
                    __syncthreads();
                    for (int i = tid; i < ns; i += kThreads) {
                        const unsigned c = (cb[i >> 2] >> (2 * (i & 3))) & 3u;
                        float h = eh[i], l = el[i];
                        df_add(h, l, s_dfl[2 * c], s_dfl[2 * c + 1]);
                        eh[i] = h;
                        el[i] = l;
                    }
                    __syncthreads();
                    slice_sum();
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
        start += last + 1;
        ++r;
    }
    cp_async_wait_all();
    __syncthreads();

    // ---- epilogue: residual back to HBM, per-slice sums, sweep statistics
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
    }
    if (blockIdx.x == 0) {
        for (int i = tid; i < a.n_groups * kMaxK; i += kThreads)
            a.stats_out[i] = (double)s_v[i];
        if (tid < a.n_groups)
            a.stats_out[a.n_groups * kMaxK + tid] = fixed_join((long long)s_bsq[tid][0], (long long)s_bsq[tid][1]);
        if (tid == 0) {
            a.stats_out[a.n_groups * kMaxK + a.n_groups] = s_scal[1];
            *a.rounds_out = r;
        }
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
                          const int32_t *group, SweepRec *rec, cudaStream_t st)
{
    k_gather<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(form, kind, order, M, table, scale, beta, u, z, group, rec);
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

size_t sweep_smem_bytes(int form, int kind, const SweepArgs &a)
{
    return make_plan(form, kind, a.slice_max, a.slot_bytes, a.B, a.n_groups).total;
}

template <int FORM, int KIND>
static cudaError_t launch_one(const SweepArgs &a, size_t smem, cudaStream_t st)
{
    cudaError_t e = cudaFuncSetAttribute(k_sweep<FORM, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    SweepArgs args = a;
    void *params[] = {&args};
    return cudaLaunchCooperativeKernel((const void *)k_sweep<FORM, KIND>, dim3(a.G), dim3(kThreads), params, smem, st);
}

cudaError_t launch_sweep(int form, int kind, const SweepArgs &a, size_t smem, cudaStream_t st)
{
    if (form == kFormFP64 && kind == kKindDense)
        return launch_one<kFormFP64, kKindDense>(a, smem, st);
    if (form == kFormFP32C && kind == kKindDense)
        return launch_one<kFormFP32C, kKindDense>(a, smem, st);
    if (form == kFormFP64 && kind == kKindRagged)
        return launch_one<kFormFP64, kKindRagged>(a, smem, st);
    return launch_one<kFormFP32C, kKindRagged>(a, smem, st);
}

int sweep_max_ctas_per_sm(int form, int kind, size_t smem)
{
    int n = 0;
    const void *f = form == kFormFP64 ? (kind == kKindDense ? (const void *)k_sweep<kFormFP64, kKindDense>
                                                             : (const void *)k_sweep<kFormFP64, kKindRagged>)
                                      : (kind == kKindDense ? (const void *)k_sweep<kFormFP32C, kKindDense>
                                                            : (const void *)k_sweep<kFormFP32C, kKindRagged>);
    cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, kThreads, smem) != cudaSuccess)
        return 0;
    return n;
}

}  // namespace brr
