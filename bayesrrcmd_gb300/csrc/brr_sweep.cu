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
//
// Pair-resolved ragged rounds (FP32C, ragged markers): a round resolves all its
// B <= 32 markers.  Besides the dot products, every CTA sums over its slice the
// integer pair terms A[p][t] = sum_i g_p(i) g_t(i) and Bm[p][t] = sum over the
// individuals missing at p of g_t(i) for p < t, by population counts of the
// markers' bit masks (ones, twos, missing) over the slice; after a change at marker p the
// later markers' num move by the exact linear correction these terms give, and
// every changing marker's residual update is applied in order at the end of the
// round.
//
// The cluster variant runs the same sweep as one thread-block cluster of up to
// 16 CTAs: each CTA stores its partial sums straight into every CTA's shared
// memory (distributed shared memory, st.async completing on the receiver's
// mbarrier), so a round needs no global atomics and no grid-wide barrier.
#include "brr_device.cuh"
#include "brr_internal.h"
#include "brr_pick.cuh"
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
    size_t gcf;             // FP32C: FP32 sampler constants, n_groups x kMaxK x 2 floats
    size_t gtab;            // FP32C dense: 256 float4 + 256 bytes
    size_t xch;             // cluster: [2][cluster][B] exchange records of 32 bytes
    size_t gmap;            // pair-resolved ragged rounds: [slice_max][32] codes of the round's markers
    size_t bmask;           // pair-resolved rounds: [3][words][32] bit masks of the round's markers
    size_t pterm;           // pair-resolved rounds: [2][32][32] pair terms of the round
    size_t gdfo;            // pair-resolved rounds: n_groups x kMaxK x {sd_k, 1/den_k} double-float
    size_t total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline SmemPlan make_plan(int form, int kind, int slice_max, int slot_bytes, int B, int n_groups,
                                              int cluster = 0, bool pair_rounds = false,
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
    p.gcf = o;
    if (form != kFormFP64)
        o += align16((size_t)n_groups * kMaxK * 2 * sizeof(float));
    p.gtab = o;
    if (form != kFormFP64 && kind == kKindDense)
        o += 256 * 16 + 256;
    o = align16(o);
    p.xch = o;
    o += (size_t)2 * cluster * B * 32;
    p.gmap = o;
    if (pair_rounds && kind == kKindRagged)
        o += align16((size_t)slice_max * 32);
    p.bmask = o;
    // ragged: a word holds 32 individuals; dense: a 32-bit code word, 16
    if (pair_rounds)
        o += align16((size_t)3 * 32 * (kind == kKindRagged ? slice_max / 32 : slot_bytes / 4) * sizeof(unsigned));
    p.pterm = o;
    if (pair_rounds)
        o += 2 * 32 * 32 * sizeof(unsigned long long);
    p.gdfo = o;
    if (pair_rounds)
        o += align16((size_t)n_groups * kMaxK * 4 * sizeof(float));
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

// ---- thread-block-cluster primitives (distributed shared memory)
__device__ __forceinline__ unsigned cl_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ unsigned cl_map(unsigned addr, unsigned rank)
{
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

// 16-byte store into a CTA's shared memory that completes as 16 transaction
// bytes on that CTA's mbarrier `rbar`.
__device__ __forceinline__ void cl_push16(unsigned raddr, unsigned long long w0, unsigned long long w1, unsigned rbar)
{
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b64 [%0], {%1, %2}, [%3];" ::"r"(raddr),
                 "l"(w0), "l"(w1), "r"(rbar)
                 : "memory");
}

__device__ __forceinline__ void cl_bar_init(uint64_t *m)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(cl_addr(m)) : "memory");
}

// The receiver's own arrival of a round: one arrival plus the bytes it expects.
__device__ __forceinline__ void cl_expect(uint64_t *m, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(cl_addr(m)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool cl_test(uint64_t *m, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(cl_addr(m)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Waits for phase `parity` of m at most timeout_ns; false on timeout.
__device__ __forceinline__ bool cl_wait(uint64_t *m, unsigned parity, uint64_t timeout_ns)
{
    if (cl_test(m, parity))
        return true;
    const uint64_t t0 = global_timer_ns();
    unsigned spins = 0;
    while (!cl_test(m, parity)) {
        if ((++spins & 63u) == 0 && global_timer_ns() - t0 > timeout_ns)
            return false;
    }
    return true;
}

// All threads of all CTAs of the cluster (release / acquire at cluster scope).
// Used once after the mbarriers are initialised and once before the CTAs
// exit; every wait between the two is bounded, so every CTA reaches both.
__device__ __forceinline__ void cl_sync_all()
{
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

__device__ __forceinline__ unsigned cl_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ __int128 u128_join(unsigned long long lo, unsigned long long hi)
{
    return (__int128)(((unsigned __int128)hi << 64) | (unsigned __int128)lo);
}

// --------------------------------------------------------------------------
// The sweep of one chain over its G CTAs; sidx is this CTA's slice.  Run by
// k_sweep (one chain per launch) and k_sweep_multi (several chains of
// different sizes, each on its own group of CTAs, in one launch).  PROF: the
// variant that counts phase cycles on the first CTA (the plain variant reads no
// clock, whose reads would constrain the scheduling of every CTA's code).
// CL: the G CTAs are one thread-block cluster and exchange the round's partial
// sums through distributed shared memory (k_sweep_cl).  PR: pair-resolved
// rounds of FP32C ragged markers (k_sweep_pr).
template <int FORM, int KIND, int KM, bool PROF, bool CL = false, bool PR = false>
__device__ __forceinline__ void sweep_body(const SweepArgs &a, const int sidx)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_beta[kMaxSpec];
    __shared__ double s_acum[kMaxSpec];
    __shared__ int s_comp[kMaxSpec];
    __shared__ int s_chg[kMaxSpec];       // pair-resolved rounds: the marker changes the residual
    __shared__ float s_pdf[32][8];        // pair-resolved rounds: its residual deltas (ragged: ones, twos,
                                          // missing; dense: per 2-bit code)
    __shared__ float s_nf[32][2];         // pair-resolved rounds: the marker's final num (double-float)
    __shared__ int s_fbd[32];             // pair-resolved rounds: the decision came from the FP64 sampler
    __shared__ int s_first;
    __shared__ int s_abort;
    __shared__ double s_scal[4];          // ragged: shift, epsSum; dense FP32C: residual total
    __shared__ double s_delta[4];         // update coefficients of the current round
    __shared__ float s_dfl[8];            // double-float split of the update coefficients
    __shared__ double s_red[kThreads / 32][2];
    // a chain on one CTA exchanges nothing: its round's sums stay in shared memory
    __shared__ unsigned long long s_acc[kMaxSpec * 4];
    // cluster: the exchange's mbarrier of each round parity
    __shared__ __align__(8) uint64_t s_xbar[2];
    const bool solo = !CL && a.G == 1 && a.phantom == 0;

    const int B = a.B;
    const int lpm = kThreads / B;
    const int R = 4 * B;
    const int tid = threadIdx.x;
    if (a.t_out && sidx == 0 && tid == 0)
        a.t_out[0] = global_timer_ns();
    const int lo = a.slice_lo[sidx];
    const int ns = a.slice_lo[sidx + 1] - lo;
    const int nbytes = ((ns + kChunk - 1) / kChunk) * 16;
    const int64_t byte_lo = lo / 4;
    const SmemPlan plan = make_plan(FORM, KIND, a.slice_max, a.slot_bytes, B, a.n_groups, CL ? a.G : 0, PR);

    double *eps64 = reinterpret_cast<double *>(smem + plan.eps0);
    float *eh = reinterpret_cast<float *>(smem + plan.eps0);
    float *el = reinterpret_cast<float *>(smem + plan.eps1);
    uint8_t *ring_codes = smem + plan.ring_codes;
    SweepRec *ring_rec = reinterpret_cast<SweepRec *>(smem + plan.ring_rec);
    int32_t *ring_roff = reinterpret_cast<int32_t *>(smem + plan.ring_roff);
    double *gconst = reinterpret_cast<double *>(smem + plan.gconst);
    int32_t *gk = reinterpret_cast<int32_t *>(smem + plan.gk);
    float *gcf = reinterpret_cast<float *>(smem + plan.gcf);
    float4 *gtab = reinterpret_cast<float4 *>(smem + plan.gtab);
    uint8_t *mtab = smem + plan.gtab + 256 * 16;
    // cluster exchange records [round parity][source CTA][marker]: the partial
    // sum and the missing-genotype sum, each a 128-bit fixed-point integer
    ulonglong2 *xch = reinterpret_cast<ulonglong2 *>(smem + plan.xch);
    // pair-resolved rounds.  Ragged: per individual of the slice the codes of
    // the round's markers (0 absent, 1 or 2 listed genotype, 3 missing) and
    // their bit masks over the slice [ones | twos | missing][word][marker];
    // the round's pair terms [p][t] summed over the CTAs (A low, Bm high
    // word).  Dense: bit masks of the code words [genotype >= 1 | genotype 2
    // | missing][word][marker] at the even bit of each individual, and two
    // words of pair terms [P | MM][p][t], [Gmp | Gmt][p][t], the diagonal
    // holding each marker's genotype sum and missing count.
    const int mw = KIND == kKindRagged ? a.slice_max / 32 : a.slot_bytes / 4;
    uint8_t *gmap = smem + plan.gmap;
    unsigned *bmask = reinterpret_cast<unsigned *>(smem + plan.bmask);
    unsigned long long *s_pt = reinterpret_cast<unsigned long long *>(smem + plan.pterm);
    float4 *gdf = reinterpret_cast<float4 *>(smem + plan.gdfo);

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
    if (FORM != kFormFP64) {
        // FP32 constants of the certified sampler: logL_k - logL_0 constant and h_k
        for (int i = tid; i < a.n_groups * kMaxK; i += kThreads) {
            const int k = i % kMaxK;
            const double *row = a.gconst + (size_t)(i / kMaxK) * kMaxK * 4;
            gcf[2 * i] = k == 0 ? 0.f : __double2float_rn(row[4 * k] - row[0]);
            gcf[2 * i + 1] = k == 0 ? 0.f : __double2float_rn(row[4 * k + 2]);
        }
    }
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
        if (CL) {
            cl_bar_init(&s_xbar[0]);
            cl_bar_init(&s_xbar[1]);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
    }
    if (CL)
        cl_sync_all();   // every CTA's mbarriers exist before the first store into it
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
    const bool prof = PROF && sidx == 0 && tid == 0;
    long long ph[8] = {0, 0, 0, 0, 0, 0, 0, 0};
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
        if (solo) {
            atomicAdd(acc, (unsigned long long)f.hi);
            atomicAdd(acc + 1, f.lo);
        } else {
            red_add_u64(acc, (unsigned long long)f.hi);
            red_add_u64(acc + 1, f.lo);
        }
    };
    for (int i = tid; i < kMaxSpec * 4; i += kThreads)
        s_acc[i] = 0ull;
    if (PR) {
        if (KIND == kKindRagged)
            for (int i = tid; i < a.slice_max * 2; i += kThreads)
                reinterpret_cast<uint4 *>(gmap)[i] = make_uint4(0u, 0u, 0u, 0u);
        // beta = z sd_k + num / den_k of a non-zero component in double-float
        for (int i = tid; i < a.n_groups * kMaxK; i += kThreads) {
            const int k = i % kMaxK;
            const double *row = a.gconst + (size_t)(i / kMaxK) * kMaxK * 4;
            float4 v;
            df_from_double(row[4 * k + 3], v.x, v.y);
            df_from_double(row[4 * k + 1], v.z, v.w);
            gdf[i] = v;
        }
    }

    unsigned start = 0;
    long long r = 0;
    int rb = 0;   // r % 3
    // cluster: the team's lanes store marker t's two sums (those of the team's
    // first lane) into CTAs lane, lane + lpm, ... of the cluster; the copy for
    // this CTA is a plain shared-memory store, made visible by the CTA barrier
    // after the round's wait
    auto push = [&](int t, __int128 x, __int128 xm) {
        unsigned long long w[4] = {(unsigned long long)x, (unsigned long long)(x >> 64), (unsigned long long)xm,
                                   (unsigned long long)(xm >> 64)};
#pragma unroll
        for (int k = 0; k < 4; ++k)
            w[k] = __shfl_sync(tm.mask, w[k], tm.base);
        ulonglong2 *rec2 = xch + ((size_t)((r & 1) * a.G + sidx) * B + t) * 2;
        const unsigned off = cl_addr(rec2);
        const unsigned bar = cl_addr(&s_xbar[r & 1]);
        for (int d = tm.lane; d < a.G; d += lpm) {
            if (d == sidx) {
                rec2[0] = make_ulonglong2(w[0], w[1]);
                rec2[1] = make_ulonglong2(w[2], w[3]);
            } else {
                const unsigned ra = cl_map(off, (unsigned)d);
                const unsigned rbar = cl_map(bar, (unsigned)d);
                cl_push16(ra, w[0], w[1], rbar);
                cl_push16(ra + 16, w[2], w[3], rbar);
            }
        }
    };
    while (start < M32) {
        cp_async_wait_all();
        __syncthreads();
        issue_codes(start + 2u * B);
        issue_recs(start + 3u * B);
        cp_async_commit();
        // a synchronous round resolves up to B markers and ends at the first
        // that changes the residual; an asynchronous batch takes T markers
        // that all read the same residual, and applies every change
        const int nb = (int)min((unsigned)(a.async_batch > 0 ? a.async_batch : B), M32 - start);
        if (tid == 0)
            s_first = kMaxSpec;
        mark(0);

        // ---- partial dot products of this slice, published as exact fixed point
        if (team < nb) {
            const unsigned slot = (start + team) & Rm;
            const SweepRec &rc = ring_rec[slot];
            unsigned long long *acc = solo ? s_acc + team * 4 : a.acc + (rb * kMaxSpec + team) * 4;
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
                    __int128 x = 0;
                    if (tm.lane == 0) {
                        ok = fx_from_double(p, x);
                        if (!ok)
                            x = 0;
                        else if (!CL)
                            publish(acc, x);
                    }
                    if (CL)
                        push(team, x, 0);
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
                    __int128 xs = 0, xms = 0;
                    if (tm.lane == 0) {
                        __int128 x1, x2, m1, m2;
                        ok = fx_from_float(Ah, x1) && fx_from_float(Al, x2) && fx_from_float(mh, m1) &&
                             fx_from_float(ml, m2);
                        if (ok) {
                            xs = x1 + x2;
                            xms = m1 + m2;
                            if (!CL) {
                                publish(acc, xs);
                                if (mh != 0.f || ml != 0.f)
                                    publish(acc + 2, xms);
                            }
                        }
                    }
                    if (CL)
                        push(team, xs, xms);
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
                    // Eigen markers: the residual over missing genotypes, weighted
                    // by the marker mean when the round is resolved
                    double pm = 0.0;
                    if (a.eigen) {
                        for (int e = ro[4] + tm.lane; e < ro[5]; e += lpm)
                            pm += eps64[a.ridx[2][e]];
                        pm = team_sum_d(pm, tm, lpm);
                    }
                    __int128 xs = 0, xms = 0;
                    if (tm.lane == 0) {
                        __int128 x, xm;
                        ok = fx_from_double(p, x) && fx_from_double(pm, xm);
                        if (ok) {
                            xs = x;
                            xms = xm;
                            if (!CL) {
                                publish(acc, x);
                                if (pm != 0.0)
                                    publish(acc + 2, xm);
                            }
                        }
                    }
                    if (CL)
                        push(team, xs, xms);
                } else {
                    float h = 0.f, l = 0.f;
                    for (int e = ro[0] + tm.lane; e < ro[1]; e += lpm) {
                        const int i = a.ridx[0][e];
                        df_add(h, l, eh[i], el[i]);
                        if (PR)
                            gmap[i * 32 + team] = 1;
                    }
                    for (int e = ro[2] + tm.lane; e < ro[3]; e += lpm) {
                        const int i = a.ridx[1][e];
                        df_add(h, l, 2.f * eh[i], 2.f * el[i]);
                        if (PR)
                            gmap[i * 32 + team] = 2;
                    }
                    if (PR)
                        for (int e = ro[4] + tm.lane; e < ro[5]; e += lpm)
                            gmap[a.ridx[2][e] * 32 + team] = 3;
                    team_df_sum(h, l, tm, lpm);
                    float mh = 0.f, ml = 0.f;
                    if (a.eigen) {
                        for (int e = ro[4] + tm.lane; e < ro[5]; e += lpm) {
                            const int i = a.ridx[2][e];
                            df_add(mh, ml, eh[i], el[i]);
                        }
                        team_df_sum(mh, ml, tm, lpm);
                    }
                    __int128 xs = 0, xms = 0;
                    if (tm.lane == 0) {
                        __int128 x1, x2, m1, m2;
                        ok = fx_from_float(h, x1) && fx_from_float(l, x2) && fx_from_float(mh, m1) &&
                             fx_from_float(ml, m2);
                        if (ok) {
                            xs = x1 + x2;
                            xms = m1 + m2;
                            if (!CL) {
                                publish(acc, xs);
                                if (mh != 0.f || ml != 0.f)
                                    publish(acc + 2, xms);
                            }
                        }
                    }
                    if (CL)
                        push(team, xs, xms);
                }
            }
            if (!ok)
                atomicCAS(a.err, kDevOk, kDevRange);
        }
        __syncthreads();
        if (PR && KIND == kKindDense) {
            mark(6);
            // bit masks of the round's markers from their code words (16
            // individuals each, code 0: genotype 2, 1: missing, 2: genotype 1,
            // 3: genotype 0; individuals past the slice masked), one thread per
            // (word, marker)
            const int nwd = (ns + 15) / 16;
            for (int e = tid; e < nwd * 32; e += kThreads) {
                const int w = e >> 5, t = e & 31;
                unsigned h = 0u, d = 0u, m = 0u;
                if (t < nb) {
                    const unsigned cw =
                        reinterpret_cast<const unsigned *>(ring_codes + ((start + t) & Rm) * a.slot_bytes)[w];
                    const int nv = ns - 16 * w;
                    const unsigned vm = nv >= 16 ? 0x55555555u : (0x55555555u & ((1u << (2 * nv)) - 1u));
                    h = ~cw & vm;
                    d = ~cw & ~(cw >> 1) & vm;
                    m = cw & ~(cw >> 1) & vm;
                }
                bmask[w * 32 + t] = h;
                bmask[(mw + w) * 32 + t] = d;
                bmask[(2 * mw + w) * 32 + t] = m;
            }
            __syncthreads();
            // pair terms p <= t, a pair per thread: P = sum g_p g_t, MM =
            // individuals missing at both, Gmp = sum of g_t over the
            // individuals missing at p, Gmt = sum of g_p over those missing at
            // t; on the diagonal the marker's genotype sum and missing count
            // (g = [genotype >= 1] + [genotype 2])
            unsigned long long *gp = a.pairs + (size_t)rb * 2048;
            for (int e = tid; e < 1024; e += kThreads) {
                const int p = e >> 5, t = e & 31;
                if (p > t || t >= nb)
                    continue;
                unsigned w0a = 0u, w0b = 0u, w1a = 0u, w1b = 0u;
                for (int w = 0; w < nwd; ++w) {
                    const unsigned *hh = bmask + w * 32, *dd = bmask + (mw + w) * 32, *mm = bmask + (2 * mw + w) * 32;
                    const unsigned hp = hh[p], dp = dd[p], mp = mm[p];
                    if (p == t) {
                        w0a += __popc(hp) + __popc(dp);
                        w0b += __popc(mp);
                    } else {
                        const unsigned ht = hh[t], dt = dd[t], mt = mm[t];
                        w0a += __popc(hp & ht) + __popc(hp & dt) + __popc(dp & ht) + __popc(dp & dt);
                        if (a.has_missing) {
                            w0b += __popc(mp & mt);
                            w1a += __popc(mp & ht) + __popc(mp & dt);
                            w1b += __popc(mt & hp) + __popc(mt & dp);
                        }
                    }
                }
                const unsigned long long v0 = (unsigned long long)w0a | ((unsigned long long)w0b << 32);
                const unsigned long long v1 = (unsigned long long)w1a | ((unsigned long long)w1b << 32);
                if (v0)
                    red_add_u64(gp + e, v0);
                if (v1)
                    red_add_u64(gp + 1024 + e, v1);
            }
            __syncthreads();
            mark(7);
        } else if (PR) {
            mark(6);
            // bit masks of the round's markers over the slice, one thread per
            // (word, marker): 32 consecutive individuals' codes of the marker
            const int nwd = (ns + 31) / 32;
            for (int e = tid; e < nwd * 32; e += kThreads) {
                const int w = e >> 5, t = e & 31;
                unsigned m1 = 0u, m2 = 0u, mm = 0u;
                if (t < nb) {
                    const int nj = min(32, ns - 32 * w);
                    const uint8_t *col = gmap + (size_t)32 * w * 32 + t;
                    for (int j = 0; j < nj; ++j) {
                        const unsigned c = col[j * 32];
                        m1 |= (c == 1u ? 1u : 0u) << j;
                        m2 |= (c == 2u ? 1u : 0u) << j;
                        mm |= (c == 3u ? 1u : 0u) << j;
                    }
                }
                bmask[w * 32 + t] = m1;
                bmask[(mw + w) * 32 + t] = m2;
                bmask[(2 * mw + w) * 32 + t] = mm;
            }
            __syncthreads();
            // pair terms p < t of the round's markers over the slice, a pair
            // per thread: A[p][t] = sum g_p g_t over individuals listed in
            // both, Bm[p][t] = sum of g_t over the individuals missing at p;
            // published as exact integers (ordered before the barrier's
            // release by the CTA barrier below)
            unsigned long long *gp = a.pairs + (size_t)rb * 2048;
            for (int e = tid; e < 1024; e += kThreads) {
                const int p = e >> 5, t = e & 31;
                if (p >= t || t >= nb)
                    continue;
                unsigned A = 0, Bm = 0;
                for (int w = 0; w < nwd; ++w) {
                    const unsigned *m1 = bmask + w * 32, *m2 = bmask + (mw + w) * 32, *mm = bmask + (2 * mw + w) * 32;
                    const unsigned a1 = m1[p], a2 = m2[p], am = mm[p], b1 = m1[t], b2 = m2[t];
                    A += __popc(a1 & b1) + 2u * (__popc(a1 & b2) + __popc(a2 & b1)) + 4u * __popc(a2 & b2);
                    Bm += __popc(am & b1) + 2u * __popc(am & b2);
                }
                const unsigned long long v = (unsigned long long)A | ((unsigned long long)Bm << 32);
                if (v)
                    red_add_u64(gp + e, v);
            }
            __syncthreads();
            mark(7);
        }
        mark(1);

        // ---- grid barrier: one counter; release orders this CTA's
        // accumulator updates (ordered before it by bar.sync), acquire orders
        // the reads below.  The wait is bounded.  Cluster: the round's
        // mbarrier completes when the other CTAs' records of the nb markers
        // have landed in this CTA's shared memory (phantom records never arrive).
        if (CL) {
            if (tid == 0) {
                cl_expect(&s_xbar[r & 1], (unsigned)(((a.G - 1) * nb + a.phantom) * 32));
                if (!cl_wait(&s_xbar[r & 1], (unsigned)(r >> 1) & 1u, a.timeout_ns)) {
                    atomicCAS(a.err, kDevOk, kDevTimeout);
                    s_abort = 1;
                }
            }
        } else if (tid == 0 && !solo) {
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

        if (PR) {
            // ---- pair-resolved round, identically in every CTA: lane t
            // samples marker t; after the first change p the later markers'
            // num move by dBeta_p isd_p isd_t (A[p][t] + mean_p Bm[p][t]
            // - mean_t (Zsum_p - mean_p N) - mean_p Zsum_t), the change of
            // x_t . eps that p's residual update, running sum and pending
            // shift make (src/raggedbayesrkernel.cpp:10-35), and they are
            // sampled again
            const unsigned long long *gp = a.pairs + (size_t)rb * 2048;
            for (int e = tid; e < (KIND == kKindDense ? 2048 : 1024); e += kThreads)
                s_pt[e] = ld_relaxed_u64(gp + e);
            __syncthreads();
            if (tid < 32) {
                const int t = tid;
                const bool valid = t < nb;
                const SweepRec &rc = ring_rec[(start + (valid ? t : 0)) & Rm];
                // ragged: mean, 1/sd, sum of listed genotypes; dense: sigma,
                // column mean, value of a missing genotype, sum of the column
                const double mean = rc.t[0], isd = rc.t[2], Zsum = rc.t[3];
                double num0 = 0.0;
                if (valid) {
                    const unsigned long long *acc = solo ? s_acc + t * 4 : a.acc + (rb * kMaxSpec + t) * 4;
                    auto ldw = [&](int k) -> unsigned long long { return solo ? acc[k] : ld_relaxed_u64(acc + k); };
                    const double tot = fx_join((long long)ldw(0), ldw(1));
                    if (KIND == kKindDense) {
                        const double sm = fx_join((long long)ldw(2), ldw(3));
                        num0 = (rc.t[0] * (tot - rc.t[1] * (s_scal[2] - sm)) + rc.t[2] * sm) +
                               rc.beta_old * ((double)a.N - 1.0);
                    } else {
                        num0 = (rc.beta_old * ((double)a.N - 1.0) - mean * s_scal[1] * isd) + (tot + s_scal[0] * Zsum) * isd;
                    }
                }
                // num, the marker constants and the corrections in double-float
                float nh, nl, mh, ml, ih, il;
                df_from_double(num0, nh, nl);
                df_from_double(mean, mh, ml);     // dense: sigma
                df_from_double(isd, ih, il);      // dense: value of a missing genotype
                const float Zf = (float)Zsum, Nf = (float)a.N;
                // dense: column mean, sum of the column, sigma * colmean and
                // sigma * colmean + the missing value, the marker's genotype sum
                // and missing count (the diagonal of the pair terms)
                float cmh = 0.f, cml = 0.f, csh = 0.f, csl = 0.f, sch = 0.f, scl = 0.f, sxh = 0.f, sxl = 0.f;
                float Sg = 0.f, Nm = 0.f;
                if (KIND == kKindDense) {
                    df_from_double(rc.t[1], cmh, cml);
                    df_from_double(rc.t[3], csh, csl);
                    df_mul(mh, ml, cmh, cml, sch, scl);
                    sxh = sch;
                    sxl = scl;
                    df_add(sxh, sxl, ih, il);
                    const unsigned long long dg = s_pt[t * 32 + t];
                    Sg = (float)(unsigned)dg;
                    Nm = (float)(unsigned)(dg >> 32);
                }
                const int g = valid ? rc.group : 0;
                const double *gcg = gconst + (size_t)g * kMaxK * 4;
                const float *gcfg = gcf + (size_t)g * kMaxK * 2;
                const int K = gk[g];
                const float uf = __double2float_rn(rc.u);
                // certified decisions with a stability margin in num^2: a marker
                // is sampled again only when a correction moves num^2 beyond
                // its margin (H: the spread of the group's h_k, h_0 = 0
                // included); decisions the margin sampler cannot certify are
                // taken by the guarded FP32 sampler, else in FP64
                float H = 0.f;
                {
                    float hmax = 0.f, hmin = 0.f;
                    for (int k = 1; k < K; ++k) {
                        hmax = fmaxf(hmax, gcfg[2 * k + 1]);
                        hmin = fminf(hmin, gcfg[2 * k + 1]);
                    }
                    H = (hmax - hmin) * 1.000001f;
                }
                bool done = !valid;
                int comp = -1;
                float sref = 0.f, wmar = -1.f;
                bool fbd = false;
                double fb_beta = rc.beta_old, fb_acum = 0.0;
                float boh, bol, zh, zl;
                df_from_double(rc.beta_old, boh, bol);
                df_from_double(rc.z, zh, zl);
                const float4 *gdfg = gdf + (size_t)g * kMaxK;
                for (;;) {
                    const float sx = __fmaf_rn(nh, nh, 2.f * nh * nl);
                    const float delta = fabsf(sx - sref) * 1.000001f + 4e-7f * (sx + sref);
                    if (!done && !(H * delta <= wmar)) {
                        int cm;
                        float w;
                        fbd = false;
                        if (pick_margin<KM>(sx, uf, gcfg, K, cm, w)) {
                            comp = cm;
                            sref = sx;
                            wmar = w;
                        } else {
                            float a0;
                            wmar = -1.f;
                            if (!pick_f32<KM>(nh, nl, uf, gcfg, K, comp, a0)) {
                                const Pick pk = pick_marker<true, KM>((double)nh + (double)nl, rc.u, rc.z, rc.beta_old,
                                                                      gcg, K);
                                comp = pk.comp;
                                fb_beta = pk.beta;
                                fb_acum = pk.acum0;
                                fbd = true;
                            }
                        }
                    }
                    const bool chg = !done && (rc.beta_old != 0.0 || comp > 0);
                    const unsigned mask = __ballot_sync(0xffffffffu, chg);
                    const int p = mask ? __ffs(mask) - 1 : 32;
                    float ch = 0.f, cl = 0.f;
                    if (!done && t <= p) {
                        // the decision of marker t is final (src/BayesRBase.cpp:346-366);
                        // beta, acum and the residual deltas follow after the round
                        s_nf[t][0] = nh;
                        s_nf[t][1] = nl;
                        s_comp[t] = comp;
                        s_fbd[t] = fbd ? 1 : 0;
                        s_chg[t] = t == p ? 1 : 0;
                        if (fbd) {
                            s_beta[t] = fb_beta;
                            s_acum[t] = fb_acum;
                        }
                        if (t == p) {
                            // dBeta isd of the change in double-float
                            float bh = boh, bl = bol;
                            if (fbd) {
                                df_from_double(fb_beta, bh, bl);
                            } else if (comp == 0) {
                                bh = bl = 0.f;
                            } else if (comp > 0) {
                                const float4 k4 = gdfg[comp];
                                float ah, al, xh, xl;
                                df_mul(zh, zl, k4.x, k4.y, ah, al);
                                df_mul(nh, nl, k4.z, k4.w, xh, xl);
                                df_add(ah, al, xh, xl);
                                bh = ah;
                                bl = al;
                            }
                            float dh = boh, dl = bol;
                            df_add(dh, dl, -bh, -bl);
                            if (KIND == kKindDense) {
                                ch = dh;
                                cl = dl;
                            } else {
                                df_mul(dh, dl, ih, il, ch, cl);
                            }
                        }
                        done = true;
                    }
                    if (!mask)
                        break;
                    if (KIND == kKindDense) {
                        // x_p . x_t moves num_t by dBeta_p (sigma_t dT - sigma_t cm_t dE
                        // + (sigma_t cm_t + xm_t) dSm): dT the change of the sum of
                        // g_t eps over t's genotypes, dE of the residual total, dSm of
                        // the residual over t's missing genotypes
                        ch = __shfl_sync(0xffffffffu, ch, p);
                        cl = __shfl_sync(0xffffffffu, cl, p);
                        const float sph = __shfl_sync(0xffffffffu, mh, p), spl = __shfl_sync(0xffffffffu, ml, p);
                        const float cph = __shfl_sync(0xffffffffu, cmh, p), cpl = __shfl_sync(0xffffffffu, cml, p);
                        const float xph = __shfl_sync(0xffffffffu, ih, p), xpl = __shfl_sync(0xffffffffu, il, p);
                        const float eph = __shfl_sync(0xffffffffu, csh, p), epl = __shfl_sync(0xffffffffu, csl, p);
                        if (!done) {
                            const unsigned long long v0 = s_pt[p * 32 + t], v1 = s_pt[1024 + p * 32 + t];
                            const float P = (float)(unsigned)v0, MM = (float)(unsigned)(v0 >> 32);
                            const float Gmp = (float)(unsigned)v1, Gmt = (float)(unsigned)(v1 >> 32);
                            // dT = sigma_p (P - cm_p (S_t - Gmp)) + xm_p Gmp
                            float th, tl, uh, ul;
                            df_mul(cph, cpl, Sg - Gmp, 0.f, th, tl);
                            th = -th;
                            tl = -tl;
                            df_add(th, tl, P, 0.f);
                            df_mul(sph, spl, th, tl, uh, ul);
                            df_mul(xph, xpl, Gmp, 0.f, th, tl);
                            df_add(uh, ul, th, tl);
                            // sigma_t dT - sigma_t cm_t dE
                            float rh, rl, qh, ql;
                            df_mul(mh, ml, uh, ul, rh, rl);
                            df_mul(sch, scl, eph, epl, qh, ql);
                            df_add(rh, rl, -qh, -ql);
                            if (a.has_missing) {
                                // dSm = sigma_p (Gmt - cm_p (nmiss_t - MM)) + xm_p MM
                                df_mul(cph, cpl, Nm - MM, 0.f, th, tl);
                                th = -th;
                                tl = -tl;
                                df_add(th, tl, Gmt, 0.f);
                                df_mul(sph, spl, th, tl, uh, ul);
                                df_mul(xph, xpl, MM, 0.f, th, tl);
                                df_add(uh, ul, th, tl);
                                df_mul(sxh, sxl, uh, ul, qh, ql);
                                df_add(rh, rl, qh, ql);
                            }
                            float xh2, xl2;
                            df_mul(ch, cl, rh, rl, xh2, xl2);
                            df_add(nh, nl, xh2, xl2);
                        }
                        continue;
                    }
                    // num_t += dBeta_p isd_p isd_t (A + mean_p Bm - mean_t (Zsum_p
                    // - mean_p N) - mean_p Zsum_t)
                    ch = __shfl_sync(0xffffffffu, ch, p);
                    cl = __shfl_sync(0xffffffffu, cl, p);
                    const float mph = __shfl_sync(0xffffffffu, mh, p), mpl = __shfl_sync(0xffffffffu, ml, p);
                    const float Zp = __shfl_sync(0xffffffffu, Zf, p);
                    if (!done) {
                        const unsigned long long v = s_pt[p * 32 + t];
                        const float A = (float)(unsigned)v, Bm = (float)(unsigned)(v >> 32);
                        float t1h, t1l, t2h, t2l, t3h, t3l, t4h, t4l;
                        df_mul(mph, mpl, Bm, 0.f, t1h, t1l);
                        df_add(t1h, t1l, A, 0.f);
                        df_mul(mph, mpl, Nf, 0.f, t2h, t2l);
                        t2h = -t2h;
                        t2l = -t2l;
                        df_add(t2h, t2l, Zp, 0.f);
                        df_mul(mh, ml, t2h, t2l, t3h, t3l);
                        df_mul(mph, mpl, Zf, 0.f, t4h, t4l);
                        df_add(t1h, t1l, -t3h, -t3l);
                        df_add(t1h, t1l, -t4h, -t4l);
                        float kh, kl, xh, xl;
                        df_mul(ch, cl, ih, il, kh, kl);
                        df_mul(kh, kl, t1h, t1l, xh, xl);
                        df_add(nh, nl, xh, xl);
                    }
                }
            }
            __syncthreads();
            // beta and acum of every marker at its final num, and the residual
            // deltas (ones, twos, missing genotypes) of every change, as the
            // pass per marker forms them
            if (tid < nb) {
                const SweepRec &rc = ring_rec[(start + tid) & Rm];
                if (!s_fbd[tid]) {
                    const int g = rc.group;
                    const double *gcg = gconst + (size_t)g * kMaxK * 4;
                    const int comp = s_comp[tid];
                    const float nh = s_nf[tid][0], nl = s_nf[tid][1];
                    double bnew = comp == 0 ? 0.0 : rc.beta_old;
                    if (comp > 0)
                        bnew = __dadd_rn(__dmul_rn(rc.z, gcg[4 * comp + 3]),
                                         __dmul_rn((double)nh + (double)nl, gcg[4 * comp + 1]));
                    int c2;
                    float a0;
                    pick_f32<KM>(nh, nl, __double2float_rn(rc.u), gcf + (size_t)g * kMaxK * 2, gk[g], c2, a0);
                    s_beta[tid] = bnew;
                    s_acum[tid] = (double)a0;
                }
            }
            if (tid < nb && s_chg[tid]) {
                const SweepRec &rc = ring_rec[(start + tid) & Rm];
                const double dBeta = rc.beta_old - s_beta[tid];
                if (KIND == kKindDense) {
                    // delta per 2-bit code: dBeta (g - colmean) sigma, a missing genotype dBeta xm
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const double gv = c == 0 ? 2.0 : (c == 2 ? 1.0 : 0.0);
                        const double d = c == 1 ? dBeta * rc.t[2] : dBeta * ((gv - rc.t[1]) * rc.t[0]);
                        df_from_double(d, s_pdf[tid][2 * c], s_pdf[tid][2 * c + 1]);
                    }
                } else {
                    const double oneAdj = dBeta * rc.t[2];
                    const double dk[3] = {oneAdj, 2.0 * oneAdj, dBeta * rc.t[0] * rc.t[2]};
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        df_from_double(dk[k], s_pdf[tid][2 * k], s_pdf[tid][2 * k + 1]);
                }
            }
            __syncthreads();
        } else if (tid < nb) {
            // ---- redundant sampling of the round's markers in every CTA, one thread per marker
            const SweepRec &rc = ring_rec[(start + tid) & Rm];
            const unsigned long long *acc = solo ? s_acc + tid * 4 : a.acc + (rb * kMaxSpec + tid) * 4;
            unsigned long long cw[4] = {0ull, 0ull, 0ull, 0ull};
            if (CL) {
                // the exact sums over the cluster's CTAs, in the accumulator format
                __int128 t0 = 0, t1 = 0;
                const ulonglong2 *xr = xch + ((size_t)(r & 1) * a.G * B + tid) * 2;
                for (int s = 0; s < a.G; ++s) {
                    const ulonglong2 w0 = xr[(size_t)s * B * 2], w1 = xr[(size_t)s * B * 2 + 1];
                    t0 += u128_join(w0.x, w0.y);
                    t1 += u128_join(w1.x, w1.y);
                }
                const Fx f0 = fx_split(t0), f1 = fx_split(t1);
                cw[0] = (unsigned long long)f0.hi;
                cw[1] = f0.lo;
                cw[2] = (unsigned long long)f1.hi;
                cw[3] = f1.lo;
            }
            auto ldacc = [&](int k) -> unsigned long long {
                return CL ? cw[k] : (solo ? acc[k] : ld_relaxed_u64(acc + k));
            };
            const double tot = fx_join((long long)ldacc(0), ldacc(1));
            double num;
            if (KIND == kKindDense) {
                if (FORM == kFormFP64) {
                    num = tot + rc.beta_old * Nm1;
                } else {
                    const double sm = fx_join((long long)ldacc(2), ldacc(3));
                    const double sigma = rc.t[0], cm = rc.t[1], xm = rc.t[2];
                    num = (sigma * (tot - cm * (s_scal[2] - sm)) + xm * sm) + rc.beta_old * Nm1;
                }
            } else {
                const double mean = rc.t[0], isd = rc.t[2], Zsum = rc.t[3];
                // Eigen markers (src/eigenbayesrkernel.cpp:17-20): Zg holds the
                // mean at missing genotypes, so their residual sum enters times
                // the mean; Zsum includes the imputed values, which carries the
                // pending uniform shift over the missing genotypes too
                const double t12 =
                    a.eigen ? tot + mean * fx_join((long long)ldacc(2), ldacc(3)) : tot;
                num = (rc.beta_old * ((double)a.N - 1.0) - mean * s_scal[1] * isd) + (t12 + s_scal[0] * Zsum) * isd;
            }
            const int g = rc.group;
            const double *gcg = gconst + (size_t)g * kMaxK * 4;
            Pick pk;
            if (FORM == kFormFP64) {
                pk = pick_marker<false, KM>(num, rc.u, rc.z, rc.beta_old, gcg, gk[g]);
            } else {
                // certified FP32 decision; FP64 where the bound cannot certify it
                float xh, xl, a0;
                int comp;
                df_from_double(num, xh, xl);
                if (pick_f32<KM>(xh, xl, __double2float_rn(rc.u), gcf + (size_t)g * kMaxK * 2, gk[g], comp, a0)) {
                    pk.comp = comp;
                    pk.acum0 = (double)a0;
                    pk.beta = comp == 0 ? 0.0 : rc.beta_old;
                    if (comp > 0)
                        pk.beta = __dadd_rn(__dmul_rn(rc.z, gcg[4 * comp + 3]), __dmul_rn(num, gcg[4 * comp + 1]));
                } else {
                    pk = pick_marker<true, KM>(num, rc.u, rc.z, rc.beta_old, gcg, gk[g]);
                }
            }
            s_beta[tid] = pk.beta;
            s_acum[tid] = pk.acum0;
            s_comp[tid] = pk.comp;
            if (rc.beta_old != 0.0 || pk.beta != 0.0)
                atomicMin(&s_first, tid);
        }
        __syncthreads();
        mark(3);

        const int first = (a.async_batch > 0 || PR) ? nb : s_first;
        const int last = first < nb ? first : nb - 1;
        if (sidx == 0) {
            // outputs of the resolved markers, only from CTA 0
            if (tid <= last) {
                const SweepRec &rc = ring_rec[(start + tid) & Rm];
                const int c = s_comp[tid];
                a.beta[rc.j] = s_beta[tid];
                if (a.async_batch == 0)   // processColumnAsync leaves acum as it was
                    a.acum[rc.j] = s_acum[tid];
                a.chosen[rc.j] = c >= 0 ? 1 : 0;
                if (c >= 0)
                    a.comp[rc.j] = c;
            }
            // all CTAs have read the accumulators of round r-1: recycle them
            if (!CL && tid < 4 * kMaxSpec)
                a.acc[((rb + 2) % 3) * kMaxSpec * 4 + tid] = 0ull;
            if (PR)
                for (int e = tid; e < 2048; e += kThreads)
                    a.pairs[(size_t)((rb + 2) % 3) * 2048 + e] = 0ull;
        }
        if (solo)   // the sampling has read this round's sums (barrier above)
            for (int i = tid; i < kMaxSpec * 4; i += kThreads)
                s_acc[i] = 0ull;

        // ---- apply the residual update of marker u of the round (the first
        // changing marker of a synchronous round; every changing marker of an
        // asynchronous batch, in order).  The decision of whether to apply is
        // the same in every thread (shared memory), so the barriers inside are
        // reached by all.
        auto apply_one = [&](const int u) {
            const unsigned slot = (start + u) & Rm;
            const SweepRec &rc = ring_rec[slot];
            const double dBeta = rc.beta_old - s_beta[u];
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
        };
        if (PR) {
            // every changing marker's residual update, in sweep order, by the
            // owner of each individual from the round's bit masks (the same
            // operations as a pass per marker, with the deltas the resolve
            // formed); the pending shift and the running sum in order by one
            // thread, one without individuals when there is one
            unsigned chm = 0u;
            for (int u = 0; u < nb; ++u)
                chm |= s_chg[u] ? 1u << u : 0u;
            if (tid == (ns < kThreads ? kThreads - 1 : 0)) {
                for (unsigned m = chm; m; m &= m - 1u) {
                    const int u = __ffs(m) - 1;
                    const SweepRec &rc = ring_rec[(start + u) & Rm];
                    const double dBeta = rc.beta_old - s_beta[u];
                    if (KIND == kKindDense) {
                        // the residual total moves by dBeta times the column sum
                        s_scal[2] = s_scal[2] + dBeta * rc.t[3];
                    } else {
                        const double mean = rc.t[0], isd = rc.t[2], Zsum = rc.t[3];
                        s_scal[0] = s_scal[0] - dBeta * mean * isd;
                        s_scal[1] = s_scal[1] + ((dBeta * Zsum) * isd - ((dBeta * mean) * (double)a.N) * isd);
                    }
                }
            }
            if (chm && KIND == kKindDense) {
                // every individual of the slice moves with every change: the
                // delta of its code, marker by marker in sweep order
                for (int i = tid; i < ns; i += kThreads) {
                    float h = eh[i], l = el[i];
                    for (unsigned m = chm; m; m &= m - 1u) {
                        const int u = __ffs(m) - 1;
                        const unsigned c = (ring_codes[((start + u) & Rm) * a.slot_bytes + (i >> 2)] >> (2 * (i & 3))) & 3u;
                        df_add(h, l, s_pdf[u][2 * c], s_pdf[u][2 * c + 1]);
                    }
                    eh[i] = h;
                    el[i] = l;
                }
            } else if (chm) {
                for (int i = tid; i < ns; i += kThreads) {
                    const int w = i >> 5;
                    const unsigned bit = 1u << (i & 31);
                    float h = eh[i], l = el[i];
                    bool any = false;
                    for (unsigned m = chm; m; m &= m - 1u) {
                        const int u = __ffs(m) - 1;
                        const int k = (bmask[w * 32 + u] & bit) ? 0
                                      : (bmask[(mw + w) * 32 + u] & bit) ? 1
                                      : (bmask[(2 * mw + w) * 32 + u] & bit) ? 2 : -1;
                        if (k >= 0) {
                            df_add(h, l, s_pdf[u][2 * k], s_pdf[u][2 * k + 1]);
                            any = true;
                        }
                    }
                    if (any) {
                        eh[i] = h;
                        el[i] = l;
                    }
                }
            }
            __syncthreads();
            // the next round's codes start from zero
            if (KIND == kKindRagged)
                for (int i = tid; i < ns * 2; i += kThreads)
                    reinterpret_cast<uint4 *>(gmap)[i] = make_uint4(0u, 0u, 0u, 0u);
        } else if (a.async_batch > 0) {
            for (int u = 0; u < nb; ++u) {
                if (ring_rec[(start + u) & Rm].beta_old != 0.0 || s_beta[u] != 0.0) {
                    apply_one(u);
                    __syncthreads();
                }
            }
        } else if (first < nb) {
            apply_one(first);
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
        a.prof[6] = ph[6];   // pair-resolved rounds: the dot products (phase 1 is then the publication)
        a.prof[7] = ph[7];   // pair-resolved rounds: the pair terms
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
        if (sidx == 0) {
            a.stats_out[0] = s_scal[1];
            *a.rounds_out = r;
            if (a.t_out)
                a.t_out[1] = global_timer_ns();
        }
    }
    if (CL)
        cl_sync_all();   // no CTA exits while another may still store into its shared memory
}

template <int FORM, int KIND, int KM, bool PROF>
__global__ void __launch_bounds__(kThreads, 1) k_sweep(SweepArgs a)
{
    sweep_body<FORM, KIND, KM, PROF>(a, (int)blockIdx.x);
}

// Pair-resolved rounds over FP32C dense or ragged markers.
template <int KIND, int KM, bool PROF>
__global__ void __launch_bounds__(kThreads, 1) k_sweep_pr(SweepArgs a)
{
    sweep_body<kFormFP32C, KIND, KM, PROF, false, true>(a, (int)blockIdx.x);
}

// The sweep as one thread-block cluster of G CTAs (the whole grid); the
// slice of a CTA is its rank in the cluster.
template <int FORM, int KIND, int KM, bool PROF>
__global__ void __launch_bounds__(kThreads, 1) k_sweep_cl(SweepArgs a)
{
    sweep_body<FORM, KIND, KM, PROF, true>(a, (int)cl_rank());
}

// Several independent chains of different sizes in one cooperative launch:
// CTAs [cta_start[i], cta_start[i+1]) run instance i's sweep over its slices,
// with its own barrier counter, records and residual; the instances share no
// data, so one chain's progress never waits on another's.
template <int FORM, int KM>
__global__ void __launch_bounds__(kThreads, 1) k_sweep_multi(const __grid_constant__ MultiSweepArgs m)
{
    int i = 0;
    while (i + 1 < m.n && (int)blockIdx.x >= m.cta_start[i + 1])
        ++i;
    const int sidx = (int)blockIdx.x - m.cta_start[i];
    if (m.kind[i] == kKindDense)
        sweep_body<FORM, kKindDense, KM, false>(m.inst[i], sidx);
    else
        sweep_body<FORM, kKindRagged, KM, false>(m.inst[i], sidx);
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

// The double-float residual as doubles (hi + lo), for the state read-back.
__global__ void k_df_to_double(int64_t N, const float *__restrict__ hi, const float *__restrict__ lo, double *out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N)
        out[i] = (double)hi[i] + (double)lo[i];
}

cudaError_t launch_df_to_double(int64_t N, const float *hi, const float *lo, double *out, cudaStream_t st)
{
    k_df_to_double<<<(unsigned)((N + kThreads - 1) / kThreads), kThreads, 0, st>>>(N, hi, lo, out);
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
    return make_plan(form, kind, a.slice_max, a.slot_bytes, a.B, a.n_groups, a.cluster, a.pairs != nullptr).total;
}

// Clusters above 8 CTAs are a non-portable size, allowed per kernel.
static cudaError_t cluster_attrs(const void *f, size_t smem)
{
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}

static cudaLaunchConfig_t cluster_config(int G, size_t smem, cudaStream_t st, cudaLaunchAttribute *attr)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)G);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

template <int FORM, int KIND, int KM>
static cudaError_t launch_one_cl(const SweepArgs &a, size_t smem, cudaStream_t st)
{
    const void *f = a.prof ? (const void *)k_sweep_cl<FORM, KIND, KM, true> : (const void *)k_sweep_cl<FORM, KIND, KM, false>;
    cudaError_t e = cluster_attrs(f, smem);
    if (e != cudaSuccess)
        return e;
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = cluster_config(a.G, smem, st, attr);
    SweepArgs args = a;
    void *params[] = {&args};
    return cudaLaunchKernelExC(&cfg, f, params);
}

template <int FORM, int KIND, int KM>
static cudaError_t launch_one(const SweepArgs &a, size_t smem, cudaStream_t st)
{
    if (a.cluster > 0)
        return launch_one_cl<FORM, KIND, KM>(a, smem, st);
    const void *f = a.prof ? (const void *)k_sweep<FORM, KIND, KM, true> : (const void *)k_sweep<FORM, KIND, KM, false>;
    if (FORM == kFormFP32C && a.pairs)
        f = a.prof ? (const void *)k_sweep_pr<KIND, KM, true> : (const void *)k_sweep_pr<KIND, KM, false>;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    SweepArgs args = a;
    void *params[] = {&args};
    return cudaLaunchCooperativeKernel(f, dim3(a.G), dim3(kThreads), params, smem, st);
}

template <int KM, bool PROF>
static const void *sweep_fn(int form, int kind)
{
    if (form == kFormFP64)
        return kind == kKindDense ? (const void *)k_sweep<kFormFP64, kKindDense, KM, PROF>
                                  : (const void *)k_sweep<kFormFP64, kKindRagged, KM, PROF>;
    return kind == kKindDense ? (const void *)k_sweep<kFormFP32C, kKindDense, KM, PROF>
                              : (const void *)k_sweep<kFormFP32C, kKindRagged, KM, PROF>;
}

template <int KM, bool PROF>
static const void *sweep_cl_fn(int form, int kind)
{
    if (form == kFormFP64)
        return kind == kKindDense ? (const void *)k_sweep_cl<kFormFP64, kKindDense, KM, PROF>
                                  : (const void *)k_sweep_cl<kFormFP64, kKindRagged, KM, PROF>;
    return kind == kKindDense ? (const void *)k_sweep_cl<kFormFP32C, kKindDense, KM, PROF>
                              : (const void *)k_sweep_cl<kFormFP32C, kKindRagged, KM, PROF>;
}

int sweep_cluster_fits(int form, int kind, int G, size_t smem)
{
    int n = 1 << 30;
    const void *fs[4] = {sweep_cl_fn<4, false>(form, kind), sweep_cl_fn<kMaxK, false>(form, kind),
                         sweep_cl_fn<4, true>(form, kind), sweep_cl_fn<kMaxK, true>(form, kind)};
    for (const void *f : fs) {
        int m = 0;
        cudaLaunchAttribute attr[1];
        const cudaLaunchConfig_t cfg = cluster_config(G, smem, nullptr, attr);
        if (cluster_attrs(f, smem) != cudaSuccess || cudaOccupancyMaxActiveClusters(&m, f, &cfg) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        n = m < n ? m : n;
    }
    return n;
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

static const void *multi_fn(int form, int kmax)
{
    if (form == kFormFP64)
        return kmax <= 4 ? (const void *)k_sweep_multi<kFormFP64, 4> : (const void *)k_sweep_multi<kFormFP64, kMaxK>;
    return kmax <= 4 ? (const void *)k_sweep_multi<kFormFP32C, 4> : (const void *)k_sweep_multi<kFormFP32C, kMaxK>;
}

size_t sweep_multi_static_smem(int form, int kmax)
{
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, multi_fn(form, kmax)) != cudaSuccess) {
        cudaGetLastError();
        return 16384;
    }
    return fa.sharedSizeBytes;
}

int sweep_multi_max_ctas_per_sm(int form, int kmax, size_t smem)
{
    const void *fn = multi_fn(form, kmax);
    int n = 0;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kThreads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// The cooperative launch goes through cudaLaunchKernelEx with the cooperative
// attribute, which stream capture records as a cooperative graph node.  The
// shared-memory attribute is set by sweep_multi_max_ctas_per_sm beforehand,
// outside any capture.
cudaError_t launch_sweep_multi(int form, int kmax, const MultiSweepArgs &m, size_t smem, cudaStream_t st)
{
    const void *fn = multi_fn(form, kmax);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)m.cta_start[m.n]);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    MultiSweepArgs args = m;
    void *params[] = {&args};
    return cudaLaunchKernelExC(&cfg, fn, params);
}

int sweep_max_ctas_per_sm(int form, int kind, size_t smem, bool pair_rounds)
{
    int n = 1 << 30;
    const void *fs[4] = {sweep_fn<4, false>(form, kind), sweep_fn<kMaxK, false>(form, kind),
                         sweep_fn<4, true>(form, kind), sweep_fn<kMaxK, true>(form, kind)};
    if (pair_rounds && kind == kKindDense) {
        fs[0] = (const void *)k_sweep_pr<kKindDense, 4, false>;
        fs[1] = (const void *)k_sweep_pr<kKindDense, kMaxK, false>;
        fs[2] = (const void *)k_sweep_pr<kKindDense, 4, true>;
        fs[3] = (const void *)k_sweep_pr<kKindDense, kMaxK, true>;
    } else if (pair_rounds) {
        fs[0] = (const void *)k_sweep_pr<kKindRagged, 4, false>;
        fs[1] = (const void *)k_sweep_pr<kKindRagged, kMaxK, false>;
        fs[2] = (const void *)k_sweep_pr<kKindRagged, 4, true>;
        fs[3] = (const void *)k_sweep_pr<kKindRagged, kMaxK, true>;
    }
    for (const void *f : fs) {
        int m = 0;
        cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, f, kThreads, smem) != cudaSuccess)
            return 0;
        n = m < n ? m : n;
    }
    return n;
}

}  // namespace brr
