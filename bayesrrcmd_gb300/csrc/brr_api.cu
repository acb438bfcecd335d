// C ABI of libbrr_gpu.so and the host-side chain driver.
//
// The driver restates the per-iteration body of BayesRBase::runGibbs
// (src/BayesRBase.cpp:186-247): updateMu, the per-marker draws, the shuffle,
// the sweep (AnalysisGraph::exec -> processColumn for every marker), the
// sigmaE draw and the per-group sigmaG / pi draws.  The sweep and all O(N) or
// O(M) work run on the device; the handful of scalar draws per iteration run
// on the host from the same counter-based stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <future>
#include <string>
#include <vector>

#include "brr_device.cuh"
#include "brr_internal.h"
#include "brr_stream.h"

using namespace brr;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

#define BRR_CUDA(call)                                                                                  \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(BRR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));              \
    } while (0)

template <class T>
cudaError_t dalloc(T **p, size_t n)
{
    *p = nullptr;
    if (n == 0)
        n = 1;
    return cudaMalloc((void **)p, n * sizeof(T));
}

}  // namespace

namespace brr {

int api_fail(int code, const std::string &msg) { return fail(code, msg); }

// Sweep permutation: Fisher-Yates from the counter-based stream.  The
// reference shuffles with std::random_shuffle (src/BayesRBase.cpp:198); any
// uniform permutation is equivalent in law, this one is replayable.
void make_permutation(StreamKey key, uint32_t it, uint32_t M, uint32_t *perm)
{
    for (uint32_t i = 0; i < M; ++i)
        perm[i] = i;
    for (uint32_t i = M; i-- > 1;) {
        const U4 b = stream_block(key, i, it, kPurposePerm, 0);
        const uint64_t r = ((uint64_t)b.x << 32) | b.y;
        const uint64_t j = (uint64_t)(((unsigned __int128)r * (uint64_t)(i + 1)) >> 64);
        std::swap(perm[i], perm[j]);
    }
}

}  // namespace brr

#include "brr_ctx.h"


namespace {

template <class T>
void drop_dev(T *&p)
{
    cudaFree(p);
    p = nullptr;
}

template <class T>
void drop_host(T *&p)
{
    cudaFreeHost(p);
    p = nullptr;
}

// Releases the buffers the first brr_pack_bed_device call allocates and
// nulls their pointers, so that a call that ran out of memory part-way leaves
// the context as before and a later call allocates them all again.
void release_pack_buffers(brr_ctx &c)
{
    drop_dev(c.d_codes);
    drop_dev(c.d_counts);
    drop_dev(c.d_table);
    drop_dev(c.d_scale);
    drop_dev(c.d_colsum);
    drop_dev(c.d_chosen);
    drop_dev(c.d_vstat);
    drop_dev(c.d_slice_lo);
    drop_dev(c.d_beta);
    drop_dev(c.d_comp);
    drop_dev(c.d_acum);
    drop_dev(c.d_order);
    drop_dev(c.d_u);
    drop_dev(c.d_z);
    drop_dev(c.d_rec);
    drop_dev(c.d_acc);
    drop_dev(c.d_gconst);
    drop_dev(c.d_gK);
    drop_dev(c.d_stats);
    drop_dev(c.d_part);
    drop_dev(c.d_err);
    drop_dev(c.d_rounds);
    drop_dev(c.d_prof);
    drop_dev(c.d_gstage);
    drop_dev(c.d_group);
    drop_dev(c.d_ystd);
    drop_dev(c.d_nzj);
    drop_dev(c.d_nzb);
    drop_dev(c.d_eps);
    drop_dev(c.d_eps_hi);
    drop_dev(c.d_eps_lo);
    drop_host(c.h_order);
    drop_host(c.h_stats);
    drop_host(c.h_part);
    drop_host(c.h_gc);
    drop_host(c.h_gK);
    drop_host(c.h_vstat);
    drop_host(c.h_misc);
}

void free_all(brr_ctx *c)
{
    if (c->perm_future.valid())
        c->perm_future.wait();
    cudaFree(c->d_slice_lo);
    cudaFree(c->d_codes);
    cudaFree(c->d_counts);
    cudaFree(c->d_table);
    cudaFree(c->d_scale);
    cudaFree(c->d_colsum);
    cudaFree(c->d_chosen);
    cudaFree(c->d_vstat);
    cudaFree(c->d_roff);
    for (auto &p : c->d_ridx)
        cudaFree(p);
    cudaFree(c->d_group);
    cudaFree(c->d_ystd);
    cudaFree(c->d_beta);
    cudaFree(c->d_comp);
    cudaFree(c->d_acum);
    cudaFree(c->d_eps);
    cudaFree(c->d_eps_dl);
    cudaFree(c->d_eps_hi);
    cudaFree(c->d_eps_lo);
    cudaFree(c->d_order);
    cudaFree(c->d_u);
    cudaFree(c->d_z);
    cudaFree(c->d_rec);
    cudaFree(c->d_acc);
    cudaFree(c->d_gconst);
    cudaFree(c->d_gK);
    cudaFree(c->d_stats);
    cudaFree(c->d_part);
    cudaFree(c->d_err);
    cudaFree(c->d_rounds);
    cudaFree(c->d_prof);
    cudaFree(c->d_tline);
    cudaFree(c->d_nzj);
    cudaFree(c->d_nzb);
    cudaFree(c->d_gram);
    cudaFree(c->d_gstage);
    cudaFree(c->d_brec);
    cudaFree(c->d_bdf);
    cudaFreeHost(c->h_order);
    cudaFreeHost(c->h_stats);
    cudaFreeHost(c->h_part);
    cudaFreeHost(c->h_gc);
    cudaFreeHost(c->h_gK);
    cudaFreeHost(c->h_vstat);
    cudaFreeHost(c->h_misc);
    for (auto &e : c->ev)
        if (e)
            cudaEventDestroy(e);
    if (c->st)
        cudaStreamDestroy(c->st);
}

// fixed-point accumulators: 3 rotating buffers of the restart sweep, 8 buffers
// of 8 copies for the blocked sweep; followed by the barrier counters (restart
// sweep: the first word; blocked sweep: 2 x 8 counters 16 words apart)

// Per-group sampler constants for the current sigmaE, sigmaG, pi
// (src/BayesRBase.cpp:309-333): c_k = log(pi_k) - log(sigmaG/sigmaE*(N-1)*cVa_k + 1)/2,
// invden_k = 1/denom_k with denom_k = N-1 + sigmaE/sigmaG/cVa_k,
// h_k = invden_k/(2 sigmaE), sdk_k = sqrt(sigmaE/denom_k).
void group_constants(const brr_ctx *c, std::vector<double> &gc, std::vector<int32_t> &gK)
{
    const int ng = c->cfg.n_groups;
    gc.assign((size_t)ng * kMaxK * 4, 0.0);
    gK.assign(ng, 0);
    const double NM1 = (double)(c->cfg.N - 1);
    for (int g = 0; g < ng; ++g) {
        const int K = c->cfg.K[g];
        gK[g] = K;
        const double sigmaG = c->sigmaG[g];
        const double sEsG = c->sigmaE / sigmaG;
        const double logLScale = sigmaG / c->sigmaE * NM1;
        double *row = gc.data() + (size_t)g * kMaxK * 4;
        row[0] = std::log(c->pi[g * BRR_MAX_K]);
        for (int k = 1; k < K; ++k) {
            const double cVa = c->cfg.S[g * (BRR_MAX_K - 1) + (k - 1)];
            const double cVaI = 1.0 / cVa;
            const double denom = NM1 + sEsG * cVaI;
            row[4 * k + 0] = std::log(c->pi[g * BRR_MAX_K + k]) - 0.5 * std::log(logLScale * cVa + 1.0);
            row[4 * k + 1] = 1.0 / denom;
            row[4 * k + 2] = 0.5 / denom / c->sigmaE;
            row[4 * k + 3] = std::sqrt(c->sigmaE / denom);
        }
    }
}

int check_device_status(brr_ctx *c)
{
    int h = 0;
    BRR_CUDA(cudaMemcpyAsync(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    BRR_CUDA(cudaStreamSynchronize(c->st));
    if (h == kDevTimeout)
        return fail(BRR_ERR_TIMEOUT, "a grid barrier of the sweep exceeded its wait limit");
    if (h == kDevRange)
        return fail(BRR_ERR_RANGE, "a partial dot product left the fixed-point exchange range");
    return BRR_OK;
}

int upload_state_eps(brr_ctx *c, const double *eps_host)
{
    const int64_t N = c->cfg.N;
    if (c->cfg.form == BRR_FORM_FP64) {
        BRR_CUDA(cudaMemcpy(c->d_eps, eps_host, sizeof(double) * N, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> h(N), l(N);
        for (int64_t i = 0; i < N; ++i) {
            h[i] = (float)eps_host[i];
            l[i] = (float)(eps_host[i] - (double)h[i]);
        }
        BRR_CUDA(cudaMemcpy(c->d_eps_hi, h.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
        BRR_CUDA(cudaMemcpy(c->d_eps_lo, l.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
    }
    return BRR_OK;
}

int download_eps(brr_ctx *c, double *eps_host)
{
    const int64_t N = c->cfg.N;
    if (c->cfg.form == BRR_FORM_FP64) {
        BRR_CUDA(cudaMemcpy(eps_host, c->d_eps, sizeof(double) * N, cudaMemcpyDeviceToHost));
    } else {
        // hi + lo formed on the device, one copy of N doubles
        if (!c->d_eps_dl && cudaMalloc((void **)&c->d_eps_dl, sizeof(double) * N) != cudaSuccess) {
            cudaGetLastError();
            return fail(BRR_ERR_OOM, "device allocation failed");
        }
        BRR_CUDA(launch_df_to_double(N, c->d_eps_hi, c->d_eps_lo, c->d_eps_dl, c->st));
        BRR_CUDA(cudaMemcpyAsync(eps_host, c->d_eps_dl, sizeof(double) * N, cudaMemcpyDeviceToHost, c->st));
        BRR_CUDA(cudaStreamSynchronize(c->st));
    }
    return BRR_OK;
}

// Slices of individuals for G CTAs in whole 64-individual chunks.
void compute_slices(brr_ctx *x, int G)
{
    G = (int)std::min<int64_t>(std::max(G, 1), x->chunks);
    x->G = G;
    x->slice_lo.assign(G + 1, 0);
    int64_t maxch = 0;
    for (int s = 0; s <= G; ++s) {
        const int64_t ch = (int64_t)s * x->chunks / G;
        x->slice_lo[s] = (int32_t)std::min<int64_t>(ch * kChunk, x->cfg.N);
        if (s > 0)
            maxch = std::max<int64_t>(maxch, ch - (int64_t)(s - 1) * x->chunks / G);
    }
    x->slice_max = (int)(maxch * kChunk);
    x->slot_bytes = (int)(maxch * 16);
}

// Per (marker, slice) ragged index lists from the packed codes for the current slices.
int build_ragged_lists(brr_ctx &c)
{
    const int64_t M = c.cfg.M;
    const int64_t MG1 = M * (int64_t)c.G + 1;
    if (3 * MG1 > (int64_t)INT_MAX)
        return fail(BRR_ERR_ARG, "ragged offset table too large for int32");
    cudaFree(c.d_roff);
    c.d_roff = nullptr;
    if (dalloc(&c.d_roff, (size_t)(3 * MG1)))
        return fail(BRR_ERR_OOM, "device allocation failed");
    BRR_CUDA(cudaMemsetAsync(c.d_roff, 0, sizeof(int32_t) * 3 * MG1, c.st));
    BRR_CUDA(launch_ragged_slice_counts(c.d_codes, c.col_stride, M, c.G, c.d_slice_lo, c.d_roff, c.st));
    int32_t *tmp = nullptr;
    if (dalloc(&tmp, (size_t)((MG1 + 1023) / 1024 + 1)))
        return fail(BRR_ERR_OOM, "device allocation failed");
    // totals must fit int32: the counts bound them by the genotype counts
    std::vector<int64_t> cnt(M * 4);
    BRR_CUDA(cudaMemcpyAsync(cnt.data(), c.d_counts, sizeof(int64_t) * M * 4, cudaMemcpyDeviceToHost, c.st));
    BRR_CUDA(cudaStreamSynchronize(c.st));
    int64_t tot[3] = {0, 0, 0};
    for (int64_t j = 0; j < M; ++j) {
        tot[0] += cnt[4 * j + 1];
        tot[1] += cnt[4 * j + 2];
        tot[2] += cnt[4 * j + 3];
    }
    for (int k = 0; k < 3; ++k) {
        if (tot[k] > (int64_t)INT_MAX) {
            cudaFree(tmp);
            return fail(BRR_ERR_ARG, "ragged index list longer than 2^31 entries");
        }
        BRR_CUDA(launch_exclusive_scan_i32(c.d_roff + k * MG1, MG1, tmp, c.st));
        cudaFree(c.d_ridx[k]);
        c.d_ridx[k] = nullptr;
        if (dalloc(&c.d_ridx[k], (size_t)tot[k] + 1)) {
            cudaFree(tmp);
            return fail(BRR_ERR_OOM, "device allocation failed");
        }
        c.rtot[k] = tot[k];
    }
    BRR_CUDA(cudaStreamSynchronize(c.st));
    cudaFree(tmp);
    BRR_CUDA(launch_ragged_fill(c.d_codes, c.col_stride, M, c.G, c.d_slice_lo, c.d_roff, c.d_roff + MG1,
                                c.d_roff + 2 * MG1, c.d_ridx[0], c.d_ridx[1], c.d_ridx[2], c.st));
    return BRR_OK;
}

}  // namespace

// New slicing (G CTAs) and round width B of a packed chain; the residual and
// the chain state are per individual and marker, so they carry over.
int brr::reslice(brr_ctx *c, int G, int B)
{
    if (!c->packed)
        return fail(BRR_ERR_ARG, "markers are not packed");
    BRR_CUDA(cudaSetDevice(c->dev));
    BRR_CUDA(cudaStreamSynchronize(c->st));
    compute_slices(c, G);
    if (B > 0)
        c->B = B;
    cudaFree(c->d_slice_lo);
    c->d_slice_lo = nullptr;
    cudaFree(c->d_part);
    c->d_part = nullptr;
    cudaFreeHost(c->h_part);
    c->h_part = nullptr;
    if (dalloc(&c->d_slice_lo, (size_t)c->G + 1) || dalloc(&c->d_part, (size_t)std::max(2 * c->G, kPartBlocks)) ||
        cudaMallocHost((void **)&c->h_part, sizeof(double) * std::max(2 * c->G, kPartBlocks)) != cudaSuccess)
        return fail(BRR_ERR_OOM, "allocation for the new slices failed");
    BRR_CUDA(cudaMemcpy(c->d_slice_lo, c->slice_lo.data(), sizeof(int32_t) * (c->G + 1), cudaMemcpyHostToDevice));
    if (c->kind == BRR_KIND_RAGGED) {
        const int rc = build_ragged_lists(*c);
        if (rc)
            return rc;
    }
    BRR_CUDA(cudaStreamSynchronize(c->st));
    return BRR_OK;
}

// The sampler constants of the current sigmaE, sigmaG and pi into the pinned
// staging the sweep's inputs are copied from.
void brr::sweep_stage(brr_ctx *c)
{
    std::vector<double> gc;
    std::vector<int32_t> gK;
    group_constants(c, gc, gK);
    std::memcpy(c->h_gc, gc.data(), sizeof(double) * gc.size());
    std::memcpy(c->h_gK, gK.data(), sizeof(int32_t) * gK.size());
}

// Device work before the sweep, on stream st: the staged constants, the records
// in sweep order (order in d_order, draws in d_u/d_z), cleared accumulators.
int brr::sweep_enqueue_inputs(brr_ctx *c, double eps_total, cudaStream_t st)
{
    const brr_config &cf = c->cfg;
    const size_t ng = (size_t)cf.n_groups;
    BRR_CUDA(cudaMemcpyAsync(c->d_gconst, c->h_gc, sizeof(double) * ng * kMaxK * 4, cudaMemcpyHostToDevice, st));
    BRR_CUDA(cudaMemcpyAsync(c->d_gK, c->h_gK, sizeof(int32_t) * ng, cudaMemcpyHostToDevice, st));
    if (c->blocked)
        BRR_CUDA(launch_gather_block(c->d_order, cf.M, cf.N, c->d_table, c->d_scale, c->d_beta, c->d_u, c->d_z,
                                     c->d_group, eps_total, c->d_brec, st));
    else
        BRR_CUDA(launch_gather(cf.form, c->kind, c->d_order, cf.M, c->d_table, c->d_scale, c->d_beta, c->d_u,
                               c->d_z, c->d_group, c->d_colsum, c->d_rec, st));
    BRR_CUDA(cudaMemsetAsync(c->d_acc, 0, sizeof(unsigned long long) * (kAccWords + kCounterWords), st));
    BRR_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(int), st));
    BRR_CUDA(cudaMemsetAsync(c->d_prof, 0, sizeof(long long) * 16, st));
    return BRR_OK;
}

// Pair-resolved rounds pay a fixed cost per round of 32 markers; restart
// rounds pay one round per residual-changing marker.  Measured on ragged
// markers (N = 20,000, M = 50,000) the pair-resolved sweep is faster while more
// than about one marker in forty carries a non-zero effect, so the choice
// follows the chain's state after the last sweep (a deterministic function of
// the chain, which keeps it reproducible).  Dense pair terms (population counts
// over every code word of the slice for each pair) grow with the square of the
// round width and cost more than the dot products on large slices, so dense
// markers take them only when asked (pair_rounds = 1, as every kind does).
static bool use_pair_rounds(const brr_ctx *c)
{
    if (!c->pair_rounds || c->blocked)
        return false;
    if (c->cfg.pair_rounds > 0)
        return true;
    return c->kind != BRR_KIND_DENSE && (c->last_nnz < 0 || c->last_nnz * 40 > c->cfg.M);
}

// The sweep kernel's arguments and shared memory.
void brr::sweep_args(brr_ctx *c, double mu_new, double eps_total, SweepArgs &a, size_t &smem)
{
    const brr_config &cf = c->cfg;
    a = SweepArgs{};
    a.N = cf.N;
    a.M = cf.M;
    a.G = c->G;
    a.B = c->B;
    a.n_groups = cf.n_groups;
    a.kmax = 0;
    for (int g = 0; g < cf.n_groups; ++g)
        a.kmax = std::max(a.kmax, cf.K[g]);
    a.slot_bytes = c->slot_bytes;
    a.slice_max = c->slice_max;
    a.slice_lo = c->d_slice_lo;
    a.codes = c->d_codes;
    a.col_stride = c->col_stride;
    const int64_t MG1 = cf.M * (int64_t)c->G + 1;
    for (int k = 0; k < 3; ++k) {
        a.roff[k] = c->d_roff ? c->d_roff + k * MG1 : nullptr;
        a.ridx[k] = c->d_ridx[k];
    }
    a.rec = c->d_rec;
    a.gconst = c->d_gconst;
    a.gK = c->d_gK;
    a.beta = c->d_beta;
    a.comp = c->d_comp;
    a.acum = c->d_acum;
    a.eps = c->d_eps;
    a.eps_hi = c->d_eps_hi;
    a.eps_lo = c->d_eps_lo;
    a.mu_new = mu_new;
    a.epsSum = c->epsSum;
    a.eps_total = eps_total;
    a.chosen = c->d_chosen;
    a.acc = c->d_acc;
    a.counter = c->d_acc + kAccWords;
    a.stats_out = c->d_stats;
    a.eigen = c->eigen ? 1 : 0;
    a.part = c->d_part;
    a.err = c->d_err;
    a.rounds_out = c->d_rounds;
    a.prof = c->profile ? c->d_prof : nullptr;
    // the timeline holds one row per SM: a sweep on more CTAs records none
    a.tline = c->profile && c->timeline && c->G <= c->sms ? c->d_tline : nullptr;
    a.async_batch = cf.async_batch;
    a.cluster = cf.cluster > 0 && c->G > 1 ? c->G : 0;
    a.pairs = use_pair_rounds(c) ? c->d_acc + kPairOffset : nullptr;
    c->last_pair = a.pairs != nullptr;
    a.timeout_ns = c->wait_limit_ns;
    a.phantom = c->phantom;
    a.gram = c->d_gram;
    a.gstage = c->d_gstage;
    a.has_missing = c->has_missing ? 1 : 0;
    a.brec = c->d_brec;
    a.order = c->d_order;
    a.beta_df = c->d_bdf;
    a.acum_df = c->d_bdf ? c->d_bdf + cf.M : nullptr;
    smem = c->blocked ? sweep_block_smem_bytes(a) : sweep_smem_bytes(cf.form, c->kind, a);
}

// Sampler constants, records in sweep order and the sweep arguments for the
// order in d_order and the draws in d_u/d_z.
int brr::sweep_prepare(brr_ctx *c, double mu_new, double eps_total, SweepArgs &a, size_t &smem)
{
    sweep_stage(c);
    const int rc = sweep_enqueue_inputs(c, eps_total, c->st);
    if (rc)
        return rc;
    sweep_args(c, mu_new, eps_total, a, smem);
    return BRR_OK;
}


// Device work after the sweep, on stream st: the statistics kernel and the
// read-back of counts, square sums, residual sums, rounds, cycles and status
// into pinned staging.
int brr::sweep_enqueue_outputs(brr_ctx *c, cudaStream_t st)
{
    const brr_config &cf = c->cfg;
    const int ng = cf.n_groups;
    BRR_CUDA(launch_sweep_stats(cf.M, c->d_group, c->d_comp, c->d_chosen, c->d_beta, ng, c->d_vstat, st));
    const size_t nv = (size_t)ng * kMaxK + 2 * ng;
    BRR_CUDA(cudaMemcpyAsync(c->h_vstat, c->d_vstat, sizeof(unsigned long long) * nv, cudaMemcpyDeviceToHost, st));
    BRR_CUDA(cudaMemcpyAsync(c->h_stats, c->d_stats, sizeof(double), cudaMemcpyDeviceToHost, st));
    BRR_CUDA(cudaMemcpyAsync(c->h_part, c->d_part, sizeof(double) * 2 * c->G, cudaMemcpyDeviceToHost, st));
    BRR_CUDA(cudaMemcpyAsync(c->h_misc, c->d_rounds, sizeof(long long), cudaMemcpyDeviceToHost, st));
    BRR_CUDA(cudaMemcpyAsync(c->h_misc + 1, c->d_prof, sizeof(long long) * 16, cudaMemcpyDeviceToHost, st));
    BRR_CUDA(cudaMemcpyAsync(c->h_misc + 17, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    return BRR_OK;
}

// Statistics of the sweep just run from the staging, once the stream is synchronised.
int brr::sweep_collect(brr_ctx *c, brr_sweep_out *out)
{
    const brr_config &cf = c->cfg;
    const int ng = cf.n_groups;
    int h = 0;
    std::memcpy(&h, c->h_misc + 17, sizeof(int));
    if (h == kDevTimeout)
        return fail(BRR_ERR_TIMEOUT, "a grid barrier of the sweep exceeded its wait limit");
    if (h == kDevRange)
        return fail(BRR_ERR_RANGE, "a partial dot product left the fixed-point exchange range");
    const unsigned long long *vstat = c->h_vstat;
    const long long rounds = c->h_misc[0];
    for (int k = 0; k < 16; ++k)
        c->phase[k] += c->h_misc[1 + k];

    for (int g = 0; g < ng; ++g)
        for (int k = 0; k < BRR_MAX_K; ++k)
            out->v[g * BRR_MAX_K + k] = k < kMaxK ? (double)vstat[g * kMaxK + k] : 0.0;
    for (int g = 0; g < ng; ++g)
        out->betasqnG[g] = fx_join((long long)vstat[(size_t)ng * kMaxK + 2 * g], vstat[(size_t)ng * kMaxK + 2 * g + 1]);
    double s1 = 0.0, s2 = 0.0;
    for (int s = 0; s < c->G; ++s) {
        s1 += c->h_part[2 * s];
        s2 += c->h_part[2 * s + 1];
    }
    out->eps_sum = s1;
    out->eps_sqnorm = s2;
    out->rounds = rounds;
    if (c->kind == BRR_KIND_RAGGED)
        c->epsSum = c->h_stats[0];
    c->sweeps += 1;
    int64_t nnz = 0;
    for (int g = 0; g < ng; ++g)
        for (int k = 1; k < kMaxK; ++k)
            nnz += (int64_t)vstat[g * kMaxK + k];
    c->last_nnz = nnz;
    return BRR_OK;
}

// Statistics of the sweep just run: component counts, squared betas, residual
// sums, rounds, device status.
int brr::sweep_finish(brr_ctx *c, brr_sweep_out *out)
{
    int rc = sweep_enqueue_outputs(c, c->st);
    if (rc)
        return rc;
    BRR_CUDA(cudaStreamSynchronize(c->st));
    return sweep_collect(c, out);
}

namespace {

// One sweep over the order already in d_order with draws in d_u/d_z.
int run_sweep(brr_ctx *c, double mu_new, double eps_total, brr_sweep_out *out, float *sweep_ms)
{
    const brr_config &cf = c->cfg;
    SweepArgs a{};
    size_t smem = 0;
    int rc = sweep_prepare(c, mu_new, eps_total, a, smem);
    if (rc)
        return rc;
    BRR_CUDA(cudaEventRecord(c->ev[0], c->st));
    if (c->blocked)
        BRR_CUDA(launch_sweep_block(a, smem, c->st));
    else
        BRR_CUDA(launch_sweep(cf.form, c->kind, a, smem, c->st));
    BRR_CUDA(cudaEventRecord(c->ev[1], c->st));
    if (c->blocked)
        BRR_CUDA(launch_block_finish(cf.M, c->d_chosen, a.beta_df, a.acum_df, c->d_beta, c->d_acum, c->st));

    rc = sweep_finish(c, out);
    if (rc)
        return rc;
    BRR_CUDA(cudaEventElapsedTime(sweep_ms, c->ev[0], c->ev[1]));
    return BRR_OK;
}

int post_sweep_draws(brr_ctx *c, const brr_sweep_out &so, uint32_t it)
{
    const brr_config &cf = c->cfg;
    const double Nd = (double)cf.N;
    // sigmaE (src/BayesRBase.cpp:238-239)
    if (!inv_scaled_chisq(c->key(), it, kPurposeSigmaE, 0, cf.v0E + Nd,
                          (so.eps_sqnorm + cf.v0E * cf.s02E) / (cf.v0E + Nd), &c->sigmaE))
        return fail(BRR_ERR_STREAM, "sigmaE gamma draw exceeded its attempt cap");
    // sigmaG, pi per group (src/BayesRBase.cpp:243-247)
    for (int g = 0; g < cf.n_groups; ++g) {
        const int K = cf.K[g];
        double vs = 0.0;
        for (int k = 0; k < K; ++k)
            vs += so.v[g * BRR_MAX_K + k];
        const double m0 = vs - so.v[g * BRR_MAX_K];
        if (!inv_scaled_chisq(c->key(), it, kPurposeSigmaG, (uint32_t)g, cf.v0G + m0,
                              (so.betasqnG[g] * m0 + cf.v0G * cf.s02G) / (cf.v0G + m0), &c->sigmaG[g]))
            return fail(BRR_ERR_STREAM, "sigmaG gamma draw exceeded its attempt cap");
        double r[BRR_MAX_K], rs = 0.0;
        for (int k = 0; k < K; ++k) {
            double gk;
            if (!gamma_draw(c->key(), it, kPurposePi, (uint32_t)(g * 256 + k), so.v[g * BRR_MAX_K + k] + 1.0, &gk))
                return fail(BRR_ERR_STREAM, "Dirichlet gamma draw exceeded its attempt cap");
            r[k] = 1.0 * gk;
            rs += r[k];
        }
        for (int k = 0; k < K; ++k)
            c->pi[g * BRR_MAX_K + k] = r[k] / rs;
    }
    return BRR_OK;
}

void schedule_permutation(brr_ctx *c, uint32_t it)
{
    if (c->perm_future.valid())
        c->perm_future.wait();
    c->perm_next.resize(c->cfg.M);
    c->perm_next_it = it;
    const StreamKey k = c->key();
    const uint32_t M = (uint32_t)c->cfg.M;
    uint32_t *dst = c->perm_next.data();
    c->perm_future = std::async(std::launch::async, [k, it, M, dst]() { make_permutation(k, it, M, dst); });
}

// The FP32C dense form resolves whole blocks of markers per grid round with
// the precomputed marker Gram when it fits in device memory (2 GB left free).
int prepare_blocked(brr_ctx *c)
{
    const brr_config &cf = c->cfg;
    if (cf.pair_rounds > 0 && !c->pair_rounds)
        return fail(BRR_ERR_ARG, "pair_rounds = 1 needs the FP32C form, ragged (not Eigen) or dense markers, at most "
                                 "32 markers per round, no cluster and slices whose pair data fit shared memory");
    if (cf.pair_rounds > 0 && cf.kind == BRR_KIND_DENSE && cf.gram > 0)
        return fail(BRR_ERR_ARG, "pair_rounds = 1 takes the restart sweep, gram = 1 the Gram-blocked one");
    if (cf.pair_rounds > 0 && cf.kind == BRR_KIND_DENSE) {
        c->blocked = false;
        return BRR_OK;
    }
    if (cf.form != BRR_FORM_FP32C || cf.kind != BRR_KIND_DENSE || cf.gram < 0 || cf.M < 2 || cf.cluster > 0) {
        c->blocked = false;
        if (cf.gram > 0)
            return fail(BRR_ERR_ARG, "the Gram-blocked sweep needs the FP32C form, dense markers and M >= 2");
        return BRR_OK;
    }
    if (c->d_gram) {
        c->blocked = true;
        return BRR_OK;
    }
    // the combination's 64-bit numerators hold 16 N^3
    if (cf.N > 800000) {
        if (cf.gram > 0)
            return fail(BRR_ERR_ARG, "the marker Gram needs N <= 800,000");
        c->blocked = false;
        return BRR_OK;
    }
    size_t gram_bytes = 0, work = 0, free_b = 0, total_b = 0;
    gram_bytes_needed(cf.N, cf.M, c->has_missing, &gram_bytes, &work);
    BRR_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t margin = (size_t)2 << 30;
    if (gram_bytes + work + margin > free_b) {
        if (cf.gram > 0)
            return fail(BRR_ERR_OOM, "the marker Gram (" + std::to_string(gram_bytes >> 20) + " MiB) does not fit");
        c->blocked = false;
        return BRR_OK;
    }
    if (cf.spec_width == 0)
        c->B = 64;
    SweepArgs a{};
    a.B = c->B;
    a.n_groups = cf.n_groups;
    a.slice_max = c->slice_max;
    a.slot_bytes = c->slot_bytes;
    const size_t smem = sweep_block_smem_bytes(a);
    std::string occ_why;
    const int per_sm = sweep_block_max_ctas_per_sm(smem, &occ_why);
    if (per_sm < 1 || (int64_t)per_sm * c->sms < c->G) {
        if (cf.gram > 0)
            return fail(BRR_ERR_ARG, "the blocked sweep does not fit its CTAs: " +
                                         (occ_why.empty() ? std::to_string(per_sm) + " per SM" : occ_why));
        c->blocked = false;
        return BRR_OK;
    }
    if (cudaMalloc((void **)&c->d_gram, gram_bytes) != cudaSuccess ||
        (!c->d_brec && cudaMalloc((void **)&c->d_brec, sizeof(BlockRec) * (size_t)cf.M) != cudaSuccess) ||
        (!c->d_bdf && cudaMalloc((void **)&c->d_bdf, sizeof(float2) * 2 * (size_t)cf.M) != cudaSuccess)) {
        cudaGetLastError();
        cudaFree(c->d_gram);
        c->d_gram = nullptr;
        if (cf.gram > 0)
            return fail(BRR_ERR_OOM, "allocation of the marker Gram failed");
        c->blocked = false;
        return BRR_OK;
    }
    std::string why;
    float ms = 0.f;
    if (build_gram(c->d_codes, c->col_stride, cf.N, cf.M, c->d_scale, c->d_counts, c->has_missing, c->d_gram, c->st,
                   why, &ms) != 0) {
        cudaFree(c->d_gram);
        c->d_gram = nullptr;
        return fail(BRR_ERR_CUDA, "building the marker Gram failed: " + why);
    }
    c->gram_ms = ms;
    c->gram_bits = gram_route_bits();
    c->blocked = true;
    return BRR_OK;
}

int refresh_eps_impl(brr_ctx *c)
{
    const brr_config &cf = c->cfg;
    std::vector<double> beta(cf.M);
    BRR_CUDA(cudaMemcpy(beta.data(), c->d_beta, sizeof(double) * cf.M, cudaMemcpyDeviceToHost));
    std::vector<uint32_t> nzj;
    std::vector<double> nzb;
    for (int64_t j = 0; j < cf.M; ++j)
        if (beta[j] != 0.0) {
            nzj.push_back((uint32_t)j);
            nzb.push_back(beta[j]);
        }
    if (!nzj.empty()) {
        BRR_CUDA(cudaMemcpy(c->d_nzj, nzj.data(), sizeof(uint32_t) * nzj.size(), cudaMemcpyHostToDevice));
        BRR_CUDA(cudaMemcpy(c->d_nzb, nzb.data(), sizeof(double) * nzb.size(), cudaMemcpyHostToDevice));
    }
    BRR_CUDA(launch_refresh(cf.form, c->kind, cf.N, c->d_ystd, c->mu, c->d_codes, c->col_stride, c->d_table, c->d_nzj,
                            c->d_nzb, (int64_t)nzj.size(), c->d_eps, c->d_eps_hi, c->d_eps_lo, c->st));
    BRR_CUDA(cudaStreamSynchronize(c->st));
    return BRR_OK;
}

}  // namespace

// FP64 refresh when due, updateMu (dense src/DenseBayesRRmz.cpp:36-42, ragged
// src/SparseBayesRRG.cpp:106-113), the per-marker draws and the permutation
// (src/BayesRBase.cpp:196-198) of iteration it.
int brr::iter_pre(brr_ctx &c, uint32_t it, double &mu_new, double &eps_total)
{
    int rc = iter_pre_dev(c, it);
    if (rc)
        return rc;
    BRR_CUDA(cudaStreamSynchronize(c.st));
    rc = iter_pre_host(c, it, mu_new, eps_total);
    if (rc)
        return rc;
    return iter_enqueue_draws(c, it, c.st);
}

// Device part of updateMu: FP64 refresh when due, the residual total into h_part.
int brr::iter_pre_dev(brr_ctx &c, uint32_t it)
{
    const brr_config &cf = c.cfg;
    if (c.perm_next_it != it)
        schedule_permutation(&c, it);
    if (cf.form == BRR_FORM_FP32C && cf.refresh_every > 0 && c.sweeps > 0 && c.sweeps % cf.refresh_every == 0) {
        const int rc = refresh_eps_impl(&c);
        if (rc)
            return rc;
    }
    BRR_CUDA(launch_mu_prep(cf.form, cf.N, c.mu, c.d_eps, c.d_eps_hi, c.d_eps_lo, c.d_part, kPartBlocks, c.st));
    if (cf.kind == BRR_KIND_DENSE)
        BRR_CUDA(cudaMemcpyAsync(c.h_part, c.d_part, sizeof(double) * kPartBlocks, cudaMemcpyDeviceToHost, c.st));
    return BRR_OK;
}

// Host part of updateMu (after the stream is synchronised) and the sweep order
// of iteration it into the pinned order buffer.
int brr::iter_pre_host(brr_ctx &c, uint32_t it, double &mu_new, double &eps_total)
{
    const brr_config &cf = c.cfg;
    const int64_t N = cf.N, M = cf.M;
    const double Nd = (double)N;
    const double old_mu = c.mu;
    double mean, esum = 0.0;
    if (cf.kind == BRR_KIND_DENSE) {
        for (int b = 0; b < kPartBlocks; ++b)
            esum += c.h_part[b];
        mean = esum / Nd;
    } else {
        c.epsSum += old_mu * Nd;
        mean = c.epsSum / Nd;
    }
    c.mu = mean + std::sqrt(c.sigmaE / Nd) * normal_mu(c.key(), it);
    if (c.kind == BRR_KIND_RAGGED)
        c.epsSum -= c.mu * Nd;
    c.perm_future.wait();
    std::memcpy(c.h_order, c.perm_next.data(), sizeof(uint32_t) * M);
    schedule_permutation(&c, it + 1);
    mu_new = c.mu;
    eps_total = esum - c.mu * Nd;
    return BRR_OK;
}

// Device work of the draws, on stream st: the per-marker draws of iteration it
// and the sweep order from the pinned buffer.
int brr::iter_enqueue_draws(brr_ctx &c, uint32_t it, cudaStream_t st)
{
    const brr_config &cf = c.cfg;
    BRR_CUDA(launch_draws(cf.seed, cf.chain, it, cf.M, c.d_u, c.d_z, st));
    BRR_CUDA(cudaMemcpyAsync(c.d_order, c.h_order, sizeof(uint32_t) * cf.M, cudaMemcpyHostToDevice, st));
    return BRR_OK;
}

// sigmaE, sigmaG and pi draws after the sweep (src/BayesRBase.cpp:237-247).
int brr::iter_post(brr_ctx &c, const brr_sweep_out &so, uint32_t it)
{
    const int rc = post_sweep_draws(&c, so, it);
    if (rc)
        return rc;
    c.iteration = it + 1;
    return BRR_OK;
}

extern "C" {

const char *brr_last_error(void) { return g_last_error.c_str(); }

int brr_ctx_create(const brr_config *cfg, brr_ctx **out)
{
    if (!cfg || !out)
        return fail(BRR_ERR_ARG, "null argument");
    *out = nullptr;
    const brr_config &c = *cfg;
    if (c.N < 2 || c.M < 1 || c.M > (int64_t)UINT32_MAX)
        return fail(BRR_ERR_ARG, "need N >= 2 individuals and 1 <= M < 2^32 markers");
    if (c.kind != BRR_KIND_DENSE && c.kind != BRR_KIND_RAGGED && c.kind != BRR_KIND_EIGEN)
        return fail(BRR_ERR_ARG, "unknown marker kind");
    if (c.form != BRR_FORM_FP64 && c.form != BRR_FORM_FP32C)
        return fail(BRR_ERR_ARG, "unknown sweep form");
    if (c.n_groups < 1 || c.n_groups > BRR_MAX_GROUPS)
        return fail(BRR_ERR_ARG, "n_groups must be in 1..64");
    for (int g = 0; g < c.n_groups; ++g) {
        if (c.K[g] < 2 || c.K[g] > BRR_MAX_K)
            return fail(BRR_ERR_ARG, "every group needs 2..16 mixture components");
        for (int k = 0; k + 1 < c.K[g]; ++k)
            if (!(c.S[g * (BRR_MAX_K - 1) + k] > 0.0))
                return fail(BRR_ERR_ARG, "variance ratios S must be positive");
    }
    int spec = c.spec_width ? c.spec_width : (c.form == BRR_FORM_FP64 ? 16 : 32);
    if (spec != 8 && spec != 16 && spec != 32 && spec != 64)
        return fail(BRR_ERR_ARG, "spec_width must be 8, 16, 32 or 64");
    if (c.async_batch < 0 || c.async_batch > kMaxSpec)
        return fail(BRR_ERR_ARG, "async_batch must be in 0..64");
    if (c.async_batch > 0 && c.form != BRR_FORM_FP64)
        return fail(BRR_ERR_ARG, "the asynchronous schedule runs the FP64 form");
    if (c.cluster < 0 || c.cluster == 1 || c.cluster > 16)
        return fail(BRR_ERR_ARG, "cluster must be 0 or 2..16");
    if (c.cluster > 0 && c.gram > 0)
        return fail(BRR_ERR_ARG, "the cluster sweep is the restart sweep: gram cannot be required");
    // an asynchronous batch is one round: the round width covers it
    while (spec < c.async_batch)
        spec *= 2;

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(BRR_ERR_DEVICE, "no CUDA device");
    if (c.device < 0 || c.device >= ndev)
        return fail(BRR_ERR_DEVICE, "device ordinal out of range");
    cudaDeviceProp prop;
    BRR_CUDA(cudaGetDeviceProperties(&prop, c.device));
    if (prop.major != 10 || prop.minor != 3)
        return fail(BRR_ERR_DEVICE, std::string("libbrr_gpu is built for sm_103a only; device is ") + prop.name);

    brr_ctx *x = new brr_ctx();
    x->cfg = c;
    x->kind = c.kind == BRR_KIND_DENSE ? BRR_KIND_DENSE : BRR_KIND_RAGGED;
    x->eigen = c.kind == BRR_KIND_EIGEN;
    x->dev = c.device;
    x->sms = prop.multiProcessorCount;
    x->B = spec;
    cudaError_t e = cudaSetDevice(c.device);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&x->st, cudaStreamNonBlocking);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i)
        e = cudaEventCreate(&x->ev[i]);
    if (e != cudaSuccess) {
        free_all(x);
        delete x;
        return fail(BRR_ERR_CUDA, cudaGetErrorString(e));
    }
    // slices of individuals in 64-individual chunks (16 bytes of codes)
    x->chunks = (c.N + kChunk - 1) / kChunk;
    x->col_stride = x->chunks * 16;
    compute_slices(x, c.cluster > 0 ? c.cluster : (c.grid > 0 ? c.grid : x->sms));
    if (c.kind != BRR_KIND_DENSE && x->slice_max > 65536) {
        free_all(x);
        delete x;
        return fail(BRR_ERR_ARG, "ragged slices are limited to 65536 individuals; raise grid");
    }
    *out = x;
    return BRR_OK;
}

int brr_ctx_destroy(brr_ctx *ctx)
{
    if (!ctx)
        return BRR_OK;
    cudaSetDevice(ctx->dev);
    free_all(ctx);
    delete ctx;
    return BRR_OK;
}

int brr_pack_bed(brr_ctx *ctx, const uint8_t *bed, int64_t nbytes)
{
    if (!ctx || !bed)
        return fail(BRR_ERR_ARG, "null argument");
    const int64_t need = ctx->cfg.M * ((ctx->cfg.N + 3) / 4);
    if (nbytes != need)
        return fail(BRR_ERR_ARG, "BED payload size does not match M*ceil(N/4) (has the FAM/BIM been changed?)");
    BRR_CUDA(cudaSetDevice(ctx->dev));
    uint8_t *d = nullptr;
    if (dalloc(&d, (size_t)nbytes) != cudaSuccess)
        return fail(BRR_ERR_OOM, "device allocation of the BED payload failed");
    cudaError_t e = cudaMemcpy(d, bed, (size_t)nbytes, cudaMemcpyHostToDevice);
    int rc = e == cudaSuccess ? brr_pack_bed_device(ctx, d, nbytes) : fail(BRR_ERR_CUDA, cudaGetErrorString(e));
    cudaFree(d);
    return rc;
}

int brr_pack_bed_device(brr_ctx *ctx, const uint8_t *d_bed, int64_t nbytes)
{
    if (!ctx || !d_bed)
        return fail(BRR_ERR_ARG, "null argument");
    brr_ctx &c = *ctx;
    const brr_config &cf = c.cfg;
    if (nbytes != cf.M * ((cf.N + 3) / 4))
        return fail(BRR_ERR_ARG, "BED payload size does not match M*ceil(N/4)");
    BRR_CUDA(cudaSetDevice(c.dev));
    {
        // the packer reads nbytes from d_bed: refuse a buffer it would overrun
        std::string why;
        if (!device_range_check(c.dev, d_bed, (size_t)nbytes, "d_bed", why))
            return fail(BRR_ERR_ARG, why);
    }
    const int64_t M = cf.M;
    if (!c.d_codes) {
        if (dalloc(&c.d_codes, (size_t)(M * c.col_stride)) != cudaSuccess || dalloc(&c.d_counts, (size_t)M * 4) ||
            dalloc(&c.d_table, (size_t)M * 4) || dalloc(&c.d_scale, (size_t)M * 2) ||
            dalloc(&c.d_colsum, (size_t)M) || dalloc(&c.d_chosen, (size_t)M) ||
            dalloc(&c.d_vstat, (size_t)cf.n_groups * kMaxK + 2 * cf.n_groups) ||
            dalloc(&c.d_slice_lo, (size_t)c.G + 1) || dalloc(&c.d_beta, (size_t)M) || dalloc(&c.d_comp, (size_t)M) ||
            dalloc(&c.d_acum, (size_t)M) || dalloc(&c.d_order, (size_t)M) || dalloc(&c.d_u, (size_t)M) ||
            dalloc(&c.d_z, (size_t)M) || dalloc(&c.d_rec, (size_t)M) || dalloc(&c.d_acc, kAccWords + kCounterWords) ||
            dalloc(&c.d_gconst, (size_t)cf.n_groups * kMaxK * 4) || dalloc(&c.d_gK, (size_t)cf.n_groups) ||
            dalloc(&c.d_stats, (size_t)cf.n_groups * kMaxK + cf.n_groups + 1) ||
            dalloc(&c.d_part, (size_t)std::max(2 * c.G, kPartBlocks)) || dalloc(&c.d_err, 1) ||
            dalloc(&c.d_rounds, 1) || dalloc(&c.d_prof, 16) || dalloc(&c.d_gstage, sweep_block_stage_bytes(kMaxSpec) / sizeof(double)) || dalloc(&c.d_group, (size_t)M) || dalloc(&c.d_ystd, (size_t)cf.N) ||
            dalloc(&c.d_nzj, (size_t)M) || dalloc(&c.d_nzb, (size_t)M)) {
            release_pack_buffers(c);
            return fail(BRR_ERR_OOM, "device allocation failed");
        }
        if (cf.form == BRR_FORM_FP64) {
            if (dalloc(&c.d_eps, (size_t)cf.N)) {
                release_pack_buffers(c);
                return fail(BRR_ERR_OOM, "device allocation failed");
            }
        } else {
            if (dalloc(&c.d_eps_hi, (size_t)cf.N) || dalloc(&c.d_eps_lo, (size_t)cf.N)) {
                release_pack_buffers(c);
                return fail(BRR_ERR_OOM, "device allocation failed");
            }
        }
        if (cudaMallocHost((void **)&c.h_order, sizeof(uint32_t) * M) != cudaSuccess ||
            cudaMallocHost((void **)&c.h_stats, sizeof(double) * ((size_t)cf.n_groups * kMaxK + cf.n_groups + 1)) !=
                cudaSuccess ||
            cudaMallocHost((void **)&c.h_part, sizeof(double) * std::max(2 * c.G, kPartBlocks)) != cudaSuccess ||
            cudaMallocHost((void **)&c.h_gc, sizeof(double) * (size_t)cf.n_groups * kMaxK * 4) != cudaSuccess ||
            cudaMallocHost((void **)&c.h_gK, sizeof(int32_t) * (size_t)cf.n_groups) != cudaSuccess ||
            cudaMallocHost((void **)&c.h_vstat, sizeof(unsigned long long) * ((size_t)cf.n_groups * kMaxK + 2 * cf.n_groups)) !=
                cudaSuccess ||
            cudaMallocHost((void **)&c.h_misc, sizeof(long long) * 18) != cudaSuccess) {
            release_pack_buffers(c);
            return fail(BRR_ERR_OOM, "pinned host allocation failed");
        }
        BRR_CUDA(cudaMemset(c.d_group, 0, sizeof(int32_t) * M));
        c.group.assign(M, 0);
    }
    BRR_CUDA(cudaMemcpy(c.d_slice_lo, c.slice_lo.data(), sizeof(int32_t) * (c.G + 1), cudaMemcpyHostToDevice));
    BRR_CUDA(launch_pack_counts(d_bed, cf.N, M, c.d_codes, c.col_stride, c.d_counts, c.st));
    int *d_bad = nullptr;
    if (dalloc(&d_bad, 1))
        return fail(BRR_ERR_OOM, "device allocation failed");
    const int big = INT_MAX;
    int bad = INT_MAX;
    cudaError_t le = cudaMemcpy(d_bad, &big, sizeof(int), cudaMemcpyHostToDevice);
    if (le == cudaSuccess)
        le = cf.kind == BRR_KIND_DENSE
                 ? launch_dense_tables(c.d_counts, cf.N, M, c.d_table, c.d_scale, c.d_colsum, d_bad, c.st)
                 : launch_ragged_stats(c.d_counts, cf.N, M, c.eigen ? 1 : 0, c.d_table, d_bad, c.st);
    if (le == cudaSuccess)
        le = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, c.st);
    if (le == cudaSuccess)
        le = cudaStreamSynchronize(c.st);
    cudaFree(d_bad);
    if (le != cudaSuccess)
        return fail(BRR_ERR_CUDA, std::string("marker statistics: ") + cudaGetErrorString(le));
    BRR_CUDA(cudaGetLastError());
    if (bad != INT_MAX)
        return fail(BRR_ERR_MARKER, "marker " + std::to_string(bad) +
                                        " does not vary or is all missing; SNPs that do not vary should be "
                                        "removed prior to analysis");
    {
        std::vector<int64_t> cnt(M * 4);
        BRR_CUDA(cudaMemcpy(cnt.data(), c.d_counts, sizeof(int64_t) * M * 4, cudaMemcpyDeviceToHost));
        c.has_missing = false;
        for (int64_t j = 0; j < M && !c.has_missing; ++j)
            c.has_missing = cnt[4 * j + 3] != 0;
    }
    if (c.kind == BRR_KIND_RAGGED) {
        const int rc = build_ragged_lists(c);
        if (rc)
            return rc;
    }
    BRR_CUDA(cudaStreamSynchronize(c.st));
    // the sweep kernel must fit one CTA per slice on the GPU at once
    SweepArgs a{};
    a.B = c.B;
    a.n_groups = cf.n_groups;
    a.slice_max = c.slice_max;
    a.slot_bytes = c.slot_bytes;
    a.cluster = cf.cluster > 0 && c.G > 1 ? c.G : 0;
    // FP32C restart sweeps resolve whole rounds with pair terms when the round
    // is one warp wide and the slice's code map or masks fit beside the ring
    c.pair_rounds = cf.form == BRR_FORM_FP32C && !c.eigen && c.B <= 32 && cf.pair_rounds >= 0 && a.cluster == 0 &&
                    cf.async_batch == 0 && cf.N < (1 << 24);
    if (c.pair_rounds) {
        a.pairs = c.d_acc + kPairOffset;
        const size_t sp = sweep_smem_bytes(cf.form, c.kind, a);
        const int per = sp <= (size_t)200 * 1024 ? sweep_max_ctas_per_sm(cf.form, c.kind, sp, true) : 0;
        if (per < 1 || (int64_t)per * c.sms < c.G) {
            c.pair_rounds = false;
            a.pairs = nullptr;
        }
    }
    const size_t smem = sweep_smem_bytes(cf.form, c.kind, a);
    if (a.cluster > 0) {
        if (sweep_cluster_fits(cf.form, c.kind, c.G, smem) < 1)
            return fail(BRR_ERR_ARG, "a cluster of " + std::to_string(c.G) + " CTAs with " + std::to_string(smem) +
                                         " bytes of shared memory each cannot be scheduled");
        c.packed = true;
        return BRR_OK;
    }
    const int per_sm = sweep_max_ctas_per_sm(cf.form, c.kind, smem);
    if (per_sm < 1 || (int64_t)per_sm * c.sms < c.G)
        return fail(BRR_ERR_ARG, "the sweep kernel does not fit " + std::to_string(c.G) +
                                     " co-resident CTAs (shared memory " + std::to_string(smem) + " bytes)");
    c.packed = true;
    return BRR_OK;
}

int brr_get_marker_table(brr_ctx *ctx, double *table, int64_t *counts)
{
    if (!ctx || !ctx->packed)
        return fail(BRR_ERR_ARG, "markers are not packed");
    const int64_t M = ctx->cfg.M;
    if (table)
        BRR_CUDA(cudaMemcpy(table, ctx->d_table, sizeof(double) * M * 4, cudaMemcpyDeviceToHost));
    if (counts)
        BRR_CUDA(cudaMemcpy(counts, ctx->d_counts, sizeof(int64_t) * M * 4, cudaMemcpyDeviceToHost));
    return BRR_OK;
}

int brr_get_ragged_lists(brr_ctx *ctx, int64_t *off_ones, int32_t *ones, int64_t *off_twos, int32_t *twos,
                         int64_t *off_miss, int32_t *miss)
{
    if (!ctx || !ctx->packed || ctx->kind != BRR_KIND_RAGGED)
        return fail(BRR_ERR_ARG, "no ragged markers packed");
    const int64_t M = ctx->cfg.M, G = ctx->G, MG1 = M * G + 1;
    std::vector<int32_t> off(3 * MG1);
    BRR_CUDA(cudaMemcpy(off.data(), ctx->d_roff, sizeof(int32_t) * 3 * MG1, cudaMemcpyDeviceToHost));
    int64_t *offs[3] = {off_ones, off_twos, off_miss};
    int32_t *outs[3] = {ones, twos, miss};
    for (int k = 0; k < 3; ++k) {
        std::vector<uint16_t> idx(ctx->rtot[k] + 1);
        BRR_CUDA(cudaMemcpy(idx.data(), ctx->d_ridx[k], sizeof(uint16_t) * (ctx->rtot[k] + 1), cudaMemcpyDeviceToHost));
        const int32_t *o = off.data() + k * MG1;
        for (int64_t j = 0; j < M; ++j) {
            if (offs[k])
                offs[k][j] = o[j * G];
            for (int64_t s = 0; s < G; ++s)
                for (int32_t e = o[j * G + s]; e < o[j * G + s + 1]; ++e)
                    if (outs[k])
                        outs[k][e] = ctx->slice_lo[s] + idx[e];
        }
        if (offs[k])
            offs[k][M] = o[M * G];
    }
    return BRR_OK;
}

int brr_set_groups(brr_ctx *ctx, const int32_t *group)
{
    if (!ctx || !group || !ctx->packed)
        return fail(BRR_ERR_ARG, "pack markers before setting groups");
    for (int64_t j = 0; j < ctx->cfg.M; ++j)
        if (group[j] < 0 || group[j] >= ctx->cfg.n_groups)
            return fail(BRR_ERR_ARG, "group id out of range at marker " + std::to_string(j));
    ctx->group.assign(group, group + ctx->cfg.M);
    BRR_CUDA(cudaMemcpy(ctx->d_group, group, sizeof(int32_t) * ctx->cfg.M, cudaMemcpyHostToDevice));
    return BRR_OK;
}

// y standardisation of BayesRBase::init (src/BayesRBase.cpp:85-86) on the
// single-precision phenotype (src/data.cpp:348).
int brr_set_phenotype(brr_ctx *ctx, const float *y)
{
    if (!ctx || !y || !ctx->packed)
        return fail(BRR_ERR_ARG, "pack markers before setting the phenotype");
    const int64_t N = ctx->cfg.N;
    double ysum = 0.0;
    for (int64_t i = 0; i < N; ++i) {
        if (!std::isfinite(y[i]))
            return fail(BRR_ERR_ARG, "phenotype value " + std::to_string(i) + " is not finite");
        ysum += (double)y[i];
    }
    const double ymean = ysum / (double)N;
    std::vector<double> d(N);
    double sq = 0.0;
    for (int64_t i = 0; i < N; ++i) {
        d[i] = (double)y[i] - ymean;
        sq += d[i] * d[i];
    }
    if (!(sq > 0.0))
        return fail(BRR_ERR_ARG, "phenotype has zero variance");
    const double scale = std::sqrt(sq / (double)(N - 1));
    ctx->ystd.resize(N);
    for (int64_t i = 0; i < N; ++i)
        ctx->ystd[i] = d[i] / scale;
    BRR_CUDA(cudaMemcpy(ctx->d_ystd, ctx->ystd.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
    ctx->pheno = true;
    return BRR_OK;
}

// BayesRBase::init (src/BayesRBase.cpp:39-99).
int brr_init_chain(brr_ctx *ctx)
{
    if (!ctx || !ctx->packed || !ctx->pheno)
        return fail(BRR_ERR_ARG, "pack markers and set the phenotype before init");
    brr_ctx &c = *ctx;
    const brr_config &cf = c.cfg;
    const int64_t N = cf.N, M = cf.M;
    for (int g = 0; g < cf.n_groups; ++g) {
        const int K = cf.K[g];
        for (int k = 0; k < BRR_MAX_K; ++k)
            c.pi[g * BRR_MAX_K + k] = k < K ? 0.5 / (double)K : 0.0;
        c.pi[g * BRR_MAX_K] = 0.5;
        c.sigmaG[g] = uniform_init(c.key(), (uint32_t)g);
    }
    c.mu = 0.0;
    std::vector<double> eps(N);
    double esq = 0.0, esum = 0.0;
    for (int64_t i = 0; i < N; ++i) {
        eps[i] = c.ystd[i] - c.mu;
        esq += eps[i] * eps[i];
        esum += eps[i];
    }
    c.sigmaE = esq / (double)N * 0.5;
    c.epsSum = esum;
    BRR_CUDA(cudaMemset(c.d_beta, 0, sizeof(double) * M));
    BRR_CUDA(cudaMemset(c.d_comp, 0, sizeof(int32_t) * M));
    BRR_CUDA(cudaMemset(c.d_acum, 0, sizeof(double) * M));
    int rc = upload_state_eps(&c, eps.data());
    if (rc)
        return rc;
    rc = prepare_blocked(&c);
    if (rc)
        return rc;
    c.iteration = 0;
    c.sweeps = 0;
    c.last_nnz = -1;
    c.inited = true;
    return BRR_OK;
}

int brr_iterate(brr_ctx *ctx, int32_t n_iter)
{
    if (!ctx || !ctx->inited)
        return fail(BRR_ERR_ARG, "chain not initialised");
    brr_ctx &c = *ctx;
    BRR_CUDA(cudaSetDevice(c.dev));
    double sweep_total = 0.0;
    int64_t rounds_total = 0;
    std::memset(c.phase, 0, sizeof(c.phase));
    BRR_CUDA(cudaEventRecord(c.ev[2], c.st));
    for (int32_t n = 0; n < n_iter; ++n) {
        const uint32_t it = c.iteration;
        double mu_new = 0.0, eps_total = 0.0;
        int rc = iter_pre(c, it, mu_new, eps_total);
        if (rc)
            return rc;
        brr_sweep_out so{};
        float ms = 0.f;
        rc = run_sweep(&c, mu_new, eps_total, &so, &ms);
        if (rc)
            return rc;
        sweep_total += ms;
        rounds_total += so.rounds;
        rc = iter_post(c, so, it);
        if (rc)
            return rc;
    }
    BRR_CUDA(cudaEventRecord(c.ev[3], c.st));
    BRR_CUDA(cudaEventSynchronize(c.ev[3]));
    float tot = 0.f;
    BRR_CUDA(cudaEventElapsedTime(&tot, c.ev[2], c.ev[3]));
    c.last_sweep_ms = sweep_total;
    c.last_total_ms = tot;
    c.last_rounds = rounds_total;
    return BRR_OK;
}

int brr_sweep(brr_ctx *ctx, const uint32_t *order, const double *u, const double *z, brr_sweep_out *out)
{
    if (!ctx || !ctx->inited || !order || !u || !z || !out)
        return fail(BRR_ERR_ARG, "chain not initialised or null argument");
    brr_ctx &c = *ctx;
    const int64_t M = c.cfg.M;
    std::vector<uint8_t> seen(M, 0);
    for (int64_t q = 0; q < M; ++q) {
        if (order[q] >= (uint32_t)M || seen[order[q]])
            return fail(BRR_ERR_ARG, "order is not a permutation of 0..M-1");
        seen[order[q]] = 1;
    }
    BRR_CUDA(cudaSetDevice(c.dev));
    BRR_CUDA(cudaMemcpyAsync(c.d_order, order, sizeof(uint32_t) * M, cudaMemcpyHostToDevice, c.st));
    BRR_CUDA(cudaMemcpyAsync(c.d_u, u, sizeof(double) * M, cudaMemcpyHostToDevice, c.st));
    BRR_CUDA(cudaMemcpyAsync(c.d_z, z, sizeof(double) * M, cudaMemcpyHostToDevice, c.st));
    BRR_CUDA(cudaEventRecord(c.ev[2], c.st));
    std::memset(c.phase, 0, sizeof(c.phase));
    double esum = 0.0;
    if (c.cfg.kind == BRR_KIND_DENSE) {
        // current residual total (adding zero leaves the residual unchanged)
        BRR_CUDA(launch_mu_prep(c.cfg.form, c.cfg.N, 0.0, c.d_eps, c.d_eps_hi, c.d_eps_lo, c.d_part, kPartBlocks, c.st));
        BRR_CUDA(cudaMemcpyAsync(c.h_part, c.d_part, sizeof(double) * kPartBlocks, cudaMemcpyDeviceToHost, c.st));
        BRR_CUDA(cudaStreamSynchronize(c.st));
        for (int b = 0; b < kPartBlocks; ++b)
            esum += c.h_part[b];
    }
    float ms = 0.f;
    const int rc = run_sweep(&c, 0.0, esum, out, &ms);
    if (rc)
        return rc;
    BRR_CUDA(cudaEventRecord(c.ev[3], c.st));
    BRR_CUDA(cudaEventSynchronize(c.ev[3]));
    float tot = 0.f;
    BRR_CUDA(cudaEventElapsedTime(&tot, c.ev[2], c.ev[3]));
    c.last_sweep_ms = ms;
    c.last_total_ms = tot;
    c.last_rounds = out->rounds;
    return BRR_OK;
}

int brr_get_state(brr_ctx *ctx, brr_state *st)
{
    if (!ctx || !st || !ctx->inited)
        return fail(BRR_ERR_ARG, "chain not initialised");
    brr_ctx &c = *ctx;
    const int64_t M = c.cfg.M;
    BRR_CUDA(cudaStreamSynchronize(c.st));
    if (st->beta)
        BRR_CUDA(cudaMemcpy(st->beta, c.d_beta, sizeof(double) * M, cudaMemcpyDeviceToHost));
    if (st->comp)
        BRR_CUDA(cudaMemcpy(st->comp, c.d_comp, sizeof(int32_t) * M, cudaMemcpyDeviceToHost));
    if (st->acum)
        BRR_CUDA(cudaMemcpy(st->acum, c.d_acum, sizeof(double) * M, cudaMemcpyDeviceToHost));
    if (st->eps) {
        const int rc = download_eps(&c, st->eps);
        if (rc)
            return rc;
    }
    st->mu = c.mu;
    st->sigmaE = c.sigmaE;
    st->epsSum = c.epsSum;
    std::memcpy(st->sigmaG, c.sigmaG, sizeof(c.sigmaG));
    std::memcpy(st->pi, c.pi, sizeof(c.pi));
    st->iteration = c.iteration;
    return BRR_OK;
}

int brr_set_state(brr_ctx *ctx, const brr_state *st)
{
    if (!ctx || !st || !ctx->packed || !ctx->pheno || !st->beta || !st->comp || !st->acum || !st->eps)
        return fail(BRR_ERR_ARG, "pack and set the phenotype first; all state arrays are required");
    brr_ctx &c = *ctx;
    const int64_t M = c.cfg.M;
    BRR_CUDA(cudaStreamSynchronize(c.st));
    BRR_CUDA(cudaMemcpy(c.d_beta, st->beta, sizeof(double) * M, cudaMemcpyHostToDevice));
    BRR_CUDA(cudaMemcpy(c.d_comp, st->comp, sizeof(int32_t) * M, cudaMemcpyHostToDevice));
    BRR_CUDA(cudaMemcpy(c.d_acum, st->acum, sizeof(double) * M, cudaMemcpyHostToDevice));
    const int rc = upload_state_eps(&c, st->eps);
    if (rc)
        return rc;
    c.mu = st->mu;
    c.sigmaE = st->sigmaE;
    c.epsSum = st->epsSum;
    std::memcpy(c.sigmaG, st->sigmaG, sizeof(c.sigmaG));
    std::memcpy(c.pi, st->pi, sizeof(c.pi));
    c.iteration = st->iteration;
    c.last_nnz = -1;
    const int rb = prepare_blocked(&c);
    if (rb)
        return rb;
    c.inited = true;
    return BRR_OK;
}

int brr_refresh_eps(brr_ctx *ctx)
{
    if (!ctx || !ctx->inited)
        return fail(BRR_ERR_ARG, "chain not initialised");
    BRR_CUDA(cudaSetDevice(ctx->dev));
    return refresh_eps_impl(ctx);
}

int brr_get_timing(brr_ctx *ctx, double *sweep_ms, double *total_ms, int64_t *rounds)
{
    if (!ctx)
        return fail(BRR_ERR_ARG, "null context");
    if (sweep_ms)
        *sweep_ms = ctx->last_sweep_ms;
    if (total_ms)
        *total_ms = ctx->last_total_ms;
    if (rounds)
        *rounds = ctx->last_rounds;
    return BRR_OK;
}

int brr_synth_bed_device(uint8_t *d_bed, int64_t N, int64_t M, uint32_t seed, double p_lo, double p_hi,
                         double missing)
{
    if (!d_bed || N < 2 || M < 1 || !(p_lo > 0.0) || !(p_hi <= 0.5) || !(p_lo <= p_hi) || !(missing >= 0.0) ||
        !(missing < 0.5))
        return fail(BRR_ERR_ARG, "invalid synthetic genotype parameters");
    {
        // the generator writes M * ceil(N/4) bytes to d_bed on the current device
        int dev = 0;
        BRR_CUDA(cudaGetDevice(&dev));
        std::string why;
        if (!device_range_check(dev, d_bed, (size_t)(M * ((N + 3) / 4)), "d_bed", why))
            return fail(BRR_ERR_ARG, why);
    }
    BRR_CUDA(launch_synth_bed(d_bed, N, M, seed, p_lo, p_hi, missing, 0));
    BRR_CUDA(cudaDeviceSynchronize());
    return BRR_OK;
}

int brr_synth_bed_device_beta(uint8_t *d_bed, int64_t N, int64_t M, uint32_t seed, double a, double b, double p_lo,
                              double p_hi, double missing)
{
    if (!d_bed || N < 2 || M < 1 || !(a > 0.0) || !(b > 0.0) || !(p_lo > 0.0) || !(p_hi <= 0.5) ||
        !(p_lo <= p_hi) || !(missing >= 0.0) || !(missing < 0.5))
        return fail(BRR_ERR_ARG, "invalid synthetic genotype parameters");
    {
        // the generator writes M * ceil(N/4) bytes to d_bed on the current device
        int dev = 0;
        BRR_CUDA(cudaGetDevice(&dev));
        std::string why;
        if (!device_range_check(dev, d_bed, (size_t)(M * ((N + 3) / 4)), "d_bed", why))
            return fail(BRR_ERR_ARG, why);
    }
    BRR_CUDA(launch_synth_bed(d_bed, N, M, seed, p_lo, p_hi, missing, 0, a, b));
    BRR_CUDA(cudaDeviceSynchronize());
    return BRR_OK;
}

int brr_xbeta(brr_ctx *ctx, const uint32_t *idx, const double *b, int64_t n, double *out)
{
    if (!ctx || !ctx->packed || (n > 0 && (!idx || !b)) || !out || n < 0 || n > ctx->cfg.M)
        return fail(BRR_ERR_ARG, "pack markers first; idx/b/out required");
    brr_ctx &c = *ctx;
    const int64_t N = c.cfg.N;
    for (int64_t q = 0; q < n; ++q)
        if (idx[q] >= (uint32_t)c.cfg.M)
            return fail(BRR_ERR_ARG, "marker index out of range");
    BRR_CUDA(cudaSetDevice(c.dev));
    double *zero = nullptr, *res = nullptr;
    if (dalloc(&zero, (size_t)N) || dalloc(&res, (size_t)N)) {
        cudaFree(zero);
        return fail(BRR_ERR_OOM, "device allocation failed");
    }
    int rc = BRR_OK;
    cudaError_t e = cudaMemsetAsync(zero, 0, sizeof(double) * N, c.st);
    if (e == cudaSuccess && n > 0)
        e = cudaMemcpyAsync(c.d_nzj, idx, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, c.st);
    if (e == cudaSuccess && n > 0)
        e = cudaMemcpyAsync(c.d_nzb, b, sizeof(double) * n, cudaMemcpyHostToDevice, c.st);
    if (e == cudaSuccess)
        e = launch_refresh(BRR_FORM_FP64, c.kind, N, zero, 0.0, c.d_codes, c.col_stride, c.d_table, c.d_nzj,
                           c.d_nzb, n, res, nullptr, nullptr, c.st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, res, sizeof(double) * N, cudaMemcpyDeviceToHost, c.st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c.st);
    if (e != cudaSuccess)
        rc = fail(BRR_ERR_CUDA, cudaGetErrorString(e));
    cudaFree(zero);
    cudaFree(res);
    if (rc == BRR_OK)
        for (int64_t i = 0; i < N; ++i)
            out[i] = -out[i];
    return rc;
}

// Allocation-free variant of brr_xbeta for callers that cannot allocate
// device memory; the term list goes through the static array of
// brr_noalloc.cu and the result into the caller's device buffer, which is
// checked first (device memory of this context's GPU, N doubles long).
int brr_xbeta_noalloc(brr_ctx *ctx, const uint32_t *idx, const double *b, int64_t n, double *d_out)
{
    if (!ctx || !ctx->packed || !d_out || n < 0 || (n > 0 && (!idx || !b)))
        return fail(BRR_ERR_ARG, "pack markers first; idx/b (host) and d_out (device, N doubles) required");
    if (n > BRR_NOALLOC_MAX_TERMS)
        return fail(BRR_ERR_ARG, "brr_xbeta_noalloc takes at most " + std::to_string(BRR_NOALLOC_MAX_TERMS) +
                                     " terms (the size of its static device array); got " + std::to_string(n));
    for (int64_t q = 0; q < n; ++q)
        if (idx[q] >= (uint32_t)ctx->cfg.M)
            return fail(BRR_ERR_ARG, "marker index out of range");
    BRR_CUDA(cudaSetDevice(ctx->dev));
    std::string why;
    if (!noalloc_check_output(ctx->dev, d_out, sizeof(double) * (size_t)ctx->cfg.N, why))
        return fail(BRR_ERR_ARG, why);
    if (noalloc_xbeta(ctx->st, ctx->kind, ctx->cfg.N, ctx->d_codes, ctx->col_stride, ctx->d_table, idx, b, n, d_out,
                      why) != cudaSuccess)
        return fail(BRR_ERR_CUDA, why);
    return BRR_OK;
}

int brr_set_wait_limit(brr_ctx *ctx, uint64_t timeout_ns, int32_t phantom_arrivals)
{
    if (!ctx || timeout_ns == 0 || phantom_arrivals < 0)
        return fail(BRR_ERR_ARG, "invalid wait limit");
    ctx->wait_limit_ns = timeout_ns;
    ctx->phantom = phantom_arrivals;
    return BRR_OK;
}

int brr_get_gram_info(brr_ctx *ctx, int32_t *blocked, double *build_ms, int64_t *bytes)
{
    if (!ctx)
        return fail(BRR_ERR_ARG, "null context");
    if (blocked)
        *blocked = ctx->blocked ? 1 : 0;
    if (build_ms)
        *build_ms = ctx->gram_ms;
    if (bytes)
        *bytes = ctx->d_gram ? (int64_t)(ctx->cfg.M * (ctx->cfg.M - 1) / 2) * (int64_t)sizeof(float2) : 0;
    return BRR_OK;
}

int brr_get_gram_bits(brr_ctx *ctx, int32_t *bits)
{
    if (!ctx || !bits)
        return fail(BRR_ERR_ARG, "null argument");
    *bits = ctx->d_gram ? ctx->gram_bits : 0;
    return BRR_OK;
}

int brr_get_round_info(brr_ctx *ctx, int32_t *pair_rounds, int32_t *last_sweep_pair_rounds)
{
    if (!ctx)
        return fail(BRR_ERR_ARG, "null context");
    if (pair_rounds)
        *pair_rounds = ctx->pair_rounds && !ctx->blocked ? 1 : 0;
    if (last_sweep_pair_rounds)
        *last_sweep_pair_rounds = ctx->last_pair ? 1 : 0;
    return BRR_OK;
}

int brr_get_gram_entries(brr_ctx *ctx, const int64_t *j, const int64_t *k, int64_t n, double *out)
{
    if (!ctx || !j || !k || !out || n < 0)
        return fail(BRR_ERR_ARG, "null argument");
    if (!ctx->d_gram)
        return fail(BRR_ERR_ARG, "the chain holds no marker Gram");
    const int64_t M = ctx->cfg.M;
    for (int64_t i = 0; i < n; ++i)
        if (!(j[i] > k[i] && k[i] >= 0 && j[i] < M))
            return fail(BRR_ERR_ARG, "Gram entries need M > j > k >= 0");
    BRR_CUDA(cudaSetDevice(ctx->dev));
    BRR_CUDA(cudaStreamSynchronize(ctx->st));
    for (int64_t i = 0; i < n; ++i) {
        float2 v;
        BRR_CUDA(cudaMemcpy(&v, ctx->d_gram + j[i] * (j[i] - 1) / 2 + k[i], sizeof(float2), cudaMemcpyDeviceToHost));
        out[i] = (double)v.x + (double)v.y;
    }
    return BRR_OK;
}

int brr_set_profiling(brr_ctx *ctx, int32_t on)
{
    if (!ctx || on < 0 || on > 2)
        return fail(BRR_ERR_ARG, "profiling is 0, 1 or 2");
    if (on == 2 && !ctx->d_tline) {
        BRR_CUDA(cudaSetDevice(ctx->dev));
        const size_t n = (size_t)kTimelineIters * (size_t)ctx->sms * kTimelineEvents;
        if (cudaMalloc((void **)&ctx->d_tline, sizeof(unsigned long long) * n) != cudaSuccess) {
            cudaGetLastError();
            ctx->d_tline = nullptr;
            return fail(BRR_ERR_OOM, "device allocation failed");
        }
        BRR_CUDA(cudaMemset(ctx->d_tline, 0, sizeof(unsigned long long) * n));
    }
    ctx->profile = on != 0;
    ctx->timeline = on == 2;
    return BRR_OK;
}

int brr_get_sweep_timeline(brr_ctx *ctx, uint64_t *events, int64_t capacity, int32_t *iterations, int32_t *ctas)
{
    if (!ctx || !events || !iterations || !ctas)
        return fail(BRR_ERR_ARG, "null argument");
    if (!ctx->d_tline)
        return fail(BRR_ERR_ARG, "the timeline is recorded with brr_set_profiling(ctx, 2)");
    const int64_t n = (int64_t)kTimelineIters * ctx->G * kTimelineEvents;
    if (capacity < n)
        return fail(BRR_ERR_ARG, "the timeline needs " + std::to_string(n) + " values");
    if (ctx->G > ctx->sms)
        return fail(BRR_ERR_ARG, "more CTAs than the timeline holds");
    BRR_CUDA(cudaSetDevice(ctx->dev));
    BRR_CUDA(cudaStreamSynchronize(ctx->st));
    BRR_CUDA(cudaMemcpy(events, ctx->d_tline, sizeof(uint64_t) * (size_t)n, cudaMemcpyDeviceToHost));
    *iterations = kTimelineIters;
    *ctas = ctx->G;
    return BRR_OK;
}

int brr_get_phase_cycles(brr_ctx *ctx, int64_t *cycles)
{
    if (!ctx || !cycles)
        return fail(BRR_ERR_ARG, "null argument");
    for (int k = 0; k < 16; ++k)
        cycles[k] = ctx->phase[k];
    return BRR_OK;
}

}  // extern "C"
