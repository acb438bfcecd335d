// C ABI of the batched form: C chains with distinct seeds and phenotypes on
// shared genotypes, one shared marker order per iteration.  Per chain the
// iteration body is the reference's BayesRBase::runGibbs loop body
// (src/BayesRBase.cpp:186-247): updateMu, the per-marker draws, the sweep, the
// sigmaE draw and the per-group sigmaG / pi draws.  The sweep of all chains is
// one cooperative launch of k_sweep_batch (brr_batch.cu); the scalar draws run
// on the host from each chain's counter-based stream.
#include <cuda_runtime.h>

#include <algorithm>
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

#define BATCH_CUDA(call)                                                                                \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return api_fail(BRR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));          \
    } while (0)

template <class T>
cudaError_t balloc(T **p, size_t n)
{
    *p = nullptr;
    return cudaMalloc((void **)p, (n ? n : 1) * sizeof(T));
}

constexpr double kTwoF = (double)(1ll << kBatchFrac);
constexpr long long kEMax = 1ll << 43;   // four balanced 11-bit limbs

}  // namespace

struct brr_batch {
    brr_config cfg{};
    int C = 0, dev = 0, sms = 0, G = 0, kext = 0;
    int64_t col_stride = 0;
    std::vector<int32_t> slice_lo;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[4] = {};
    uint64_t wait_limit_ns = 2000000000ull;
    int phantom = 0;

    uint8_t *d_codes = nullptr;
    int64_t *d_counts = nullptr;
    double *d_lut = nullptr, *d_scale = nullptr, *d_colsum = nullptr;
    int32_t *d_slice_lo = nullptr, *d_group = nullptr, *d_gK = nullptr;
    uint32_t *d_order = nullptr;
    BatchRec *d_rec = nullptr;
    ChainRec *d_crec = nullptr;
    float *d_gcf = nullptr;
    float4 *d_gdf = nullptr;
    double *d_beta = nullptr, *d_acum = nullptr, *d_gconst = nullptr;
    int32_t *d_comp = nullptr;
    uint8_t *d_chosen = nullptr;
    long long *d_E = nullptr, *d_dmu = nullptr, *d_sumE = nullptr, *d_wx = nullptr, *d_prof = nullptr;
    unsigned long long *d_acc = nullptr, *d_counter = nullptr, *d_stats = nullptr;
    unsigned *d_pacc = nullptr;
    double *d_part = nullptr;
    int *d_err = nullptr;

    uint32_t *h_order = nullptr;
    std::vector<int32_t> group;
    std::vector<double> ystd;             // [C][N]
    std::vector<double> mu, sigmaE;       // [C]
    std::vector<double> sigmaG, pi;       // [C][BRR_MAX_GROUPS], [C][BRR_MAX_GROUPS*BRR_MAX_K]
    std::vector<long long> sumE;          // [C] exact residual totals
    uint32_t iteration = 0;
    bool packed = false, pheno = false, inited = false;
    std::vector<uint32_t> perm_next;
    std::future<void> perm_future;
    uint32_t perm_next_it = UINT32_MAX;
    double last_sweep_ms = 0.0, last_total_ms = 0.0;
    long long phase[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    bool profile = false;   // phase counters on (brr_batch_set_profiling)

    StreamKey key(int c) const { return StreamKey{cfg.seed, cfg.chain + (uint32_t)c}; }
};

namespace {

void free_batch(brr_batch *b)
{
    if (b->perm_future.valid())
        b->perm_future.wait();
    void *dev[] = {b->d_codes, b->d_counts, b->d_lut,  b->d_scale, b->d_colsum, b->d_slice_lo, b->d_group,
                   b->d_gK,    b->d_order,  b->d_rec,  b->d_crec,  b->d_gcf,    b->d_gdf,      b->d_beta,     b->d_acum,
                   b->d_gconst, b->d_comp,  b->d_chosen, b->d_E,    b->d_dmu,   b->d_sumE,   b->d_wx,       b->d_prof,
                   b->d_acc,   b->d_counter, b->d_stats, b->d_pacc, b->d_part,  b->d_err};
    for (void *p : dev)
        cudaFree(p);
    cudaFreeHost(b->h_order);
    for (auto &e : b->ev)
        if (e)
            cudaEventDestroy(e);
    if (b->st)
        cudaStreamDestroy(b->st);
}

template <class T>
void drop_dev(T *&p)
{
    cudaFree(p);
    p = nullptr;
}

// Releases the buffers the first pack call allocates and nulls their
// pointers, so that a call that ran out of memory part-way leaves the batch as
// before and a later call allocates them all again.
void release_pack_buffers(brr_batch *b)
{
    drop_dev(b->d_codes);
    drop_dev(b->d_counts);
    drop_dev(b->d_lut);
    drop_dev(b->d_scale);
    drop_dev(b->d_colsum);
    drop_dev(b->d_slice_lo);
    drop_dev(b->d_group);
    drop_dev(b->d_gK);
    drop_dev(b->d_order);
    drop_dev(b->d_rec);
    drop_dev(b->d_crec);
    drop_dev(b->d_gcf);
    drop_dev(b->d_gdf);
    drop_dev(b->d_beta);
    drop_dev(b->d_acum);
    drop_dev(b->d_comp);
    drop_dev(b->d_chosen);
    drop_dev(b->d_gconst);
    drop_dev(b->d_E);
    drop_dev(b->d_dmu);
    drop_dev(b->d_sumE);
    drop_dev(b->d_wx);
    drop_dev(b->d_prof);
    drop_dev(b->d_acc);
    drop_dev(b->d_counter);
    drop_dev(b->d_stats);
    drop_dev(b->d_pacc);
    drop_dev(b->d_part);
    drop_dev(b->d_err);
    cudaFreeHost(b->h_order);
    b->h_order = nullptr;
}

size_t acc_words(int C) { return (size_t)kBatchCopies * C * kBatchBlock; }
size_t pacc_words() { return (size_t)2 * kBatchPCopies * kBatchBlock * kBatchBlock; }
size_t stats_words(int C, int ng) { return (size_t)C * (ng * kMaxK + 2 * ng); }

// Sampler constants of chain c (src/BayesRBase.cpp:309-333), as in the
// single-chain driver, and their FP32 form for the certified sampler:
// {logL_k - logL_0 constant, h_k} per component.
void chain_constants(const brr_batch *b, int c, double *gc, float *gcf, float4 *gdf, int32_t *gK)
{
    const brr_config &cf = b->cfg;
    const double NM1 = (double)(cf.N - 1);
    const double sE = b->sigmaE[c];
    for (int g = 0; g < cf.n_groups; ++g) {
        const int K = cf.K[g];
        gK[g] = K;
        const double sigmaG = b->sigmaG[(size_t)c * BRR_MAX_GROUPS + g];
        const double *pi = &b->pi[((size_t)c * BRR_MAX_GROUPS + g) * BRR_MAX_K];
        const double sEsG = sE / sigmaG;
        const double logLScale = sigmaG / sE * NM1;
        double *row = gc + (size_t)g * kMaxK * 4;
        for (int k = 0; k < kMaxK * 4; ++k)
            row[k] = 0.0;
        row[0] = std::log(pi[0]);
        for (int k = 1; k < K; ++k) {
            const double cVa = cf.S[g * (BRR_MAX_K - 1) + (k - 1)];
            const double denom = NM1 + sEsG * (1.0 / cVa);
            row[4 * k + 0] = std::log(pi[k]) - 0.5 * std::log(logLScale * cVa + 1.0);
            row[4 * k + 1] = 1.0 / denom;
            row[4 * k + 2] = 0.5 / denom / sE;
            row[4 * k + 3] = std::sqrt(sE / denom);
        }
        float *frow = gcf + (size_t)g * kMaxK * 2;
        float4 *drow = gdf + (size_t)g * kMaxK;
        auto split = [](double v, float &h, float &l) {
            h = (float)v;
            l = (float)(v - (double)h);
        };
        for (int k = 0; k < kMaxK; ++k) {
            frow[2 * k] = (k == 0 || k >= K) ? 0.f : (float)(row[4 * k] - row[0]);
            frow[2 * k + 1] = (k == 0 || k >= K) ? 0.f : (float)row[4 * k + 2];
            float4 d4{0.f, 0.f, 0.f, 0.f};
            split(row[4 * k + 3], d4.x, d4.y);
            split(row[4 * k + 1], d4.z, d4.w);
            drow[k] = d4;
        }
    }
}

void schedule_perm(brr_batch *b, uint32_t it)
{
    if (b->perm_future.valid())
        b->perm_future.wait();
    b->perm_next.resize(b->cfg.M);
    b->perm_next_it = it;
    const StreamKey k = b->key(0);
    const uint32_t M = (uint32_t)b->cfg.M;
    uint32_t *dst = b->perm_next.data();
    b->perm_future = std::async(std::launch::async, [k, it, M, dst]() { make_permutation(k, it, M, dst); });
}

int check_batch_status(brr_batch *b)
{
    int h = 0;
    BATCH_CUDA(cudaMemcpyAsync(&h, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->st));
    BATCH_CUDA(cudaStreamSynchronize(b->st));
    if (h == kDevTimeout)
        return api_fail(BRR_ERR_TIMEOUT, "a grid barrier or tensor-core wait of the batched sweep exceeded its limit");
    if (h == kDevRange)
        return api_fail(BRR_ERR_RANGE, "a residual left the fixed-point range of the batched sweep (|eps| < 8)");
    return BRR_OK;
}

}  // namespace

extern "C" {

int brr_batch_create(const brr_config *cfg, int32_t chains, brr_batch **out)
{
    if (!cfg || !out)
        return api_fail(BRR_ERR_ARG, "null argument");
    *out = nullptr;
    const brr_config &c = *cfg;
    if (c.N < 2 || c.M < 1 || c.M > (int64_t)UINT32_MAX || c.N > (int64_t)INT_MAX)
        return api_fail(BRR_ERR_ARG, "need N >= 2 individuals and 1 <= M < 2^32 markers");
    if (c.kind != BRR_KIND_DENSE)
        return api_fail(BRR_ERR_ARG, "the batched form runs dense markers");
    if (chains != 32 && chains != 64)
        return api_fail(BRR_ERR_ARG, "the batched form runs 32 or 64 chains");
    if (c.async_batch != 0)
        return api_fail(BRR_ERR_ARG, "the batched form runs the synchronous schedule");
    if (c.cluster != 0)
        return api_fail(BRR_ERR_ARG, "the batched form runs on the whole GPU, not as one cluster");
    if (c.n_groups < 1 || c.n_groups > BRR_MAX_GROUPS)
        return api_fail(BRR_ERR_ARG, "n_groups must be in 1..64");
    for (int g = 0; g < c.n_groups; ++g) {
        if (c.K[g] < 2 || c.K[g] > BRR_MAX_K)
            return api_fail(BRR_ERR_ARG, "every group needs 2..16 mixture components");
        for (int k = 0; k + 1 < c.K[g]; ++k)
            if (!(c.S[g * (BRR_MAX_K - 1) + k] > 0.0))
                return api_fail(BRR_ERR_ARG, "variance ratios S must be positive");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return api_fail(BRR_ERR_DEVICE, "no CUDA device");
    if (c.device < 0 || c.device >= ndev)
        return api_fail(BRR_ERR_DEVICE, "device ordinal out of range");
    cudaDeviceProp prop;
    BATCH_CUDA(cudaGetDeviceProperties(&prop, c.device));
    if (prop.major != 10 || prop.minor != 3)
        return api_fail(BRR_ERR_DEVICE, std::string("libbrr_gpu is built for sm_103a only; device is ") + prop.name);

    brr_batch *b = new brr_batch();
    b->cfg = c;
    b->C = chains;
    b->dev = c.device;
    b->sms = prop.multiProcessorCount;
    cudaError_t e = cudaSetDevice(c.device);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i)
        e = cudaEventCreate(&b->ev[i]);
    if (e != cudaSuccess) {
        free_batch(b);
        delete b;
        return api_fail(BRR_ERR_CUDA, cudaGetErrorString(e));
    }
    // slices of 16-individual chunks (4 bytes of codes), one CTA each
    const int64_t chunks = (c.N + 15) / 16;
    int G = c.grid > 0 ? c.grid : b->sms;
    G = (int)std::min<int64_t>(G, chunks);
    b->G = G;
    b->slice_lo.resize(G + 1);
    int64_t maxch = 0;
    for (int s = 0; s <= G; ++s) {
        const int64_t ch = (int64_t)s * chunks / G;
        b->slice_lo[s] = (int32_t)std::min<int64_t>(ch * 16, c.N);
        if (s > 0)
            maxch = std::max<int64_t>(maxch, ch - (int64_t)(s - 1) * chunks / G);
    }
    b->kext = (int)(maxch * 16);
    b->col_stride = 16 * ((c.N + 63) / 64);
    const size_t smem = batch_smem_bytes(chains, b->kext, G);
    const int per_sm = smem <= (size_t)prop.sharedMemPerBlockOptin ? batch_max_ctas_per_sm(chains, b->kext, smem) : 0;
    if (per_sm < 1 || (int64_t)per_sm * b->sms < G) {
        // shared memory per individual of a slice: genotypes 64 B, residual limbs 8 B per chain, codes 8 B
        const int64_t fixed = 256 * (int64_t)chains + 2048;
        const int64_t per_ind = 72 + 8 * (int64_t)chains;
        const int64_t cap = (int64_t)b->sms * (((int64_t)prop.sharedMemPerBlockOptin - fixed) / per_ind / 16 * 16);
        free_batch(b);
        delete b;
        return api_fail(BRR_ERR_ARG, "the batched sweep does not fit: " + std::to_string(smem) +
                                         " bytes of shared memory per CTA for " + std::to_string(chains) +
                                         " chains over slices of " + std::to_string(maxch * 16) +
                                         " individuals (at most about " + std::to_string(cap) + " individuals)");
    }
    *out = b;
    return BRR_OK;
}

int brr_batch_destroy(brr_batch *b)
{
    if (!b)
        return BRR_OK;
    cudaSetDevice(b->dev);
    free_batch(b);
    delete b;
    return BRR_OK;
}

int brr_batch_pack_bed_device(brr_batch *b, const uint8_t *d_bed, int64_t nbytes)
{
    if (!b || !d_bed)
        return api_fail(BRR_ERR_ARG, "null argument");
    const brr_config &cf = b->cfg;
    const int64_t M = cf.M, C = b->C;
    if (nbytes != M * ((cf.N + 3) / 4))
        return api_fail(BRR_ERR_ARG, "BED payload size does not match M*ceil(N/4)");
    BATCH_CUDA(cudaSetDevice(b->dev));
    {
        // the packer reads nbytes from d_bed: refuse a buffer it would overrun
        std::string why;
        if (!device_range_check(b->dev, d_bed, (size_t)nbytes, "d_bed", why))
            return api_fail(BRR_ERR_ARG, why);
    }
    if (!b->d_codes) {
        if (balloc(&b->d_codes, (size_t)(M * b->col_stride)) || balloc(&b->d_counts, (size_t)M * 4) ||
            balloc(&b->d_lut, (size_t)M * 4) || balloc(&b->d_scale, (size_t)M * 2) || balloc(&b->d_colsum, (size_t)M) ||
            balloc(&b->d_slice_lo, (size_t)b->G + 1) || balloc(&b->d_group, (size_t)M) ||
            balloc(&b->d_gK, (size_t)kMaxGroups) || balloc(&b->d_order, (size_t)M) || balloc(&b->d_rec, (size_t)M) ||
            balloc(&b->d_crec, (size_t)(C * M)) || balloc(&b->d_gcf, (size_t)C * cf.n_groups * kMaxK * 2) ||
            balloc(&b->d_gdf, (size_t)C * cf.n_groups * kMaxK) ||
            balloc(&b->d_beta, (size_t)(C * M)) ||
            balloc(&b->d_acum, (size_t)(C * M)) || balloc(&b->d_comp, (size_t)(C * M)) ||
            balloc(&b->d_chosen, (size_t)(C * M)) ||
            balloc(&b->d_gconst, (size_t)C * cf.n_groups * kMaxK * 4) || balloc(&b->d_E, (size_t)(C * cf.N)) ||
            balloc(&b->d_dmu, (size_t)C) || balloc(&b->d_sumE, (size_t)C) ||
            balloc(&b->d_wx, (size_t)C * (kBatchBlock + 1)) || balloc(&b->d_prof, 8) ||
            balloc(&b->d_acc, acc_words(b->C)) || balloc(&b->d_counter, 64) ||
            balloc(&b->d_stats, stats_words(b->C, cf.n_groups)) || balloc(&b->d_pacc, pacc_words()) ||
            balloc(&b->d_part, (size_t)b->G * C * 2) || balloc(&b->d_err, 1) ||
            cudaMallocHost((void **)&b->h_order, sizeof(uint32_t) * M) != cudaSuccess) {
            cudaGetLastError();
            release_pack_buffers(b);
            return api_fail(BRR_ERR_OOM, "device allocation for the batched chains failed");
        }
        BATCH_CUDA(cudaMemset(b->d_group, 0, sizeof(int32_t) * M));
        b->group.assign(M, 0);
    }
    BATCH_CUDA(cudaMemcpy(b->d_slice_lo, b->slice_lo.data(), sizeof(int32_t) * (b->G + 1), cudaMemcpyHostToDevice));
    BATCH_CUDA(launch_pack_counts(d_bed, cf.N, M, b->d_codes, b->col_stride, b->d_counts, b->st));
    int *d_bad = nullptr;
    if (balloc(&d_bad, 1))
        return api_fail(BRR_ERR_OOM, "device allocation failed");
    const int big = INT_MAX;
    int bad = INT_MAX;
    cudaError_t le = cudaMemcpy(d_bad, &big, sizeof(int), cudaMemcpyHostToDevice);
    if (le == cudaSuccess)
        le = launch_dense_tables(b->d_counts, cf.N, M, b->d_lut, b->d_scale, b->d_colsum, d_bad, b->st);
    if (le == cudaSuccess)
        le = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, b->st);
    if (le == cudaSuccess)
        le = cudaStreamSynchronize(b->st);
    cudaFree(d_bad);
    if (le != cudaSuccess)
        return api_fail(BRR_ERR_CUDA, std::string("marker statistics: ") + cudaGetErrorString(le));
    BATCH_CUDA(cudaGetLastError());
    if (bad != INT_MAX)
        return api_fail(BRR_ERR_MARKER, "marker " + std::to_string(bad) +
                                            " does not vary or is all missing; SNPs that do not vary should be "
                                            "removed prior to analysis");
    std::vector<int64_t> cnt((size_t)M * 4);
    BATCH_CUDA(cudaMemcpy(cnt.data(), b->d_counts, sizeof(int64_t) * M * 4, cudaMemcpyDeviceToHost));
    for (int64_t j = 0; j < M; ++j)
        if (cnt[4 * j + 3] != 0)
            return api_fail(BRR_ERR_ARG, "marker " + std::to_string(j) +
                                             " has missing genotypes; the batched form runs complete genotypes");
    b->packed = true;
    return BRR_OK;
}

int brr_batch_pack_bed(brr_batch *b, const uint8_t *bed, int64_t nbytes)
{
    if (!b || !bed)
        return api_fail(BRR_ERR_ARG, "null argument");
    BATCH_CUDA(cudaSetDevice(b->dev));
    uint8_t *d = nullptr;
    if (balloc(&d, (size_t)nbytes))
        return api_fail(BRR_ERR_OOM, "device allocation of the BED payload failed");
    cudaError_t e = cudaMemcpy(d, bed, (size_t)nbytes, cudaMemcpyHostToDevice);
    int rc = e == cudaSuccess ? brr_batch_pack_bed_device(b, d, nbytes)
                              : api_fail(BRR_ERR_CUDA, std::string("BED upload: ") + cudaGetErrorString(e));
    cudaFree(d);
    return rc;
}

int brr_batch_set_groups(brr_batch *b, const int32_t *group)
{
    if (!b || !group || !b->packed)
        return api_fail(BRR_ERR_ARG, "pack markers before setting groups");
    for (int64_t j = 0; j < b->cfg.M; ++j)
        if (group[j] < 0 || group[j] >= b->cfg.n_groups)
            return api_fail(BRR_ERR_ARG, "group id out of range at marker " + std::to_string(j));
    b->group.assign(group, group + b->cfg.M);
    BATCH_CUDA(cudaMemcpy(b->d_group, group, sizeof(int32_t) * b->cfg.M, cudaMemcpyHostToDevice));
    return BRR_OK;
}

// One phenotype per chain (chain-major, C x N values), each standardised as
// BayesRBase::init does (src/BayesRBase.cpp:85-86).
int brr_batch_set_phenotypes(brr_batch *b, const float *y)
{
    if (!b || !y || !b->packed)
        return api_fail(BRR_ERR_ARG, "pack markers before setting the phenotypes");
    const int64_t N = b->cfg.N;
    b->ystd.assign((size_t)b->C * N, 0.0);
    for (int c = 0; c < b->C; ++c) {
        const float *yc = y + (size_t)c * N;
        double ysum = 0.0;
        for (int64_t i = 0; i < N; ++i) {
            if (!std::isfinite(yc[i]))
                return api_fail(BRR_ERR_ARG, "phenotype " + std::to_string(c) + " value " + std::to_string(i) +
                                                 " is not finite");
            ysum += (double)yc[i];
        }
        const double ymean = ysum / (double)N;
        double sq = 0.0;
        for (int64_t i = 0; i < N; ++i) {
            const double d = (double)yc[i] - ymean;
            sq += d * d;
        }
        if (!(sq > 0.0))
            return api_fail(BRR_ERR_ARG, "phenotype " + std::to_string(c) + " has zero variance");
        const double scale = std::sqrt(sq / (double)(N - 1));
        for (int64_t i = 0; i < N; ++i)
            b->ystd[(size_t)c * N + i] = ((double)yc[i] - ymean) / scale;
    }
    b->pheno = true;
    return BRR_OK;
}

// BayesRBase::init per chain (src/BayesRBase.cpp:39-99).
int brr_batch_init(brr_batch *b)
{
    if (!b || !b->packed || !b->pheno)
        return api_fail(BRR_ERR_ARG, "pack markers and set the phenotypes before init");
    const brr_config &cf = b->cfg;
    const int64_t N = cf.N, M = cf.M;
    const int C = b->C;
    BATCH_CUDA(cudaSetDevice(b->dev));
    b->mu.assign(C, 0.0);
    b->sigmaE.assign(C, 0.0);
    b->sigmaG.assign((size_t)C * BRR_MAX_GROUPS, 0.0);
    b->pi.assign((size_t)C * BRR_MAX_GROUPS * BRR_MAX_K, 0.0);
    b->sumE.assign(C, 0);
    std::vector<long long> E((size_t)C * N);
    for (int c = 0; c < C; ++c) {
        for (int g = 0; g < cf.n_groups; ++g) {
            const int K = cf.K[g];
            double *pi = &b->pi[((size_t)c * BRR_MAX_GROUPS + g) * BRR_MAX_K];
            for (int k = 0; k < K; ++k)
                pi[k] = 0.5 / (double)K;
            pi[0] = 0.5;
            b->sigmaG[(size_t)c * BRR_MAX_GROUPS + g] = uniform_init(b->key(c), (uint32_t)g);
        }
        double esq = 0.0;
        long long se = 0;
        for (int64_t i = 0; i < N; ++i) {
            const double e = b->ystd[(size_t)c * N + i];
            esq += e * e;
            const long long x = llrint(e * kTwoF);
            if (x <= -kEMax || x >= kEMax)
                return api_fail(BRR_ERR_RANGE, "a standardised phenotype value is outside the batched form's range");
            E[(size_t)c * N + i] = x;
            se += x;
        }
        b->sigmaE[c] = esq / (double)N * 0.5;
        b->sumE[c] = se;
    }
    BATCH_CUDA(cudaMemcpy(b->d_E, E.data(), sizeof(long long) * E.size(), cudaMemcpyHostToDevice));
    BATCH_CUDA(cudaMemset(b->d_beta, 0, sizeof(double) * C * M));
    BATCH_CUDA(cudaMemset(b->d_acum, 0, sizeof(double) * C * M));
    BATCH_CUDA(cudaMemset(b->d_comp, 0, sizeof(int32_t) * C * M));
    b->iteration = 0;
    b->inited = true;
    return BRR_OK;
}

int brr_batch_iterate(brr_batch *b, int32_t n_iter)
{
    if (!b || !b->inited)
        return api_fail(BRR_ERR_ARG, "batch not initialised");
    const brr_config &cf = b->cfg;
    const int64_t N = cf.N, M = cf.M;
    const int C = b->C, ng = cf.n_groups;
    const double Nd = (double)N;
    BATCH_CUDA(cudaSetDevice(b->dev));
    int kmax = 2;
    for (int g = 0; g < ng; ++g)
        kmax = std::max(kmax, cf.K[g]);
    std::vector<double> gc((size_t)C * ng * kMaxK * 4);
    std::vector<float> gcf((size_t)C * ng * kMaxK * 2);
    std::vector<float4> gdf((size_t)C * ng * kMaxK);
    std::vector<int32_t> gK(ng);
    std::vector<long long> dmu(C);
    std::vector<double> part((size_t)b->G * C * 2);
    std::vector<unsigned long long> stats(stats_words(C, ng));
    std::vector<long long> sumE_dev(C);
    double sweep_total = 0.0;
    std::memset(b->phase, 0, sizeof(b->phase));
    BATCH_CUDA(cudaEventRecord(b->ev[2], b->st));
    if (b->perm_next_it != b->iteration)
        schedule_perm(b, b->iteration);
    for (int32_t n = 0; n < n_iter; ++n) {
        const uint32_t it = b->iteration;
        // updateMu per chain (src/DenseBayesRRmz.cpp:36-42) on the exact residual total
        for (int c = 0; c < C; ++c) {
            const double mean = (double)b->sumE[c] / kTwoF / Nd + b->mu[c];
            const double mu_new = mean + std::sqrt(b->sigmaE[c] / Nd) * normal_mu(b->key(c), it);
            dmu[c] = llrint((b->mu[c] - mu_new) * kTwoF);
            b->sumE[c] += (long long)N * dmu[c];
            b->mu[c] = mu_new;
        }
        // the shared permutation and every chain's per-marker draws, laid out
        // in sweep order with beta_old (src/BayesRBase.cpp:196-198)
        b->perm_future.wait();
        std::memcpy(b->h_order, b->perm_next.data(), sizeof(uint32_t) * M);
        BATCH_CUDA(cudaMemcpyAsync(b->d_order, b->h_order, sizeof(uint32_t) * M, cudaMemcpyHostToDevice, b->st));
        BATCH_CUDA(launch_batch_draws(cf.seed, cf.chain, it, M, C, b->d_order, b->d_beta, b->d_crec, b->st));
        for (int c = 0; c < C; ++c)
            chain_constants(b, c, gc.data() + (size_t)c * ng * kMaxK * 4, gcf.data() + (size_t)c * ng * kMaxK * 2,
                            gdf.data() + (size_t)c * ng * kMaxK, gK.data());
        BATCH_CUDA(cudaMemcpyAsync(b->d_gconst, gc.data(), sizeof(double) * gc.size(), cudaMemcpyHostToDevice, b->st));
        BATCH_CUDA(cudaMemcpyAsync(b->d_gcf, gcf.data(), sizeof(float) * gcf.size(), cudaMemcpyHostToDevice, b->st));
        BATCH_CUDA(cudaMemcpyAsync(b->d_gdf, gdf.data(), sizeof(float4) * gdf.size(), cudaMemcpyHostToDevice, b->st));
        BATCH_CUDA(cudaMemcpyAsync(b->d_gK, gK.data(), sizeof(int32_t) * ng, cudaMemcpyHostToDevice, b->st));
        BATCH_CUDA(cudaMemcpyAsync(b->d_dmu, dmu.data(), sizeof(long long) * C, cudaMemcpyHostToDevice, b->st));
        BATCH_CUDA(cudaMemcpyAsync(b->d_sumE, b->sumE.data(), sizeof(long long) * C, cudaMemcpyHostToDevice, b->st));
        BATCH_CUDA(launch_batch_gather(b->d_order, M, b->d_scale, b->d_counts, b->d_group, b->d_rec, b->st));
        BATCH_CUDA(cudaMemsetAsync(b->d_acc, 0, sizeof(unsigned long long) * acc_words(C), b->st));
        BATCH_CUDA(cudaMemsetAsync(b->d_pacc, 0, sizeof(unsigned) * pacc_words(), b->st));
        BATCH_CUDA(cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned long long) * 64, b->st));
        BATCH_CUDA(cudaMemsetAsync(b->d_err, 0, sizeof(int), b->st));
        BATCH_CUDA(cudaMemsetAsync(b->d_prof, 0, sizeof(long long) * 8, b->st));
        schedule_perm(b, it + 1);

        BatchArgs a{};
        a.N = N;
        a.M = M;
        a.G = b->G;
        a.C = C;
        a.kext = b->kext;
        a.n_groups = ng;
        a.slice_lo = b->d_slice_lo;
        a.codes = b->d_codes;
        a.col_stride = b->col_stride;
        a.rec = b->d_rec;
        a.gconst = b->d_gconst;
        a.gcf = b->d_gcf;
        a.gdf = b->d_gdf;
        a.gK = b->d_gK;
        a.crec = b->d_crec;
        a.beta = b->d_beta;
        a.acum = b->d_acum;
        a.comp = b->d_comp;
        a.chosen = b->d_chosen;
        a.E = b->d_E;
        a.dmu = b->d_dmu;
        a.sumE = b->d_sumE;
        a.acc = b->d_acc;
        a.pacc = b->d_pacc;
        a.wx = b->d_wx;
        a.counter = b->d_counter;
        a.part = b->d_part;
        a.err = b->d_err;
        a.timeout_ns = b->wait_limit_ns;
        a.phantom = b->phantom;
        a.prof = b->profile ? b->d_prof : nullptr;
        BATCH_CUDA(cudaEventRecord(b->ev[0], b->st));
        BATCH_CUDA(launch_sweep_batch(a, kmax, b->st));
        BATCH_CUDA(cudaEventRecord(b->ev[1], b->st));
        BATCH_CUDA(cudaMemsetAsync(b->d_stats, 0, sizeof(unsigned long long) * stats.size(), b->st));
        BATCH_CUDA(launch_batch_stats(M, C, b->d_group, b->d_comp, b->d_chosen, b->d_beta, ng, b->d_stats, b->st));
        BATCH_CUDA(cudaMemcpyAsync(stats.data(), b->d_stats, sizeof(unsigned long long) * stats.size(),
                                   cudaMemcpyDeviceToHost, b->st));
        BATCH_CUDA(cudaMemcpyAsync(part.data(), b->d_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, b->st));
        BATCH_CUDA(cudaMemcpyAsync(sumE_dev.data(), b->d_sumE, sizeof(long long) * C, cudaMemcpyDeviceToHost, b->st));
        long long prof[8];
        BATCH_CUDA(cudaMemcpyAsync(prof, b->d_prof, sizeof(prof), cudaMemcpyDeviceToHost, b->st));
        const int rc = check_batch_status(b);
        if (rc)
            return rc;
        float ms = 0.f;
        BATCH_CUDA(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
        sweep_total += ms;
        for (int k = 0; k < 8; ++k)
            b->phase[k] += prof[k];

        // per chain: the residual total from the slices must equal the one the
        // resolve carried (both exact), then sigmaE, sigmaG and pi
        for (int c = 0; c < C; ++c) {
            long long se = 0;
            double sq = 0.0;
            for (int s = 0; s < b->G; ++s) {
                long long v;
                std::memcpy(&v, &part[((size_t)s * C + c) * 2], sizeof v);
                se += v;
                sq += part[((size_t)s * C + c) * 2 + 1];
            }
            if (se != sumE_dev[c])
                return api_fail(BRR_ERR_RANGE, "batched sweep: residual total of chain " + std::to_string(c) +
                                                   " differs from the carried total");
            b->sumE[c] = se;
            const StreamKey k = b->key(c);
            if (!inv_scaled_chisq(k, it, kPurposeSigmaE, 0, cf.v0E + Nd, (sq + cf.v0E * cf.s02E) / (cf.v0E + Nd),
                                  &b->sigmaE[c]))
                return api_fail(BRR_ERR_STREAM, "sigmaE gamma draw exceeded its attempt cap");
            const unsigned long long *so = stats.data() + (size_t)c * (ng * kMaxK + 2 * ng);
            for (int g = 0; g < ng; ++g) {
                const int K = cf.K[g];
                double v[BRR_MAX_K], vs = 0.0;
                for (int kk = 0; kk < K; ++kk) {
                    v[kk] = (double)so[g * kMaxK + kk];
                    vs += v[kk];
                }
                const double m0 = vs - v[0];
                const double bsq = fx_join((long long)so[ng * kMaxK + 2 * g], so[ng * kMaxK + 2 * g + 1]);
                if (!inv_scaled_chisq(k, it, kPurposeSigmaG, (uint32_t)g, cf.v0G + m0,
                                      (bsq * m0 + cf.v0G * cf.s02G) / (cf.v0G + m0),
                                      &b->sigmaG[(size_t)c * BRR_MAX_GROUPS + g]))
                    return api_fail(BRR_ERR_STREAM, "sigmaG gamma draw exceeded its attempt cap");
                double r[BRR_MAX_K], rs = 0.0;
                for (int kk = 0; kk < K; ++kk) {
                    double gk;
                    if (!gamma_draw(k, it, kPurposePi, (uint32_t)(g * 256 + kk), v[kk] + 1.0, &gk))
                        return api_fail(BRR_ERR_STREAM, "Dirichlet gamma draw exceeded its attempt cap");
                    r[kk] = gk;
                    rs += gk;
                }
                for (int kk = 0; kk < K; ++kk)
                    b->pi[((size_t)c * BRR_MAX_GROUPS + g) * BRR_MAX_K + kk] = r[kk] / rs;
            }
        }
        b->iteration = it + 1;
    }
    BATCH_CUDA(cudaEventRecord(b->ev[3], b->st));
    BATCH_CUDA(cudaEventSynchronize(b->ev[3]));
    float tot = 0.f;
    BATCH_CUDA(cudaEventElapsedTime(&tot, b->ev[2], b->ev[3]));
    b->last_sweep_ms = sweep_total;
    b->last_total_ms = tot;
    return BRR_OK;
}

int brr_batch_get_chain_state(brr_batch *b, int32_t chain, brr_state *st)
{
    if (!b || !st || !b->inited || chain < 0 || chain >= b->C)
        return api_fail(BRR_ERR_ARG, "batch not initialised or chain out of range");
    const int64_t N = b->cfg.N, M = b->cfg.M;
    BATCH_CUDA(cudaSetDevice(b->dev));
    BATCH_CUDA(cudaStreamSynchronize(b->st));
    const size_t off = (size_t)chain * M;
    if (st->beta)
        BATCH_CUDA(cudaMemcpy(st->beta, b->d_beta + off, sizeof(double) * M, cudaMemcpyDeviceToHost));
    if (st->comp)
        BATCH_CUDA(cudaMemcpy(st->comp, b->d_comp + off, sizeof(int32_t) * M, cudaMemcpyDeviceToHost));
    if (st->acum)
        BATCH_CUDA(cudaMemcpy(st->acum, b->d_acum + off, sizeof(double) * M, cudaMemcpyDeviceToHost));
    if (st->eps) {
        std::vector<long long> E(N);
        BATCH_CUDA(cudaMemcpy(E.data(), b->d_E + (size_t)chain * N, sizeof(long long) * N, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < N; ++i)
            st->eps[i] = (double)E[i] / kTwoF;
    }
    st->mu = b->mu[chain];
    st->sigmaE = b->sigmaE[chain];
    st->epsSum = (double)b->sumE[chain] / kTwoF;
    for (int g = 0; g < BRR_MAX_GROUPS; ++g)
        st->sigmaG[g] = b->sigmaG[(size_t)chain * BRR_MAX_GROUPS + g];
    for (int k = 0; k < BRR_MAX_GROUPS * BRR_MAX_K; ++k)
        st->pi[k] = b->pi[(size_t)chain * BRR_MAX_GROUPS * BRR_MAX_K + k];
    st->iteration = b->iteration;
    return BRR_OK;
}

int brr_batch_get_timing(brr_batch *b, double *sweep_ms, double *total_ms, int64_t *cycles)
{
    if (!b)
        return api_fail(BRR_ERR_ARG, "null batch");
    if (sweep_ms)
        *sweep_ms = b->last_sweep_ms;
    if (total_ms)
        *total_ms = b->last_total_ms;
    if (cycles)
        for (int k = 0; k < 8; ++k)
            cycles[k] = b->phase[k];
    return BRR_OK;
}

int brr_batch_set_profiling(brr_batch *b, int32_t on)
{
    if (!b || (on != 0 && on != 1))
        return api_fail(BRR_ERR_ARG, "profiling is 0 or 1");
    b->profile = on != 0;
    return BRR_OK;
}

int brr_batch_set_wait_limit(brr_batch *b, uint64_t timeout_ns, int32_t phantom_arrivals)
{
    if (!b || timeout_ns == 0 || phantom_arrivals < 0)
        return api_fail(BRR_ERR_ARG, "null batch, zero limit or negative phantom arrivals");
    b->wait_limit_ns = timeout_ns;
    b->phantom = phantom_arrivals;
    return BRR_OK;
}

int brr_batch_get_geometry(brr_batch *b, int32_t *ctas, int32_t *slice, int64_t *smem_bytes)
{
    if (!b)
        return api_fail(BRR_ERR_ARG, "null batch");
    if (ctas)
        *ctas = b->G;
    if (slice)
        *slice = b->kext;
    if (smem_bytes)
        *smem_bytes = (int64_t)batch_smem_bytes(b->C, b->kext, b->G);
    return BRR_OK;
}

}  // extern "C"
