// The single-chain context behind brr_ctx and the phases of one iteration that
// the multi-instance driver (brr_multi_api.cu) reuses.
#pragma once
#include <future>
#include <vector>

#include "brr_device.cuh"
#include "brr_internal.h"
#include "brr_stream.h"

struct brr_ctx {
    brr_config cfg{};
    int dev = 0;
    int sms = 0;
    cudaStream_t st = nullptr;
    int G = 0;
    int B = 16;
    int64_t chunks = 0;
    int64_t col_stride = 0;
    int slice_max = 0;
    int slot_bytes = 0;
    std::vector<int32_t> slice_lo;
    bool packed = false, pheno = false, inited = false;

    // device buffers
    int32_t *d_slice_lo = nullptr;
    uint8_t *d_codes = nullptr;
    int64_t *d_counts = nullptr;
    double *d_table = nullptr;
    double *d_scale = nullptr;
    double *d_colsum = nullptr;
    uint8_t *d_chosen = nullptr;
    unsigned long long *d_vstat = nullptr;   // sweep statistics: counts, fixed-point square sums
    int32_t *d_roff = nullptr;          // 3 x (M*G+1)
    uint16_t *d_ridx[3] = {nullptr, nullptr, nullptr};
    int64_t rtot[3] = {0, 0, 0};
    int32_t *d_group = nullptr;
    double *d_ystd = nullptr;
    double *d_beta = nullptr;
    int32_t *d_comp = nullptr;
    double *d_acum = nullptr;
    double *d_eps = nullptr;
    float *d_eps_hi = nullptr, *d_eps_lo = nullptr;
    uint32_t *d_order = nullptr;
    double *d_u = nullptr, *d_z = nullptr;
    brr::SweepRec *d_rec = nullptr;
    unsigned long long *d_acc = nullptr;   // accumulators followed by the counter
    double *d_gconst = nullptr;
    int32_t *d_gK = nullptr;
    double *d_stats = nullptr;
    double *d_part = nullptr;
    int *d_err = nullptr;
    long long *d_rounds = nullptr;
    long long *d_prof = nullptr;        // per-phase cycles of the last sweep (CTA 0)
    uint32_t *d_nzj = nullptr;
    double *d_nzb = nullptr;
    float2 *d_gram = nullptr;           // blocked FP32C: packed marker Gram (double-float entries)
    double *d_eps_dl = nullptr;         // FP32C: the residual as doubles for its read-back (allocated on use)
    double *d_gstage = nullptr;         // blocked FP32C: staged Gram entries (8 blocks)
    brr::BlockRec *d_brec = nullptr;         // blocked FP32C: records in sweep order
    float2 *d_bdf = nullptr;            // blocked FP32C: [2][M] new beta, acum (double-float)
    bool blocked = false;
    bool pair_rounds = false;   // FP32C restart sweep: pair-resolved rounds available (pair terms in
                                // d_acc + kPairOffset)
    bool last_pair = false;     // the last sweep took pair-resolved rounds
    int gram_bits = 0;          // element bits of the marker Gram's GEMM operands (FP4, FP8 or BF16)
    int64_t last_nnz = -1;      // markers in a non-zero component after the last sweep (-1: not known)
    bool has_missing = false;
    int kind = BRR_KIND_DENSE;          // storage: dense codes, or ragged lists (Ragged and Eigen markers)
    bool eigen = false;                 // Eigen sparse markers (BRR_KIND_EIGEN)
    double gram_ms = 0.0;

    // pinned host staging
    uint32_t *h_order = nullptr;
    double *h_stats = nullptr;
    double *h_part = nullptr;
    double *h_gc = nullptr;               // sampler constants for the next sweep
    int32_t *h_gK = nullptr;
    unsigned long long *h_vstat = nullptr;   // sweep statistics read back
    long long *h_misc = nullptr;          // [0] rounds, [1..16] cycles, [17] device status

    // host chain state
    std::vector<int32_t> group;
    std::vector<double> ystd;
    double mu = 0.0, sigmaE = 0.0, epsSum = 0.0;
    double sigmaG[BRR_MAX_GROUPS] = {};
    double pi[BRR_MAX_GROUPS * BRR_MAX_K] = {};
    uint32_t iteration = 0;
    int64_t sweeps = 0;

    // timing
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    double last_sweep_ms = 0.0, last_total_ms = 0.0;
    int64_t last_rounds = 0;
    long long phase[16] = {};   // summed over the sweeps of the last call
    bool profile = false;       // phase counters on (brr_set_profiling)
    bool timeline = false;      // and the per-CTA event timeline of the blocked sweep
    unsigned long long *d_tline = nullptr;
    uint64_t wait_limit_ns = 2000000000ull;
    int phantom = 0;

    // permutation prepared one iteration ahead on a host thread
    std::future<void> perm_future;
    std::vector<uint32_t> perm_next;
    uint32_t perm_next_it = UINT32_MAX;

    brr::StreamKey key() const { return brr::StreamKey{cfg.seed, cfg.chain}; }
};

namespace brr {

constexpr size_t kAccWords = 8 * 8 * kMaxSpec * 4;
constexpr size_t kCounterWords = 2 * 8 * 16;
// The restart sweep's accumulators take the first 3 x kMaxSpec x 4 words; the
// pair terms of pair-resolved rounds (3 x 2048 words) follow.
constexpr size_t kPairOffset = 4096;
static_assert(kPairOffset + 3 * 2048 <= kAccWords, "pair terms must fit the accumulator block");
constexpr int kPartBlocks = 608;   // 4 x 152 SMs for the updateMu reduction

// Phases of one iteration of a chain (BayesRBase::runGibbs loop body,
// src/BayesRBase.cpp:186-247), as brr_iterate runs them:
//   iter_pre      FP64 refresh when due, updateMu, per-marker draws, permutation
//                 (= iter_pre_dev, synchronise, iter_pre_host, iter_enqueue_draws)
//   sweep_prepare sampler constants, records in sweep order, sweep arguments
//                 (= sweep_stage, sweep_enqueue_inputs, sweep_args)
//   (the sweep kernel launch)
//   sweep_finish  sweep statistics, residual sums, device status
//                 (= sweep_enqueue_outputs, synchronise, sweep_collect)
//   iter_post     sigmaE, sigmaG and pi draws, next iteration
// The enqueue steps do device work only, from and to pinned staging, on the
// given stream, so that the multi-instance driver can capture them in a graph.
int iter_pre(brr_ctx &c, uint32_t it, double &mu_new, double &eps_total);
int iter_pre_dev(brr_ctx &c, uint32_t it);
int iter_pre_host(brr_ctx &c, uint32_t it, double &mu_new, double &eps_total);
int iter_enqueue_draws(brr_ctx &c, uint32_t it, cudaStream_t st);
int sweep_prepare(brr_ctx *c, double mu_new, double eps_total, SweepArgs &a, size_t &smem);
void sweep_stage(brr_ctx *c);
int sweep_enqueue_inputs(brr_ctx *c, double eps_total, cudaStream_t st);
void sweep_args(brr_ctx *c, double mu_new, double eps_total, SweepArgs &a, size_t &smem);
int sweep_finish(brr_ctx *c, brr_sweep_out *out);
int sweep_enqueue_outputs(brr_ctx *c, cudaStream_t st);
int sweep_collect(brr_ctx *c, brr_sweep_out *out);
int iter_post(brr_ctx &c, const brr_sweep_out &so, uint32_t it);
// New slicing (G CTAs) and, if B > 0, round width of a packed chain.
int reslice(brr_ctx *c, int G, int B);

}  // namespace brr
