// Internal declarations shared by the translation units of libbrr_gpu.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/brr_gpu.h"

namespace brr {

// One record per sweep position, gathered before each sweep so that the
// persistent kernel streams them contiguously.  t[] holds the marker table
// in the layout the sweep form needs:
//   FP64 dense : standardised value per 2-bit code (4 doubles)
//   FP32C dense: {sigma, colmean, value of a missing genotype, column sum}
//   ragged     : {mean, sd, sqrdZ, Zsum}
struct alignas(16) SweepRec {
    double t[4];
    double beta_old;
    double u;
    double z;
    uint32_t j;
    int32_t group;
};
static_assert(sizeof(SweepRec) == 64, "SweepRec must be 64 bytes");

// Record of the Gram-blocked FP32C dense sweep.  FP64 arithmetic issues at a
// small fraction of the FP32 rate on this GPU, so every per-marker quantity the
// resolve and the residual update need is prepared here once per sweep, by a
// kernel over all markers, as a double-float pair (hi, lo):
//   num = sigma * sum(g*eps) + cst + dm * sum_missing(eps)
// with cst = beta_old*(N-1) - sigma*colmean*S and dm = sigma*colmean + xm
// (S: sum of the residual at the sweep start, xm: value of a missing genotype).
struct alignas(16) BlockRec {
    float x[8];          // standardised value per 2-bit code c at x[2c], x[2c+1]
    float sig[2];        // sigma
    float cst[2];        // constant part of num
    float dm[2];         // coefficient of the missing-genotype sum
    float bo[2];         // beta_old
    float zf[2];         // z
    float uf;            // u rounded to FP32 (certified sampler)
    uint32_t bnz;        // beta_old != 0
    double beta_old;     // FP64 draws for the sampler's FP64 fallback
    double u;
    double z;
    uint32_t j;
    int32_t group;
    uint32_t pad[4];
};
static_assert(sizeof(BlockRec) == 128, "BlockRec must be 128 bytes");

struct SweepArgs {
    int64_t N, M;
    int G;                       // CTAs (slices of individuals)
    int B;                       // markers resolved per grid round
    int n_groups;
    int kmax;                    // largest mixture size over the groups
    int slot_bytes;              // bytes of one ring slot (max slice code bytes)
    int slice_max;               // max individuals of a slice (multiple of 64)
    const int32_t *slice_lo;     // G+1 slice boundaries in individuals
    const uint8_t *codes;        // M x col_stride 2-bit codes
    int64_t col_stride;
    const int32_t *roff[3];      // ragged: (M*G+1) offsets of ones/twos/missing per (marker, slice)
    const uint16_t *ridx[3];     // ragged: slice-local indices
    const SweepRec *rec;         // M records in sweep order
    const double *gconst;        // [n_groups][kMaxK][4] {c, invden, h, sdk}
    const int32_t *gK;           // [n_groups]
    double *beta;
    int32_t *comp;
    double *acum;
    double *eps;                 // FP64 residual (FP64 form)
    float *eps_hi, *eps_lo;      // double-float residual (FP32C form)
    double mu_new;               // subtracted from eps while it is loaded (updateMu, second half)
    double epsSum;               // ragged running sum at sweep start (after updateMu)
    double eps_total;            // dense FP32C: sum of the residual at sweep start (after updateMu)
    unsigned long long *acc;     // [kAccBuffers][kMaxSpec][4] fixed-point accumulators (sum, missing sum)
    unsigned long long *counter; // grid round counter(s), zero at launch (blocked sweep: two)
    double *stats_out;           // [0]: ragged running sum at sweep end
    uint8_t *chosen;             // M flags: marker chose a component in this sweep
    double *part;                // [G][2] per-slice sum(eps), sum(eps^2) after the sweep
    int *err;                    // device status word
    long long *rounds_out;
    long long *prof;             // optional: cycles per round phase of CTA 0 (diagnostics), or null
    uint64_t timeout_ns;         // limit of any single wait
    int phantom;                 // extra arrivals the barrier waits for (tests of the timeout path)
    const float2 *gram;          // blocked FP32C sweep: packed lower-triangle marker Gram (double-float)
    double *gstage;              // blocked FP32C sweep: staged Gram entries (sweep_block_stage_bytes)
    int has_missing;             // any missing genotype in the packed markers
    const BlockRec *brec;        // blocked FP32C sweep: M records in sweep order
    const uint32_t *order;       // blocked FP32C sweep: the M marker ids in sweep order
    float2 *beta_df;             // blocked FP32C sweep: new beta per marker (hi, lo)
    float2 *acum_df;             // blocked FP32C sweep: acum per marker (hi, lo)
    int eigen;                   // ragged sweep: Eigen sparse markers (missing genotypes enter
                                 // the dot product at the marker's mean)
    unsigned long long *t_out;   // optional [2]: global timer (ns) at the start and end of the sweep (CTA 0)
    int async_batch;             // restart sweep: 0 synchronous; T > 0 asynchronous batches of T markers
    int cluster;                 // restart sweep: 0 grid-wide exchange; G: the G CTAs are one thread-block
                                 // cluster exchanging through distributed shared memory
    unsigned long long *pairs;   // pair-resolved ragged rounds: [3][32][32] integer pair terms of the
                                 // round's markers, A in the low and Bm in the high word (zero at
                                 // launch), else null
    unsigned long long *tline;   // blocked sweep, counting variant, optional: per-CTA event timeline
                                 // [kTimelineIters][G][kTimelineEvents] of global-timer stamps (ns)
};
// Event timeline of the counting variant of the blocked sweep: iterations
// nblk/2 - 32 .. nblk/2 + 31 (or all, fewer blocks), per CTA: 0 the others'
// iteration start, 1 the dot warps' grid-barrier arrival, 2 the input warp
// past the barrier, 3 the input warp's GO signal, 4 the chore warp's signal to
// the dot warps, 5 the chore warp's GO signal, 6 the resolve's start, 7 its end,
// 8 the dot warps' residual update done, 9 their dot products done, 10 the
// input warp's far corrections done, 11 the chore warp's Gram loads issued,
// 12-15 inside the residual update: the update terms computed, the dot warps
// synchronised, the residual slice updated, synchronised again.
constexpr int kTimelineIters = 64;
constexpr int kTimelineEvents = 16;

// ---------------------------------------------------------------------------
// Batched chains on shared genotypes (brr_batch.cu).
//
// C chains (distinct seeds and phenotypes) sweep the markers in one shared
// order, 32 markers per block.  Each chain's residual is held exactly in fixed
// point, E = eps * 2^kBatchFrac (int64), and on chip as kBatchLimbs balanced
// 11-bit limbs stored as FP16, so that the dot products X_block^T E and the
// rank-32 residual update are FP16 tensor-core GEMMs with FP32 accumulation
// whose every partial sum is an integer below 2^24, i.e. exact.
constexpr int kBatchFrac = 40;
constexpr int kBatchLimbs = 4;
constexpr int kBatchBlock = 32;          // markers per block
constexpr int kBatchMaxChains = 64;
constexpr int kBatchCopies = 8;          // copies of the dot accumulators (CTA s adds into s % 8)
constexpr int kBatchPCopies = 4;         // copies of the block Gram accumulators (CTA s adds into s % 4)

struct alignas(16) BatchRec {
    double sigma;        // 1 / sd of the marker column
    double colmean;      // column mean
    double S;            // sum of the genotypes over all individuals (exact integer)
    uint32_t j;          // marker id
    int32_t group;
};
static_assert(sizeof(BatchRec) == 32, "BatchRec must be 32 bytes");

// Per chain and sweep position: beta_old of the marker and its draws.
struct alignas(32) ChainRec {
    double beta_old;
    double u;
    double z;
    double pad;
};
static_assert(sizeof(ChainRec) == 32, "ChainRec must be 32 bytes");

struct BatchArgs {
    int64_t N, M;
    int G;                           // CTAs: slices of individuals
    int C;                           // chains (32 or 64)
    int kext;                        // individuals per slice, padded to a multiple of 16
    int n_groups;
    const int32_t *slice_lo;         // G+1 slice boundaries
    const uint8_t *codes;            // M x col_stride 2-bit codes
    int64_t col_stride;
    const BatchRec *rec;             // M records in sweep order
    const double *gconst;            // [C][n_groups][kMaxK][4] sampler constants per chain
    const float *gcf;                // [C][n_groups][kMaxK][2] FP32 {logL_k - logL_0 constant, h_k}
    const float4 *gdf;               // [C][n_groups][kMaxK] double-float {sdk hi, lo, invden hi, lo}
    const int32_t *gK;               // [n_groups] mixture sizes
    const ChainRec *crec;            // [C][M] in sweep order
    double *beta, *acum;             // [C][M] by marker id
    int32_t *comp;                   // [C][M]
    uint8_t *chosen;                 // [C][M] the sampler chose a component in this sweep
    long long *E;                    // [C][N] fixed-point residual (in at sweep start, out at the end)
    const long long *dmu;            // [C] fixed-point shift added to E at the start (updateMu)
    long long *sumE;                 // [C] exact residual total, carried through the sweep
    unsigned long long *acc;         // [kBatchCopies][C][32] dot-product accumulators (zero at launch)
    unsigned *pacc;                  // [2][kBatchPCopies][32][32] integer block Gram accumulators (zero at launch)
    long long *wx;                   // [C][33] per block: W per marker, then the constant
    unsigned long long *counter;     // 2 barrier counters, 32 words apart (zero at launch)
    double *part;                    // [G][C][2] per slice: sum(E) (bits of an int64) and sum(eps^2)
    int *err;
    uint64_t timeout_ns;
    int phantom;                     // extra arrivals the dot barrier waits for (tests of the timeout path)
    long long *prof;                 // optional [8] cycle counters of CTA 0
};

// Sets the string brr_last_error() returns and passes the status code through.
int api_fail(int code, const std::string &msg);

cudaError_t launch_batch_gather(const uint32_t *order, int64_t M, const double *scale, const int64_t *counts,
                                const int32_t *group, BatchRec *rec, cudaStream_t st);
// Per chain c and sweep position q: beta_old of marker order[q] and its draws
// (u, z) from chain (chain0 + c)'s stream for iteration it.
cudaError_t launch_batch_draws(uint32_t seed, uint32_t chain0, uint32_t it, int64_t M, int C, const uint32_t *order,
                               const double *beta, ChainRec *crec, cudaStream_t st);
cudaError_t launch_batch_stats(int64_t M, int C, const int32_t *group, const int32_t *comp, const uint8_t *chosen,
                               const double *beta, int n_groups, unsigned long long *out, cudaStream_t st);
size_t batch_smem_bytes(int C, int kext, int G);
int batch_max_ctas_per_sm(int C, int kext, size_t smem);
cudaError_t launch_sweep_batch(const BatchArgs &a, int kmax, cudaStream_t st);

// Several chains of different sizes in one cooperative launch (k_sweep_multi).
constexpr int kMaxInstances = 32;
struct MultiSweepArgs {
    int n;                               // instances
    int cta_start[kMaxInstances + 1];    // CTAs [cta_start[i], cta_start[i+1]) run instance i
    int kind[kMaxInstances];             // sweep kind of each instance (dense or ragged lists)
    SweepArgs inst[kMaxInstances];
};
int sweep_multi_max_ctas_per_sm(int form, int kmax, size_t smem);
size_t sweep_multi_static_smem(int form, int kmax);
cudaError_t launch_sweep_multi(int form, int kmax, const MultiSweepArgs &m, size_t smem, cudaStream_t st);

// Kernel launchers (defined in brr_pack.cu / brr_sweep.cu).
cudaError_t launch_pack_counts(const uint8_t *bed, int64_t N, int64_t M, uint8_t *codes,
                               int64_t col_stride, int64_t *counts, cudaStream_t st);
cudaError_t launch_dense_tables(const int64_t *counts, int64_t N, int64_t M, double *lut,
                                double *scale, double *colsum, int *bad, cudaStream_t st);
cudaError_t launch_ragged_stats(const int64_t *counts, int64_t N, int64_t M, int eigen, double *stats,
                                int *bad, cudaStream_t st);
cudaError_t launch_ragged_slice_counts(const uint8_t *codes, int64_t col_stride, int64_t M, int G,
                                       const int32_t *slice_lo, int32_t *cnt3, cudaStream_t st);
cudaError_t launch_exclusive_scan_i32(int32_t *data, int64_t n, int32_t *tmp, cudaStream_t st);
cudaError_t launch_ragged_fill(const uint8_t *codes, int64_t col_stride, int64_t M, int G,
                               const int32_t *slice_lo, const int32_t *off0, const int32_t *off1,
                               const int32_t *off2, uint16_t *idx0, uint16_t *idx1, uint16_t *idx2,
                               cudaStream_t st);
cudaError_t launch_draws(uint32_t seed, uint32_t chain, uint32_t it, int64_t M, double *u, double *z,
                         cudaStream_t st);
cudaError_t launch_gather(int form, int kind, const uint32_t *order, int64_t M, const double *table,
                          const double *scale, const double *beta, const double *u, const double *z,
                          const int32_t *group, const double *colsum, SweepRec *rec, cudaStream_t st);
cudaError_t launch_sweep_stats(int64_t M, const int32_t *group, const int32_t *comp, const uint8_t *chosen,
                               const double *beta, int n_groups, unsigned long long *out, cudaStream_t st);
cudaError_t launch_mu_prep(int form, int64_t N, double mu_old, double *eps, float *eps_hi,
                           float *eps_lo, double *part, int nblocks, cudaStream_t st);
cudaError_t launch_refresh(int form, int kind, int64_t N, const double *ystd, double mu,
                           const uint8_t *codes, int64_t col_stride, const double *table,
                           const uint32_t *nz_j, const double *nz_beta, int64_t n_nz, double *eps,
                           float *eps_hi, float *eps_lo, cudaStream_t st);
cudaError_t launch_synth_bed(uint8_t *out, int64_t N, int64_t M, uint32_t seed, double p_lo, double p_hi,
                             double miss, cudaStream_t st, double beta_a = 0.0, double beta_b = 0.0);
cudaError_t launch_sweep(int form, int kind, const SweepArgs &a, size_t smem, cudaStream_t st);
size_t sweep_smem_bytes(int form, int kind, const SweepArgs &a);
cudaError_t launch_df_to_double(int64_t N, const float *hi, const float *lo, double *out, cudaStream_t st);
cudaError_t noalloc_xbeta(cudaStream_t st, int kind, int64_t N, const uint8_t *codes, int64_t col_stride,
                          const double *table, const uint32_t *idx, const double *b, int64_t n, double *d_out,
                          std::string &why);
bool noalloc_check_output(int dev, const void *d_out, size_t bytes, std::string &why);
// Whether p is device or managed memory of device dev with `bytes` bytes to the
// end of its allocation (no allocation, no launch); the message names `name`.
bool device_range_check(int dev, const void *p, size_t bytes, const char *name, std::string &why);
int sweep_max_ctas_per_sm(int form, int kind, size_t smem, bool pair_rounds = false);
// Clusters of G CTAs of the cluster sweep that can be resident at once (0: none).
int sweep_cluster_fits(int form, int kind, int G, size_t smem);
size_t sweep_block_smem_bytes(const SweepArgs &a);
cudaError_t launch_gather_block(const uint32_t *order, int64_t M, int64_t N, const double *table,
                                const double *scale, const double *beta, const double *u, const double *z,
                                const int32_t *group, double eps_total, BlockRec *rec, cudaStream_t st);
cudaError_t launch_block_finish(int64_t M, const uint8_t *chosen, const float2 *beta_df, const float2 *acum_df,
                                double *beta, double *acum, cudaStream_t st);
cudaError_t launch_sweep_block(const SweepArgs &a, size_t smem, cudaStream_t st);
size_t sweep_block_stage_bytes(int B);   // global Gram staging of the blocked sweep
int sweep_block_threads();
int sweep_block_max_ctas_per_sm(size_t smem, std::string *why = nullptr);
cudaError_t gram_bytes_needed(int64_t N, int64_t M, bool missing, size_t *gram, size_t *work);
int build_gram(const uint8_t *codes, int64_t col_stride, int64_t N, int64_t M, const double *scale,
               const int64_t *counts, bool missing, float2 *G, cudaStream_t st, std::string &why,
               float *device_ms);
// Element bits of the last successful Gram build's GEMM operands (4, 8 or 16).
int gram_route_bits();

}  // namespace brr
