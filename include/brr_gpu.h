/*
 * libbrr_gpu.so — C ABI of the GB300 (sm_103a) BayesR Gibbs-sweep path.
 *
 * One context = one Markov chain on one GPU.  Calls on a context are not
 * re-entrant; every function returns an int status (BRR_OK = 0, negative on
 * error) and brr_last_error() returns a message for the calling thread.
 * No C++ exception crosses this boundary and no torch type appears in it.
 *
 * Reference interfaces replaced (paths inside the BayesRRcmd project):
 *   brr_pack_bed          PreprocessGraph::preprocessBedFile + the per-genotype
 *                         MarkerBuilder::initialise/processAllele/endColumn/build
 *                         calls (src/preprocessgraph.cpp:10-73, :152-244;
 *                         src/markerbuilder.h:11-42;
 *                         src/densemarkerbuilder.cpp:6-60;
 *                         src/raggedsparsemarkerbuilder.cpp:5-55)
 *   brr_get_marker_table  the per-marker statistics of the built Marker objects
 *                         (DenseMarker::Cx values; SparseMarker mean/sd/sqrdZ/Zsum,
 *                         src/densemarker.h:7-20, src/sparsemarker.h:6-18)
 *   brr_get_ragged_lists  RaggedSparseMarker::Zones/Ztwos/Zmissing
 *                         (src/raggedsparsemarker.h:7-23); for the Eigen kind the
 *                         entries of EigenSparseMarker::Zg by value
 *                         (src/eigensparsemarker.h:6-16)
 *   brr_set_phenotype     Data::readPhenotypeFile result + BayesRBase::init's
 *                         standardisation (src/data.cpp:334-365,
 *                         src/BayesRBase.cpp:85-90)
 *   brr_set_groups        Data::readGroupFile result (src/data.cpp:424-453)
 *   brr_init_chain        BayesRBase::init (src/BayesRBase.cpp:39-99)
 *   brr_iterate           one pass of the BayesRBase::runGibbs chain loop body
 *                         (src/BayesRBase.cpp:186-247), i.e. updateMu,
 *                         prepareForAnylsis, the shuffle, AnalysisGraph::exec
 *                         (-> BayesRBase::processColumn -> BayesRKernel::computeNum /
 *                         calculateEpsilonChange for every marker) and the
 *                         sigmaE / sigmaG / pi draws
 *   brr_sweep             AnalysisGraph::exec(analysis, N, M, markerIndices)
 *                         alone (src/analysisgraph.hpp:18-21,
 *                         src/sequential.cpp:10-27, src/limitsequencegraph.cpp:79-106)
 *                         with caller-supplied per-marker draws
 *   brr_get_state /       the BayesRBase members written to the sample file
 *   brr_set_state         (src/BayesRBase.hpp:63-96, src/BayesRBase.cpp:251)
 *   brr_ctx_create /      construction of the analysis from Data and Options
 *   brr_ctx_destroy       (src/BayesRBase.cpp:18, src/DenseBayesRRmz.cpp:13,
 *                         src/SparseBayesRRG.cpp:8; the option fields used are
 *                         those of src/options.hpp:21-105)
 *   brr_pack_bed_device   brr_pack_bed with the payload already on the device
 *   brr_get_timing        the per-iteration and flow-graph durations runGibbs
 *                         measures and prints (src/BayesRBase.cpp:178-184,
 *                         :208-210, :257-260, :277-282)
 *   brr_refresh_eps       no counterpart: the FP64 residual refresh of the
 *                         FP32-compensated form (the reference keeps eps in FP64)
 *   brr_xbeta             no counterpart: genetic values X b of the packed
 *                         markers, for simulating phenotypes and for prediction
 *   brr_synth_bed_device* no counterpart: seeded synthetic BED payloads on the
 *                         device, a data source for benchmarks
 *   brr_set_wait_limit,   no counterpart: limits of the device-side waits, the
 *   brr_get_gram_info,    marker Gram of the blocked sweep, and phase counters
 *   brr_get_gram_entries,
 *   brr_get_round_info,
 *   brr_get_gram_bits,
 *   brr_get_phase_cycles, (the device counterpart of the timing log above)
 *   brr_set_profiling
 *   brr_batch_*,          no single counterpart: each chain (instance) is
 *   brr_multi_*           BayesRBase::runGibbs (src/BayesRBase.cpp:186-274) on its
 *                         own phenotype and seed; the reference runs them as
 *                         separate processes
 */
#ifndef BRR_GPU_H
#define BRR_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BRR_OK 0
#define BRR_ERR_ARG -1       /* invalid argument or call order */
#define BRR_ERR_CUDA -2      /* CUDA runtime error */
#define BRR_ERR_OOM -3       /* device or host allocation failed */
#define BRR_ERR_TIMEOUT -4   /* a device-side wait exceeded its limit */
#define BRR_ERR_MARKER -5    /* a marker does not vary or is all missing */
#define BRR_ERR_RANGE -6     /* a device value left the exchange range */
#define BRR_ERR_STREAM -7    /* a gamma draw exceeded its attempt cap */
#define BRR_ERR_DEVICE -8    /* no usable sm_103 device */

#define BRR_KIND_DENSE 0     /* 2-bit packed genotypes, standardised on the fly */
#define BRR_KIND_RAGGED 1    /* index lists of ones / twos / missing */
#define BRR_KIND_EIGEN 2     /* the same index lists with the Eigen sparse marker's
                              * statistics: missing genotypes imputed at the mean in
                              * sqrdZ, Zsum, sd and the dot product
                              * (src/eigensparsemarkerbuilder.cpp:40-75,
                              * src/eigenbayesrkernel.cpp:10-20) */

#define BRR_FORM_FP64 0      /* plain FP64 sweep: the drop-in */
#define BRR_FORM_FP32C 1     /* FP32 compensated dots and residual, FP64 refresh */

#define BRR_MAX_GROUPS 64
#define BRR_MAX_K 16

typedef struct brr_config {
    int64_t N;                 /* individuals */
    int64_t M;                 /* markers */
    int32_t kind;              /* BRR_KIND_* */
    int32_t form;              /* BRR_FORM_* */
    int32_t n_groups;          /* marker groups (>= 1) */
    int32_t K[BRR_MAX_GROUPS]; /* mixture components per group, incl. the zero component */
    double S[BRR_MAX_GROUPS * (BRR_MAX_K - 1)]; /* S[g*(BRR_MAX_K-1)+k]: variance ratios */
    uint32_t seed;
    uint32_t chain;
    double v0E, s02E, v0G, s02G;   /* priors (reference defaults 1e-4) */
    int32_t refresh_every;     /* FP32C: FP64 residual refresh every this many sweeps (0: never) */
    int32_t spec_width;        /* markers resolved per grid round (0: form default) */
    int32_t grid;              /* CTAs of the persistent sweep (0: one per SM) */
    int32_t device;            /* CUDA device ordinal */
    int32_t gram;              /* FP32C dense: 0 blocked sweep with a precomputed marker Gram when it fits
                                  in device memory, -1 never, 1 required */
    int32_t async_batch;       /* 0: the synchronous sweep (ppbayes); T in 1..64: the asyncppbayes
                                  schedule of the reference's ParallelGraph with T analysis tokens
                                  (src/parallelgraph.cpp:51-150): the T markers of a batch all read
                                  the residual before any of them updates it, acum is not written
                                  (src/BayesRBase.cpp:394-524); FP64 form only */
    int32_t cluster;           /* 0: the restart sweep exchanges its partial sums through L2 across `grid`
                                  CTAs with a grid-wide barrier; C in 2..16: the restart sweep runs as
                                  one thread-block cluster of C CTAs, each holding its slice of the
                                  residual in shared memory and storing its partial sums into every
                                  CTA's shared memory (no Gram-blocked form; gram must not be 1) */
    int32_t pair_rounds;       /* FP32C restart sweep (ragged markers other than Eigen, and dense markers
                                  without the Gram-blocked sweep): rounds of up to 32 markers resolved
                                  whole with exact integer pair terms of the round's markers.  0: ragged
                                  markers in the first sweep and after any sweep that leaves more than
                                  M/40 non-zero effects, dense markers never; 1: in every sweep;
                                  -1: never */
} brr_config;

/* Chain state; arrays are caller-owned, sized M (beta, comp, acum) and N (eps).
 * sigmaG[g] and pi[g*BRR_MAX_K+k] are filled for g < n_groups, k < K[g]. */
typedef struct brr_state {
    double *beta;
    int32_t *comp;
    double *acum;
    double *eps;
    double mu;
    double sigmaE;
    double epsSum;             /* ragged kind: the running residual sum */
    double sigmaG[BRR_MAX_GROUPS];
    double pi[BRR_MAX_GROUPS * BRR_MAX_K];
    uint32_t iteration;        /* next iteration index */
} brr_state;

/* Per-sweep statistics returned by brr_sweep (src/BayesRBase.cpp:200-202, :238). */
typedef struct brr_sweep_out {
    double v[BRR_MAX_GROUPS * BRR_MAX_K];  /* component counts */
    double betasqnG[BRR_MAX_GROUPS];       /* sum of squared non-zero betas */
    double eps_sqnorm;                     /* ||eps||^2 after the sweep */
    double eps_sum;                        /* sum(eps) after the sweep */
    int64_t rounds;                        /* grid rounds used by the sweep */
} brr_sweep_out;

typedef struct brr_ctx brr_ctx;

const char *brr_last_error(void);

int brr_ctx_create(const brr_config *cfg, brr_ctx **out);
int brr_ctx_destroy(brr_ctx *ctx);

/* Pack a PLINK SNP-major BED payload (M columns of ceil(N/4) bytes, the 3-byte
 * magic header already removed) from host memory; the decode, genotype counts,
 * standardisation or ragged index lists all run on the device. */
int brr_pack_bed(brr_ctx *ctx, const uint8_t *bed, int64_t nbytes);
/* Same, from a device pointer: device or managed memory of the context's GPU
 * with nbytes to the end of its allocation, else BRR_ERR_ARG before any launch. */
int brr_pack_bed_device(brr_ctx *ctx, const uint8_t *d_bed, int64_t nbytes);

/* Per-marker table, M x 4 doubles.  Dense: the standardised value of each
 * 2-bit code {0: g=2, 1: missing, 2: g=1, 3: g=0}.  Ragged and Eigen: {mean,
 * sd, sqrdZ, Zsum} (Eigen: sqrdZ, Zsum and sd include the imputed missing values).  counts (optional): M x 4 int64 {n0, n1, n2, nmissing}. */
int brr_get_marker_table(brr_ctx *ctx, double *table, int64_t *counts);
/* Ragged (and Eigen) index lists in ascending individual order.  off_*: M+1 offsets;
 * ones/twos/miss sized from the counts. */
int brr_get_ragged_lists(brr_ctx *ctx, int64_t *off_ones, int32_t *ones,
                         int64_t *off_twos, int32_t *twos,
                         int64_t *off_miss, int32_t *miss);

int brr_set_groups(brr_ctx *ctx, const int32_t *group);      /* M ids in 0..n_groups-1 */
int brr_set_phenotype(brr_ctx *ctx, const float *y);         /* N values */
int brr_init_chain(brr_ctx *ctx);

/* Run n_iter iterations of the chain. */
int brr_iterate(brr_ctx *ctx, int32_t n_iter);

/* One sweep over `order` (M marker ids) with per-marker draws u, z (indexed by
 * marker id), using the context's current mu/sigmaE/sigmaG/pi.  Host arrays. */
int brr_sweep(brr_ctx *ctx, const uint32_t *order, const double *u, const double *z,
              brr_sweep_out *out);

int brr_get_state(brr_ctx *ctx, brr_state *st);
int brr_set_state(brr_ctx *ctx, const brr_state *st);

/* FP64 residual refresh eps = y - mu - X beta (the FP32C form also runs it
 * every refresh_every sweeps). */
int brr_refresh_eps(brr_ctx *ctx);

/* Device time of the last brr_iterate / brr_sweep call, split into the sweep
 * kernels and everything else, in milliseconds; rounds = grid rounds. */
int brr_get_timing(brr_ctx *ctx, double *sweep_ms, double *total_ms, int64_t *rounds);

/* Genetic values out[i] = sum_q b[q] * x[i, idx[q]] of the packed, standardised
 * markers (dense: the DenseMarker column; ragged: the column its residual
 * update uses, missing = 0).  out: N doubles on the host.  Used to simulate
 * phenotypes and to predict from posterior-mean effects. */
int brr_xbeta(brr_ctx *ctx, const uint32_t *idx, const double *b, int64_t n, double *out);

/* Seeded synthetic genotypes written as a BED payload (M x ceil(N/4) bytes,
 * no header) into a device buffer: allele frequency of marker j uniform in
 * [p_lo, p_hi], genotypes Binomial(2, p_j), missing at rate `missing`.  A data
 * source for benchmarks at sizes where host generation is too slow.  d_bed must
 * be device or managed memory of the current GPU with M x ceil(N/4) bytes to the
 * end of its allocation, else BRR_ERR_ARG before any launch. */
int brr_synth_bed_device(uint8_t *d_bed, int64_t N, int64_t M, uint32_t seed, double p_lo, double p_hi,
                         double missing);
/* The same with allele frequencies p_j ~ Beta(a, b) clipped to [p_lo, p_hi]. */
int brr_synth_bed_device_beta(uint8_t *d_bed, int64_t N, int64_t M, uint32_t seed, double a, double b, double p_lo,
                              double p_hi, double missing);

/* Allocation-free genetic values.  No counterpart in the reference: it serves
 * callers that cannot allocate device memory when they need the values (a
 * host runtime that owns the whole GPU through its own pool and forbids
 * further cudaMalloc, a serving loop that must not block on the allocator or
 * synchronise the device).  Computes the same d_out[i] = sum_q b[q] *
 * x[i, idx[q]] as brr_xbeta, but into a caller-owned device buffer of N
 * doubles, with idx/b (host arrays) staged in a fixed static device array
 * of BRR_NOALLOC_MAX_TERMS terms; n above that limit is rejected with
 * BRR_ERR_ARG.  Calls no cudaMalloc/cudaFree.  d_out is checked before any
 * launch, without allocating: it must be device or managed memory of the
 * context's GPU, 8-byte aligned, with N doubles to the end of its allocation;
 * otherwise BRR_ERR_ARG.  The first call on a device (and in each new CUDA
 * context) looks up the array's device address, so make it before any stream
 * capture.  Every call is synchronous on the context's stream: it returns
 * once d_out is written.  Calls that overlap on the GPU share the array and
 * race. */
#define BRR_NOALLOC_MAX_TERMS 65536
int brr_xbeta_noalloc(brr_ctx *ctx, const uint32_t *idx, const double *b, int64_t n, double *d_out);

/* Limit of every device-side wait of the sweep (default 2 s); a wait that
 * runs out makes the call return BRR_ERR_TIMEOUT and leaves the context
 * usable (re-initialise or set the state before continuing).
 * phantom_arrivals > 0 makes the grid barrier wait for that many CTAs more
 * than exist, so that tests can exercise the timeout path without a fault. */
int brr_set_wait_limit(brr_ctx *ctx, uint64_t timeout_ns, int32_t phantom_arrivals);

/* Whether the chain runs the Gram-blocked FP32C dense sweep, the device time of
 * building the packed marker Gram (ms: decode, GEMMs and combine, without the
 * allocations and the library's initialisation) and its size in bytes. */
int brr_get_gram_info(brr_ctx *ctx, int32_t *blocked, double *build_ms, int64_t *bytes);

/* Element bits of the GEMM operands the marker Gram was built from: 4 (FP4
 * E2M1), 8 (FP8 E4M3) or 16 (BF16); 0 without a Gram. */
int brr_get_gram_bits(brr_ctx *ctx, int32_t *bits);

/* Whether the chain can take pair-resolved rounds, and whether its last sweep
 * took them. */
int brr_get_round_info(brr_ctx *ctx, int32_t *pair_rounds, int32_t *last_sweep_pair_rounds);

/* Entries G[j[i], k[i]] = x_j . x_k (j > k) of the marker Gram of a blocked
 * chain, for i < n, into out (a check of the build; one copy per entry). */
int brr_get_gram_entries(brr_ctx *ctx, const int64_t *j, const int64_t *k, int64_t n, double *out);

/* ---- Batched chains on shared genotypes (the C4 batching form) -------------
 * C = 32 or 64 chains with distinct seeds (chain ids cfg.chain .. cfg.chain+C-1)
 * and one phenotype each sweep the same dense markers in one shared order per
 * iteration (the permutation of chain cfg.chain's stream); per chain the
 * iteration is BayesRBase::runGibbs's loop body (src/BayesRBase.cpp:186-247).
 * The dot products X_block^T E and the residual updates run on the tensor
 * cores with each residual held exactly as fixed point eps * 2^40 (|eps| < 8);
 * markers with missing genotypes are rejected.  Sizes: N up to about
 * 152 x 336 individuals for 64 chains, 152 x 660 for 32. */
typedef struct brr_batch brr_batch;
int brr_batch_create(const brr_config *cfg, int32_t chains, brr_batch **out);
int brr_batch_destroy(brr_batch *b);
int brr_batch_pack_bed(brr_batch *b, const uint8_t *bed, int64_t nbytes);
/* d_bed: device or managed memory of the batch's GPU with nbytes to the end of
 * its allocation, else BRR_ERR_ARG before any launch. */
int brr_batch_pack_bed_device(brr_batch *b, const uint8_t *d_bed, int64_t nbytes);
int brr_batch_set_groups(brr_batch *b, const int32_t *group);
/* chains x N phenotype values, chain-major */
int brr_batch_set_phenotypes(brr_batch *b, const float *y);
int brr_batch_init(brr_batch *b);
int brr_batch_iterate(brr_batch *b, int32_t n_iter);
/* One chain's state; eps is the exact fixed-point residual as doubles. */
int brr_batch_get_chain_state(brr_batch *b, int32_t chain, brr_state *st);
/* Device time of the sweeps and of the whole last brr_batch_iterate call (ms);
 * cycles (optional, 8 values), summed over the sweeps of that call, measured on
 * CTA 0 (indicative): the dot, publish, resolve and update phases; then, of
 * the resolve phase, the wait for all CTAs' dot products, chain 0's own
 * resolve, chain 0's sampling steps, and the wait for the slowest chain. */
int brr_batch_get_timing(brr_batch *b, double *sweep_ms, double *total_ms, int64_t *cycles);
/* Phase counters on (1) or off (0, the default; the cycles then read zero):
 * the counting runs a variant of the sweep kernel with clock reads. */
int brr_batch_set_profiling(brr_batch *b, int32_t on);
/* Limit of every device-side wait of the batched sweep (default 2 s);
 * phantom_arrivals > 0 makes the barrier before the resolve wait for that many
 * CTAs more than exist (tests of the timeout path).  A wait that runs out
 * makes brr_batch_iterate return BRR_ERR_TIMEOUT; brr_batch_init then starts
 * the chains again. */
int brr_batch_set_wait_limit(brr_batch *b, uint64_t timeout_ns, int32_t phantom_arrivals);
/* CTAs of the sweep, individuals per slice and shared memory per CTA. */
int brr_batch_get_geometry(brr_batch *b, int32_t *ctas, int32_t *slice, int64_t *smem_bytes);

/* ---- Uneven batch: independent regressions of different sizes (C5 form) ----
 * Up to 32 instances, each with its own configuration (N, M, kind, groups, S,
 * seed, chain) but one sweep form and device, swept together: per iteration
 * one CUDA graph holds every instance's draws, records and statistics and one
 * cooperative launch that runs every instance's sweep on its own group of CTAs.
 * Per instance the chain is the single-chain one (the same draws and results
 * as brr_iterate up to the order of floating-point sums).  brr_multi_tune runs
 * 3 + rounds real iterations to choose each instance's round width and CTAs. */
typedef struct brr_multi brr_multi;
int brr_multi_create(const brr_config *cfgs, int32_t n, brr_multi **out);
int brr_multi_destroy(brr_multi *m);
int brr_multi_pack_bed(brr_multi *m, int32_t i, const uint8_t *bed, int64_t nbytes);
int brr_multi_pack_bed_device(brr_multi *m, int32_t i, const uint8_t *d_bed, int64_t nbytes);
int brr_multi_set_groups(brr_multi *m, int32_t i, const int32_t *group);
int brr_multi_set_phenotype(brr_multi *m, int32_t i, const float *y);
int brr_multi_init(brr_multi *m);
int brr_multi_tune(brr_multi *m, int32_t rounds);
int brr_multi_iterate(brr_multi *m, int32_t n_iter);
int brr_multi_get_state(brr_multi *m, int32_t i, brr_state *st);
/* Limit of every device-side wait of instance i's sweep (i < 0: every
 * instance; default 2 s); phantom_arrivals > 0 makes its grid barrier wait for
 * that many CTAs more than it has (tests of the timeout path).  A wait that
 * runs out makes brr_multi_iterate return BRR_ERR_TIMEOUT; brr_multi_init then
 * starts every instance again. */
int brr_multi_set_wait_limit(brr_multi *m, int32_t i, uint64_t timeout_ns, int32_t phantom_arrivals);
/* Device time of the iteration graphs and wall time of the last
 * brr_multi_iterate call (ms); per instance (optional, n values each): CTAs,
 * round width and the last sweep's time (ms). */
int brr_multi_get_timing(brr_multi *m, double *sweep_ms, double *total_ms, int32_t *ctas, int32_t *width,
                         double *inst_ms);

/* Per-phase SM cycles of the sweeps of the last brr_iterate / brr_sweep call,
 * measured on the first CTA (the counterpart of the reference's per-column
 * timing log, src/BayesRBase.cpp:381-389), 16 values.  Restart sweep: [0] ring
 * prefetch and wait, [1] partial dot products, [2] grid barrier, [3]
 * component sampling, [4] outputs and residual update, [5] grid rounds.
 * Gram-blocked sweep: [0] ring wait and waiting for the other warps, [1] dot
 * products of the next block and their publication, [2] waiting for the grid
 * barrier, [3] sampling, [4] residual update, [5] blocks, [6] sampling steps,
 * [7] block inputs on the sampling warp (corrections of the previous block,
 * Gram copy wait), [8] samples the FP32 sampler handed to FP64, [9] cycles of
 * [3] in component picks, [10] cycles of [3] resolving steps, [11] assembling
 * the next block's inputs, [12]-[15] cycles from each iteration's start to the
 * end of the work of the dot warps, the Gram warp, the sampling warp and the
 * input warp.  The
 * per-thread clock is read around long code regions, so the values are
 * indicative. */
int brr_get_phase_cycles(brr_ctx *ctx, int64_t *cycles);
/* Phase counters on (1) or off (0, the default).  The counting runs a variant
 * of the Gram-blocked sweep that reads the SM clock on the first CTA; the
 * clock reads constrain the scheduling of the sweep's sampling chain, so timed
 * runs leave the counters off and brr_get_phase_cycles returns zeros. */
int brr_set_profiling(brr_ctx *ctx, int32_t on);
/* on = 2: the counters of on = 1 and, in the Gram-blocked sweep, a per-CTA
 * event timeline of 64 iterations around the sweep's middle (global timer,
 * ns): events[(it * ctas + cta) * 16 + e] for e = 0 the iteration's start on
 * the warps other than the sampling warp, 1 the grid-barrier arrival of the
 * dot products, 2 the input warp past the barrier, 3 the next block's inputs
 * ready, 4 the Gram warp's staging done, 5 the Gram warp's work done, 6 and 7
 * the start and end of the block's sampling, 8 the residual update done, 9 the
 * dot products done, 10 the far corrections done, 11 the Gram loads issued,
 * 12-15 the residual update's terms computed, first barrier, slice updated,
 * second barrier.  capacity: values available (64 x ctas x 16).  Diagnostics
 * of the pipeline's critical path. */
int brr_get_sweep_timeline(brr_ctx *ctx, uint64_t *events, int64_t capacity, int32_t *iterations, int32_t *ctas);

#ifdef __cplusplus
}
#endif
#endif
