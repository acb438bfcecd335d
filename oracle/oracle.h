/*
 * CPU oracle for the BayesR Gibbs-sweep path (TEST INFRASTRUCTURE ONLY).
 *
 * This library is a plain-C, FP64 restatement of the reference algorithm of
 * BayesRRcmd (BayesRPlus) for the `ppbayes` analysis on dense and
 * ragged-sparse markers, plus its preprocess (BED decode + marker builders).
 * It exists to check the CUDA product; only the test-suite, the smoke check
 * and the CPU-baseline leg of the benchmark may load it.  The product path
 * (libbrr_gpu.so) never links or calls it.
 *
 * Parity status: the reference itself cannot be compiled here (it needs
 * Eigen, Boost.Random and TBB, none of which are installed), so the chain
 * outputs of this oracle are NOT pinned against reference runs.  What is
 * pinned (see tests/test_oracle_pins.py):
 *   - BED decode + per-marker allele counting against the GeneFrq column that
 *     the reference ships for its uk10k test fixture (test.zip test/res);
 *   - the `--S` parsing cases of test/optionstest.cpp;
 *   - the sparse epsilon-update identity of test/eigenSparseTest.cpp:69-81;
 *   - the sample-file row count 1 + ceil(chain/thin) of
 *     test/ppbayestest.cpp:138-149.
 * Summation orders that the reference leaves to Eigen (vector sums, dot
 * products, squared norms) are restated as left-to-right loops; the random
 * stream (Boost mt19937 in the reference) is replaced by the counter-based
 * Philox4x32-10 draw stream defined below, which both the oracle and the GPU
 * product replay.
 */
#ifndef BRR_ORACLE_H
#define BRR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAX_GROUPS 64
#define OR_MAX_K 16
#define OR_MAX_ASYNC 64     /* largest asyncppbayes batch (markers in flight) */

/* Marker storage kinds (reference: src/common.h:27-32 PreprocessDataType). */
#define OR_KIND_DENSE 0
#define OR_KIND_RAGGED 1
#define OR_KIND_EIGEN 2   /* ragged lists with mean-imputed statistics and dot (src/common.h:30) */

/* Status codes. */
#define OR_OK 0
#define OR_ERR_ARG -1
#define OR_ERR_MARKER -2   /* a marker that does not vary (sd == 0) or is all missing */
#define OR_ERR_STREAM -3   /* gamma sampler exceeded its attempt cap */

/* ---------------- draw stream (Philox4x32-10, Salmon et al., SC'11) ---------------- */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double or_u53(uint32_t a, uint32_t b);
/* marker j's (u, z) pair at iteration it (reference: src/BayesRBase.cpp:101-110) */
void or_marker_draws(uint32_t seed, uint32_t chain, uint32_t it, uint32_t j, double *u, double *z);
/* Fisher-Yates permutation of 0..M-1 for iteration it (reference: src/BayesRBase.cpp:198) */
void or_permutation(uint32_t seed, uint32_t chain, uint32_t it, uint32_t M, uint32_t *perm);
/* Gamma(shape, 1) from stream (it, purpose, sub); returns OR_ERR_STREAM on attempt cap */
int or_gamma(uint32_t seed, uint32_t chain, uint32_t it, uint32_t purpose, uint32_t sub,
             double shape, double *out);

/* ---------------- preprocess ---------------- */
/* BED decode (reference: src/preprocessgraph.cpp:43-56).  bed is SNP-major,
 * WITHOUT the 3-byte magic header; M columns of ceil(N/4) bytes.  Output g is
 * M x N int8 with values 0,1,2 and -1 for missing. */
int or_decode_bed(const uint8_t *bed, int64_t N, int64_t M, int8_t *g);
/* Per-marker genotype counts n0,n1,n2,nmiss (out: M x 4 int64). */
int or_marker_counts(const uint8_t *bed, int64_t N, int64_t M, int64_t *counts);
/* Dense standardized value table per marker, indexed by the 2-bit BED code
 * (reference: src/densemarkerbuilder.cpp:23-60).  out: M x 4 doubles. */
int or_dense_lut(const uint8_t *bed, int64_t N, int64_t M, double *lut);
/* Dense standardized columns (M x N doubles, the reference .ppbed payload). */
int or_dense_columns(const uint8_t *bed, int64_t N, int64_t M, double *x);
/* Ragged marker statistics (reference: src/raggedsparsemarkerbuilder.cpp:25-55,
 * src/sparsemarker.cpp:8-19).  stats: M x 4 doubles {mean, sd, sqrdZ, Zsum}. */
int or_ragged_stats(const uint8_t *bed, int64_t N, int64_t M, double *stats);
/* Eigen sparse marker statistics (reference: src/eigensparsemarkerbuilder.cpp:40-56):
 * as above with the missing genotypes imputed at the mean in sqrdZ and Zsum,
 * and the sd formed from those. */
int or_eigen_stats(const uint8_t *bed, int64_t N, int64_t M, double *stats);
/* Ragged index lists.  off: M+1 offsets per list kind (3 x (M+1), kinds
 * ones, twos, missing); idx: concatenated int32 indices for each kind, sized by
 * the caller from or_marker_counts (3 buffers). */
int or_ragged_lists(const uint8_t *bed, int64_t N, int64_t M,
                    int64_t *off_ones, int32_t *ones,
                    int64_t *off_twos, int32_t *twos,
                    int64_t *off_miss, int32_t *miss);

/* ---------------- chain ---------------- */
typedef struct {
    int64_t N, M;
    int32_t kind;                /* OR_KIND_DENSE, OR_KIND_RAGGED or OR_KIND_EIGEN */
    int32_t n_groups;
    const int32_t *group;        /* M group ids in 0..n_groups-1 */
    const int32_t *K;            /* n_groups: mixture components incl. the zero one */
    const double *S;             /* n_groups x (OR_MAX_K-1): S[g*(OR_MAX_K-1)+k] */
    const float *y;              /* N phenotype values (single precision, as read) */
    const uint8_t *bed;          /* M x ceil(N/4) SNP-major BED payload */
    uint32_t seed, chain;
    double v0E, s02E, v0G, s02G;
    /* batched chains: when shared_perm != 0 the sweep order of every
     * iteration is the permutation of chain perm_chain's stream */
    int32_t shared_perm;
    uint32_t perm_chain;
    /* dense markers: 0 stores the standardized columns (M x N doubles, as the
     * reference's DenseMarker does); 1 keeps the four standardized values per
     * marker and reads the codes from `bed` (which must outlive the markers),
     * for problems whose columns do not fit in host memory.  Both read the
     * same value for every genotype, in the same order: identical results. */
    int32_t dense_lut;
    /* 0: the synchronous sweep (ppbayes); T > 0: the asyncppbayes schedule with
     * T markers in flight (at most OR_MAX_ASYNC) */
    int32_t async_batch;
} or_problem;

typedef struct {
    double *beta;                /* M */
    int32_t *comp;               /* M */
    double *acum;                /* M */
    double *eps;                 /* N */
    double mu, sigmaE, epsSum;
    double sigmaG[OR_MAX_GROUPS];
    double pi[OR_MAX_GROUPS * OR_MAX_K];
    /* per-iteration sweep statistics */
    double v[OR_MAX_GROUPS * OR_MAX_K];
    double betasqnG[OR_MAX_GROUPS];
    double m0;
} or_state;

typedef struct or_markers or_markers;
/* Build the marker store for the problem (dense columns or ragged lists). */
int or_markers_create(const or_problem *p, or_markers **out);
void or_markers_destroy(or_markers *m);
/* Initialise state (reference: src/BayesRBase.cpp:39-99).  State buffers are
 * owned by the caller. */
int or_init(const or_problem *p, or_state *s);
/* One Gibbs iteration `it` (reference: src/BayesRBase.cpp:186-247). */
int or_iterate(const or_problem *p, const or_markers *mk, or_state *s, uint32_t it);
/* Only the sweep over markers in `order` with per-marker draws (u, z) indexed
 * by marker id (reference: analysis->exec + processColumn). */
int or_sweep(const or_problem *p, const or_markers *mk, or_state *s,
             const uint32_t *order, const double *u, const double *z);

#ifdef __cplusplus
}
#endif
#endif
